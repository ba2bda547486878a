"""Mesh boundaries: OBJ loading (CPU) and GPU sampling against the reference's own sampling
kernels (MPSParticleSamplingUtil.cuh, MPSMeshObject.cuh) run through the headless driver."""
import numpy as np
import pytest


def write_box_obj(path, n=3):
    """A closed box surface: each face an n x n grid of quads (split into triangles by the loader)."""
    verts, faces, index = [], [], {}

    def vid(p):
        key = tuple(round(c, 9) for c in p)
        if key not in index:
            index[key] = len(verts)
            verts.append(p)
        return index[key] + 1

    for axis in range(3):
        for side in (0.0, 1.0):
            u, v = [a for a in range(3) if a != axis]
            for i in range(n):
                for j in range(n):
                    quad = []
                    for di, dj in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        p = [0.0, 0.0, 0.0]
                        p[axis] = side
                        p[u] = (i + di) / n
                        p[v] = (j + dj) / n
                        quad.append(vid(tuple(p)))
                    faces.append(quad)
    with open(path, "w") as f:
        f.write("# box\n")
        for p in verts:
            f.write(f"v {p[0]} {p[1]} {p[2]}\n")
        for q in faces:
            f.write("f " + " ".join(f"{k}/{k}" for k in q) + "\n")
    return len(verts), len(faces)


def test_obj_loading_and_box_fit(mps, tmp_path):
    from mps_cuda_gb300 import scenes
    path = tmp_path / "box.obj"
    nv, nq = write_box_obj(path, n=2)
    V, F = scenes.load_obj(path)
    assert V.shape == (nv, 3) and F.shape == (2 * nq, 3)
    assert V.min() == 0.0 and V.max() == 1.0
    V2, _ = scenes.load_obj(path, center=(1.0, 2.0, 3.0), size=(4.0, 2.0, 1.0))
    assert np.allclose(V2.min(0), [-1.0, 1.0, 2.5]) and np.allclose(V2.max(0), [3.0, 3.0, 3.5])
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 3\n")
    from mps_cuda_gb300 import MpsError
    with pytest.raises(MpsError):
        scenes.load_obj(bad)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [2, 5])
def test_mesh_sampling_matches_reference(mps, tmp_path, n):
    from mps_cuda_gb300 import scenes
    from oracle import refstep
    path = tmp_path / "box.obj"
    write_box_obj(path, n=n)
    V, F = scenes.load_obj(path, center=(0.0, 0.0, 0.0), size=(9.0, 9.0, 9.0))  # a box like System::Initalize's
    ours, fid = scenes.sample_mesh(V, F, 0.4, with_faces=True)
    ref = refstep.sample_mesh(V, F, 0.4)
    assert ours.shape[0] == ref.shape[0]
    assert np.abs(ours[:, :3].astype(np.float64) - ref).max() <= 1e-6 * np.abs(ref).max()
    assert np.all(ours[:, 3] == np.float32(0.1))
    assert np.all(np.diff(fid.astype(np.int64)) >= 0)  # written face by face
    # every sample lies on the box surface
    assert np.abs(np.abs(ours[:, :3]).max(1) - 4.5).max() < 1e-5


@pytest.mark.gpu
def test_step_with_mesh_sampled_boundary(mps, orc, tmp_path):
    """A fluid block inside a box whose boundary particles come from mesh sampling: full steps
    against the oracle (fixed iteration counts)."""
    from mps_cuda_gb300 import Simulation, scenes
    path = tmp_path / "box.obj"
    write_box_obj(path, n=4)
    V, F = scenes.load_obj(path, center=(0.25, 0.25, 0.25), size=(0.5, 0.5, 0.5))
    sc = scenes.dam_break_small(8, seed=3)
    sc.bpos4 = scenes.sample_mesh(V, F, 0.04)      # spacing 0.02, particle radius 0.01
    sim = Simulation.from_scene(sc, fixed_iters=4)
    o = orc.from_scene(sc, config=dict(fixed_iters=4))
    sim.step(3)
    o.step(3)
    p, v = sim.get_fluid()
    rp, rv = o.get("pos"), o.get("vel")
    assert np.abs(p[:, :3] - rp).max() / np.abs(rp).max() < 1e-5
    assert np.abs(v[:, :3] - rv).max() / np.abs(rv).max() < 1e-4
