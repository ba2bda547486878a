"""The benchmark configurations at full size.

- 1M dam break (1,000,000 fluid, ~210k wall particles): one step phase by phase against the FP64
  oracle from the GPU's state after a few steps (density, alpha after the density pass; the
  first-iteration stiffness of each pressure solve; velocities after each solve, at 1e-5); and
  size-independent properties of the step's neighbour lists: every slot's list is sorted, the
  fluid lists are symmetric (j lists i whenever i lists j), and the counts equal the oracle's FP32
  restatement bit for bit.
- 4M colliding blocks: two runs give the same bits, and the graph step equals the host-driven
  phases bit for bit.
- 256 batched scenes (2k-64k particles each, 4.9M in all): the batch equals single-scene runs of
  its smallest, median and largest scene bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-5


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


class Views(C.Structure):
    """mps_device_views of include/mps_c.h."""
    _fields_ = [("n", C.c_int64), ("nb", C.c_int64), ("slots", C.c_int64)] + \
               [(k, C.c_void_p) for k in ("pos4", "vel4", "ids", "density", "pressure", "alpha", "delta", "color4",
                                          "scratch4", "bpos4", "bvol", "nbr_fluid", "nbr_boundary", "nbr_count")] + \
               [("nbr_stride", C.c_int64), ("cap_fluid", C.c_int32), ("cap_boundary", C.c_int32),
                ("volume_accumulate", C.c_int32)]


def fluid_lists(sim):
    """(counts, lists[cap, slots]) of the step's fluid neighbour lists, copied from the device."""
    v = Views()
    assert sim.lib.mps_get_device_views(sim.h, C.addressof(v)) == 0
    cudart = C.CDLL("libcudart.so")
    cudart.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    lists = np.empty((v.cap_fluid, v.nbr_stride), np.uint32)
    assert cudart.cudaMemcpy(lists.ctypes.data, v.nbr_fluid, lists.nbytes, 2) == 0   # device to host
    counts = sim.get_field("nbr_count", order="slot")
    return counts, lists


def gpu_state_to_oracle(sim, o):
    p, v = sim.get_fluid()
    o.set_fluid(p[:, :3].astype(np.float64), v[:, :3].astype(np.float64), v[:, 3].astype(np.float64),
                p[:, 3].astype(np.float64))


@pytest.fixture(scope="module")
def scene_1m():
    from mps_cuda_gb300 import scenes
    return scenes.dam_break_1m(seed=0)


def test_dam_break_1m_phase_by_phase(mps, orc, scene_1m):
    """One step of the 1M dam break after 5 GPU steps, phase by phase on both sides from the GPU's
    state; each solve starts from the GPU's velocities on both sides.  Where an adaptive solve
    stops on another iteration than the oracle's (a threshold decision at r.r ~ tol), the
    oracle's solve is repeated with the GPU's number of updates and compared."""
    from mps_cuda_gb300 import Simulation
    sc = scene_1m
    for fixed in (1, 0):
        sim = Simulation.from_scene(sc, fixed_iters=fixed)
        sim.step(5)
        o = orc.from_scene(sc, config=dict(fixed_iters=fixed))
        gpu_state_to_oracle(sim, o)
        for ph in (mps.PHASE_SORT, mps.PHASE_NEIGHBORS, mps.PHASE_BVOLUME, mps.PHASE_DENSITY_ALPHA):
            sim.phase(ph)
        for ph in (orc.ZSORT, orc.NEIGHBORS, orc.BVOLUME, orc.DENSITY, orc.ALPHA, orc.GRAVITY):
            o.phase(ph)
        rho0 = sc.material["density"]
        assert np.abs(sim.get_field("density") - o.get("density")).max() / rho0 < REL
        assert rel_err(sim.get_field("alpha"), o.get("alpha")) < REL
        for gph, oph, name in ((mps.PHASE_DF, orc.DF, "df_iters"), (mps.PHASE_VISCST, orc.VISCST, "cg_iters"),
                               (mps.PHASE_CD, orc.CD, "cd_iters")):
            v_in = sim.get_field("vel")[:, :3].astype(np.float64)
            o.put("vel", v_in)
            sim.phase(gph)
            o.phase(oph)
            gi, oi = sim.stats()[name], o.stats()[name]
            assert abs(gi - oi) <= (0 if fixed else 1), (name, gi, oi)
            vo = o.get("vel")
            if gi != oi and name == "cg_iters":
                # the CG's loop counter is its number of updates plus one
                o.put("vel", v_in)
                o.set_fixed_iters(gi - 1)
                o.phase(oph)
                o.set_fixed_iters(0)
                vo = o.get("vel")
                o.put("vel", vo)
            if gi == oi or name == "cg_iters":
                assert rel_err(sim.get_field("vel")[:, :3], vo) < REL, (name, fixed)
            if fixed and name != "cg_iters":
                assert rel_err(sim.get_field("pressure"), o.get("pressure")) < REL, name
        sim.close()


def test_dam_break_1m_neighbour_lists(mps, orc, scene_1m):
    """After 3 steps: lists sorted by slot, fluid lists symmetric, counts equal to the oracle's
    FP32 restatement of the search on the same sorted positions."""
    from mps_cuda_gb300 import Simulation
    sc = scene_1m
    sim = Simulation.from_scene(sc)
    sim.step(3)
    sim.phase(mps.PHASE_SORT)
    sim.phase(mps.PHASE_NEIGHBORS)
    counts, lists = fluid_lists(sim)
    n, S = sc.n, lists.shape[1]
    nf = (counts & 0xFFFF).astype(np.int64)
    assert nf.max() <= lists.shape[0]
    k = np.arange(lists.shape[0])[:, None]
    live = k < nf[None, :n]
    sub = lists[:, :n]
    # sorted by slot within each list, no self, no duplicates
    inc = (sub[1:] > sub[:-1]) | ~live[1:]
    assert inc.all()
    ii = np.broadcast_to(np.arange(n, dtype=np.int64)[None, :], sub.shape)[live]
    jj = sub[live].astype(np.int64)
    assert jj.max() < n and not np.any(ii == jj)
    # symmetric: the pair set equals its transpose
    a = np.sort(ii * S + jj)
    b = np.sort(jj * S + ii)
    assert np.array_equal(a, b)
    assert sim.stats()["fluid_pairs"] == a.size
    # counts against the oracle's restatement (sorted positions of the GPU's current state)
    g = sim.grid()
    grid = orc.grid(g["origin"], g["cell"], g["dims"])
    q4 = sim.get_field("pos", order="slot")   # w holds the support radius h = 4 r on the device
    b4 = sc.bpos4.copy()
    b4[:, 3] *= 4
    kq = sim.get_field("cell_key", order="slot")
    assert np.all(np.diff(kq.astype(np.int64)) >= 0)
    kb_s, border = orc.new_stable_sort(orc.new_keys(b4, grid), np.arange(sc.nb, dtype=np.uint32))
    cf = orc.new_nbr_counts(q4, q4, kq, grid, True)
    cb = orc.new_nbr_counts(q4, b4[border], kb_s, grid, False)
    assert np.array_equal(counts & 0xFFFF, cf)
    assert np.array_equal(counts >> 16, cb)
    sim.close()


def test_colliding_4m_deterministic_and_graph_equals_phases(mps):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.colliding_4m(seed=0)
    a = Simulation.from_scene(sc)
    b = Simulation.from_scene(sc)
    a.step(2)
    b.step(2)
    pa, va = a.get_fluid()
    pb, vb = b.get_fluid()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    b.close()
    # one more step: graph on one handle, the phases with host-driven loops on a copy of the state
    e = Simulation.from_scene(sc, use_graph=0)
    e.set_fluid(pa, va)
    a2 = Simulation.from_scene(sc)
    a2.set_fluid(pa, va)
    a2.step(1)
    for ph in (mps.PHASE_SORT, mps.PHASE_NEIGHBORS, mps.PHASE_BVOLUME, mps.PHASE_DENSITY_ALPHA, mps.PHASE_DF,
               mps.PHASE_VISCST, mps.PHASE_CD, mps.PHASE_ADVECT):
        e.phase(ph)
    pg, vg = a2.get_fluid()
    pe, ve = e.get_fluid()
    assert np.array_equal(pg, pe) and np.array_equal(vg, ve)
    ids = a2.get_field("ids", order="slot")
    assert np.array_equal(np.sort(ids), np.arange(sc.n, dtype=ids.dtype))
    for s in (a, e, a2):
        s.close()


def test_batched_256_equals_single_scenes(mps):
    from mps_cuda_gb300 import BatchedSimulation, Simulation, scenes
    scs = scenes.batched_scenes(256, seed=0)
    bat = BatchedSimulation(scs)
    bat.step(2)
    p, v = bat.get_fluid()
    its = bat.scene_iters()
    sizes = np.array([s.n for s in scs])
    order = np.argsort(sizes, kind="stable")
    for k in (order[0], order[len(order) // 2], order[-1]):
        one = Simulation.from_scene(scs[k])
        one.step(2)
        p1, v1 = one.get_fluid()
        lo, hi = bat.offsets[k], bat.offsets[k + 1]
        assert np.array_equal(p[lo:hi], p1) and np.array_equal(v[lo:hi], v1), k
        st = one.stats()
        assert (st["df_iters"], st["cg_iters"], st["cd_iters"]) == tuple(its[k])
        one.close()
    bat.close()
