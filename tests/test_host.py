"""Host-side checks of the C ABI library (CPU only: no kernel launches)."""
import ctypes as C
import hashlib
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, has_gpu


def declared_symbols():
    text = (ROOT / "include" / "mps_c.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mps_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(mps):
    lib = mps._lib.load()
    syms = declared_symbols()
    assert len(syms) >= 28
    for s in syms:
        assert hasattr(lib, s), s
    assert lib.mps_abi_version() == 1


def test_python_binding_covers_the_header(mps):
    assert set(declared_symbols()) == set(mps._lib.EXPORTS)


def test_default_config_matches_reference_literals(mps):
    c = mps._lib.default_config()
    assert (c.df_tol, c.cd_tol, c.df_min_iter, c.cd_min_iter, c.max_iter) == (1e-3, 1e-4, 1, 2, 100)
    assert (c.cg_tol, c.cg_max_iter, c.cg_factor) == (1e-2, 100, 0.01)


def test_reference_material_mirror(mps):
    from mps_cuda_gb300 import SPHMaterial
    m = SPHMaterial()
    m.SetRadius(0.4)
    out = mps._lib.Material()
    mps._lib.load().mps_reference_material(0.4, 1.0, C.byref(out))
    p = m.GetParam()
    for k in ("radius", "mass", "density", "volume", "viscosity", "xsph", "surface_tension"):
        assert getattr(out, k) == pytest.approx(p[k], rel=0, abs=0), k


def test_invalid_arguments_rejected_without_device(mps):
    lib = mps._lib.load()
    mat = mps._lib.Material(0.4, 1.0, 1.0, 1.0, 0.0, 0.0, 0.0)
    phys = mps._lib.Physics()
    phys.dt = 0.0
    h = C.c_void_p()
    assert lib.mps_create(C.byref(mat), C.byref(phys), None, 0, C.byref(h)) == -1
    phys.dt = 0.001
    r = lib.mps_create(C.byref(mat), C.byref(phys), None, 0, C.byref(h))
    if not has_gpu():
        assert r == -2 and b"no CUDA device" in lib.mps_last_error()
    else:
        assert r == 0
        lib.mps_destroy(h)
    assert lib.mps_step(None, 1, None) == -1
    assert lib.mps_get_stats(None, None, None) == -1


def _digest(*arrays):
    m = hashlib.sha256()
    for a in arrays:
        m.update(np.ascontiguousarray(a).tobytes())
    return m.hexdigest()[:16]


def test_scene_generation_is_deterministic(mps):
    from mps_cuda_gb300 import scenes
    a = scenes.dam_break_small(6, seed=11)
    b = scenes.dam_break_small(6, seed=11)
    c = scenes.dam_break_small(6, seed=12)
    assert _digest(a.pos4, a.bpos4) == _digest(b.pos4, b.bpos4)
    assert _digest(a.pos4) != _digest(c.pos4)
    # the jitter stays within the bound and the lattice is where it should be
    d = a.pos4[:, :3] - (0.02 * (1 + np.stack(np.meshgrid(np.arange(6), np.arange(6), np.arange(6), indexing="ij"),
                                                -1)[..., ::-1].reshape(-1, 3)))
    assert np.abs(d).max() <= 0.002 + 1e-7


def test_scene_generation_platform_digest(mps):
    """Fixed digest: the generators give identical bits on x86 and Arm."""
    from mps_cuda_gb300 import scenes
    a = scenes.dam_break_small(6, seed=11)
    assert _digest(a.pos4, a.bpos4) == "63304c2dc7b11b63"


def test_wall_counts(mps):
    from mps_cuda_gb300 import scenes
    w = scenes.gen_walls((0, 0, 0), (1, 1, 1), 0.02, 0.01)
    assert w.shape[0] == 51 ** 3 - 49 ** 3  # six closed faces of a 51^3 lattice
    w = scenes.gen_walls((0, 0, 0), (3.0, 1.5, 2.0), 0.01, 0.005, scenes.FACE_PY)
    assert 205_000 < w.shape[0] < 215_000  # the ~210k single-layer tank of the 1M dam break
    s = scenes.gen_sphere((0, 0, 0), 0.2, 0.01, 0.005)
    assert abs(np.linalg.norm(s[:, :3], axis=1) - 0.2).max() < 1e-6


def test_reference_scene_matches_reference_setup(mps):
    from mps_cuda_gb300 import scenes
    sc = scenes.reference_surface_tension()
    assert sc.n == 250
    # two 5^3 blocks, stride 2 * 0.09 + 0.001 (MPSSystem.cpp:567-570)
    p = sc.meta["pos_f64"]
    xs = np.unique(np.round(p[:, 0], 6))
    assert len(xs) == 10
    assert sc.material["volume"] == pytest.approx(0.4 ** 3 / 48 * 3.141592, rel=1e-15)


def test_partition_scenes():
    from mps_cuda_gb300.sharding import imbalance, partition_scenes
    rng = np.random.default_rng(0)
    counts = [int(c) for c in np.exp(rng.uniform(np.log(2000), np.log(64000), 256))]
    for world in (1, 2, 4, 8):
        parts = partition_scenes(counts, world)
        assert sorted(i for p in parts for i in p) == list(range(256))
        assert imbalance(counts, parts) < 1.02
    assert partition_scenes([5, 1, 1], 2) == [[0], [1, 2]]
