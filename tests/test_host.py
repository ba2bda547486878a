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
    cfg = mps._lib.default_config(max_fluid_neighbors=70000)   # above the 16-bit counts
    assert lib.mps_create(C.byref(mat), C.byref(phys), C.byref(cfg), 0, C.byref(h)) == -1
    assert b"65535" in lib.mps_last_error()


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


def _lib_block(lib, dims, origin, spacing, radius, mass, jitter, seed):
    n = dims[0] * dims[1] * dims[2]
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    o = (C.c_double * 3)(*origin)
    assert lib.mps_gen_block(dims[0], dims[1], dims[2], o, spacing, radius, mass, jitter, seed,
                             pos.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p)) == 0
    return pos, vel


def _lib_walls(lib, lo, hi, spacing, radius, open_mask):
    clo, chi = (C.c_double * 3)(*lo), (C.c_double * 3)(*hi)
    n = lib.mps_gen_box_walls(clo, chi, spacing, radius, open_mask, None)
    out = np.zeros((n, 4), np.float32)
    lib.mps_gen_box_walls(clo, chi, spacing, radius, open_mask, out.ctypes.data_as(C.c_void_p))
    return out


def _lib_sphere(lib, center, R, spacing, radius):
    c = (C.c_double * 3)(*center)
    n = lib.mps_gen_sphere(c, R, spacing, radius, None)
    out = np.zeros((n, 4), np.float32)
    lib.mps_gen_sphere(c, R, spacing, radius, out.ctypes.data_as(C.c_void_p))
    return out


def test_numpy_generators_equal_the_library(mps):
    """The NumPy scene generators (which build every scene without loading a CUDA library) give the
    same bits as the library's C-ABI generators, on the benchmark configurations' arguments."""
    from mps_cuda_gb300 import scenes
    lib = mps._lib.load()
    for args in (((32, 32, 32), (0.0, 0.0, 0.0), 0.02, 0.01, 1.0e-3 * 8, 0.002, 0),
                 ((100, 100, 100), (0.0, 0.0, 0.0), 0.01, 0.005, 1.0e-3, 0.001, 0),
                 ((7, 3, 5), (1.25, -0.5, 0.1), 0.02, 0.01, 8.0, 0.002, 123456789012345),
                 ((128, 125, 125), (0.49, 0.365, 0.365), 0.01, 0.005, 1.0e-3, 0.001, 1)):
        pa, va = scenes.gen_block(*args)
        pb, vb = _lib_block(lib, *args)
        assert np.array_equal(pa.view(np.uint32), pb.view(np.uint32)), args[0]
        assert np.array_equal(va.view(np.uint32), vb.view(np.uint32)), args[0]
    for args in (((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.02, 0.01, 0),
                 ((0.0, 0.0, 0.0), (3.0, 1.5, 2.0), 0.01, 0.005, scenes.FACE_PY),
                 ((0.0, 0.0, 0.0), (4.0, 2.0, 2.0), 0.01, 0.005, 0),
                 ((-4.1, -3.9, -4.2), (3.3, 3.1, 3.05), 0.2, 0.1, 0b101001)):
        a = scenes.gen_walls(*args)
        b = _lib_walls(lib, *args)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), args
    for args in (((2.0, 1.0, 1.0), 0.2, 0.01, 0.005), ((0.0, 0.0, 0.0), 1.0, 0.05, 0.01)):
        a = scenes.gen_sphere(*args)
        b = _lib_sphere(lib, *args)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), args


def test_scene_construction_loads_no_cuda_library():
    """Building the benchmark scenes maps no CUDA library, so the reference arm of bench.py can
    build its inputs and map only the reference's own step (checked in a fresh interpreter)."""
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from mps_cuda_gb300 import scenes\n"
            "scenes.dam_break_32k(); scenes.colliding_4m(scale=0.05); scenes.reference_surface_tension()\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libmps_gb300' not in maps and 'libcudart' not in maps, 'a CUDA library was mapped'\n"
            "print('ok')\n") % str(ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr


def test_noalloc_sort_rejects_bad_arguments_before_device_work(mps):
    """The allocation-free cell sort checks its sizes and its pointers' alignment on the host and
    touches no device before rejecting them (pointer values here are never dereferenced)."""
    lib = mps._lib.load()
    origin = (C.c_float * 3)(0.0, 0.0, 0.0)
    dims = (C.c_int32 * 3)(4, 4, 4)
    ok = dict(pos=0x10000, keys=0x20000, order=0x30000)

    def call(n, pos=ok["pos"], keys=ok["keys"], order=ok["order"], cell=1.0):
        return lib.mps_cell_sort_noalloc(C.c_void_p(pos), n, origin, C.c_float(cell), dims, C.c_void_p(keys),
                                         C.c_void_p(order), None)

    assert call(262145) == -1                 # beyond the fixed scratch
    assert call(-1) == -1
    assert call(16, pos=0x10008) == -1        # float4 reads need 16-byte alignment
    assert call(16, keys=0x20004) == -1       # 64-bit keys
    assert call(16, order=0x30002) == -1      # 32-bit indices
    assert call(16, cell=0.0) == -1
