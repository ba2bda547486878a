"""ctypes wrapper of the FP64 CPU oracle (oracle/mps_oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the
checker of the CUDA path.  The product (mps_cuda_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libmps_oracle.so"

ZSORT, NEIGHBORS, BVOLUME, DENSITY, ALPHA, GRAVITY, DF, VISCST, CD, ADVECT = range(10)


class Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("gravity", C.c_double * 3), ("bmin", C.c_double * 3), ("bmax", C.c_double * 3),
                ("mat_radius", C.c_double), ("mat_mass", C.c_double), ("mat_density", C.c_double),
                ("mat_volume", C.c_double), ("viscosity", C.c_double), ("xsph", C.c_double),
                ("surface_tension", C.c_double), ("hash_cell", C.c_double), ("hash_size", C.c_uint32 * 3),
                ("cubic", C.c_int32), ("df_tol", C.c_double), ("cd_tol", C.c_double), ("df_min_iter", C.c_int32),
                ("cd_min_iter", C.c_int32), ("max_iter", C.c_int32), ("cg_tol", C.c_double),
                ("cg_max_iter", C.c_int32), ("volume_accumulate", C.c_int32), ("zsort", C.c_int32),
                ("threads", C.c_int32), ("fixed_iters", C.c_int32), ("visc_solver", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("df_iters", C.c_int32), ("cg_iters", C.c_int32), ("cd_iters", C.c_int32), ("df_err", C.c_double),
                ("cd_err", C.c_double), ("cg_rr", C.c_double), ("nei_ff", C.c_int64), ("nei_fb", C.c_int64),
                ("nei_bb", C.c_int64), ("frame", C.c_int32)]


class Grid(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("cell", C.c_float), ("inv_cell", C.c_float), ("dims", C.c_int32 * 3),
                ("key_base", C.c_uint64)]


def build() -> Path:
    """Compiles the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        vp = C.c_void_p
        lib.orc_create.restype = vp
        lib.orc_create.argtypes = [C.POINTER(Params)]
        lib.orc_destroy.argtypes = [vp]
        lib.orc_set_params.argtypes = [vp, C.POINTER(Params)]
        lib.orc_set_fluid.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp]
        lib.orc_set_boundary.argtypes = [vp, C.c_int64, vp, vp, vp]
        lib.orc_set_frame.argtypes = [vp, C.c_int32]
        lib.orc_phase.argtypes = [vp, C.c_int32]
        lib.orc_step.argtypes = [vp, C.c_int32]
        lib.orc_get_stats.argtypes = [vp, C.POINTER(Stats)]
        lib.orc_get.restype = C.c_int64
        lib.orc_get.argtypes = [vp, C.c_char_p, vp]
        lib.orc_put.argtypes = [vp, C.c_char_p, vp, C.c_int64]
        lib.orc_new_keys.argtypes = [C.c_int64, vp, C.POINTER(Grid), vp]
        lib.orc_new_stable_sort.argtypes = [C.c_int64, vp, vp]
        lib.orc_new_cell_ranges.restype = C.c_int64
        lib.orc_new_cell_ranges.argtypes = [C.c_int64, vp, vp, vp, vp]
        lib.orc_new_nbr_counts.argtypes = [C.c_int64, vp, C.c_int64, vp, vp, C.POINTER(Grid), C.c_int, vp]
        _lib = lib
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def params(material: dict, physics: dict, config: dict | None = None, hash_cell: float | None = None,
           hash_size=(64, 64, 64), **kw) -> Params:
    """Oracle parameters; defaults are the reference's shipped literals."""
    cfg = dict(kernel=0, df_tol=1e-3, cd_tol=1e-4, df_min_iter=1, cd_min_iter=2, max_iter=100, cg_tol=1e-2,
               cg_max_iter=100)
    cfg.update(config or {})
    p = Params()
    p.dt = physics["dt"]
    for k in range(3):
        p.gravity[k] = physics["gravity"][k]
        p.bmin[k] = physics["min"][k]
        p.bmax[k] = physics["max"][k]
        p.hash_size[k] = hash_size[k]
    p.mat_radius = material["radius"]
    p.mat_mass = material["mass"]
    p.mat_density = material["density"]
    p.mat_volume = material["volume"]
    p.viscosity = material["viscosity"]
    p.xsph = material["xsph"]
    p.surface_tension = material["surface_tension"]
    p.hash_cell = hash_cell if hash_cell is not None else material["radius"]
    p.cubic = int(cfg["kernel"])
    p.df_tol, p.cd_tol = cfg["df_tol"], cfg["cd_tol"]
    p.df_min_iter, p.cd_min_iter = cfg["df_min_iter"], cfg["cd_min_iter"]
    p.max_iter, p.cg_tol, p.cg_max_iter = cfg["max_iter"], cfg["cg_tol"], cfg["cg_max_iter"]
    p.volume_accumulate = int(kw.get("volume_accumulate", 0))
    p.zsort = int(kw.get("zsort", 0))
    p.threads = int(kw.get("threads", 0))
    p.fixed_iters = int(cfg.get("fixed_iters", 0))
    p.visc_solver = int(cfg.get("visc_solver", 0))
    return p


class Oracle:
    """Stateful FP64 replay of the reference step."""

    VEC = {"pos", "vel", "force", "gradsum", "cg_b", "bpos"}

    def __init__(self, p: Params):
        self.lib = load()
        self.p = p
        self.h = self.lib.orc_create(C.byref(p))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def set_fluid(self, pos, vel, mass, radius):
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.ascontiguousarray(vel, np.float64)
        mass = np.ascontiguousarray(mass, np.float64)
        radius = np.ascontiguousarray(radius, np.float64)
        self.n = pos.shape[0]
        self.lib.orc_set_fluid(self.h, self.n, _p(pos), _p(vel), _p(mass), _p(radius), None)

    def set_boundary(self, pos, radius, volume=None):
        pos = np.ascontiguousarray(pos, np.float64)
        radius = np.ascontiguousarray(radius, np.float64)
        vol = None if volume is None else np.ascontiguousarray(volume, np.float64)
        self.nb = pos.shape[0]
        self.lib.orc_set_boundary(self.h, self.nb, _p(pos), _p(radius), None if vol is None else _p(vol))

    def set_fixed_iters(self, n: int):
        """fixed_iters of the following phases (0: adaptive loops)."""
        self.p.fixed_iters = int(n)
        self.lib.orc_set_params(self.h, C.byref(self.p))

    def set_frame(self, f: int):
        self.lib.orc_set_frame(self.h, f)

    def phase(self, ph: int):
        assert self.lib.orc_phase(self.h, ph) == 0

    def step(self, n: int = 1):
        self.lib.orc_step(self.h, n)

    def stats(self) -> dict:
        s = Stats()
        self.lib.orc_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def get(self, name: str) -> np.ndarray:
        cnt = self.lib.orc_get(self.h, name.encode(), None)
        if cnt < 0:
            raise KeyError(name)
        if name == "color":
            out = np.zeros(cnt, np.float32)
        elif name.startswith("nei") or name == "ids":
            out = np.zeros(cnt, np.uint32)
        else:
            out = np.zeros(cnt, np.float64)
        self.lib.orc_get(self.h, name.encode(), _p(out))
        if name in self.VEC:
            out = out.reshape(-1, 3)
        if name == "color":
            out = out.reshape(-1, 4)
        return out

    def put(self, name: str, values: np.ndarray):
        a = np.ascontiguousarray(values, np.float64).ravel()
        assert self.lib.orc_put(self.h, name.encode(), _p(a), a.size) == 0, name


def from_scene(scene, config: dict | None = None, f32_inputs: bool = True, **kw) -> Oracle:
    """Oracle loaded with a scene's arrays (FP32 values widened to FP64 unless f32_inputs=False)."""
    cfg = dict(scene.config)
    cfg.update(config or {})
    hc = scene.meta.get("hash_cell")
    hs = scene.meta.get("hash_size")
    if hs is None:
        # a power-of-two table that covers the box without wrapping
        ext = np.asarray(scene.physics["max"]) - np.asarray(scene.physics["min"])
        cell = hc or scene.material["radius"]
        hs = tuple(int(2 ** np.ceil(np.log2(max(4, e / cell * 2 + 4)))) for e in ext)
    o = Oracle(params(scene.material, scene.physics, cfg, hash_cell=hc, hash_size=hs, **kw))
    pos = scene.meta["pos_f64"] if (not f32_inputs and "pos_f64" in scene.meta) else scene.pos4[:, :3].astype(np.float64)
    o.set_boundary(scene.bpos4[:, :3].astype(np.float64), scene.bpos4[:, 3].astype(np.float64))
    o.set_fluid(pos, scene.vel4[:, :3].astype(np.float64), scene.vel4[:, 3].astype(np.float64),
                scene.pos4[:, 3].astype(np.float64))
    return o


# ------------------------------------------------------------------ new integer scheme
def grid(origin, cell, dims, key_base=0) -> Grid:
    g = Grid()
    for k in range(3):
        g.origin[k] = origin[k]
        g.dims[k] = dims[k]
    g.cell = cell
    g.inv_cell = float(np.float32(1.0) / np.float32(cell))
    g.key_base = key_base
    return g


def new_keys(pos4: np.ndarray, g: Grid) -> np.ndarray:
    p = np.ascontiguousarray(pos4, np.float32)
    out = np.zeros(p.shape[0], np.uint64)
    load().orc_new_keys(p.shape[0], _p(p), C.byref(g), _p(out))
    return out


def new_stable_sort(keys: np.ndarray, vals: np.ndarray):
    k = np.ascontiguousarray(keys, np.uint64).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    load().orc_new_stable_sort(k.size, _p(k), _p(v))
    return k, v


def new_cell_ranges(sorted_keys: np.ndarray):
    sk = np.ascontiguousarray(sorted_keys, np.uint64)
    n = sk.size
    cells = np.zeros(n, np.uint64)
    st = np.zeros(n, np.uint32)
    en = np.zeros(n, np.uint32)
    m = load().orc_new_cell_ranges(n, _p(sk), _p(cells), _p(st), _p(en))
    return cells[:m], st[:m], en[:m]


def new_nbr_counts(q4: np.ndarray, p4: np.ndarray, p_sorted_keys: np.ndarray, g: Grid, same_set: bool) -> np.ndarray:
    q = np.ascontiguousarray(q4, np.float32)
    p = np.ascontiguousarray(p4, np.float32)
    k = np.ascontiguousarray(p_sorted_keys, np.uint64)
    out = np.zeros(q.shape[0], np.uint32)
    load().orc_new_nbr_counts(q.shape[0], _p(q), p.shape[0], _p(p), _p(k), C.byref(g), int(same_set), _p(out))
    return out
