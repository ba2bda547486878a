"""ctypes wrapper of the reference's own CUDA step rebuilt headless (oracle/_ref) -- TEST
INFRASTRUCTURE ONLY: the checker that pins the FP64 oracle, and the reference arm of bench.py.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"


def lib_path(variant: str) -> Path:
    return REF_DIR / variant / "libmpsref.so"


def available(variant: str = "shipped") -> bool:
    return lib_path(variant).exists() or (REF_DIR / "src" / "MPS_Computer").exists()


def build() -> None:
    subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True, stdout=subprocess.DEVNULL)


_libs: dict[str, C.CDLL] = {}


def load(variant: str = "shipped") -> C.CDLL:
    if variant in _libs:
        return _libs[variant]
    p = lib_path(variant)
    if not p.exists():
        build()
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    lib.ref_create.restype = vp
    lib.ref_create.argtypes = [C.c_longlong, vp, vp, vp, vp, C.c_longlong, vp, vp, vp, vp, C.c_double, vp]
    lib.ref_destroy.argtypes = [vp]
    lib.ref_set_frame.argtypes = [vp, C.c_int]
    lib.ref_loops.argtypes = [vp]
    lib.ref_phase.argtypes = [vp, C.c_int]
    lib.ref_step.argtypes = [vp, C.c_int]
    lib.ref_get.restype = C.c_longlong
    lib.ref_get.argtypes = [vp, C.c_char_p, vp]
    lib.ref_put.argtypes = [vp, C.c_char_p, vp, C.c_longlong]
    lib.ref_sample_mesh.restype = C.c_longlong
    lib.ref_sample_mesh.argtypes = [vp, C.c_longlong, vp, C.c_longlong, C.c_double, vp, C.c_longlong]
    _libs[variant] = lib
    return lib


def sample_mesh(V: np.ndarray, F: np.ndarray, mesh_radius: float, variant: str = "shipped") -> np.ndarray:
    """The reference's own ParticleSampling on a mesh: (N, 3) float64 positions."""
    lib = load(variant)
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.uint32)
    n = lib.ref_sample_mesh(_p(V), V.shape[0], _p(F), F.shape[0], mesh_radius, None, 0)
    if n < 0:
        raise RuntimeError("reference mesh sampling failed")
    out = np.zeros((n, 3), np.float64)
    lib.ref_sample_mesh(_p(V), V.shape[0], _p(F), F.shape[0], mesh_radius, _p(out), n)
    return out


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class RefStep:
    """The reference's step on the GPU, fed with FP64 arrays."""

    VEC = {"pos", "vel", "bpos"}

    def __init__(self, scene, variant: str = "shipped", hash_cell=None, hash_size=None, f32_inputs: bool = True):
        self.lib = load(variant)
        mat, ph = scene.material, scene.physics
        pos = scene.meta["pos_f64"] if (not f32_inputs and "pos_f64" in scene.meta) else scene.pos4[:, :3].astype(np.float64)
        self._keep = [np.ascontiguousarray(pos, np.float64), np.ascontiguousarray(scene.vel4[:, :3], np.float64),
                      np.ascontiguousarray(scene.vel4[:, 3], np.float64), np.ascontiguousarray(scene.pos4[:, 3], np.float64),
                      np.ascontiguousarray(scene.bpos4[:, :3], np.float64), np.ascontiguousarray(scene.bpos4[:, 3], np.float64)]
        sm = np.array([mat["radius"], mat["mass"], mat["density"], mat["volume"], mat["viscosity"], mat["xsph"],
                       mat["surface_tension"]], np.float64)
        phv = np.array([ph["dt"], *ph["gravity"], *ph["min"], *ph["max"]], np.float64)
        hc = hash_cell or scene.meta.get("hash_cell") or mat["radius"]
        if hash_size is None:
            hash_size = scene.meta.get("hash_size")
        if hash_size is None:
            ext = np.asarray(ph["max"]) - np.asarray(ph["min"])
            hash_size = tuple(int(2 ** np.ceil(np.log2(max(4, e / hc * 2 + 4)))) for e in ext)
        hs = np.array(hash_size, np.uint32)
        k = self._keep
        self.n, self.nb = scene.n, scene.nb
        self.h = self.lib.ref_create(self.n, _p(k[0]), _p(k[1]), _p(k[2]), _p(k[3]), self.nb, _p(k[4]), _p(k[5]),
                                     _p(sm), _p(phv), hc, _p(hs))
        if not self.h:
            raise RuntimeError("reference step: device set-up failed")

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_frame(self, f: int):
        self.lib.ref_set_frame(self.h, f)

    def phase(self, ph: int):
        r = self.lib.ref_phase(self.h, ph)
        if r:
            raise RuntimeError(f"reference phase {ph} failed ({r})")

    def step(self, n: int = 1):
        r = self.lib.ref_step(self.h, n)
        if r:
            raise RuntimeError(f"reference step failed ({r})")

    def loops(self) -> tuple[int, int, int]:
        out = np.zeros(3, np.int32)
        self.lib.ref_loops(_p(out))
        return tuple(int(v) for v in out)

    def get(self, name: str) -> np.ndarray:
        cnt = self.lib.ref_get(self.h, name.encode(), None)
        if cnt < 0:
            raise KeyError(name)
        dt = np.float32 if name == "color" else (np.uint32 if name.startswith("nei") else np.float64)
        out = np.zeros(cnt, dt)
        self.lib.ref_get(self.h, name.encode(), _p(out))
        if name in self.VEC:
            out = out.reshape(-1, 3)
        if name == "color":
            out = out.reshape(-1, 4)
        return out

    def put(self, name: str, values: np.ndarray):
        a = np.ascontiguousarray(values, np.float64).ravel()
        if self.lib.ref_put(self.h, name.encode(), _p(a), a.size):
            raise KeyError(name)
