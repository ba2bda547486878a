"""Python mirror of the reference's step interface on top of the C ABI.

Names follow the reference (moonsh5009/MPS_CUDA):
- ``SPHMaterial`` mirrors mps::SPHMaterial (src/MPS_Object/MPSSPHMaterial.{h,cpp}): SetParam,
  SetRadius, SetViscosity, SetXSPH, SetSurfaceTension, GetParam.
- ``Simulation.OnUpdate`` is one frame of mps::System::OnUpdate (src/MPS_System/MPSSystem.cpp:191-291);
  ``Simulation.phase`` runs one of its sub-phases (the free functions of mps::kernel::SPH / Advect).
Errors are raised as MpsError carrying the library's status code and message (the reference
returns void and drops errors; this interface reports them).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L
from .scenes import Scene

FIELD_DTYPES = {
    "density": (np.float32, 1), "alpha": (np.float32, 1), "pressure": (np.float32, 1), "delta": (np.float32, 1),
    "density_deviation": (np.float32, 1),
    "aux": (np.float32, 2), "color": (np.float32, 4), "pos": (np.float32, 4), "vel": (np.float32, 4),
    "ids": (np.uint32, 1), "nbr_count": (np.uint32, 1), "cell_key": (np.uint64, 1), "cg_b": (np.float32, 4),
    "cg_x": (np.float32, 4), "bvol": (np.float32, 1), "bpos": (np.float32, 4),
}
BOUNDARY_FIELDS = {"bvol", "bpos"}


class SPHMaterial:
    """mps::SPHMaterial: defaults SetParam(0.01, 1.0), viscosity 0.025, XSPH 0.1, ST 100."""

    def __init__(self):
        self._p = {}
        self.SetParam(0.01, 1.0)
        self.SetViscosity(0.025)
        self.SetXSPH(0.1)
        self.SetSurfaceTension(100.0)

    def SetParam(self, radius: float, density: float) -> None:
        self._p["radius"] = radius
        self._p["volume"] = radius * radius * radius / 48.0 * 3.141592
        self._p["density"] = density
        self._p["mass"] = density * self._p["volume"]

    def SetRadius(self, radius: float) -> None:
        self.SetParam(radius, self._p["density"])

    def SetViscosity(self, v: float) -> None:
        self._p["viscosity"] = v

    def SetXSPH(self, v: float) -> None:
        self._p["xsph"] = v

    def SetSurfaceTension(self, v: float) -> None:
        self._p["surface_tension"] = v

    def GetParam(self) -> dict:
        return dict(self._p)


def _material(d: dict) -> L.Material:
    return L.Material(d["radius"], d["mass"], d["density"], d["volume"], d["viscosity"], d["xsph"], d["surface_tension"])


def _physics(d: dict) -> L.Physics:
    p = L.Physics()
    p.dt = d["dt"]
    for k in range(3):
        p.gravity[k] = d["gravity"][k]
        p.min[k] = d["min"][k]
        p.max[k] = d["max"][k]
    return p


def _stream(stream) -> Optional[int]:
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


class Simulation:
    """One fluid + one static boundary on one GPU (the reference's SPHModel + ObstacleModel)."""

    def __init__(self, material: dict, physics: dict, config: Optional[dict] = None, device: int = 0):
        self.lib = L.load()
        self.cfg = L.default_config(**(config or {}))
        h = C.c_void_p()
        m, p = _material(material), _physics(physics)
        L.check(self.lib.mps_create(C.byref(m), C.byref(p), C.byref(self.cfg), device, C.byref(h)))
        self.h = h
        self.n = 0
        self.nb = 0
        self.nscenes = 1
        self.material = dict(material)

    @classmethod
    def from_scene(cls, scene: Scene, device: int = 0, **config) -> "Simulation":
        cfg = dict(scene.config)
        cfg.update(config)
        sim = cls(scene.material, scene.physics, cfg, device)
        sim.set_boundary(scene.bpos4)
        sim.set_fluid(scene.pos4, scene.vel4)
        return sim

    def close(self) -> None:
        if self.h:
            self.lib.mps_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ state
    def set_boundary(self, bpos4: np.ndarray, volume: Optional[np.ndarray] = None) -> None:
        b = np.ascontiguousarray(bpos4, np.float32)
        nb = b.shape[0]
        pos3 = np.ascontiguousarray(b[:, :3], np.float64)
        rad = np.ascontiguousarray(b[:, 3], np.float64)
        vol = None if volume is None else np.ascontiguousarray(volume, np.float64)
        L.check(self.lib.mps_set_boundary(self.h, nb, pos3.ctypes.data_as(C.c_void_p), rad.ctypes.data_as(C.c_void_p),
                                          None if vol is None else vol.ctypes.data_as(C.c_void_p)))
        self.nb = nb

    def set_fluid(self, pos4: np.ndarray, vel4: np.ndarray, stream=None) -> None:
        p = np.ascontiguousarray(pos4, np.float32)
        v = np.ascontiguousarray(vel4, np.float32)
        L.check(self.lib.mps_set_fluid_f32(self.h, p.shape[0], p.ctypes.data_as(C.c_void_p),
                                           v.ctypes.data_as(C.c_void_p), 0, _stream(stream)))
        self.n = p.shape[0]

    def set_fluid_device(self, pos4_ptr: int, vel4_ptr: int, n: int, stream=None) -> None:
        L.check(self.lib.mps_set_fluid_f32(self.h, n, C.c_void_p(pos4_ptr), C.c_void_p(vel4_ptr), 1, _stream(stream)))

    def get_fluid(self, stream=None) -> tuple[np.ndarray, np.ndarray]:
        p = np.zeros((self.n, 4), np.float32)
        v = np.zeros((self.n, 4), np.float32)
        L.check(self.lib.mps_get_fluid_f32(self.h, p.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p), 0,
                                           _stream(stream)))
        return p, v

    def get_fluid_device(self, pos4_ptr: int, vel4_ptr: int, stream=None) -> None:
        L.check(self.lib.mps_get_fluid_f32(self.h, C.c_void_p(pos4_ptr), C.c_void_p(vel4_ptr), 1, _stream(stream)))

    def get_field(self, name: str, order: str = "id") -> np.ndarray:
        dt, comps = FIELD_DTYPES[name]
        count = self.nb if name in BOUNDARY_FIELDS else self.n
        out = np.zeros((count, comps) if comps > 1 else (count,), dt)
        L.check(self.lib.mps_get_field(self.h, name.encode(), out.ctypes.data_as(C.c_void_p), 1 if order == "id" else 0))
        return out

    def put_field(self, name: str, values: np.ndarray, order: str = "id") -> None:
        dt, comps = FIELD_DTYPES[name]
        a = np.ascontiguousarray(values, dt)
        L.check(self.lib.mps_put_field(self.h, name.encode(), a.ctypes.data_as(C.c_void_p), 1 if order == "id" else 0))

    def grid(self) -> dict:
        o = (C.c_float * 3)()
        c = C.c_float()
        d = (C.c_int32 * 3)()
        L.check(self.lib.mps_get_grid(self.h, o, C.byref(c), d))
        return dict(origin=tuple(o), cell=c.value, dims=tuple(d))

    def set_material(self, **changes) -> None:
        """Updates material constants (e.g. viscosity, surface_tension); graphs are re-captured."""
        self.material.update(changes)
        m = _material(self.material)
        L.check(self.lib.mps_set_material(self.h, C.byref(m)))

    # ------------------------------------------------------------------ stepping
    def step(self, nsteps: int = 1, stream=None) -> None:
        L.check(self.lib.mps_step(self.h, nsteps, _stream(stream)))

    def OnUpdate(self, stream=None) -> None:
        """One frame of mps::System::OnUpdate."""
        self.step(1, stream)

    def step_host(self, pos4: np.ndarray, vel4: np.ndarray, nsteps: int = 1, stream=None) -> None:
        """Host-buffer step: copies pos4/vel4 (float32, ID order) in, steps, copies them back in place."""
        assert pos4.dtype == np.float32 and vel4.dtype == np.float32 and pos4.flags.c_contiguous
        L.check(self.lib.mps_step_host(self.h, pos4.ctypes.data_as(C.c_void_p), vel4.ctypes.data_as(C.c_void_p),
                                       nsteps, _stream(stream)))

    def profile_kernel(self, kernel: int, reps: int = 10, stream=None) -> float:
        """Mean ms per launch of one kernel of the step (CUDA events on `stream`)."""
        ms = C.c_double()
        L.check(self.lib.mps_profile_kernel(self.h, kernel, reps, _stream(stream), C.byref(ms)))
        return ms.value

    def phase(self, ph: int, stream=None) -> None:
        L.check(self.lib.mps_phase(self.h, ph, _stream(stream)))

    def stats(self, stream=None, check: bool = True) -> dict:
        s = L.Stats()
        r = self.lib.mps_get_stats(self.h, C.byref(s), _stream(stream))
        if check:
            L.check(r)
        out = {}
        for k, _ in L.Stats._fields_:
            v = getattr(s, k)
            out[k] = list(v) if isinstance(v, C.Array) else v
        return out

    def launches_per_step(self, runs: tuple[int, int, int], radix_passes: int) -> int:
        """Kernel launches of one graph step given its launched solver passes (DF, CG, CD; the
        stats' passes_total)."""
        # keys + radix (4 per pass) + reorder, lists, [volume], density, DF init + condition
        static = 2 + 4 * radix_passes + 1 + (1 if self.cfg.volume_accumulate else 0) + 1 + 2
        jacobi = self.cfg.visc_solver == L.VISC_JACOBI
        # DF finish + solve set-up (ST factor, coefficients + r0, init, condition), solve finish +
        # CD set-up, CD finish + advect
        static += 5 + 4 + 2
        if self.cfg.stage == 1:
            static += 1   # the neighbourhood tiles, built with the neighbour lists
        # per pass: pressure A + its decision + pressure B; three-pass CG: operator + decision +
        # update + beta + direction; two-pass: operator + decision + update; Jacobi: one sweep
        cg = 1 if jacobi else (3 if self.cfg.cg_form == L.CG_TWO_PASS else 5)
        return static + 3 * runs[0] + cg * runs[1] + 3 * runs[2]


class BatchedSimulation(Simulation):
    """Many independent scenes advanced by one set of launches per pass."""

    def __init__(self, scenes: list[Scene], device: int = 0, **config):
        self.lib = L.load()
        base = scenes[0]
        cfg = dict(base.config)
        cfg.update(config)
        self.cfg = L.default_config(**cfg)
        fo = np.zeros(len(scenes) + 1, np.int64)
        bo = np.zeros(len(scenes) + 1, np.int64)
        boxes = np.zeros((len(scenes), 6), np.float64)
        for s, sc in enumerate(scenes):
            fo[s + 1] = fo[s] + sc.n
            bo[s + 1] = bo[s] + sc.nb
            boxes[s, :3] = sc.physics["min"]
            boxes[s, 3:] = sc.physics["max"]
        h = C.c_void_p()
        m, p = _material(base.material), _physics(base.physics)
        L.check(self.lib.mps_create_batched(C.byref(m), C.byref(p), C.byref(self.cfg), device, len(scenes),
                                            fo.ctypes.data_as(C.c_void_p), bo.ctypes.data_as(C.c_void_p),
                                            boxes.ctypes.data_as(C.c_void_p), C.byref(h)))
        self.h = h
        self.material = dict(base.material)
        self.n = int(fo[-1])
        self.nb = int(bo[-1])
        self.offsets = fo
        self.nscenes = len(scenes)
        pos = np.ascontiguousarray(np.concatenate([s.pos4 for s in scenes]), np.float32)
        vel = np.ascontiguousarray(np.concatenate([s.vel4 for s in scenes]), np.float32)
        bpos = np.ascontiguousarray(np.concatenate([s.bpos4 for s in scenes]), np.float32)
        L.check(self.lib.mps_set_batched(self.h, pos.ctypes.data_as(C.c_void_p), vel.ctypes.data_as(C.c_void_p),
                                         bpos.ctypes.data_as(C.c_void_p), None))

    def scene_iters(self) -> np.ndarray:
        out = np.zeros((self.nscenes, 3), np.int32)
        L.check(self.lib.mps_get_scene_iters(self.h, out.ctypes.data_as(C.c_void_p)))
        return out
