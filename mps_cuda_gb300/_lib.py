"""ctypes binding of libmps_gb300.so (declared in include/mps_c.h).

The library is the product: it is loaded from this package directory and never replaced by a
Python or CPU implementation.  Importing works on a machine without a GPU (scene generation
and configuration are host code); creating a simulation needs a CUDA device and fails loudly
otherwise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libmps_gb300.so"

MPS_OK = 0
ERRORS = {
    -1: "MPS_E_INVALID",
    -2: "MPS_E_CUDA",
    -3: "MPS_E_NOMEM",
    -4: "MPS_E_STATE",
    -5: "MPS_E_OVERFLOW",
    -6: "MPS_E_NONFINITE",
}

PHASE_SORT, PHASE_NEIGHBORS, PHASE_BVOLUME, PHASE_DENSITY_ALPHA, PHASE_DF, PHASE_VISCST, PHASE_CD, PHASE_ADVECT = range(8)
KERNEL_POLY6_SPIKY, KERNEL_CUBIC_SPLINE = 0, 1
K_PRESSURE_A, K_PRESSURE_B, K_CG_AP, K_DENSITY_ALPHA, K_BUILD_NBRS, K_SORT, K_CG_VECTOR = range(7)
VISC_CG, VISC_JACOBI = 0, 1
CG_THREE_PASS, CG_TWO_PASS = 0, 1


class MpsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Material(C.Structure):
    _fields_ = [("radius", C.c_double), ("mass", C.c_double), ("density", C.c_double), ("volume", C.c_double),
                ("viscosity", C.c_double), ("xsph", C.c_double), ("surface_tension", C.c_double)]


class Physics(C.Structure):
    _fields_ = [("dt", C.c_double), ("gravity", C.c_double * 3), ("min", C.c_double * 3), ("max", C.c_double * 3)]


class Config(C.Structure):
    _fields_ = [("kernel", C.c_int32), ("df_tol", C.c_double), ("cd_tol", C.c_double), ("df_min_iter", C.c_int32),
                ("cd_min_iter", C.c_int32), ("max_iter", C.c_int32), ("cg_tol", C.c_double), ("cg_max_iter", C.c_int32),
                ("cg_factor", C.c_double), ("fixed_iters", C.c_int32), ("max_fluid_neighbors", C.c_int32),
                ("max_boundary_neighbors", C.c_int32), ("volume_accumulate", C.c_int32), ("use_graph", C.c_int32),
                ("block_size", C.c_int32), ("stage", C.c_int32), ("sort_digit_bits", C.c_int32),
                ("visc_solver", C.c_int32), ("cg_form", C.c_int32), ("cg_unroll", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("df_iters", C.c_int32), ("cg_iters", C.c_int32), ("cd_iters", C.c_int32), ("flags", C.c_int32),
                ("df_err", C.c_double), ("cd_err", C.c_double), ("cg_rr", C.c_double), ("fluid_pairs", C.c_int64),
                ("boundary_pairs", C.c_int64), ("steps", C.c_int64), ("iters_total", C.c_int64 * 3),
                ("runs_total", C.c_int64 * 3), ("passes_total", C.c_int64 * 3), ("tile_blocks", C.c_int64 * 2),
                ("sort_passes", C.c_int64)]


EXPORTS = {
    "mps_last_error": (C.c_char_p, []),
    "mps_abi_version": (C.c_int, []),
    "mps_default_config": (None, [C.POINTER(Config)]),
    "mps_reference_material": (None, [C.c_double, C.c_double, C.POINTER(Material)]),
    "mps_create": (C.c_int, [C.POINTER(Material), C.POINTER(Physics), C.POINTER(Config), C.c_int, C.POINTER(C.c_void_p)]),
    "mps_destroy": (C.c_int, [C.c_void_p]),
    "mps_set_physics": (C.c_int, [C.c_void_p, C.POINTER(Physics)]),
    "mps_set_material": (C.c_int, [C.c_void_p, C.POINTER(Material)]),
    "mps_set_fluid": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mps_set_boundary": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mps_set_fluid_f32": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "mps_get_fluid_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "mps_get_fluid": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mps_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mps_step_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "mps_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats), C.c_void_p]),
    "mps_phase": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mps_field_size": (C.c_int64, [C.c_void_p, C.c_char_p]),
    "mps_get_field": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_int]),
    "mps_put_field": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_int]),
    "mps_get_grid": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mps_profile_kernel": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_double)]),
    "mps_cell_sort_noalloc": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
    "mps_create_batched": (C.c_int, [C.POINTER(Material), C.POINTER(Physics), C.POINTER(Config), C.c_int, C.c_int32,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "mps_set_batched": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mps_get_batched": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mps_get_scene_iters": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mps_gen_block": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                C.c_double, C.c_uint64, C.c_void_p, C.c_void_p]),
    "mps_gen_box_walls": (C.c_int64, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int32, C.c_void_p]),
    "mps_gen_sphere": (C.c_int64, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_void_p]),
    "mps_mesh_load_obj": (C.c_int, [C.c_char_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.c_void_p, C.c_void_p]),
    "mps_mesh_sample": (C.c_int64, [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_double, C.c_void_p,
                                    C.c_void_p]),
    "mps_adjoint_forward": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "mps_adjoint_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "mps_adjoint_memory": (C.c_int64, [C.c_void_p, C.c_int32, C.c_int32]),
    "mps_adjoint_reserve": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "mps_op": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "mps_get_device_views": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mps_device_zero": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
}

_lib = None


def load() -> C.CDLL:
    """Loads libmps_gb300.so; raises if it has not been built (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with mps_cuda_gb300.build.build()")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != MPS_OK:
        msg = load().mps_last_error()
        raise MpsError(code, msg.decode() if msg else "")


def default_config(**overrides) -> Config:
    c = Config()
    load().mps_default_config(C.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c
