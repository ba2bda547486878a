"""Scene and configuration table.

Scenes are built with deterministic generators (NumPy restatements of the library's mps_gen_block /
mps_gen_box_walls / mps_gen_sphere, bit-identical to them) so that every implementation (this
package, the FP64 oracle, the reference's own CUDA step) gets bit-identical inputs, and building a
scene loads no CUDA library.

- ``reference_surface_tension``: the reference's active scene, mps::System::SurfaceTensionTestScene
  (src/MPS_System/MPSSystem.cpp:552-651) with the constants of System::Initalize (:26-72); its
  mesh-sampled cube boundary (cube.obj, not shipped with the reference) is replaced by the box walls
  sampled at the reference's boundary spacing 2 * (0.25 * 0.4) (MPSParticleSamplingUtil.cuh:31).
- ``dam_break_32k`` / ``dam_break_1m``: the plain FP32 dam breaks (32^3 fluid in a unit box; 100^3
  fluid in a 3 x 1.5 x 2 tank, y up, open top, ~210k wall particles).
- ``colliding_4m``: two 2M-particle blocks at +-1 m/s around a sampled sphere in a 4 x 2 x 2 tank.
- ``batched_256``: 256 independent dam breaks, fluid counts log-uniform in [2k, 64k].
- ``adjoint_16k``: 32 x 32 x 16 block in a unit box, 30 fixed solver iterations.
- ``reference_viscosity``: mps::System::ViscosityTestScene (MPSSystem.cpp:455-551), a 5 x 5 x height
  column, with the surface-tension scene's walls.

Material of the physical configs: rest density 1000, particle volume V = spacing^3 (so the rest
lattice sums to about rho0), mass = rho0 V, viscosity 0.01, surface tension 0.05, XSPH 0.1 (the
reference default), cubic spline kernel, tolerances 0.1 % density and 0.1 % divergence.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

FACE_NX, FACE_PX, FACE_NY, FACE_PY, FACE_NZ, FACE_PZ = (1 << k for k in range(6))


@dataclass
class Scene:
    name: str
    pos4: np.ndarray            # (N, 4) float32: x, y, z, particle radius
    vel4: np.ndarray            # (N, 4) float32: vx, vy, vz, mass
    bpos4: np.ndarray           # (B, 4) float32: x, y, z, particle radius
    material: dict
    physics: dict
    config: dict = field(default_factory=dict)
    steps: int = 1
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos4.shape[0])

    @property
    def nb(self) -> int:
        return int(self.bpos4.shape[0])


def _ptr(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


# ---- generators (host set-up code).  NumPy restatements of the library's C-ABI generators
# mps_gen_block / mps_gen_box_walls / mps_gen_sphere (csrc/scene.cpp), bit-identical to them (a CPU
# test compares the two), so that building a scene loads no CUDA library: the reference arm of the
# benchmark builds its inputs with these and maps only the reference's own step.
_M64 = (1 << 64) - 1


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic), as in csrc/scene.cpp."""
    x = x + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def _uniform01(seed: int, counter: np.ndarray) -> np.ndarray:
    """Uniform doubles in [0, 1) from (seed, counter): the top 53 bits of splitmix64(seed ^ splitmix64(counter))."""
    r = _splitmix64(np.uint64(seed & _M64) ^ _splitmix64(counter.astype(np.uint64)))
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def gen_block(dims, origin, spacing, radius, mass, jitter, seed):
    """Jittered lattice block: particle i = (x, y, z) with x fastest sits at
    origin + spacing * (index + 1) + jitter * U(-1, 1) per axis (FP64, then rounded to FP32)."""
    nx, ny, nz = (int(d) for d in dims)
    if nx <= 0 or ny <= 0 or nz <= 0:
        raise ValueError("bad block dimensions")
    n = nx * ny * nz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    idx = (x.ravel(), y.ravel(), z.ravel())
    i = np.arange(n, dtype=np.uint64)
    pos = np.zeros((n, 4), np.float32)
    for a in range(3):
        u = _uniform01(int(seed), np.uint64(3) * i + np.uint64(a))
        j = float(jitter) * (2.0 * u - 1.0)
        pos[:, a] = (float(origin[a]) + float(spacing) * (idx[a] + 1).astype(np.float64) + j).astype(np.float32)
    pos[:, 3] = np.float32(radius)
    vel = np.zeros((n, 4), np.float32)
    vel[:, 3] = np.float32(mass)
    return pos, vel


def _llround(v: float) -> int:
    """Round half away from zero (C's llround) for v >= 0."""
    f = math.floor(v)
    return int(f) + (1 if v - f >= 0.5 else 0)


def gen_walls(lo, hi, spacing, radius, open_mask=0):
    """Single-layer box walls: lattice points of the box surface (per-axis spacing stretched so that
    both faces are hit exactly), point (i, j, k) kept when it lies on a face that is not open
    (bit 2a: the low face of axis a, bit 2a + 1: the high face)."""
    if not spacing > 0.0:
        raise ValueError("bad wall arguments")
    n, step = [], []
    for a in range(3):
        ext = float(hi[a]) - float(lo[a])
        if not ext > 0.0:
            raise ValueError("bad wall arguments")
        na = max(2, _llround(ext / float(spacing)) + 1)
        n.append(na)
        step.append(ext / float(na - 1))
    k, j, i = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    c = (i.ravel(), j.ravel(), k.ravel())
    on = np.zeros(c[0].shape, bool)
    for a in range(3):
        if not open_mask & (1 << (2 * a)):
            on |= c[a] == 0
        if not open_mask & (1 << (2 * a + 1)):
            on |= c[a] == n[a] - 1
    out = np.zeros((int(on.sum()), 4), np.float32)
    for a in range(3):
        ca = c[a][on]
        v = float(lo[a]) + step[a] * ca.astype(np.float64)
        out[:, a] = np.where(ca == n[a] - 1, float(hi[a]), v).astype(np.float32)
    out[:, 3] = np.float32(radius)
    return out


def gen_sphere(center, R, spacing, radius):
    """Fibonacci lattice on a sphere, about one point per spacing^2 of area (the C library's math
    functions through Python's math module, so the points equal the C-ABI generator's)."""
    if not (R > 0.0 and spacing > 0.0):
        raise ValueError("bad sphere arguments")
    pi = math.acos(-1.0)
    count = _llround(4.0 * pi * R * R / (spacing * spacing))
    out = np.zeros((max(count, 0), 4), np.float32)
    golden = pi * (3.0 - math.sqrt(5.0))
    for i in range(count):
        y = 1.0 - 2.0 * (float(i) + 0.5) / float(count)
        r = math.sqrt(max(0.0, 1.0 - y * y))
        th = golden * float(i)
        out[i, 0] = center[0] + R * r * math.cos(th)
        out[i, 1] = center[1] + R * y
        out[i, 2] = center[2] + R * r * math.sin(th)
    out[:, 3] = np.float32(radius)
    return out


def load_obj(path: str, center=None, size=None) -> tuple[np.ndarray, np.ndarray]:
    """OBJ mesh -> (vertices (V, 3) float64, faces (F, 3) uint32), optionally fitted to a box."""
    lib = L.load()
    nv, nf = C.c_int64(), C.c_int64()
    c = None if center is None else (C.c_double * 3)(*center)
    s = None if size is None else (C.c_double * 3)(*size)
    L.check(lib.mps_mesh_load_obj(str(path).encode(), c, s, C.byref(nv), C.byref(nf), None, None))
    V = np.zeros((nv.value, 3), np.float64)
    F = np.zeros((nf.value, 3), np.uint32)
    L.check(lib.mps_mesh_load_obj(str(path).encode(), c, s, C.byref(nv), C.byref(nf), _ptr(V), _ptr(F)))
    return V, F


def sample_mesh(V: np.ndarray, F: np.ndarray, mesh_radius: float, with_faces: bool = False):
    """Boundary particles (N, 4) float32 on a triangle mesh (GPU), as the reference samples its obstacles."""
    lib = L.load()
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.uint32)
    n = lib.mps_mesh_sample(_ptr(V), V.shape[0], _ptr(F), F.shape[0], mesh_radius, None, None)
    if n < 0:
        L.check(int(n))
    out = np.zeros((n, 4), np.float32)
    fid = np.zeros(n, np.uint32)
    m = lib.mps_mesh_sample(_ptr(V), V.shape[0], _ptr(F), F.shape[0], mesh_radius, _ptr(out), _ptr(fid))
    if m < 0:
        L.check(int(m))
    return (out, fid) if with_faces else out


def physical_material(spacing: float, rho0: float = 1000.0, visc: float = 0.01, sigma: float = 0.05,
                      xsph: float = 0.1, radius: float | None = None) -> dict:
    V = spacing ** 3
    r = radius if radius is not None else spacing / 2
    return dict(radius=4 * r, mass=rho0 * V, density=rho0, volume=V, viscosity=visc, xsph=xsph, surface_tension=sigma)


def reference_material(h: float, density: float = 1.0) -> dict:
    """SPHMaterial() + SetRadius(h) (MPSSPHMaterial.cpp:4-19)."""
    V = h * h * h / 48.0 * 3.141592
    return dict(radius=h, mass=density * V, density=density, volume=V, viscosity=0.025, xsph=0.1,
                surface_tension=100.0)


PHYS_CONFIG = dict(kernel=L.KERNEL_CUBIC_SPLINE, df_tol=1.0e-3, cd_tol=1.0e-3, df_min_iter=1, cd_min_iter=2,
                   max_iter=100)


def dam_break(dims, spacing, radius, jitter, lo, hi, open_mask=0, seed=0, dt=1.0e-3, name="dam_break",
              steps=1, origin=None, wall_spacing=None, material=None, config=None) -> Scene:
    mat = material or physical_material(spacing, radius=radius)
    org = origin if origin is not None else lo
    pos, vel = gen_block(dims, org, spacing, radius, mat["mass"], jitter, seed)
    walls = gen_walls(lo, hi, wall_spacing or spacing, radius, open_mask)
    phys = dict(dt=dt, gravity=(0.0, -9.81, 0.0), min=tuple(lo), max=tuple(hi))
    cfg = dict(PHYS_CONFIG)
    cfg.update(config or {})
    return Scene(name, pos, vel, walls, mat, phys, cfg, steps, dict(dims=tuple(dims), spacing=spacing, seed=seed))


def dam_break_32k(seed: int = 0) -> Scene:
    return dam_break((32, 32, 32), 0.02, 0.01, 0.002, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), seed=seed, dt=1.0e-3,
                     name="dam_break_32k", steps=1000)


def dam_break_1m(seed: int = 0) -> Scene:
    return dam_break((100, 100, 100), 0.01, 0.005, 0.001, (0.0, 0.0, 0.0), (3.0, 1.5, 2.0), open_mask=FACE_PY,
                     seed=seed, dt=5.0e-4, name="dam_break_1m", steps=2000)


def dam_break_512k(seed: int = 0) -> Scene:
    """80^3 fluid in the 1M dam break's tank (profiling size: working set just above L2)."""
    return dam_break((80, 80, 80), 0.01, 0.005, 0.001, (0.0, 0.0, 0.0), (3.0, 1.5, 2.0), open_mask=FACE_PY,
                     seed=seed, dt=5.0e-4, name="dam_break_512k", steps=2000)


def dam_break_small(n: int = 10, seed: int = 0, box: float = 0.5, kernel=L.KERNEL_CUBIC_SPLINE) -> Scene:
    """Small dam break with the dam_break_32k constants (for tests)."""
    return dam_break((n, n, n), 0.02, 0.01, 0.002, (0.0, 0.0, 0.0), (box, box, box), seed=seed, dt=1.0e-3,
                     name=f"dam_break_{n}", config=dict(kernel=kernel))


def colliding_4m(seed: int = 0, scale: float = 1.0) -> Scene:
    """Two blocks (128 x 125 x 125 each at full scale) at +-1 m/s around a sampled sphere."""
    sp, r = 0.01, 0.005
    mat = physical_material(sp, radius=r)
    d = (max(2, round(128 * scale)), max(2, round(125 * scale)), max(2, round(125 * scale)))
    ext = [sp * (k + 1) for k in d]
    lo, hi = (0.0, 0.0, 0.0), (4.0, 2.0, 2.0)
    yz0 = (1.0 - ext[1] / 2, 1.0 - ext[2] / 2)
    pa, va = gen_block(d, (2.0 - 0.25 - ext[0], yz0[0], yz0[1]), sp, r, mat["mass"], 0.001, seed)
    pb, vb = gen_block(d, (2.0 + 0.25 - sp, yz0[0], yz0[1]), sp, r, mat["mass"], 0.001, seed + 1)
    va[:, 0] = 1.0
    vb[:, 0] = -1.0
    walls = gen_walls(lo, hi, sp, r)
    sph = gen_sphere((2.0, 1.0, 1.0), 0.2, sp, r)
    phys = dict(dt=5.0e-4, gravity=(0.0, -9.81, 0.0), min=lo, max=hi)
    return Scene("colliding_4m", np.concatenate([pa, pb]), np.concatenate([va, vb]), np.concatenate([walls, sph]),
                 mat, phys, dict(PHYS_CONFIG), 500, dict(dims=d, seed=seed))


def batched_scenes(nscenes: int = 256, seed: int = 0, nmin: int = 2000, nmax: int = 64000) -> list[Scene]:
    """Independent dam breaks: N log-uniform in [nmin, nmax], aspect U[0.5, 2], box 1.5-3x the block."""
    rng = np.random.default_rng(seed)
    out = []
    sp, r = 0.02, 0.01
    for s in range(nscenes):
        n = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        b, c = rng.uniform(0.5, 2.0, size=2)
        nx = max(2, round((n / (b * c)) ** (1.0 / 3.0)))
        dims = (nx, max(2, round(nx * b)), max(2, round(nx * c)))
        ext = [sp * (k + 1) for k in dims]
        f = rng.uniform(1.5, 3.0, size=3)
        hi = tuple(float(ext[a] * f[a]) for a in range(3))
        out.append(dam_break(dims, sp, r, 0.002, (0.0, 0.0, 0.0), hi, seed=seed * 1000003 + s, dt=1.0e-3,
                             name=f"batched_{s}"))
    return out


def adjoint_16k(seed: int = 0) -> Scene:
    """32 x 32 x 16 block (r = 0.01) in a unit box, v0 ~ N(0, 0.1) per component, 30 fixed
    iterations per solve (Jacobi viscosity / surface tension), 200 steps."""
    sc = dam_break((32, 32, 16), 0.02, 0.01, 0.002, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), seed=seed, dt=1.0e-3,
                   name="adjoint_16k", steps=200, config=dict(fixed_iters=30, visc_solver=L.VISC_JACOBI))
    rng = np.random.default_rng(seed + 17)
    sc.vel4[:, :3] = rng.normal(0.0, 0.1, size=(sc.n, 3)).astype(np.float32)
    sc.meta["target"] = tuple(float(t) for t in rng.uniform(0.3, 0.7, size=3))
    return sc


def adjoint_scenes(nscenes: int = 32, seed: int = 0) -> list[Scene]:
    """The adjoint benchmark's batch: `nscenes` seeded adjoint_16k scenes, each with its target."""
    return [adjoint_16k(seed * 1000003 + s) for s in range(nscenes)]


def reference_surface_tension(size: int = 5) -> Scene:
    """mps::System::SurfaceTensionTestScene (MPSSystem.cpp:552-651) with Initalize's constants."""
    radius = 0.1
    f32 = lambda v: float(np.float32(v))  # the reference writes 0.9f and 0.001f literals
    gap = radius * f32(0.9)
    offset = f32(0.001)
    stride = gap + gap + offset
    l = stride * (size - 1) + gap + gap
    start = -l
    lo = (start - l * 0.025 + gap - 3.5, start + gap - 3.5, start + gap - 3.5)
    hi = (l * 0.025 + (size - 1) * stride + gap + 3.5, start + (size - 1) * stride + gap + 3.5,
          start + (size - 1) * stride + gap + 3.5)
    mat = reference_material(4 * radius)
    pos = []
    for z in range(size):
        for y in range(size):
            for x in range(size):
                pos.append((start - l * 0.025 + x * stride + gap, start + y * stride + gap, start + z * stride + gap))
                pos.append((l * 0.025 + x * stride + gap, start + y * stride + gap, start + z * stride + gap))
    pos = np.array(pos, np.float64)
    n = pos.shape[0]
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos
    pos4[:, 3] = radius
    vel4 = np.zeros((n, 4), np.float32)
    vel4[:, 3] = mat["mass"]
    walls = gen_walls(lo, hi, 2 * (0.25 * mat["radius"]), 0.25 * mat["radius"])
    phys = dict(dt=0.005, gravity=(0.0, -9.8, 0.0), min=lo, max=hi)
    cfg = dict(kernel=L.KERNEL_POLY6_SPIKY)
    return Scene("reference_surface_tension", pos4, vel4, walls, mat, phys, cfg, 1,
                 dict(pos_f64=pos, hash_cell=4 * radius, hash_size=(64, 64, 64)))


def reference_viscosity(height: int = 300, size: int = 5) -> Scene:
    """mps::System::ViscosityTestScene (MPSSystem.cpp:455-551, commented out in Initalize): a
    size x size x height column with the reference's literals (0.9f, 0.001f), unit mass as the
    scene sets it before the material's mass overrides it, box walls as in the surface-tension
    scene (the mesh-sampled cube of the reference is not shipped)."""
    radius = 0.1
    f32 = lambda v: float(np.float32(v))
    gap = radius * f32(0.9)
    offset = f32(0.001)
    stride = gap + gap + offset
    lw = stride * (size - 1) + gap + gap
    start = -lw * f32(0.5)
    start_h = 0.0
    lo = (start + gap - 5.5, start_h - 1.0, start + gap - 5.5)
    hi = (start + (size - 1) * stride + gap + 5.5, start_h + (height - 1) * stride + gap + 5.5,
          start + (size - 1) * stride + gap + 5.5)
    mat = reference_material(4 * radius)
    pos = [(start + x * stride + gap, start + y * stride + gap, start + z * stride + gap)
           for y in range(height) for z in range(size) for x in range(size)]
    pos = np.array(pos, np.float64)
    n = pos.shape[0]
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos
    pos4[:, 3] = radius
    vel4 = np.zeros((n, 4), np.float32)
    vel4[:, 3] = mat["mass"]
    walls = gen_walls(lo, hi, 2 * (0.25 * mat["radius"]), 0.25 * mat["radius"])
    phys = dict(dt=0.005, gravity=(0.0, -9.8, 0.0), min=lo, max=hi)
    cfg = dict(kernel=L.KERNEL_POLY6_SPIKY)
    return Scene("reference_viscosity", pos4, vel4, walls, mat, phys, cfg, 1,
                 dict(pos_f64=pos, hash_cell=4 * radius, hash_size=(64, 64, 64)))


CONFIGS = {
    "dam_break_32k": dam_break_32k,
    "dam_break_1m": dam_break_1m,
    "dam_break_512k": dam_break_512k,
    "colliding_4m": colliding_4m,
    "adjoint_16k": adjoint_16k,
    "reference_surface_tension": reference_surface_tension,
    "reference_viscosity": reference_viscosity,
}
