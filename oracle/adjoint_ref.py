"""FP64 unrolled host gradient of a DFSPH rollout -- TEST INFRASTRUCTURE ONLY (the checker of the
GPU adjoint, never a product path).

A PyTorch float64 CPU restatement of the differentiated step (the adjoint form's forward, fixed
iteration counts, 3x3 block-Jacobi viscosity / surface-tension solve): density and alpha, gravity,
K divergence-free iterations, the viscosity + surface tension + XSPH system by K block-Jacobi sweeps,
K constant-density iterations, box collision and advection.  Neighbour pairs are found by brute
force (a k-d tree for large sets) from the detached positions with the reference's test
|x_i - x_j| < (h_i + h_j) / 2
(MPSSPHKernel.cuh:17-26), so they are piecewise constant in x exactly as in the GPU adjoint.
`torch.autograd` of this forward is the FP64 reference gradient; the forward itself is pinned
against the C++ FP64 oracle (mps_oracle.cpp, visc_solver = 1) at the same settings.

Formulas: kernels MPSSPHKernel.cuh:28-84; density MPSSPHBaseUtil.cuh:88-203; alpha, divergence-free
and constant-density iterations MPSSPHDFSPHUtil.cuh:10-468 with the drivers' order
MPSSPHDFSPHUtil.cu:270-441; surface tension / XSPH / viscosity terms MPSSPHNonPressureUtil.cuh:425-648;
collision and advection MPSAdvectUtil.cuh:36-77; boundary volume MPSSPHBaseUtil.cuh:10-86.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

PI = math.pi
KW = 315.0 / (64.0 * PI)
KG = 45.0 / PI
KCW = 8.0 / PI
KCG = 48.0 / PI
KSTW = 8.0 / PI * 10.0 / 7.0 * 2.0
KSTG = 48.0 / PI * 10.0 / 7.0
FLT_EPS = 1.1920928955078125e-07
H_RATIO = 4.0


def kern_w(r, h, cubic: bool):
    q = r / h
    ih = 1.0 / h
    if cubic:
        outer = 2.0 * KCW * (1.0 - q) ** 3 * ih ** 3
        inner = KCW * ih ** 3 * ((6.0 * q - 6.0) * q * q + 1.0)
        w = torch.where(q >= 0.5, outer, inner)
    else:
        w = KW * ((1.0 - q * q) * ih) ** 3
    return torch.where(q < 1.0, w, torch.zeros_like(w))


def kern_g(r, h, cubic: bool):
    """G with grad W = G x_ij (r > 0 for every pair)."""
    q = r / h
    ih = 1.0 / h
    if cubic:
        outer = -KCG / r * ((1.0 - q) * ih * ih) ** 2
        inner = KCG * ih ** 5 * (3.0 * q - 2.0)
        g = torch.where(q > 0.5, outer, inner)
    else:
        g = -KG / r * ((1.0 - q) * ih * ih) ** 2
    return torch.where(q < 1.0, g, torch.zeros_like(g))


def kern_stw(r, h):
    q = torch.clamp(r / h, min=0.5)
    w = KSTW * ((1.0 - q) / h) ** 3
    return torch.where(q < 1.0, w, torch.zeros_like(w))


def kern_stg(r, h):
    q = r / h
    g = -KSTG / r * ((1.0 - q) / (h * h)) ** 2
    return torch.where((q > 0.5) & (q < 1.0), g, torch.zeros_like(g))


@dataclass
class RefScene:
    """One scene: fluid (N, 4) pos (x, y, z, radius) and vel (vx, vy, vz, mass), boundary (B, 4)."""
    pos4: np.ndarray
    vel4: np.ndarray
    bpos4: np.ndarray
    material: dict
    physics: dict
    cubic: bool
    iters: int
    bvol: np.ndarray | None = None


def pairs(x: torch.Tensor, h: torch.Tensor, y: torch.Tensor | None = None, hy: torch.Tensor | None = None):
    """Index pairs (i, j) with |x_i - y_j| < (h_i + h_j) / 2 (i != j when y is x)."""
    same = y is None
    y = x if same else y
    hy = h if same else hy
    if x.shape[0] * y.shape[0] > 2 ** 24:
        return _pairs_tree(x, h, y, hy, same)
    d = torch.cdist(x, y)
    m = d < 0.5 * (h[:, None] + hy[None, :])
    if same:
        m.fill_diagonal_(False)
    I, J = torch.nonzero(m, as_tuple=True)
    return I, J


def _pairs_tree(x, h, y, hy, same):
    """The same pairs through a k-d tree (large sets): candidates within the largest support, then
    the exact test."""
    from scipy.spatial import cKDTree
    xn, yn = x.numpy(), y.numpy()
    rmax = float(0.5 * (h.max() + hy.max()))
    ta = cKDTree(xn)
    tb = ta if same else cKDTree(yn)
    coo = ta.sparse_distance_matrix(tb, rmax, output_type="ndarray")
    I = torch.from_numpy(coo["i"].astype(np.int64))
    J = torch.from_numpy(coo["j"].astype(np.int64))
    d = (x[I] - y[J]).norm(dim=1)
    m = d < 0.5 * (h[I] + hy[J])
    if same:
        m &= I != J
    I, J = I[m], J[m]
    order = torch.argsort(I * y.shape[0] + J)
    return I[order], J[order]


def boundary_volume(bpos4: np.ndarray, cubic: bool) -> np.ndarray:
    """V_b = 1 / (W(0) + sum_k W(x_b - x_k)) over boundary neighbours (h of b)."""
    x = torch.tensor(bpos4[:, :3], dtype=torch.float64)
    h = torch.tensor(bpos4[:, 3], dtype=torch.float64) * H_RATIO
    I, J = pairs(x, h)
    r = (x[I] - x[J]).norm(dim=1)
    s = kern_w(torch.zeros_like(h), h, cubic).clone()
    s.index_add_(0, I, kern_w(r, h[I], cubic))
    return (1.0 / s).numpy()


class Rollout:
    """FP64 forward of `nsteps` steps; call with tensors to differentiate."""

    def __init__(self, scene: RefScene):
        self.sc = scene
        m, ph = scene.material, scene.physics
        self.rho0 = float(m["density"])
        self.V = float(m["volume"])
        self.xsph = float(m["xsph"])
        self.dt = float(ph["dt"])
        self.g = torch.tensor(ph["gravity"], dtype=torch.float64)
        self.lo = torch.tensor(ph["min"], dtype=torch.float64)
        self.hi = torch.tensor(ph["max"], dtype=torch.float64)
        self.h = torch.tensor(scene.pos4[:, 3], dtype=torch.float64) * H_RATIO
        self.mass = torch.tensor(scene.vel4[:, 3], dtype=torch.float64)
        self.bx = torch.tensor(scene.bpos4[:, :3], dtype=torch.float64)
        self.bh = torch.tensor(scene.bpos4[:, 3], dtype=torch.float64) * H_RATIO
        bv = scene.bvol if scene.bvol is not None else boundary_volume(scene.bpos4, scene.cubic)
        self.bvol = torch.tensor(bv, dtype=torch.float64)
        self.K = int(scene.iters)
        self.cubic = bool(scene.cubic)
        self.factor = 0.01

    def step(self, x, v, visc, sigma):
        dt, V, rho0, cubic, K = self.dt, self.V, self.rho0, self.cubic, self.K
        h, m = self.h, self.mass
        n = x.shape[0]
        with torch.no_grad():
            I, J = pairs(x.detach(), h)
            IB, B = pairs(x.detach(), h, self.bx, self.bh)
        hI = h[I]
        e = x[I] - x[J]
        r = e.norm(dim=1)
        eb = x[IB] - self.bx[B]
        rb = eb.norm(dim=1)
        vb = self.bvol[B]
        hb = h[IB]
        Wf, Gf = kern_w(r, hI, cubic), kern_g(r, hI, cubic)
        Wb, Gb = kern_w(rb, hb, cubic), kern_g(rb, hb, cubic)

        def ssum(vals, idx):
            out = torch.zeros((n,) + vals.shape[1:], dtype=vals.dtype)
            return out.index_add(0, idx, vals)

        # density and alpha
        rho = rho0 * (V * kern_w(torch.zeros_like(h), h, cubic) + ssum(V * Wf, I) + ssum(vb * Wb, IB))
        gp = (V * Gf)[:, None] * e
        gs = ssum(gp, I) + ssum((vb * Gb)[:, None] * eb, IB)
        f = ssum((gp * gp).sum(1), I) + (gs * gs).sum(1)
        alpha = torch.where(f > 1.0e-20, 1.0 / torch.where(f > 1.0e-20, f, torch.ones_like(f)), torch.zeros_like(f))
        massive = (m > 1.0e-10)[:, None]
        v = v + torch.where(massive, dt * self.g[None, :], torch.zeros_like(v))

        def pressure(v, divergence: bool):
            for _ in range(K):
                delta = ssum(V * Gf * (e * (v[I] - v[J])).sum(1), I) + ssum(vb * Gb * (eb * v[IB]).sum(1), IB)
                ratio = rho / rho0
                k = torch.minimum(delta * dt, ratio + dt * delta - 0.8) if divergence else ratio + dt * delta - 1.0
                kap = torch.where(k > 0.0, k * alpha / (dt * dt), torch.zeros_like(k))
                ff = -ssum((0.5 * V * (kap[I] + kap[J]) * Gf)[:, None] * e, I)
                fb = -ssum((0.5 * vb * kap[IB] * Gb)[:, None] * eb, IB)
                v = v + torch.where(massive, dt * (ff + fb), torch.zeros_like(v))
            return v

        v = pressure(v, True)

        # viscosity + surface tension + XSPH, K Jacobi sweeps
        sf = ssum(m[J] * Gf * (e * (v[I] - v[J])).sum(1), I)
        invD = 2.0 / (rho[I] + rho[J])
        stw = kern_stw(r, hI)
        stg = kern_stg(r, hI)
        vdot = stg * (e * (v[I] - v[J])).sum(1)
        gij = (stw + dt * (vdot - (sf[I] + sf[J]) * invD * 0.5 * stw)) * invD
        mbar = 0.5 * (m[I] + m[J])
        c = mbar * gij
        st_scale = dt * sigma / m
        b = v + st_scale[:, None] * ssum(-c[:, None] * e, I)
        cij = st_scale[I] * c + (self.xsph / dt) * (m[J] / rho[J]) * Wf
        cv = 10.0 * rho0 * visc / rho[I] * mbar / rho[J] / (r * r + 0.01 * hI * hI) * Gf / (r + FLT_EPS)
        fct = self.factor
        eye = torch.eye(3, dtype=torch.float64)
        D = ((1.0 + fct) + dt * ssum(cij, I))[:, None, None] * eye - dt * ssum(cv[:, None, None] * (e[:, :, None] * e[:, None, :]), I)
        ok = (torch.linalg.det(D) > 1.0e-30)[:, None, None]
        Dinv = torch.where(ok, torch.linalg.inv(torch.where(ok, D, eye)), eye / (1.0 + fct))
        x0 = v
        q = v
        for _ in range(K):
            p = q[I] - q[J]
            acc = ssum(cij[:, None] * p - (cv * (p * e).sum(1))[:, None] * e, I)
            Aq = q * (1.0 + fct) + dt * acc
            q = q + (Dinv @ (b + fct * x0 - Aq)[:, :, None])[:, :, 0]
        v = q

        v = pressure(v, False)

        # collision + position
        xn = x + v * dt
        out = ((xn < self.lo) & (v < 0.0)) | ((xn > self.hi) & (v > 0.0))
        vc = torch.where(out, torch.where(v.abs() < 1.0e-4, torch.zeros_like(v), -0.4 * v), v)
        return x + dt * vc, vc

    def run(self, x, v, visc, sigma, nsteps: int):
        for _ in range(nsteps):
            x, v = self.step(x, v, visc, sigma)
        return x, v


def gradient(scene: RefScene, nsteps: int, gx: np.ndarray, gv: np.ndarray):
    """FP64 vector-Jacobian product of the rollout: (d/dx0, d/dv0, d/dvisc, d/dsigma) of
    sum(gx * x_T) + sum(gv * v_T), and the final state."""
    R = Rollout(scene)
    x0 = torch.tensor(scene.pos4[:, :3], dtype=torch.float64, requires_grad=True)
    v0 = torch.tensor(scene.vel4[:, :3], dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(float(scene.material["viscosity"]), dtype=torch.float64, requires_grad=True)
    sg = torch.tensor(float(scene.material["surface_tension"]), dtype=torch.float64, requires_grad=True)
    xT, vT = R.run(x0, v0, mu, sg, nsteps)
    L = (xT * torch.tensor(gx, dtype=torch.float64)).sum() + (vT * torch.tensor(gv, dtype=torch.float64)).sum()
    L.backward()
    return (x0.grad.numpy(), v0.grad.numpy(), float(mu.grad), float(sg.grad), xT.detach().numpy(),
            vT.detach().numpy())


def forward(scene: RefScene, nsteps: int, x0=None, v0=None, visc=None, sigma=None):
    """FP64 forward without gradients (central finite differences)."""
    R = Rollout(scene)
    with torch.no_grad():
        x = torch.tensor(scene.pos4[:, :3] if x0 is None else x0, dtype=torch.float64)
        v = torch.tensor(scene.vel4[:, :3] if v0 is None else v0, dtype=torch.float64)
        mu = torch.tensor(float(scene.material["viscosity"] if visc is None else visc), dtype=torch.float64)
        sg = torch.tensor(float(scene.material["surface_tension"] if sigma is None else sigma), dtype=torch.float64)
        xT, vT = R.run(x, v, mu, sg, nsteps)
    return xT.numpy(), vT.numpy()
