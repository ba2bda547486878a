"""Adjoint (reverse-mode) form of the step.

CPU: the FP64 torch restatement of the differentiated step (oracle/adjoint_ref.py) is pinned
against the C++ FP64 oracle's forward (same fixed iterations, Jacobi viscosity solve), and its
torch.autograd gradient against FP64 central finite differences (eps = 1e-4 relative).

GPU (through the C ABI): the Jacobi viscosity / surface-tension solve against the oracle; the
adjoint's vector-Jacobian product against the FP64 host gradient and against FP64 central finite
differences (tolerance 1e-3 relative: FP32 kernels vs FP64); batched scenes equal single-scene
runs; the handle is left at the final state; the torch.autograd wrapper and the loss.
"""
import numpy as np
import pytest

K = 4


def small_scene(mps, dims=(6, 6, 4), seed=3, K=K, box=0.2, vel_sigma=0.1):
    from mps_cuda_gb300 import scenes
    sc = scenes.dam_break(dims, 0.02, 0.01, 0.002, (0.0, 0.0, 0.0), (box, box, box), seed=seed, dt=1.0e-3,
                          name="adjoint_small", config=dict(fixed_iters=K, visc_solver=mps.VISC_JACOBI),
                          origin=(0.02, 0.02, 0.02))
    rng = np.random.default_rng(seed + 101)
    sc.vel4[:, :3] = rng.normal(0.0, vel_sigma, size=(sc.n, 3)).astype(np.float32)
    return sc


def ref_of(sc, K=K):
    from oracle import adjoint_ref as A
    return A.RefScene(sc.pos4, sc.vel4, sc.bpos4, sc.material, sc.physics, True, K)


def rel_norm(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ----------------------------------------------------------------------------------- CPU
def test_host_forward_matches_oracle(mps, orc):
    from oracle import adjoint_ref as A
    sc = small_scene(mps)
    xT, vT = A.forward(ref_of(sc), 3)
    o = orc.from_scene(sc, config=dict(fixed_iters=K, visc_solver=1))
    o.step(3)
    assert rel_norm(xT, o.get("pos")) < 1e-10
    assert rel_norm(vT, o.get("vel")) < 1e-9


def test_host_boundary_volume_matches_oracle(mps, orc):
    from oracle import adjoint_ref as A
    sc = small_scene(mps)
    o = orc.from_scene(sc, config=dict(fixed_iters=K, visc_solver=1))
    o.phase(orc.NEIGHBORS)
    o.phase(orc.BVOLUME)
    assert rel_norm(A.boundary_volume(sc.bpos4, True), o.get("bvol")) < 1e-12


def test_host_gradient_matches_finite_differences(mps):
    from oracle import adjoint_ref as A
    sc = small_scene(mps)
    R = ref_of(sc)
    rng = np.random.default_rng(7)
    gx = rng.normal(size=(sc.n, 3))
    gv = rng.normal(size=(sc.n, 3))
    steps = 3
    dx0, dv0, dmu, dsg, _, _ = A.gradient(R, steps, gx, gv)

    def loss(**kw):
        xT, vT = A.forward(R, steps, **kw)
        return float((gx * xT).sum() + (gv * vT).sum())

    v0 = sc.vel4[:, :3].astype(np.float64)
    x0 = sc.pos4[:, :3].astype(np.float64)
    u = rng.normal(size=v0.shape)
    eps = 1e-4 * np.abs(v0).max()
    fd = (loss(v0=v0 + eps * u) - loss(v0=v0 - eps * u)) / (2 * eps)
    assert abs(fd - (dv0 * u).sum()) <= 1e-5 * abs(fd)
    # positions move densities across the stiffness clamp max(0, .) at a step of 1e-4 spacing
    # (a kink of the loss, 0.6 % off here); 1e-6 spacing stays within one smooth piece
    eps = 1e-6 * 0.02
    fd = (loss(x0=x0 + eps * u) - loss(x0=x0 - eps * u)) / (2 * eps)
    assert abs(fd - (dx0 * u).sum()) <= 1e-5 * abs(fd)
    for name, g in (("viscosity", dmu), ("surface_tension", dsg)):
        val = float(sc.material[name])
        eps = 1e-4 * val
        kw_p = {"visc" if name == "viscosity" else "sigma": val + eps}
        kw_m = {"visc" if name == "viscosity" else "sigma": val - eps}
        fd = (loss(**kw_p) - loss(**kw_m)) / (2 * eps)
        assert abs(fd - g) <= 1e-5 * abs(fd), (name, fd, g)


def test_com_loss_gradient():
    import torch
    from mps_cuda_gb300.adjoint import com_loss
    rng = np.random.default_rng(1)
    x = torch.tensor(rng.normal(size=(10, 3)), requires_grad=True)
    v = torch.tensor(rng.normal(size=(10, 3)), requires_grad=True)
    m = torch.full((10,), 2.0, dtype=torch.float64)
    t = torch.tensor([[0.1, 0.2, 0.3], [0.0, 0.0, 0.0]], dtype=torch.float64)
    L = com_loss(x, v, m, [0, 4, 10], t)
    assert L.shape == (2,)
    L.sum().backward()
    com0 = x.detach()[:4].mean(0)
    assert np.allclose(x.grad[:4].numpy(), np.tile(2 * (com0 - t[0]).numpy() / 4, (4, 1)))
    assert np.allclose(v.grad[:4].numpy(), 2e-3 * v.detach()[:4].numpy() / 4)


# ----------------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("fixed", [0, 6])
def test_jacobi_solve_vs_oracle(mps, orc, fixed):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=5)
    cfg = dict(fixed_iters=fixed, visc_solver=mps.VISC_JACOBI)
    sim = Simulation.from_scene(sc, **cfg)
    o = orc.from_scene(sc, config=dict(cfg, visc_solver=1))
    for ph in (mps.PHASE_SORT, mps.PHASE_NEIGHBORS, mps.PHASE_BVOLUME, mps.PHASE_DENSITY_ALPHA, mps.PHASE_DF):
        sim.phase(ph)
    for ph in (0, 1, 2, 3, 4, 5, orc.DF):
        o.phase(ph)
    v = sim.get_field("vel")
    v[:, :3] = o.get("vel")
    sim.put_field("vel", v)
    sim.phase(mps.PHASE_VISCST)
    o.phase(orc.VISCST)
    gi, oi = sim.stats()["cg_iters"], o.stats()["cg_iters"]
    if fixed:
        assert gi == oi == fixed + 1
    else:
        assert abs(gi - oi) <= 1, (gi, oi)
    if gi == oi:
        g, r = sim.get_field("vel")[:, :3], o.get("vel")
        assert np.abs(g - r).max() / np.abs(r).max() < 1e-5


@pytest.mark.gpu
def test_jacobi_graph_equals_eager(mps):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=9)
    a = Simulation.from_scene(sc, use_graph=1, visc_solver=mps.VISC_JACOBI)
    b = Simulation.from_scene(sc, use_graph=0, visc_solver=mps.VISC_JACOBI)
    a.step(3)
    b.step(3)
    pa, va = a.get_fluid()
    pb, vb = b.get_fluid()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    assert a.stats()["cg_iters"] == b.stats()["cg_iters"] > 1


def _gpu_vjp(mps, sc, steps, every, gx, gv):
    from mps_cuda_gb300 import Simulation
    from mps_cuda_gb300.adjoint import AdjointRollout
    sim = Simulation.from_scene(sc)
    roll = AdjointRollout(sim, steps, every)
    pT, vT = roll.forward()
    g4x = np.zeros((sc.n, 4), np.float32)
    g4v = np.zeros((sc.n, 4), np.float32)
    g4x[:, :3] = gx
    g4v[:, :3] = gv
    op, ov, par = roll.backward(g4x, g4v)
    return sim, roll, pT, vT, op, ov, par


@pytest.mark.gpu
def test_adjoint_matches_fp64_host_gradient(mps):
    from oracle import adjoint_ref as A
    sc = small_scene(mps)
    rng = np.random.default_rng(11)
    gx = rng.normal(size=(sc.n, 3)).astype(np.float32)
    gv = rng.normal(size=(sc.n, 3)).astype(np.float32)
    steps = 6
    _, _, pT, vT, op, ov, par = _gpu_vjp(mps, sc, steps, 4, gx, gv)
    dx0, dv0, dmu, dsg, xT, vTr = A.gradient(ref_of(sc), steps, gx.astype(np.float64), gv.astype(np.float64))
    assert rel_norm(pT[:, :3], xT) < 1e-5
    assert rel_norm(vT[:, :3], vTr) < 1e-3
    assert rel_norm(ov[:, :3], dv0) < 1e-3
    assert rel_norm(op[:, :3], dx0) < 1e-3
    assert abs(par[0, 0] - dmu) <= 1e-3 * abs(dmu)
    assert abs(par[0, 1] - dsg) <= 1e-3 * abs(dsg)
    assert np.all(op[:, 3] == 0) and np.all(ov[:, 3] == 0)


@pytest.mark.gpu
def test_adjoint_matches_finite_differences(mps):
    """Directional derivatives of the GPU gradient against FP64 central differences."""
    from oracle import adjoint_ref as A
    sc = small_scene(mps, seed=8)
    R = ref_of(sc)
    rng = np.random.default_rng(5)
    gx = rng.normal(size=(sc.n, 3)).astype(np.float32)
    gv = rng.normal(size=(sc.n, 3)).astype(np.float32)
    steps = 5
    _, _, _, _, op, ov, par = _gpu_vjp(mps, sc, steps, 2, gx, gv)

    def loss(**kw):
        xT, vT = A.forward(R, steps, **kw)
        return float((gx * xT).sum() + (gv * vT).sum())

    v0 = sc.vel4[:, :3].astype(np.float64)
    u = rng.normal(size=v0.shape)
    eps = 1e-4 * np.abs(v0).max()
    fd = (loss(v0=v0 + eps * u) - loss(v0=v0 - eps * u)) / (2 * eps)
    assert abs(fd - (ov[:, :3] * u).sum()) <= 1e-3 * abs(fd)
    for k, name, key in ((0, "viscosity", "visc"), (1, "surface_tension", "sigma")):
        val = float(sc.material[name])
        eps = 1e-4 * val
        fd = (loss(**{key: val + eps}) - loss(**{key: val - eps})) / (2 * eps)
        assert abs(fd - par[0, k]) <= 1e-3 * abs(fd), (name, fd, par[0, k])


@pytest.mark.gpu
def test_adjoint_batched_equals_single(mps):
    from mps_cuda_gb300 import BatchedSimulation
    from mps_cuda_gb300.adjoint import AdjointRollout
    scs = [small_scene(mps, dims=d, seed=s) for d, s in (((6, 6, 4), 1), ((5, 7, 4), 2), ((6, 5, 5), 3))]
    rng = np.random.default_rng(3)
    gxs = [rng.normal(size=(s.n, 3)).astype(np.float32) for s in scs]
    gvs = [rng.normal(size=(s.n, 3)).astype(np.float32) for s in scs]
    bs = BatchedSimulation(scs)
    roll = AdjointRollout(bs, 4, 3)
    roll.forward()
    g4x = np.zeros((bs.n, 4), np.float32)
    g4v = np.zeros((bs.n, 4), np.float32)
    g4x[:, :3] = np.concatenate(gxs)
    g4v[:, :3] = np.concatenate(gvs)
    op, ov, par = roll.backward(g4x, g4v)
    off = bs.offsets
    for s, sc in enumerate(scs):
        _, _, _, _, op1, ov1, par1 = _gpu_vjp(mps, sc, 4, 3, gxs[s], gvs[s])
        a, b = off[s], off[s + 1]
        assert np.array_equal(op[a:b], op1) and np.array_equal(ov[a:b], ov1)
        assert np.allclose(par[s], par1[0], rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_adjoint_leaves_final_state(mps):
    from mps_cuda_gb300 import Simulation
    from mps_cuda_gb300.adjoint import AdjointRollout
    sc = small_scene(mps)
    sim = Simulation.from_scene(sc)
    roll = AdjointRollout(sim, 5, 2)
    pT, vT = roll.forward()
    st = sim.stats()
    roll.backward(np.ones((sc.n, 4), np.float32), None)
    p2, v2 = sim.get_fluid()
    assert np.array_equal(pT, p2) and np.array_equal(vT, v2)
    st2 = sim.stats()
    assert st2["steps"] == st["steps"] and st2["iters_total"] == st["iters_total"]
    # a second backward from the same forward gives the same gradient
    a = roll.backward(np.ones((sc.n, 4), np.float32), None)
    b = roll.backward(np.ones((sc.n, 4), np.float32), None)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.gpu
def test_adjoint_rejects_unsupported_config(mps):
    from mps_cuda_gb300 import MpsError, Simulation
    from mps_cuda_gb300.adjoint import AdjointRollout
    sc = small_scene(mps)
    for cfg in (dict(visc_solver=mps.VISC_CG), dict(fixed_iters=0)):
        sim = Simulation.from_scene(sc, **cfg)
        with pytest.raises(MpsError):
            AdjointRollout(sim, 2, 1).forward()
    sim = Simulation.from_scene(sc)
    with pytest.raises(MpsError):
        AdjointRollout(sim, 2, 1).backward(None, None)   # no forward recorded


@pytest.mark.gpu
def test_autograd_rollout_and_com_loss(mps):
    import torch
    from mps_cuda_gb300 import Simulation
    from mps_cuda_gb300.adjoint import AdjointRollout, com_loss, rollout
    sc = small_scene(mps)
    sim = Simulation.from_scene(sc)
    roll = AdjointRollout(sim, 4, 2)
    x0 = torch.tensor(sc.pos4[:, :3], dtype=torch.float64, requires_grad=True)
    v0 = torch.tensor(sc.vel4[:, :3], dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(sc.material["viscosity"], dtype=torch.float64, requires_grad=True)
    sg = torch.tensor(sc.material["surface_tension"], dtype=torch.float64, requires_grad=True)
    xT, vT = rollout(roll, x0, v0, mu, sg)
    m = torch.tensor(sc.vel4[:, 3], dtype=torch.float64)
    L = com_loss(xT, vT, m, [0, sc.n], torch.tensor([[0.1, 0.05, 0.1]], dtype=torch.float64)).sum()
    L.backward()
    for t in (x0, v0, mu, sg):
        assert t.grad is not None and torch.isfinite(t.grad).all()
    # the same cotangents through the C ABI directly
    xT2 = xT.detach().clone().requires_grad_(True)
    vT2 = vT.detach().clone().requires_grad_(True)
    com_loss(xT2, vT2, m, [0, sc.n], torch.tensor([[0.1, 0.05, 0.1]], dtype=torch.float64)).sum().backward()
    g4x = np.zeros((sc.n, 4), np.float32)
    g4v = np.zeros((sc.n, 4), np.float32)
    g4x[:, :3] = xT2.grad.numpy()
    g4v[:, :3] = vT2.grad.numpy()
    op, ov, par = roll.backward(g4x, g4v)
    assert np.allclose(v0.grad.numpy(), ov[:, :3], rtol=0, atol=1e-12)
    assert abs(float(mu.grad) - par[0, 0]) <= 1e-12 * max(1.0, abs(par[0, 0]))


@pytest.mark.gpu
def test_adjoint_poly6_kernel_matches_host_gradient(mps):
    """The reference's shipped kernel pair (poly6 W, spiky gradient)."""
    from oracle import adjoint_ref as A
    sc = small_scene(mps, seed=12)
    sc.config["kernel"] = mps.KERNEL_POLY6_SPIKY
    rng = np.random.default_rng(21)
    gx = rng.normal(size=(sc.n, 3)).astype(np.float32)
    gv = rng.normal(size=(sc.n, 3)).astype(np.float32)
    _, _, pT, vT, op, ov, par = _gpu_vjp(mps, sc, 4, 2, gx, gv)
    R = A.RefScene(sc.pos4, sc.vel4, sc.bpos4, sc.material, sc.physics, False, K)
    dx0, dv0, dmu, dsg, xT, _ = A.gradient(R, 4, gx.astype(np.float64), gv.astype(np.float64))
    assert rel_norm(pT[:, :3], xT) < 1e-5
    assert rel_norm(ov[:, :3], dv0) < 1e-3
    assert rel_norm(op[:, :3], dx0) < 1e-3
    assert abs(par[0, 0] - dmu) <= 1e-3 * abs(dmu)
    assert abs(par[0, 1] - dsg) <= 1e-3 * abs(dsg)
