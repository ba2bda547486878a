"""Parity of the CUDA step (through the C ABI) against the FP64 oracle.

Tolerances (FP32 bulk vs FP64 oracle, same inputs):
  - integer work (cell keys, sort permutation, cell ranges, FP32 neighbour counts): bit-exact
    against the oracle's restatement of the same FP32 scheme; neighbour counts against the
    reference's FP64 test differ only for pairs within 1e-6 h of the support radius.
  - densities, alphas, pressure factors, velocities after a phase, from an identical state:
    max|a - b| / max|b| <= 1e-5 (the per-step bound: 1e-5 relative to an FP64 oracle).
    "Identical state": the GPU's FP32 state is what both sides start from (the oracle takes it
    exactly, FP32 values being FP64 values), before the step and before each solver phase.  The
    pressure factor from an identical state is the stiffness of a solve's first iteration
    (fixed_iters = 1); after further iterations the two sides' velocities already differ by their
    own rounding.
Solver phases are compared in fixed-iteration mode (same number of Jacobi / CG iterations on
both sides) and, in adaptive mode, by iteration counts within one iteration.
"""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-5


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def make(mps, orc, scene, **cfg):
    from mps_cuda_gb300 import Simulation
    sim = Simulation.from_scene(scene, **cfg)
    o = orc.from_scene(scene, config=cfg)
    return sim, o


def gpu_state_to_oracle(sim, o):
    """The oracle continues from the GPU's current (FP32) fluid state."""
    p, v = sim.get_fluid()
    o.set_fluid(p[:, :3].astype(np.float64), v[:, :3].astype(np.float64), v[:, 3].astype(np.float64),
                p[:, 3].astype(np.float64))


def gpu_vel_to_oracle(sim, o):
    o.put("vel", sim.get_field("vel")[:, :3].astype(np.float64))


def advance_to_density(sim, o, mps):
    sim.phase(mps.PHASE_SORT)
    sim.phase(mps.PHASE_NEIGHBORS)
    sim.phase(mps.PHASE_BVOLUME)
    sim.phase(mps.PHASE_DENSITY_ALPHA)
    for ph in (0, 1, 2, 3, 4, 5):  # zsort(no-op), neighbours, volume, density, alpha, gravity
        o.phase(ph)


@pytest.fixture(params=["cubic", "poly6"])
def small(request, mps):
    from mps_cuda_gb300 import scenes
    k = mps.KERNEL_CUBIC_SPLINE if request.param == "cubic" else mps.KERNEL_POLY6_SPIKY
    return scenes.dam_break_small(10, seed=5, kernel=k)


def test_sort_keys_and_ranges_bit_exact(mps, orc):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(12, seed=2)
    sim = Simulation.from_scene(sc)
    sim.phase(mps.PHASE_SORT)
    g = sim.grid()
    grid = orc.grid(g["origin"], g["cell"], g["dims"])
    q4 = sc.pos4.copy()
    q4[:, 3] *= 4
    keys = orc.new_keys(q4, grid)
    sk, order = orc.new_stable_sort(keys, np.arange(sc.n, dtype=np.uint32))
    gpu_keys = sim.get_field("cell_key", order="slot")
    gpu_ids = sim.get_field("ids", order="slot")
    assert np.array_equal(gpu_keys, sk)
    assert np.array_equal(gpu_ids, order)
    # positions were moved with their particles
    assert np.array_equal(sim.get_field("pos", order="id")[:, :3], sc.pos4[:, :3])
    # the sort processes the significant bits of the scene's key space (2 x 2 columns: ny, nz even)
    nx, ny, nz = g["dims"]
    bits = max(1, int(nx * (ny + ny % 2) * (nz + nz % 2) - 1).bit_length())
    assert sim.stats()["sort_passes"] == -(-bits // sim.cfg.sort_digit_bits)


def test_neighbour_counts_bit_exact(mps, orc, small):
    sc = small
    from mps_cuda_gb300 import Simulation
    sim = Simulation.from_scene(sc)
    sim.phase(mps.PHASE_SORT)
    sim.phase(mps.PHASE_NEIGHBORS)
    g = sim.grid()
    grid = orc.grid(g["origin"], g["cell"], g["dims"])
    q4 = sc.pos4.copy(); q4[:, 3] *= 4
    b4 = sc.bpos4.copy(); b4[:, 3] *= 4
    kq_s, order = orc.new_stable_sort(orc.new_keys(q4, grid), np.arange(sc.n, dtype=np.uint32))
    kb_s, border = orc.new_stable_sort(orc.new_keys(b4, grid), np.arange(sc.nb, dtype=np.uint32))
    cf = orc.new_nbr_counts(q4[order], q4[order], kq_s, grid, True)
    cb = orc.new_nbr_counts(q4[order], b4[border], kb_s, grid, False)
    c = sim.get_field("nbr_count", order="slot")
    assert np.array_equal(c & 0xFFFF, cf)
    assert np.array_equal(c >> 16, cb)
    st = sim.stats()
    assert st["fluid_pairs"] == int(cf.sum()) and st["boundary_pairs"] == int(cb.sum())
    # against the reference's FP64 criterion
    o = orc.from_scene(sc)
    o.phase(orc.NEIGHBORS)
    ref = np.diff(o.get("nei_ff_idx"))
    gpu = sim.get_field("nbr_count", order="id") & 0xFFFF
    assert (gpu != ref).sum() <= max(1, sc.n // 10000)


def test_boundary_volume(mps, orc, small):
    sim, o = make(mps, orc, small)
    o.phase(orc.NEIGHBORS)
    o.phase(orc.BVOLUME)
    assert rel_err(sim.get_field("bvol", order="id"), o.get("bvol")) < REL


def test_density_alpha_gravity(mps, orc, small):
    sim, o = make(mps, orc, small)
    advance_to_density(sim, o, mps)
    assert rel_err(sim.get_field("density"), o.get("density")) < REL
    assert rel_err(sim.get_field("alpha"), o.get("alpha")) < REL
    assert np.abs(sim.get_field("color") - o.get("color")).max() < 1e-5
    assert rel_err(sim.get_field("vel")[:, :3], o.get("vel")) < REL


@pytest.mark.parametrize("fixed", [0, 1, 4])
def test_pressure_and_nonpressure_solves(mps, orc, small, fixed):
    sim, o = make(mps, orc, small, fixed_iters=fixed)
    advance_to_density(sim, o, mps)
    # each solve from an identical state: the GPU's velocities go into the oracle before it
    for gph, oph, name in ((mps.PHASE_DF, orc.DF, "df_iters"), (mps.PHASE_VISCST, orc.VISCST, "cg_iters"),
                           (mps.PHASE_CD, orc.CD, "cd_iters")):
        gpu_vel_to_oracle(sim, o)
        sim.phase(gph)
        o.phase(oph)
        gi, oi = sim.stats()[name], o.stats()[name]
        if fixed:
            assert gi == oi == fixed + 1, (name, gi, oi)
        else:
            assert abs(gi - oi) <= 1, (name, gi, oi)
        if gi == oi:
            assert rel_err(sim.get_field("vel")[:, :3], o.get("vel")) < REL, name
        if fixed == 1 and name != "cg_iters":
            # the stiffness of the solve's one iteration, from an identical state
            assert rel_err(sim.get_field("pressure"), o.get("pressure")) < REL, name


def test_advect(mps, orc, small):
    sim, o = make(mps, orc, small, fixed_iters=3)
    advance_to_density(sim, o, mps)
    for gph, oph in ((mps.PHASE_DF, orc.DF), (mps.PHASE_VISCST, orc.VISCST), (mps.PHASE_CD, orc.CD)):
        sim.phase(gph)
        o.phase(oph)
    gpu_vel_to_oracle(sim, o)
    sim.phase(mps.PHASE_ADVECT)
    o.phase(orc.ADVECT)
    assert rel_err(sim.get_field("pos")[:, :3], o.get("pos")) < 1e-6
    assert rel_err(sim.get_field("vel")[:, :3], o.get("vel")) < REL


def test_graph_step_equals_eager_phases(mps):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=9)
    a = Simulation.from_scene(sc, use_graph=1)
    b = Simulation.from_scene(sc, use_graph=0)
    a.step(3)
    b.step(3)
    pa, va = a.get_fluid()
    pb, vb = b.get_fluid()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    assert a.stats() ["cd_iters"] == b.stats()["cd_iters"]


def test_launched_solver_passes(mps):
    """Graph steps launch whole CG loop bodies (several passes each; the ones after the stop return
    at once): passes_total counts them, runs_total the passes that ran.  The DF and CD bodies hold
    one pass, and the host-driven form launches one pass per iteration."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=4)
    g = Simulation.from_scene(sc)
    g.step(3)
    st = g.stats()
    runs, passes = st["runs_total"], st["passes_total"]
    assert passes[0] == runs[0] and passes[2] == runs[2]
    assert runs[1] <= passes[1] < runs[1] + 3 * 4 and passes[1] % 4 == 0
    e = Simulation.from_scene(sc, use_graph=0)
    e.step(3)
    st = e.stats()
    assert st["passes_total"] == st["runs_total"]


def test_deterministic(mps):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=4)
    outs = []
    for _ in range(2):
        s = Simulation.from_scene(sc)
        s.step(4)
        outs.append(s.get_fluid())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_full_step_vs_oracle_fixed_iterations(mps, orc, small):
    sim, o = make(mps, orc, small, fixed_iters=5)
    sim.step(1)
    o.step(1)
    p, v = sim.get_fluid()
    assert rel_err(p[:, :3], o.get("pos")) < 1e-6
    assert rel_err(v[:, :3], o.get("vel")) < REL
    assert rel_err(sim.get_field("density"), o.get("density")) < REL


def test_reference_scene_step(mps, orc):
    """The reference's own scene (poly6/spiky, reference material, shipped tolerances), frame by
    frame from an identical state: the same iteration counts (or within one where a residual
    lands on the tolerance) and, where they are equal, the same positions and velocities."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.reference_surface_tension()
    sim = Simulation.from_scene(sc)
    o = orc.from_scene(sc)
    equal = 0
    for f in range(6):
        gpu_state_to_oracle(sim, o)
        o.set_frame(f)
        sim.step(1)
        o.step(1)
        st, ost = sim.stats(), o.stats()
        its = (st["df_iters"], st["cg_iters"], st["cd_iters"])
        oits = (ost["df_iters"], ost["cg_iters"], ost["cd_iters"])
        assert all(abs(a - b) <= 1 for a, b in zip(its, oits)), (f, its, oits)
        if its == oits:
            equal += 1
            p, v = sim.get_fluid()
            assert rel_err(p[:, :3], o.get("pos")) < 1e-6, f
            assert rel_err(v[:, :3], o.get("vel")) < REL, f
    assert equal >= 4


@pytest.mark.parametrize("form", [0, 1])
def test_batched_equals_single(mps, form):
    """Scenes stepped in one batch equal the same scenes stepped alone, bit for bit, in both CG
    arrangements."""
    from mps_cuda_gb300 import BatchedSimulation, Simulation, scenes
    scs = scenes.batched_scenes(4, seed=3, nmin=500, nmax=3000)
    b = BatchedSimulation(scs, cg_form=form)
    b.step(2)
    pb, vb = b.get_fluid()
    its = b.scene_iters()
    off = 0
    for k, sc in enumerate(scs):
        s = Simulation.from_scene(sc, cg_form=form)
        s.step(2)
        p, v = s.get_fluid()
        assert np.array_equal(p, pb[off:off + sc.n]) and np.array_equal(v, vb[off:off + sc.n]), k
        st = s.stats()
        assert (st["df_iters"], st["cg_iters"], st["cd_iters"]) == tuple(its[k])
        off += sc.n


def test_step_host_matches_device_step(mps):
    """The host-buffer call (load the state, step, store it) equals the same load + step through the
    device API bit for bit; against a run that keeps its cell order between steps it differs only by
    rounding (a reload starts from particle-ID order, which changes the order within each cell and
    so the summation order)."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(8, seed=6)
    a = Simulation.from_scene(sc)
    b = Simulation.from_scene(sc)
    c = Simulation.from_scene(sc)
    a.step(2)
    p = sc.pos4.copy()
    v = sc.vel4.copy()
    b.step_host(p, v, 1)
    p1, v1 = p.copy(), v.copy()
    b.step_host(p, v, 1)
    c.step(1)
    c.set_fluid(p1, v1)
    c.step(1)
    pc, vc = c.get_fluid()
    assert np.array_equal(p, pc) and np.array_equal(v, vc)
    pa, va = a.get_fluid()
    assert rel_err(p[:, :3], pa[:, :3]) < 1e-6
    assert rel_err(v[:, :3], va[:, :3]) < REL


@pytest.mark.parametrize("form", [0, 1])
def test_graph_with_cg_cap_equals_host_loop(mps, form):
    """A CG cap of 5 ends the solve inside a graph loop body (bodies hold several passes): the
    passes after the cap must change nothing, so the graph steps equal the host-driven loop bit
    for bit, in both CG forms."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=9)
    g = Simulation.from_scene(sc, cg_max_iter=5, cg_form=form)
    e = Simulation.from_scene(sc, cg_max_iter=5, cg_form=form, use_graph=0)
    g.step(2)
    e.step(2)
    assert g.stats()["cg_iters"] == e.stats()["cg_iters"]
    pg, vg = g.get_fluid()
    pe, ve = e.get_fluid()
    assert np.array_equal(pg, pe) and np.array_equal(vg, ve)


@pytest.mark.parametrize("unroll", [1, 3, 8])
def test_cg_unroll_changes_nothing(mps, unroll):
    """CG iterations per device-loop body (the autotuner's cg_unroll): the iterations after the
    stop return at once, so every value gives the same bits as the default, with the cap reached
    inside a body and with an adaptive stop."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=9)
    for extra in ({}, {"cg_max_iter": 5}):
        ref = Simulation.from_scene(sc, **extra)
        sim = Simulation.from_scene(sc, cg_unroll=unroll, **extra)
        ref.step(3)
        sim.step(3)
        assert sim.stats()["cg_iters"] == ref.stats()["cg_iters"]
        assert sim.stats()["iters_total"] == ref.stats()["iters_total"]
        pr, vr = ref.get_fluid()
        ps, vs = sim.get_fluid()
        assert np.array_equal(pr, ps) and np.array_equal(vr, vs)


def test_overflow_and_nonfinite_are_reported(mps):
    from mps_cuda_gb300 import MpsError, Simulation, scenes
    sc = scenes.dam_break_small(6, seed=1)
    s = Simulation.from_scene(sc, max_fluid_neighbors=4)
    s.step(1)
    with pytest.raises(MpsError, match="OVERFLOW"):
        s.stats()
    sc2 = scenes.dam_break_small(6, seed=1)
    sc2.pos4[5, 0] = np.nan
    s2 = Simulation.from_scene(sc2)
    s2.step(1)
    with pytest.raises(MpsError, match="NONFINITE"):
        s2.stats()


def test_empty_boundary_and_out_of_box_particles(mps, orc):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(6, seed=8)
    sc.bpos4 = sc.bpos4[:0]
    sc.pos4[0, :3] = (-0.3, 0.1, 0.1)   # outside the box: clamped into the border cells
    sim = Simulation.from_scene(sc, fixed_iters=3)
    o = orc.from_scene(sc, config=dict(fixed_iters=3))
    sim.step(1)
    o.step(1)
    p, v = sim.get_fluid()
    assert rel_err(p[:, :3], o.get("pos")) < 1e-6


def test_single_particle_and_single_pair(mps, orc):
    """The smallest inputs: one fluid particle (no fluid neighbours) and two (one pair) against the
    oracle over two full steps."""
    base = scenes_mod().dam_break_small(4, seed=3)
    for keep in ([0], [0, 1]):
        sc = dataclasses.replace(base, pos4=base.pos4[keep].copy(), vel4=base.vel4[keep].copy(),
                                 name=f"tiny_{len(keep)}")
        sim, o = make(mps, orc, sc)
        sim.step(2)
        o.step(2)
        p, v = sim.get_fluid()
        assert rel_err(p[:, :3], o.get("pos")) < 1e-6, keep
        assert rel_err(v[:, :3], o.get("vel")) < REL, keep


def test_empty_fluid_and_limits(mps):
    """A single-scene handle without fluid is rejected (a batch accepts empty scenes, below), and so
    is a box whose cell grid would exceed the key space; both with MPS_E_INVALID."""
    from mps_cuda_gb300 import MpsError, Simulation
    base = scenes_mod().dam_break_small(4, seed=3)
    empty = dataclasses.replace(base, pos4=base.pos4[:0].copy(), vel4=base.vel4[:0].copy(), name="empty")
    with pytest.raises(MpsError, match="INVALID"):
        Simulation.from_scene(empty)
    huge = dataclasses.replace(base, physics=dict(base.physics, max=(1.0e7, 1.0e7, 1.0e7)), name="huge")
    with pytest.raises(MpsError, match="INVALID"):
        Simulation.from_scene(huge)
    with pytest.raises(MpsError, match="INVALID"):
        Simulation.from_scene(base, max_fluid_neighbors=70000)


def test_batched_with_an_empty_scene(mps):
    """A scene without fluid particles in the middle of a batch: the other scenes step exactly as
    they do alone."""
    from mps_cuda_gb300 import BatchedSimulation, Simulation
    scs = scenes_mod().batched_scenes(3, seed=5, nmin=500, nmax=2000)
    empty = dataclasses.replace(scs[1], pos4=scs[1].pos4[:0].copy(), vel4=scs[1].vel4[:0].copy())
    batch = [scs[0], empty, scs[2]]
    b = BatchedSimulation(batch)
    b.step(2)
    pb, vb = b.get_fluid()
    its = b.scene_iters()
    off = 0
    for k, sc in enumerate(batch):
        if sc.n:
            s = Simulation.from_scene(sc)
            s.step(2)
            p, v = s.get_fluid()
            assert np.array_equal(p, pb[off:off + sc.n]) and np.array_equal(v, vb[off:off + sc.n]), k
            st = s.stats()
            assert (st["df_iters"], st["cg_iters"], st["cd_iters"]) == tuple(its[k]), k
        off += sc.n


def scenes_mod():
    from mps_cuda_gb300 import scenes
    return scenes


@pytest.mark.parametrize("fixed", [0, 6])
def test_cg_forms_match_oracle(mps, orc, fixed):
    """Both arrangements of the CG iteration (three-pass as the reference, two-pass) against the
    oracle's CG from the same state."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_small(10, seed=6)
    vels = []
    for form in (mps._lib.CG_THREE_PASS, mps._lib.CG_TWO_PASS):
        sim = Simulation.from_scene(sc, fixed_iters=fixed, cg_form=form)
        o = orc.from_scene(sc, config=dict(fixed_iters=fixed))
        advance_to_density(sim, o, mps)
        sim.phase(mps.PHASE_DF)
        o.phase(orc.DF)
        gpu_vel_to_oracle(sim, o)
        sim.phase(mps.PHASE_VISCST)
        o.phase(orc.VISCST)
        gi, oi = sim.stats()["cg_iters"], o.stats()["cg_iters"]
        assert abs(gi - oi) <= (0 if fixed else 1), (form, gi, oi)
        if gi == oi:
            assert rel_err(sim.get_field("vel")[:, :3], o.get("vel")) < REL, form
        vels.append(sim.get_field("vel")[:, :3])
    assert rel_err(vels[1], vels[0]) < REL


def test_reference_viscosity_scene_step(mps, orc):
    """The reference's viscosity column scene (ViscosityTestScene) with its shipped settings."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.reference_viscosity(height=20)
    sim = Simulation.from_scene(sc, fixed_iters=4)
    o = orc.from_scene(sc, config=dict(fixed_iters=4))
    for _ in range(3):
        sim.step(1)
        o.step(1)
    p, v = sim.get_fluid()
    assert rel_err(p[:, :3], o.get("pos")) < 1e-6
    assert rel_err(v[:, :3], o.get("vel")) < REL


@pytest.mark.parametrize("warm", [0, 30])
def test_dam_break_32k_phase_by_phase(mps, orc, warm):
    """The 32k dam break configuration at full size (32^3 fluid, the 51^3 wall lattice, cubic
    spline, 0.1 % tolerances), phase by phase against the oracle from an identical state: at the
    first step and after `warm` GPU steps.  Density and alpha after the density pass; the pressure
    factor of each pressure solve's first iteration (fixed_iters = 1) and the velocities after
    each solve (adaptive, where the iteration counts agree)."""
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.dam_break_32k(seed=0)
    for fixed in (1, 0):
        sim = Simulation.from_scene(sc, fixed_iters=fixed)
        if warm:
            sim.step(warm)
        o = orc.from_scene(sc, config=dict(fixed_iters=fixed))
        gpu_state_to_oracle(sim, o)
        advance_to_density(sim, o, mps)
        rho0 = sc.material["density"]
        assert np.abs(sim.get_field("density") - o.get("density")).max() / rho0 < REL
        assert rel_err(sim.get_field("alpha"), o.get("alpha")) < REL
        for gph, oph, name in ((mps.PHASE_DF, orc.DF, "df_iters"), (mps.PHASE_VISCST, orc.VISCST, "cg_iters"),
                               (mps.PHASE_CD, orc.CD, "cd_iters")):
            gpu_vel_to_oracle(sim, o)
            sim.phase(gph)
            o.phase(oph)
            gi, oi = sim.stats()[name], o.stats()[name]
            assert abs(gi - oi) <= (0 if fixed else 1), (name, gi, oi)
            if gi == oi:
                assert rel_err(sim.get_field("vel")[:, :3], o.get("vel")) < REL, (name, fixed)
            if fixed and name != "cg_iters":
                assert rel_err(sim.get_field("pressure"), o.get("pressure")) < REL, name
        sim.close()
