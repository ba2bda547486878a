"""Precision protocol of the colliding-blocks scene at a reduced scale (two ~1.8k-particle blocks at
+-1 m/s around a sampled sphere): every few steps one step is taken phase by phase on the GPU and
on the FP64 oracle from the GPU's current state.  Densities within 1e-5 of rho0, velocities within
1e-4 relative (max-norm) whenever both sides ran the same iteration counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_colliding_blocks_per_step_error(mps, orc):
    from mps_cuda_gb300 import Simulation, scenes
    sc = scenes.colliding_4m(seed=1, scale=0.1)
    sim = Simulation.from_scene(sc)
    o = orc.from_scene(sc)
    rho0 = sc.material["density"]
    checked = 0
    for t in range(40):
        if t % 10:
            sim.step(1)
            continue
        p, v = sim.get_fluid()
        o.set_fluid(p[:, :3].astype(np.float64), v[:, :3].astype(np.float64), v[:, 3].astype(np.float64),
                    p[:, 3].astype(np.float64))
        for ph in (mps.PHASE_SORT, mps.PHASE_NEIGHBORS, mps.PHASE_BVOLUME, mps.PHASE_DENSITY_ALPHA):
            sim.phase(ph)
        for ph in (orc.ZSORT, orc.NEIGHBORS, orc.BVOLUME, orc.DENSITY, orc.ALPHA, orc.GRAVITY):
            o.phase(ph)
        assert np.abs(sim.get_field("density") - o.get("density")).max() / rho0 < 1e-5
        for gph, oph in ((mps.PHASE_DF, orc.DF), (mps.PHASE_VISCST, orc.VISCST), (mps.PHASE_CD, orc.CD)):
            sim.phase(gph)
            o.phase(oph)
        st, so = sim.stats(), o.stats()
        if (st["df_iters"], st["cg_iters"], st["cd_iters"]) == (so["df_iters"], so["cg_iters"], so["cd_iters"]):
            vg, vo = sim.get_field("vel")[:, :3], o.get("vel")
            assert np.abs(vg - vo).max() / np.abs(vo).max() < 1e-4
            checked += 1
        sim.phase(mps.PHASE_ADVECT)
    assert checked >= 2
