"""Neighbourhood tiles (mps_config.stage = 1) against the global-gather passes (stage = 0).

The tiled passes gather the neighbours' data from a shared-memory copy of each block's distinct
neighbour slots, indexed by 16-bit ranks built with the neighbour lists; the pairs, their order and
the arithmetic are those of the global-gather passes, so whole steps agree bit for bit.  A block
whose neighbourhood does not fit its tile falls back to the global gathers (tile size -1).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(sc, steps, **cfg):
    from mps_cuda_gb300 import Simulation
    sim = Simulation.from_scene(sc, **cfg)
    sim.step(steps)
    p, v = sim.get_fluid()
    st = sim.stats()
    sim.close()
    return p, v, st


@pytest.mark.parametrize("bs", [64, 128, 256])
def test_tiled_step_equals_global_gathers(mps, bs):
    from mps_cuda_gb300 import scenes
    sc = scenes.dam_break_small(14, seed=21)
    p0, v0, s0 = _run(sc, 3, block_size=bs, stage=0)
    p1, v1, s1 = _run(sc, 3, block_size=bs, stage=1)
    assert s1["flags"] & 8 == 0, s1["flags"]   # no rank outside its tile
    assert s1["tile_blocks"][0] > 0            # the tiles were used
    assert (s0["df_iters"], s0["cg_iters"], s0["cd_iters"]) == (s1["df_iters"], s1["cg_iters"], s1["cd_iters"])
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)


def test_tiled_eager_phases_equal_graph(mps):
    from mps_cuda_gb300 import scenes
    sc = scenes.dam_break_small(12, seed=5)
    pg, vg, _ = _run(sc, 2, stage=1, use_graph=1)
    pe, ve, _ = _run(sc, 2, stage=1, use_graph=0)
    assert np.array_equal(pg, pe) and np.array_equal(vg, ve)


def test_tile_overflow_falls_back_to_global_gathers(mps):
    """Spacing = particle radius puts about 270 neighbours on a particle and 64 particles in a cell,
    so a block's distinct neighbours exceed its tile (5 records a slot): those blocks keep the
    global gathers, and the step still equals the untiled one."""
    from mps_cuda_gb300 import scenes
    sc = scenes.dam_break((12, 12, 12), 0.01, 0.01, 0.001, (0.0, 0.0, 0.0), (0.3, 0.3, 0.3), seed=3, dt=1.0e-3,
                          name="dense")
    cfg = dict(max_fluid_neighbors=400, max_boundary_neighbors=256, block_size=64, fixed_iters=4)
    p0, v0, s0 = _run(sc, 1, stage=0, **cfg)
    p1, v1, s1 = _run(sc, 1, stage=1, **cfg)
    assert s1["flags"] & 8 == 0
    assert s1["tile_blocks"][1] > 0            # blocks without a tile took the global gathers
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)
