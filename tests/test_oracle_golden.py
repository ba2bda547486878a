"""Pins the FP64 oracle against the reference's OWN CUDA step (CPU only).

tests/golden/ref_*.npz hold the outputs of moonsh5009/MPS_CUDA's step rebuilt headless for
sm_103a (oracle/build_ref.sh), produced on a GB300 by tests/golden/make_golden.py.  The oracle
replays the same frames (the reference's Morton re-sort every 50 frames and its un-reset boundary
volume included) and must agree to FP64 rounding: integer neighbour structure bit-exact, solver
loop counts equal, floating-point fields within 1e-9 relative (the reference contracts
multiply-adds into FMAs on the GPU, the oracle does not).
"""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
REL = 1e-9


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _case(name):
    from mps_cuda_gb300 import scenes
    if name == "surface_tension":
        return scenes.reference_surface_tension(), {}
    return scenes.dam_break_small(8, seed=7), {}


@pytest.mark.parametrize("case", ["surface_tension", "dam_break_8"])
def test_oracle_matches_reference_golden(mps, orc, case):
    path = GOLDEN / f"ref_{case}.npz"
    assert path.exists(), f"missing golden vectors {path}; run tests/golden/make_golden.py on a GPU"
    g = np.load(path)
    sc, _ = _case(case)
    # the fixture was made from exactly these inputs
    assert np.array_equal(g["pos4"], sc.pos4) and np.array_equal(g["vel4"], sc.vel4)
    assert np.array_equal(g["bpos4"], sc.bpos4)
    o = orc.from_scene(sc, zsort=1, volume_accumulate=1)
    for f in range(int(g["frames"])):
        o.step(1)
        st = o.stats()
        loops = tuple(int(x) for x in g[f"f{f}_loops"])
        assert (st["df_iters"], st["cg_iters"], st["cd_iters"]) == loops, (f, loops)
        for k in ("nei_ff_idx", "nei_fb_idx", "nei_bb_idx"):
            assert np.array_equal(o.get(k), g[f"f{f}_{k}"]), (f, k)
        for k in ("pos", "vel", "density", "alpha", "pressure", "bvol"):
            assert rel_err(o.get(k), g[f"f{f}_{k}"]) < REL, (f, k, rel_err(o.get(k), g[f"f{f}_{k}"]))
        assert np.abs(o.get("color") - g[f"f{f}_color"]).max() <= 1e-6
