"""Generates the golden vectors that pin the FP64 oracle: outputs of the reference's OWN CUDA
step (moonsh5009/MPS_CUDA rebuilt headless for sm_103a by oracle/build_ref.sh) on small scenes.

Run on a GPU machine:  python tests/golden/make_golden.py
Writes tests/golden/ref_<case>.npz with the inputs, and per frame the reference's positions,
velocities, densities, alphas, pressures, boundary volumes, colours, neighbour CSR offsets and
solver loop counts.  tests/test_oracle_golden.py checks the oracle against these on the CPU.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mps_cuda_gb300 import scenes  # noqa: E402
from oracle import refstep  # noqa: E402

OUT = Path(__file__).resolve().parent

CASES = {
    # the reference's own scene and settings: poly6/spiky, ZSort every 50 frames, un-reset volume
    "surface_tension": dict(scene=lambda: scenes.reference_surface_tension(), variant="shipped", frames=3),
    # a small dam break with the dam_break_32k constants: cubic spline, 0.1 % tolerances
    "dam_break_8": dict(scene=lambda: scenes.dam_break_small(8, seed=7), variant="config", frames=2),
}


def run(case: str) -> Path:
    spec = CASES[case]
    sc = spec["scene"]()
    ref = refstep.RefStep(sc, variant=spec["variant"])
    rec = dict(pos4=sc.pos4, vel4=sc.vel4, bpos4=sc.bpos4, frames=np.int32(spec["frames"]))
    for f in range(spec["frames"]):
        ref.step(1)
        for k in ("pos", "vel", "density", "alpha", "pressure", "bvol", "color", "nei_ff_idx", "nei_fb_idx",
                  "nei_bb_idx"):
            rec[f"f{f}_{k}"] = ref.get(k)
        rec[f"f{f}_loops"] = np.array(ref.loops(), np.int32)
    ref.close()
    path = OUT / f"ref_{case}.npz"
    np.savez_compressed(path, **rec)
    return path


if __name__ == "__main__":
    for c in CASES:
        print(run(c))
