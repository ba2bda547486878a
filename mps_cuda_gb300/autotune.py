"""Autotuner for the launch parameters of the step.

Tries every combination of the neighbour-pass block size and the radix-sort digit width on the
caller's own scene(s), each from the same initial state, timing a few graph-launched steps with
CUDA events; then, from the fastest, the CG iterations per device-loop body (`cg_unroll`) one
value at a time, and returns the fastest configuration.  None of the knobs changes results.  (The
reference has no tunables: block sizes 128/1024 and thrust's sort are fixed,
src/MPS_Computer/MPSSPHUtilDef.h:7-11.)
"""
from __future__ import annotations

import ctypes as C
import itertools

from . import _lib as L

DEFAULT_SPACE = {"block_size": (64, 128, 256), "sort_digit_bits": (6, 7, 8)}
DEFAULT_REFINE = {"cg_unroll": (1, 2, 4, 8)}


def _time_steps(sim, warmup: int, steps: int) -> float:
    """Mean ms per step over `steps` graph-launched steps after `warmup` untimed ones."""
    cudart = C.CDLL("libcudart.so")
    ev = [C.c_void_p(), C.c_void_p()]
    for e in ev:
        assert cudart.cudaEventCreate(C.byref(e)) == 0
    sim.step(warmup)
    cudart.cudaEventRecord(ev[0], None)
    sim.step(steps)
    cudart.cudaEventRecord(ev[1], None)
    cudart.cudaEventSynchronize(ev[1])
    ms = C.c_float()
    cudart.cudaEventElapsedTime(C.byref(ms), ev[0], ev[1])
    for e in ev:
        cudart.cudaEventDestroy(e)
    return ms.value / steps


def autotune(make_sim, space: dict | None = None, warmup: int = 2, steps: int = 3,
             refine: dict | None = None) -> tuple[dict, list]:
    """make_sim(**config) -> Simulation or BatchedSimulation.  Every combination of `space`, then
    each key of `refine` in turn from the best so far.  Returns (best config, all results)."""
    space = DEFAULT_SPACE if space is None else space
    refine = DEFAULT_REFINE if refine is None else refine
    results = []

    def run(cfg):
        sim = make_sim(**cfg)
        try:
            ms = _time_steps(sim, warmup, steps)
        finally:
            sim.close()
        results.append((ms, cfg))
        return ms

    keys = sorted(space)
    for values in itertools.product(*(space[k] for k in keys)):
        run(dict(zip(keys, values)))
    best_ms, best = min(results, key=lambda r: r[0])
    for k in sorted(refine):
        for v in refine[k]:
            if k in best and best[k] == v:
                continue
            cfg = dict(best, **{k: v})
            ms = run(cfg)
            if ms < best_ms:
                best_ms, best = ms, cfg
    results.sort(key=lambda r: r[0])
    return best, results
