"""Autotuner for the launch parameters of the step.

Tries every combination of the neighbour-pass block size and the radix-sort digit width on the
caller's own scene(s), each from the same initial state, timing a few graph-launched steps with
CUDA events, and returns the fastest configuration.  (The reference has no tunables: block sizes
128/1024 and thrust's sort are fixed, src/MPS_Computer/MPSSPHUtilDef.h:7-11.)
"""
from __future__ import annotations

import ctypes as C
import itertools

from . import _lib as L

DEFAULT_SPACE = {"block_size": (64, 128, 256), "sort_digit_bits": (6, 7, 8)}


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


def autotune(make_sim, space: dict | None = None, warmup: int = 2, steps: int = 3) -> tuple[dict, list]:
    """make_sim(**config) -> Simulation or BatchedSimulation.  Returns (best config, all results)."""
    space = space or DEFAULT_SPACE
    keys = sorted(space)
    results = []
    for values in itertools.product(*(space[k] for k in keys)):
        cfg = dict(zip(keys, values))
        sim = make_sim(**cfg)
        try:
            ms = _time_steps(sim, warmup, steps)
        finally:
            sim.close()
        results.append((ms, cfg))
    results.sort(key=lambda r: r[0])
    return results[0][1], results
