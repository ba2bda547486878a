"""The allocation-free cell sort (mps_cell_sort_noalloc) against the step's own cell sort.

Callers that cannot allocate device memory (a host application recording a stream capture, a
plugin whose host owns the GPU allocator, a real-time loop that cannot afford an allocation's
device synchronisation) pass their own device buffers; the sort's scratch lives in a fixed
device array inside the library.  This file is collected last on purpose: if it fails, a run
that stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reference_sort(mps, sc):
    """Cell keys and sorted particle order from the existing entry points (mps_phase SORT)."""
    from mps_cuda_gb300 import Simulation
    sim = Simulation.from_scene(sc)
    sim.phase(mps.PHASE_SORT)
    keys = sim.get_field("cell_key", order="slot")
    ids = sim.get_field("ids", order="slot")
    grid = sim.grid()
    sim.close()
    return keys, ids, grid


def _noalloc(lib, pos_dev, n, grid, keys_dev, order_dev):
    origin = (C.c_float * 3)(*grid["origin"])
    dims = (C.c_int32 * 3)(*grid["dims"])
    return lib.mps_cell_sort_noalloc(C.c_void_p(pos_dev), n, origin, C.c_float(grid["cell"]), dims,
                                     C.c_void_p(keys_dev), C.c_void_p(order_dev), None)


def test_noalloc_cell_sort_matches_step_sort_twice(mps):
    torch = pytest.importorskip("torch")
    from mps_cuda_gb300 import scenes
    lib = mps._lib.load()
    for call, seed in enumerate((3, 4)):  # two calls in a row, different inputs
        sc = scenes.dam_break_small(24, seed=seed)
        keys_ref, ids_ref, grid = _reference_sort(mps, sc)
        pos = torch.tensor(sc.pos4, device="cuda")
        keys = torch.full((sc.n,), -1, dtype=torch.int64, device="cuda")
        order = torch.full((sc.n,), -1, dtype=torch.int32, device="cuda")
        rc = _noalloc(lib, pos.data_ptr(), sc.n, grid, keys.data_ptr(), order.data_ptr())
        assert rc == 0, (call, lib.mps_last_error())
        torch.cuda.synchronize()
        assert np.array_equal(keys.cpu().numpy().view(np.uint64), keys_ref), call
        assert np.array_equal(order.cpu().numpy().view(np.uint32), ids_ref), call


def test_noalloc_rejects_sizes_beyond_its_scratch(mps):
    torch = pytest.importorskip("torch")
    lib = mps._lib.load()
    n = 262144 + 1
    pos = torch.zeros((1, 4), device="cuda")
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    grid = dict(origin=(0.0, 0.0, 0.0), cell=1.0, dims=(4, 4, 4))
    assert _noalloc(lib, pos.data_ptr(), n, grid, out.data_ptr(), out.data_ptr()) == -1
