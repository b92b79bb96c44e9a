"""The grid sort through rrsph_sort_pairs_noalloc, the entry point that
allocates nothing, against the sort of rrsph_grid_find.

rrsph_sort_pairs_noalloc is for callers that cannot allocate device memory
(their memory belongs to another framework's pool, or their step loop must not
call cudaMalloc). It works in a fixed array inside the library, so the check
here runs it twice in a row on different inputs (a stale array from the first
call must not leak into the second), compares each result with the sorted grid
rrsph_grid_find returns for the same particles (integers: exact), and checks
that the second call leaves the device's free memory unchanged and that a size
above the limit is refused. This file is collected last on purpose.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid_of(case):
    from sph2d_gb300 import Solver

    p = case.params()
    with Solver(p, "fp64") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        keys, grid, _ = s.grid_find(with_cells_start=False)
    key_bits = int(p.max_cells - 1).bit_length()
    return keys, grid, key_bits


def _sort_noalloc(keys, key_bits):
    import torch

    from sph2d_gb300 import capi

    n = len(keys)
    d_keys = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    d_ids = torch.arange(n, dtype=torch.int32, device="cuda")
    out_keys = torch.empty_like(d_keys)
    out_ids = torch.empty_like(d_ids)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc = capi.lib().rrsph_sort_pairs_noalloc(
        C.c_void_p(d_keys.data_ptr()), C.c_void_p(d_ids.data_ptr()), C.c_void_p(out_keys.data_ptr()),
        C.c_void_p(out_ids.data_ptr()), n, key_bits, C.c_void_p(stream.cuda_stream))
    capi.check(rc)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert np.array_equal(d_keys.cpu().numpy().view(np.uint32), keys)  # inputs untouched
    return out_keys.cpu().numpy().view(np.uint32), out_ids.cpu().numpy().view(np.uint32), free_before - free_after


def test_noalloc_sort_matches_grid_find_on_two_calls(gpu_available):
    from sph2d_gb300 import capi, cases

    inputs = [cases.piston_flume_2d(nx=900, ny=60, seed=21), cases.dam_break_2d(nx=150, ny=80, seed=22)]
    for call, case in enumerate(inputs):
        keys, grid, key_bits = _grid_of(case)
        assert len(keys) <= capi.SORT_NOALLOC_MAX_PAIRS
        out_keys, out_ids, used = _sort_noalloc(keys, key_bits)
        assert np.array_equal(out_ids, grid), f"call {call}: ids differ from rrsph_grid_find"
        assert np.array_equal(out_keys, keys[grid]), f"call {call}: keys not sorted like the grid"
        if call == 1:
            assert used == 0, f"second call changed free device memory by {used} bytes"


def test_noalloc_sort_rejects_sizes_above_its_limit(gpu_available):
    import torch

    from sph2d_gb300 import RrsphError, capi

    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    out = torch.zeros(16, dtype=torch.int32, device="cuda")
    out2 = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    rc = capi.lib().rrsph_sort_pairs_noalloc(p, C.c_void_p(buf.data_ptr() + 4), C.c_void_p(out.data_ptr()),
                                             C.c_void_p(out2.data_ptr()), capi.SORT_NOALLOC_MAX_PAIRS + 1, 21, None)
    assert rc == capi.ERR_INVALID_ARGUMENT
    with pytest.raises(RrsphError, match="exceeds the maximum"):
        capi.check(rc)
