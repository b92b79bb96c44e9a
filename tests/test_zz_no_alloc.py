"""The grid sort through rrsph_sort_pairs_noalloc, the entry point that
allocates nothing, against the sort of rrsph_grid_find.

rrsph_sort_pairs_noalloc is for callers that cannot allocate device memory
(their memory belongs to another framework's pool, or their step loop must not
call cudaMalloc). It works in a fixed array inside the library, so the check
here runs it twice in a row on different inputs (a stale array from the first
call must not leak into the second), compares each result with the sorted grid
rrsph_grid_find returns for the same particles (integers: exact), and checks
that the second call leaves the device's free memory unchanged; random keys at
the largest size and at widths that take an even or an odd number of passes
are checked against numpy's stable argsort, and sizes above the limit and
overlapping buffers are refused. This file is collected last on purpose.
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


@pytest.mark.parametrize("n, key_bits", [(1 << 20, 32), (1 << 20, 24), (5000, 8), (1, 1)])
def test_noalloc_sort_pass_counts_against_numpy(gpu_available, n, key_bits):
    """Random keys whose width gives four, three, one and one 8-bit passes (an
    even and an odd number of passes write the outputs from different
    buffers), the largest n accepted among them: a stable sort by the low
    key_bits bits, as numpy's stable argsort gives it."""
    from sph2d_gb300 import capi

    assert n <= capi.SORT_NOALLOC_MAX_PAIRS
    rng = np.random.default_rng(n + key_bits)
    keys = rng.integers(0, 1 << key_bits, size=n, dtype=np.uint64).astype(np.uint32)
    for _ in range(2):  # two calls in a row on the shared working array
        out_keys, out_ids, _ = _sort_noalloc(keys, key_bits)
        order = np.argsort(keys, kind="stable").astype(np.uint32)
        assert np.array_equal(out_ids, order)
        assert np.array_equal(out_keys, keys[order])
        keys = rng.permutation(keys)


def test_noalloc_sort_refuses_overlapping_buffers(gpu_available):
    import torch

    from sph2d_gb300 import capi

    n = 64
    a = torch.zeros(8 * n, dtype=torch.int32, device="cuda")  # every range below lies inside it
    base = a.data_ptr()
    word = 4

    def call(keys_in, ids_in, keys_out, ids_out):
        return capi.lib().rrsph_sort_pairs_noalloc(C.c_void_p(keys_in), C.c_void_p(ids_in), C.c_void_p(keys_out),
                                                   C.c_void_p(ids_out), n, 8, None)

    k_in, i_in, k_out, i_out = base, base + n * word, base + 2 * n * word, base + 3 * n * word
    assert call(k_in, i_in, i_in, i_out) == capi.ERR_INVALID_ARGUMENT          # keys out = ids in
    assert call(k_in, i_in, k_out, k_in) == capi.ERR_INVALID_ARGUMENT          # ids out = keys in
    assert call(k_in, i_in, k_out, k_out + 8 * word) == capi.ERR_INVALID_ARGUMENT  # outputs overlap
    assert call(k_in, i_in, i_in + 16 * word, base + 5 * n * word) == capi.ERR_INVALID_ARGUMENT  # partly
    assert call(k_in, i_in, k_out, i_out) == capi.OK
    torch.cuda.synchronize()


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
