"""The allocation-free scan entry point (pp_decoupled_scan_device_noalloc).

It exists for callers that must not allocate device memory while they scan:
latency-critical loops that must stay out of the allocator (its calls can
synchronise the device), plug-ins whose host framework owns all device
memory through its own pool, processes whose device-memory budget is spent.
Its scratch is a fixed array in the library. Here it is called through the C
ABI and its output compared with the regular entry point's and, for integer
types, with the oracle, on two calls in a row (the second call must not see
the first call's leftovers in the shared scratch); the device's free memory
is unchanged across calls on a stream the library has never seen; and a
device-side timeout of a call is reported by pp_stream_status() instead of
being wiped by the next call. This file is collected last on purpose."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from helpers import NP, check_scan, from_dev, make_input, to_dev

pytestmark = pytest.mark.gpu

CASES = [("u32", "plus", False, (1 << 20) + 7), ("i64", "maximum", True, 300001), ("f32", "plus", False, 777777),
         ("u64", "bit_xor", False, 65536), ("i32", "multiplies", True, 4097)]


def _noalloc(pp):
    fn = pp.lib().pp_decoupled_scan_device_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_uint64]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("dtype,op,excl,n", CASES)
def test_noalloc_matches_regular_entry_point(pp, oracle, cuda, dtype, op, excl, n):
    fn = _noalloc(pp)
    s = cuda.cuda.current_stream().cuda_stream
    for call in range(2):
        x = make_input(dtype, op, n, seed=1000 * call + n)
        d_in = to_dev(cuda, x)
        d_ref = cuda.empty_like(d_in)
        d_out = cuda.empty_like(d_in)
        kind = pp.EXCLUSIVE if excl else pp.INCLUSIVE
        pp.decoupled_scan_device(kind, op, d_in.data_ptr(), d_ref.data_ptr(), n, dtype, stream=s)
        st = fn(s, kind, pp.OPS[op], pp.DTYPES[dtype], d_in.data_ptr(), d_out.data_ptr(), n)
        assert st == pp.PP_OK, pp.status_string(st)
        assert pp.stream_status(s) == pp.PP_OK
        got, ref = from_dev(d_out, NP[dtype]), from_dev(d_ref, NP[dtype])
        if dtype.startswith("f"):
            # float scans may associate differently from call to call: both
            # must sit within the error bound the scan tests use
            check_scan(got, x, dtype, op, excl, (n + 1023) // 1024)
            check_scan(ref, x, dtype, op, excl, (n + 1023) // 1024)
        else:
            np.testing.assert_array_equal(got, ref)
            np.testing.assert_array_equal(got, oracle.scan(x, op, excl))


def test_noalloc_rejects_sizes_beyond_its_scratch(pp, cuda):
    fn = _noalloc(pp)
    d = cuda.zeros(16, dtype=cuda.int32, device="cuda")
    too_many = 1_870_659_584 + 1  # one element more than 1 MiB of descriptors covers
    st = fn(cuda.cuda.current_stream().cuda_stream, pp.INCLUSIVE, pp.OPS["plus"], pp.DTYPES["u32"], d.data_ptr(),
            d.data_ptr(), too_many)
    assert st == pp.PP_ERR_WORKSPACE


def test_noalloc_leaves_free_device_memory_unchanged(pp, oracle, cuda):
    """After one call has loaded the kernels and looked up the scratch, calls
    on a stream the library has never seen (so no cached workspace could
    serve them) leave the device's free memory exactly as it was."""
    fn = _noalloc(pp)
    n = (1 << 22) + 3
    x = make_input("u32", "plus", n, seed=77)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s0 = cuda.cuda.current_stream().cuda_stream
    assert fn(s0, pp.INCLUSIVE, pp.OPS["plus"], pp.DTYPES["u32"], d_in.data_ptr(), d_out.data_ptr(), n) == pp.PP_OK
    cuda.cuda.synchronize()
    fresh = cuda.cuda.Stream()
    free_before, _ = cuda.cuda.mem_get_info()
    for _ in range(3):
        st = fn(fresh.cuda_stream, pp.INCLUSIVE, pp.OPS["plus"], pp.DTYPES["u32"], d_in.data_ptr(), d_out.data_ptr(),
                n)
        assert st == pp.PP_OK
    fresh.synchronize()
    free_after, _ = cuda.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    assert pp.stream_status(fresh.cuda_stream) == pp.PP_OK
    np.testing.assert_array_equal(from_dev(d_out, np.uint32), oracle.scan(x, "plus"))


def test_noalloc_timeout_is_reported_by_stream_status(pp, oracle, cuda):
    """A tile that never publishes its descriptor (the test-only skip knob)
    makes its successors' bounded look-back give up: the call returns, the
    timeout stays in the scratch's error word until pp_stream_status() reads
    it, and the next call is correct again."""
    fn = _noalloc(pp)
    n = 1 << 20
    x = make_input("u32", "plus", n, seed=21)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    assert pp.stream_status(s) == pp.PP_OK
    pp.set_timeout_ns(50_000_000)
    pp.debug_set_skip_tile(3)
    try:
        assert fn(s, pp.INCLUSIVE, pp.OPS["plus"], pp.DTYPES["u32"], d_in.data_ptr(), d_out.data_ptr(),
                  n) == pp.PP_OK
    finally:
        pp.debug_set_skip_tile(-1)
        pp.set_timeout_ns(1_000_000_000)
    # a second call before the status is read must not wipe the recorded timeout
    assert fn(s, pp.INCLUSIVE, pp.OPS["plus"], pp.DTYPES["u32"], d_in.data_ptr(), d_out.data_ptr(), n) == pp.PP_OK
    assert pp.stream_status(s) == pp.PP_ERR_TIMEOUT
    assert pp.stream_status(s) == pp.PP_OK  # read once, then cleared
    np.testing.assert_array_equal(from_dev(d_out, np.uint32), oracle.scan(x, "plus"))
