"""The allocation-free scan entry point (pp_decoupled_scan_device_noalloc).

It exists for callers that may not allocate device memory while they scan
(graph capture, allocator-free loops, plug-ins whose host owns all device
memory); its scratch is a fixed array in the library. Here it is called
through the C ABI and its output compared with the regular entry point's,
on two calls in a row (the second call must not see the first call's
leftovers in the shared scratch). This file is collected last on purpose."""

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
        cuda.cuda.synchronize()
        got, ref = from_dev(d_out, NP[dtype]), from_dev(d_ref, NP[dtype])
        if dtype.startswith("f"):
            # float scans may associate differently from call to call: both
            # must sit within the error bound the scan tests use
            check_scan(got, x, dtype, op, excl, (n + 1023) // 1024)
            check_scan(ref, x, dtype, op, excl, (n + 1023) // 1024)
        else:
            np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_sizes_beyond_its_scratch(pp, cuda):
    fn = _noalloc(pp)
    d = cuda.zeros(16, dtype=cuda.int32, device="cuda")
    too_many = 1_870_659_584 + 1  # one element more than 1 MiB of descriptors covers
    st = fn(cuda.cuda.current_stream().cuda_stream, pp.INCLUSIVE, pp.OPS["plus"], pp.DTYPES["u32"], d.data_ptr(),
            d.data_ptr(), too_many)
    assert st == pp.PP_ERR_WORKSPACE
