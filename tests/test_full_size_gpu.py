"""The scans at the benchmark configurations' full sizes (2^30 and 2^28
elements), compared with the oracle element by element where that is cheap
(integer scans) and through size-independent properties elsewhere: the
difference of neighbouring outputs gives back the input, the last inclusive
output is the total, and the compensated float scan stays within 1e-6 relative
error of an FP64 scan."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import from_dev, to_dev

pytestmark = pytest.mark.gpu


def test_u32_inclusive_plus_2p30_matches_oracle(pp, oracle, cuda):
    n = 1 << 30
    x = oracle.gen_u32(0x5CA72026, n, 0, 1 << 16)  # the headline input: U[0, 2^16)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=s)
    assert pp.stream_status(s) == 0
    del d_in
    got = from_dev(d_out, np.uint32)
    del d_out
    want = oracle.scan(x, "plus")
    assert np.array_equal(got, want)


def test_i32_max_scan_2p30_matches_numpy(pp, cuda):
    n = 1 << 30
    g = cuda.Generator(device="cuda")
    g.manual_seed(7)
    d_in = cuda.randint(-(1 << 31), (1 << 31) - 1, (n,), dtype=cuda.int32, device="cuda", generator=g)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.decoupled_scan_device("inclusive", "maximum", d_in.data_ptr(), d_out.data_ptr(), n, "i32", stream=s)
    assert pp.stream_status(s) == 0
    x = d_in.cpu().numpy()
    got = d_out.cpu().numpy()
    assert np.array_equal(got, np.maximum.accumulate(x))


def test_u64_exclusive_plus_2p28_properties(pp, oracle, cuda):
    n = 1 << 28
    x = oracle.gen_u64(11, n, 0, 1 << 32)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.decoupled_scan_device("exclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u64", stream=s)
    assert pp.stream_status(s) == 0
    got = from_dev(d_out, np.uint64)
    assert got[0] == 0
    assert np.array_equal(np.diff(got), x[:-1])  # wrapping differences give back the input
    assert np.add(got[-1:], x[-1:])[0] == np.sum(x, dtype=np.uint64)


def test_f32_compensated_2p28_error(pp, oracle, cuda):
    n = 1 << 28
    x = oracle.gen_f32_normal(12, n)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "f32", stream=s, precision="compensated")
    assert pp.stream_status(s) == 0
    got = from_dev(d_out, np.float32).astype(np.float64)
    want = np.cumsum(x.astype(np.float64))
    m = np.abs(want) >= 1e-3 * np.sqrt(np.mean(want * want))
    rel = np.abs(got[m] - want[m]) / np.abs(want[m])
    assert rel.max() <= 1e-6, rel.max()


def test_u32_scan_and_sum_beyond_2p32_elements(pp, cuda):
    """2^32 + 12,345 elements (16 GiB in, 16 GiB out): element and tile
    indices past 32 bits. Checked on the device through properties: wrapping
    differences of neighbouring outputs give back the input, the first output
    is the first input, the last is the total, and the reduction agrees."""
    n = (1 << 32) + 12345
    g = cuda.Generator(device="cuda")
    g.manual_seed(33)
    d_in = cuda.randint(-(1 << 31), (1 << 31) - 1, (n,), dtype=cuda.int32, device="cuda", generator=g)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=s)
    assert pp.stream_status(s) == 0
    assert int(d_out[0]) == int(d_in[0])
    step = 1 << 28  # compare in slices to bound the temporaries
    for a in range(1, n, step):
        b = min(n, a + step)
        assert cuda.equal(d_out[a:b] - d_out[a - 1:b - 1], d_in[a:b]), a  # int32 arithmetic wraps like uint32
    total = int(d_in.sum(dtype=cuda.int64)) & 0xFFFFFFFF
    assert int(d_out[-1]) & 0xFFFFFFFF == total
    r = cuda.zeros(1, dtype=cuda.int64, device="cuda")
    pp.reduce("plus", d_in.data_ptr(), n, "u32", r.data_ptr(), stream=s)
    assert pp.stream_status(s) == 0
    assert int(r[0]) & 0xFFFFFFFF == total


def test_u64_scan_beyond_2p32_elements(pp, cuda):
    """2^32 + 7 uint64 elements (32 GiB in, 32 GiB out) on the rows layout
    with the store warp: wrapping differences give back the input."""
    n = (1 << 32) + 7
    g = cuda.Generator(device="cuda")
    g.manual_seed(34)
    d_in = cuda.randint(-(1 << 62), 1 << 62, (n,), dtype=cuda.int64, device="cuda", generator=g)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u64", stream=s)
    assert pp.stream_status(s) == 0
    assert int(d_out[0]) == int(d_in[0])
    step = 1 << 27
    for a in range(1, n, step):
        b = min(n, a + step)
        assert cuda.equal(d_out[a:b] - d_out[a - 1:b - 1], d_in[a:b]), a  # int64 arithmetic wraps like uint64
