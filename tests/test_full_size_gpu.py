"""Every benchmark configuration at its full size, compared with the oracle:

* 2^30 uint32 U[0, 2^16) (the headline input): inclusive and exclusive
  plus-scans through the decoupled kernel and the inclusive plus-scan through
  the cooperative kernel, bit-exact against oracle.scan;
* 2^28 uint64 U[0, 2^32): inclusive and exclusive plus-scans, bit-exact;
* 2^30 int32 over the full range: max-scan, bit-exact;
* 2^30 float32 N(0,1): max reduction bit-exact, sum within the worst-case
  bound of the reduction's combine tree of the FP64 sum;
* 2^28 float32 N(0,1) and sign-random lognormal(0, 2): the compensated scan
  within 1e-6 relative error of the FP64 scan on every prefix not near a
  zero crossing, and every prefix (those included) within 1e-6 of
  sum_{j<=i} |x_j|;
* the batched segmented workload (65,536 segments with log-uniform lengths in
  [1, 2^16], about 385 M elements): int32 U[0, 1000) scans and reductions
  bit-exact on every segment, float32 N(0,1) ones within the scan error
  bound, against the oracle applied segment by segment;
* beyond 2^32 elements through properties (wrapping differences, totals).
Inputs come from the oracle's splitmix64 generators with the benchmark's
seeds, so they are the bytes the CPU baseline sees."""

from __future__ import annotations

import math

import numpy as np
import pytest

from helpers import EPS, from_dev, to_dev

pytestmark = pytest.mark.gpu

SEED = 0x5CA72026  # the benchmark's seed


def _stream(cuda):
    return cuda.cuda.current_stream().cuda_stream


def _scan_dev(pp, cuda, x, kind, op, dtype, algo="decoupled", precision="default"):
    """Scans numpy x on the GPU and returns the output as numpy."""
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = _stream(cuda)
    if algo == "cooperative":
        pp.cooperative_scan_device(kind, op, d_in.data_ptr(), d_out.data_ptr(), x.size, dtype, stream=s)
    elif precision != "default":
        pp.scan(kind, op, d_in.data_ptr(), d_out.data_ptr(), x.size, dtype, stream=s, precision=precision)
    else:
        pp.decoupled_scan_device(kind, op, d_in.data_ptr(), d_out.data_ptr(), x.size, dtype, stream=s)
    assert pp.stream_status(s) == 0
    del d_in
    got = from_dev(d_out, x.dtype)
    del d_out
    return got


def _assert_equal(got, want, what):
    if not np.array_equal(got, want):
        bad = np.nonzero(got != want)[0]
        raise AssertionError(f"{what}: {bad.size} mismatches, first at {bad[0]}: got {got[bad[0]]} want {want[bad[0]]}")


@pytest.fixture(scope="module")
def headline_input(oracle):
    return oracle.gen_u32(SEED, 1 << 30, 0, 1 << 16)


def test_u32_exclusive_plus_2p30_matches_oracle(pp, oracle, cuda, headline_input):
    x = headline_input
    _assert_equal(_scan_dev(pp, cuda, x, "exclusive", "plus", "u32"), oracle.scan(x, "plus", True),
                  "2^30 u32 exclusive")


def test_u32_cooperative_inclusive_plus_2p30_matches_oracle(pp, oracle, cuda, headline_input):
    x = headline_input
    _assert_equal(_scan_dev(pp, cuda, x, "inclusive", "plus", "u32", algo="cooperative"), oracle.scan(x, "plus"),
                  "2^30 u32 cooperative inclusive")


def test_u64_inclusive_plus_2p28_matches_oracle(pp, oracle, cuda):
    x = oracle.gen_u64(SEED + 2, 1 << 28, 0, 1 << 32)
    _assert_equal(_scan_dev(pp, cuda, x, "inclusive", "plus", "u64"), oracle.scan(x, "plus"), "2^28 u64 inclusive")


def test_f32_sum_and_max_reduce_2p30(pp, oracle, cuda):
    """Max is exact. The sum runs in FP32 through a fixed combine tree: every
    vector lane of every thread adds a run of at most ceil(n / (SMs * 512 *
    4)) inputs (one block of 512 threads per SM at least, 4 lanes of 16-byte
    loads), then warps, blocks and the last block's fold combine at most 64
    levels, so |sum - exact| <= (run + 64) * eps * sum |x_i| (the standard
    bound for recursive summation applied along the tree)."""
    n = 1 << 30
    x = oracle.gen_f32_normal(SEED + 3, n)
    d_in = to_dev(cuda, x)
    res = cuda.zeros(2, dtype=cuda.float32, device="cuda")
    s = _stream(cuda)
    pp.reduce("plus", d_in.data_ptr(), n, "f32", res.data_ptr(), stream=s)
    pp.reduce("maximum", d_in.data_ptr(), n, "f32", res.data_ptr() + 4, stream=s)
    assert pp.stream_status(s) == 0
    got = res.cpu().numpy()
    assert got[1] == np.max(x)
    exact = oracle.sum_fp64(x)
    sms = cuda.cuda.get_device_properties(0).multi_processor_count
    run = math.ceil(n / (sms * 512 * 4))
    bound = (run + 64) * EPS["f32"] * float(np.sum(np.abs(x), dtype=np.float64))
    err = abs(float(got[0]) - exact)
    assert err <= bound, (err, bound)
    print(f"f32 sum 2^30: {got[0]} vs FP64 {exact}: error {err:.3g}, bound {bound:.3g}")


@pytest.mark.parametrize("dist", ["normal", "lognormal"])
def test_f32_compensated_2p28_error(pp, oracle, cuda, dist):
    n = 1 << 28
    x = oracle.gen_f32_normal(12, n) if dist == "normal" else oracle.gen_f32_signed_lognormal(13, n, 0.0, 2.0)
    got = _scan_dev(pp, cuda, x, "inclusive", "plus", "f32", precision="compensated").astype(np.float64)
    want = oracle.scan_fp64(x)
    err = np.abs(got - want)
    m = np.abs(want) >= 1e-3 * np.sqrt(np.mean(want * want))
    rel = err[m] / np.abs(want[m])
    assert rel.max() <= 1e-6, rel.max()
    # the excluded prefixes (near zero crossings of the running sum), against
    # the magnitude the sum was built from
    cabs = np.cumsum(np.abs(x), dtype=np.float64)
    ex = ~m
    assert ex.sum() > 0
    rel_abs = err[ex] / cabs[ex]
    assert rel_abs.max() <= 1e-6, rel_abs.max()
    print(f"compensated {dist}: max rel {rel.max():.3g} over {m.sum()} prefixes; {ex.sum()} near-zero prefixes: "
          f"max |err| / sum|x| {rel_abs.max():.3g}")


def _c4_offsets(cuda):
    """The batched benchmark's segments: 65,536 lengths floor(exp(U[0, ln 2^16]))
    clipped to [1, 2^16] from torch's CPU generator seeded 0x5EC."""
    S = 65536
    g = cuda.Generator(device="cpu").manual_seed(0x5EC)
    lens = cuda.floor(cuda.exp(cuda.rand(S, generator=g, dtype=cuda.float64) * math.log(2 ** 16)))
    lens = lens.clamp(1, 2 ** 16).to(cuda.int64).numpy()
    return np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)


@pytest.mark.parametrize("dtype", ["i32", "f32"])
def test_batched_segments_full_workload(pp, oracle, cuda, dtype):
    off = _c4_offsets(cuda)
    S = off.size - 1
    n = int(off[-1])
    x = (oracle.gen_u32(SEED + 4, n, 0, 1000).view(np.int32) if dtype == "i32"
         else oracle.gen_f32_normal(SEED + 5, n))
    d_in, d_off = to_dev(cuda, x), cuda.from_numpy(off).cuda()
    d_out = cuda.empty_like(d_in)
    s = _stream(cuda)
    pp.segmented_scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, d_off.data_ptr(), S, dtype, stream=s)
    tot = cuda.empty(S, dtype=d_in.dtype, device="cuda")
    pp.segmented_reduce("plus", d_in.data_ptr(), n, d_off.data_ptr(), S, tot.data_ptr(), dtype, stream=s)
    assert pp.stream_status(s) == 0
    del d_in
    got = from_dev(d_out, x.dtype)
    del d_out
    got_tot = from_dev(tot, x.dtype)
    if dtype == "i32":
        _assert_equal(got, oracle.segmented_scan(x, off, "plus"), "segmented scan")
        _assert_equal(got_tot, oracle.segmented_reduce(x, off, "plus"), "segmented reduce")
        return
    # float32: |err_i| <= (64 + tiles) * eps * sum_{j<=i in the segment} |x_j|,
    # tiles = the most tiles a segment of <= 2^16 elements can span
    tiles = (1 << 16) // 1024 + 2
    want = oracle.segmented_scan_fp64(x, off)
    cabs = oracle.segmented_scan_fp64(np.abs(x), off)
    bound = (64 + tiles) * EPS["f32"] * cabs + np.finfo(np.float64).tiny
    err = np.abs(got.astype(np.float64) - want)
    assert np.all(err <= bound), float(np.max(err / bound))
    want_tot = oracle.segmented_sum_fp64(x, off)
    seg_abs = oracle.segmented_sum_fp64(np.abs(x), off)
    err_tot = np.abs(got_tot.astype(np.float64) - want_tot)
    assert np.all(err_tot <= (64 + tiles) * EPS["f32"] * seg_abs + np.finfo(np.float64).tiny)


def test_u32_inclusive_plus_2p30_matches_oracle(pp, oracle, cuda, headline_input):
    x = headline_input
    _assert_equal(_scan_dev(pp, cuda, x, "inclusive", "plus", "u32"), oracle.scan(x, "plus"), "2^30 u32 inclusive")


def test_i32_max_scan_2p30_matches_oracle(pp, oracle, cuda):
    x = oracle.gen_i32_full(SEED + 1, 1 << 30)
    _assert_equal(_scan_dev(pp, cuda, x, "inclusive", "maximum", "i32"), oracle.scan(x, "maximum"),
                  "2^30 i32 max-scan")


def test_u64_exclusive_plus_2p28_matches_oracle(pp, oracle, cuda):
    x = oracle.gen_u64(SEED + 2, 1 << 28, 0, 1 << 32)
    got = _scan_dev(pp, cuda, x, "exclusive", "plus", "u64")
    _assert_equal(got, oracle.scan(x, "plus", True), "2^28 u64 exclusive")
    assert got[0] == 0
    assert np.array_equal(np.diff(got), x[:-1])  # wrapping differences give back the input


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
