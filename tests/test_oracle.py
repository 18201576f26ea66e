"""CPU checks of the oracle itself (no GPU): the reference's own known answers,
the multi-threaded restatements of the reference's algorithms against the
sequential oracle, and the reference defects the oracle documents."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import INT_DTYPES, INT_OPS, NP, make_input


def test_reference_reduction_known_answers(oracle):
    """tests/test_reduction.cpp:4-31: uint64 iota(0..n-1) sums to n(n-1)/2, n = 4^k."""
    n = 1
    while n < 1_000_000:
        a = np.arange(n, dtype=np.uint64)
        assert int(oracle.reduce(a, "plus")) == n * (n - 1) // 2
        assert int(oracle.ref_reduce(a, "plus", threads=4)) == n * (n - 1) // 2
        n *= 4


def test_reference_scan_benchmark_known_answer(oracle):
    """benchmarks/benchmark_scan.cpp:32-51: a scan of ones ends at n."""
    n = 1 << 20
    a = np.ones(n, dtype=np.uint32)
    assert int(oracle.scan(a)[-1]) == n
    assert int(oracle.ref_decoupled_scan(a, threads=4)[-1]) == n


def test_sequential_matches_numpy(oracle):
    x = oracle.gen_u32(1, 100_000, 0, 1 << 16)
    np.testing.assert_array_equal(oracle.scan(x), np.cumsum(x, dtype=np.uint32))
    e = oracle.scan(x, exclusive=True)
    assert e[0] == 0
    np.testing.assert_array_equal(e[1:], np.cumsum(x, dtype=np.uint32)[:-1])
    y = oracle.gen_i32_full(2, 50_000)
    np.testing.assert_array_equal(oracle.scan(y, "maximum"), np.maximum.accumulate(y))
    np.testing.assert_array_equal(oracle.scan(y, "bit_xor"), np.bitwise_xor.accumulate(y))


@pytest.mark.parametrize("dtype", INT_DTYPES)
@pytest.mark.parametrize("op", INT_OPS)
def test_reference_decoupled_restatement(oracle, dtype, op):
    """The multi-threaded restatement of the reference's decoupled kernel
    (small partitions so many look-backs happen) equals the sequential scan."""
    x = make_input(dtype, op, 200_003, seed=11)
    want = oracle.scan(x, op)
    np.testing.assert_array_equal(oracle.ref_decoupled_scan(x, op, threads=6, local_mem_bytes=4096), want)
    np.testing.assert_array_equal(
        oracle.ref_decoupled_scan(x, op, threads=3, local_mem_bytes=2048, force_lookback=True), want)
    np.testing.assert_array_equal(oracle.ref_cooperative_scan(x, op, threads=5), want)
    assert oracle.ref_reduce(x, op, threads=7) == oracle.reduce(x, op)


def test_reference_exclusive_defect_is_reproduced(oracle):
    """In the reference, a partition that takes the scan-then-reduce path
    publishes the last element of its EXCLUSIVE local scan as its aggregate
    (scan_decoupled_lookback.hpp:42,163,168), so downstream prefixes miss one
    element per such partition. With every partition forced down that path the
    restatement shows the defect deterministically; with one work-group every
    partition finds its predecessor ready and the result is correct."""
    x = np.ones(10_000, dtype=np.uint32)
    want = oracle.scan(x, exclusive=True)
    bad = oracle.ref_decoupled_scan(x, exclusive=True, threads=2, local_mem_bytes=1024, force_lookback=True)
    assert not np.array_equal(bad, want)
    L = 1024 // 4 - 1
    # partition 0 always finds its (empty) predecessor ready; every later
    # partition before the last one loses one element
    assert int(want[-1] - bad[-1]) == (x.size - 1) // L - 1
    good = oracle.ref_decoupled_scan(x, exclusive=True, threads=1, local_mem_bytes=1024)
    np.testing.assert_array_equal(good, want)
    # the cooperative scan reads chunk tails of exclusive scans the same way
    coop = oracle.ref_cooperative_scan(x, exclusive=True, threads=4)
    assert not np.array_equal(coop, want)


def test_generators_are_deterministic_and_shaped(oracle):
    a = oracle.gen_u32(0x5CA72026, 1 << 16, 0, 256, threads=1)
    b = oracle.gen_u32(0x5CA72026, 1 << 16, 0, 256, threads=7)
    np.testing.assert_array_equal(a, b)
    assert a.max() == 255 and a.min() == 0
    z = oracle.gen_f32_normal(5, 1 << 20)
    assert abs(float(z.mean())) < 0.01 and abs(float(z.std()) - 1.0) < 0.01
    ln = oracle.gen_f32_signed_lognormal(6, 1 << 18, 0.0, 2.0)
    assert 0.45 < float(np.mean(ln > 0)) < 0.55
    assert abs(float(np.log(np.abs(ln)).std()) - 2.0) < 0.02
    u = oracle.gen_u64(9, 1 << 16, 0, 1 << 32)
    assert int(u.max()) < (1 << 32)


def test_fp64_oracle(oracle):
    x = np.full(1000, 0.1, dtype=np.float32)
    s = oracle.scan_fp64(x)
    assert abs(s[-1] - 1000 * float(np.float32(0.1))) < 1e-9
    assert oracle.scan_fp64(x, exclusive=True)[0] == 0.0
    y = np.array([1e16, 1.0, -1e16], dtype=np.float64)
    assert oracle.scan_fp64(y)[-1] == 1.0  # compensated for f64 inputs
    assert oracle.sum_fp64(y) == 1.0


@pytest.mark.parametrize("dtype", [np.int32, np.uint64, np.float32])
def test_segmented_oracle_is_the_scan_of_each_segment(oracle, dtype):
    """oracle.segmented_* against the single-array oracle applied to every
    segment on its own (empty segments included)."""
    rng = np.random.default_rng(3)
    lens = rng.integers(0, 40, 500)
    lens[:3] = 0
    lens[-1] = 0
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    n = int(off[-1])
    x = (rng.standard_normal(n) if dtype == np.float32 else rng.integers(0, 1 << 20, n)).astype(dtype)
    for excl in (False, True):
        got = oracle.segmented_scan(x, off, "plus", excl)
        for k in range(lens.size):
            a, b = off[k], off[k + 1]
            assert np.array_equal(got[a:b], oracle.scan(x[a:b], "plus", excl))
    red = oracle.segmented_reduce(x, off, "maximum")
    for k in range(lens.size):
        a, b = off[k], off[k + 1]
        assert red[k] == oracle.reduce(x[a:b], "maximum")  # the identity when empty
    if dtype == np.float32:
        f = oracle.segmented_scan_fp64(x, off)
        t = oracle.segmented_sum_fp64(x, off)
        for k in range(lens.size):
            a, b = off[k], off[k + 1]
            assert np.array_equal(f[a:b], oracle.scan_fp64(x[a:b]))
            assert t[k] == oracle.sum_fp64(x[a:b])
    bad = off.copy()
    bad[-1] = n + 5
    with pytest.raises(ValueError):
        oracle.segmented_scan(x, bad, "plus")  # offsets must end at n
