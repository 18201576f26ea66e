"""The look-back protocol under perturbed timing (the descriptor perturbation
knob, pp_debug_set_lookback_delay).

The reference's look-back is correct only if its descriptor protocol is
(partition_descriptor.h:115-130; the reduce-then-scan / scan-then-reduce
choice of scan_decoupled_lookback.hpp:143-174 depends on when predecessors
publish). Natural timing rarely exercises the rare branches, so here every
tile delays the publication of its aggregate and of its inclusive prefix by a
seeded pseudo-random time of up to a few microseconds, and spaces the words
of two-word descriptors (64-bit integers, compensated and FP64-carry float
scans) apart. The results must stay bit-exact (integers, min/max) or within
the scan error bound (float sums) against the oracle, and the kernel's
counters must show that both resolutions, look-backs over more than one
window of 32 predecessors and reads of half-written descriptors all
happened."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import NP, check_scan, empty_dev, from_dev, make_input, to_dev

pytestmark = pytest.mark.gpu

DELAY_NS = 3000
# (dtype, op, precision): one-word and two-word descriptors
CASES = [("u32", "plus", "default"), ("i32", "maximum", "default"), ("u64", "plus", "default"),
         ("i64", "bit_xor", "default"), ("f32", "plus", "default"), ("f32", "plus", "compensated"),
         ("f32", "plus", "fp64_carry"), ("f64", "plus", "default")]
TWO_WORD = {("u64", "plus", "default"), ("i64", "bit_xor", "default"), ("f32", "plus", "compensated"),
            ("f32", "plus", "fp64_carry"), ("f64", "plus", "default")}

_totals = {"one": {}, "two": {}}


def _add(key, c):
    d = _totals[key]
    for k, v in c.items():
        d[k] = d.get(k, 0) + v


@pytest.fixture
def perturbed(pp):
    def on(seed):
        pp.debug_set_lookback_delay(DELAY_NS, seed)
    yield on
    pp.debug_set_lookback_delay(0, 0)


@pytest.mark.parametrize("excl", [False, True])
@pytest.mark.parametrize("dtype,op,precision", CASES)
def test_scan_under_perturbed_descriptors(pp, oracle, cuda, perturbed, dtype, op, precision, excl):
    n = 3_000_001
    x = make_input(dtype, op, n, seed=n + len(op))
    s = cuda.cuda.current_stream().cuda_stream
    pp.debug_lookback_counters(s)  # start from zero
    for seed, phase in ((1, 0), (2, 1)):
        # phase 1: the input one element past a 16-byte boundary (shifted tile grid)
        d_in = empty_dev(cuda, n, NP[dtype], pad=1)
        d_in[phase:phase + n].copy_(to_dev(cuda, x))
        d_out = empty_dev(cuda, n, NP[dtype], pad=1)
        esz = x.dtype.itemsize
        perturbed(seed)
        pp.scan("exclusive" if excl else "inclusive", op, d_in.data_ptr() + phase * esz,
                d_out.data_ptr() + phase * esz, n, dtype, stream=s, precision=precision)
        assert pp.stream_status(s) == 0
        c = pp.debug_lookback_counters(s)
        pp.debug_set_lookback_delay(0, 0)
        got = from_dev(d_out, NP[dtype])[phase:phase + n]
        if precision == "default":
            check_scan(got, x, dtype, op, excl, (n + 1023) // 1024)
        else:
            want = oracle.scan_fp64(x, excl)
            cabs = np.cumsum(np.abs(x.astype(np.float64)))
            tol = (1e-6 if precision == "compensated" else 64 * np.finfo(np.float32).eps) * cabs + 1e-30
            assert np.all(np.abs(got.astype(np.float64) - want) <= tol)
        assert c["reduce_then_scan"] + c["scan_then_reduce"] > 0, c
        _add("two" if (dtype, op, precision) in TWO_WORD else "one", c)


def test_perturbation_exercised_every_branch():
    """Summed over the runs above (this test comes after them in the file)."""
    one, two = _totals["one"], _totals["two"]
    if not one or not two:
        pytest.skip("the perturbed scans did not run")
    for t in (one, two):
        assert t["reduce_then_scan"] > 0, t
        assert t["scan_then_reduce"] > 0, t
        assert t["over_32_predecessors"] > 0, t
    assert two["half_written_reads"] > 0, two
    assert one["half_written_reads"] == 0, one  # one-word descriptors cannot be half written
    print(f"one-word descriptors: {one}; two-word descriptors: {two}")


def test_counters_stay_zero_with_the_knob_off(pp, oracle, cuda):
    n = 1_000_003
    x = make_input("u32", "plus", n, seed=5)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.debug_lookback_counters(s)
    pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=s)
    assert pp.stream_status(s) == 0
    assert pp.debug_lookback_counters(s) == {"reduce_then_scan": 0, "scan_then_reduce": 0,
                                             "over_32_predecessors": 0, "half_written_reads": 0}
    np.testing.assert_array_equal(from_dev(d_out, np.uint32), oracle.scan(x, "plus"))
