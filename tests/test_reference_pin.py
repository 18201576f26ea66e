"""Pins the C restatement in oracle/oracle.c directly against the reference's
own code run on the CPU (oracle/_ref, built only where the reference checkout
exists; skipped elsewhere)."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import INT_DTYPES, INT_OPS, make_input


@pytest.fixture(scope="module")
def ref(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference checkout not available: oracle/_ref not built")
    return oracle


@pytest.mark.parametrize("dtype", INT_DTYPES)
@pytest.mark.parametrize("op", INT_OPS)
def test_inclusive_scans_and_reductions_match_reference(ref, dtype, op):
    for n in (1, 17, 16383, 16384, 70001):
        x = make_input(dtype, op, n, seed=n + len(op))
        want = ref.scan(x, op)
        np.testing.assert_array_equal(ref.reference_scan(x, op, False, "decoupled"), want)
        np.testing.assert_array_equal(ref.reference_scan(x, op, False, "cooperative"), want)
        np.testing.assert_array_equal(ref.ref_decoupled_scan(x, op, threads=4), want)
        assert ref.reference_reduce(x, op) == ref.reduce(x, op) == ref.ref_reduce(x, op, threads=3)


@pytest.mark.parametrize("op", ["minimum", "maximum"])
def test_float_min_max_match_reference(ref, op):
    x = make_input("f32", op, 50001, seed=3)
    np.testing.assert_array_equal(ref.reference_scan(x, op), ref.scan(x, op))


def test_float_plus_within_fp64_bound(ref):
    """The reference's float scan order is its own; both it and the oracle stay
    within the FP64 error bound."""
    x = make_input("f32", "plus", 200003, seed=9)
    exact = ref.scan_fp64(x)
    bound = 1e-5 * np.cumsum(np.abs(x.astype(np.float64)))
    assert np.all(np.abs(ref.reference_scan(x, "plus").astype(np.float64) - exact) <= bound)
    assert np.all(np.abs(ref.scan(x, "plus").astype(np.float64) - exact) <= bound)


def test_reference_exclusive_scans_are_defective(ref):
    """scan_over_group returns out[length-1] of the local scan as the partition
    aggregate (scan_decoupled_lookback.hpp:42,163,168), which for an exclusive
    scan omits the partition's last element; the cooperative scan reads chunk
    tails the same way (scan_cooperative.hpp:76). On many partitions the
    reference's exclusive output therefore differs from the exclusive scan."""
    x = np.ones(1 << 20, dtype=np.uint32)
    want = ref.scan(x, exclusive=True)
    assert not np.array_equal(ref.reference_scan(x, "plus", True, "cooperative"), want)
    y = ref.reference_scan(x, "plus", True, "decoupled")
    # every element is either right or short by whole partitions
    assert np.all(y <= want)
