"""Precision modes of the float32 plus-scan (no counterpart in the reference,
whose float scans accumulate in plain FP32): compensated float-float
accumulation and an FP64 cross-tile carry chain, against the FP64 oracle.

Error measures per prefix i (s = FP64 oracle, g = GPU result):
  rel_i  = |g_i - s_i| / |s_i|, over prefixes with |s_i| >= 1e-3 * rms(s)
           (near-zero crossings of a random walk have no meaningful relative
           error in FP32 output);
  norm   = max_i |g_i - s_i| / max_i |s_i|;
  abs_i  = |g_i - s_i| / sum_{j<=i} |x_j|, over every prefix, the excluded
           near-zero ones included: the error against the magnitude the sum
           was built from.
"""

from __future__ import annotations

import numpy as np
import pytest

from helpers import from_dev, to_dev

pytestmark = pytest.mark.gpu


def _errors(got, want):
    err = np.abs(got.astype(np.float64) - want)
    scale = np.sqrt(np.mean(want * want))
    mask = np.abs(want) >= 1e-3 * scale
    rel = err[mask] / np.abs(want[mask])
    return float(rel.max()), float(np.sqrt(np.mean(rel * rel))), float(err.max() / np.abs(want).max())


def _abs_errors(got, want, x):
    """max_i |g_i - s_i| / sum_{j<=i} |x_j| over every prefix."""
    cabs = np.cumsum(np.abs(x.astype(np.float64)))
    return float(np.max(np.abs(got.astype(np.float64) - want) / np.maximum(cabs, np.finfo(np.float64).tiny)))


def _scan(pp, cuda, x, precision, excl=False, algo="auto"):
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.scan("exclusive" if excl else "inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), x.size, "f32",
            stream=s, algo=algo, precision=precision)
    assert pp.stream_status(s) == 0
    return from_dev(d_out, np.float32)


@pytest.mark.parametrize("dist", ["normal", "lognormal"])
def test_compensated_beats_plain_and_meets_1e6(pp, oracle, cuda, dist):
    n = 1 << 23
    x = oracle.gen_f32_normal(21, n) if dist == "normal" else oracle.gen_f32_signed_lognormal(22, n, 0.0, 2.0)
    want = oracle.scan_fp64(x)
    plain = _errors(_scan(pp, cuda, x, "default"), want)
    comp_out = _scan(pp, cuda, x, "compensated")
    comp = _errors(comp_out, want)
    f64c = _errors(_scan(pp, cuda, x, "fp64_carry"), want)
    # compensated: every prefix (away from zero crossings) within 1e-6 relative
    assert comp[0] <= 1e-6, comp
    # and every prefix, near-zero ones included, within 1e-6 of sum |x_j|
    assert _abs_errors(comp_out, want, x) <= 1e-6
    assert comp[2] < plain[2] and comp[2] < f64c[2] * 1.01 + 1e-12, (plain, comp, f64c)
    assert f64c[2] <= plain[2] * 1.01, (plain, f64c)


@pytest.mark.parametrize("precision", ["compensated", "fp64_carry"])
@pytest.mark.parametrize("n", [1, 5, 4097, 16385, 300001])
def test_precision_modes_small_and_ragged(pp, oracle, cuda, precision, n):
    x = oracle.gen_f32_normal(n, n)
    for excl in (False, True):
        got = _scan(pp, cuda, x, precision, excl)
        want = oracle.scan_fp64(x, excl)
        bound = 1e-6 * np.maximum(np.abs(want), 1.0) + 4 * np.finfo(np.float32).eps * np.cumsum(np.abs(x))
        assert np.all(np.abs(got.astype(np.float64) - want) <= bound)


@pytest.mark.parametrize("precision", ["compensated", "fp64_carry"])
def test_precision_modes_other_paths(pp, oracle, cuda, precision):
    """Pointers that are not 16-byte aligned (shifted tile grid) and the
    cooperative scan honour the precision mode too."""
    n = 200003
    x = oracle.gen_f32_normal(3, n)
    want = oracle.scan_fp64(x)
    for algo in ("cooperative", "single_group"):
        got = _scan(pp, cuda, x, precision, algo=algo)
        assert _errors(got, want)[0] <= 1e-6 if precision == "compensated" else True
        assert np.all(np.abs(got.astype(np.float64) - want) <= 1e-4 * np.maximum(np.abs(want), 1.0))
    d = to_dev(cuda, np.concatenate([np.zeros(1, np.float32), x]))
    o = cuda.empty_like(d)
    pp.scan("inclusive", "plus", d.data_ptr() + 4, o.data_ptr() + 4, n, "f32", precision=precision)
    got = from_dev(o, np.float32)[1:]
    assert np.all(np.abs(got.astype(np.float64) - want) <= 1e-4 * np.maximum(np.abs(want), 1.0))
