"""Randomised stress of the scan kernels against the oracle: 1,000 calls with
random element type, operator, scan kind, length (log-uniform up to 2^23),
algorithm and 16-byte phases of the input and output pointers, back to back
on one stream, so that look-back races and stale-descriptor bugs that show
only under particular timings get many chances to appear."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import INT_DTYPES, NP, check_scan, empty_dev, from_dev, make_input, to_dev

pytestmark = pytest.mark.gpu

CASES = [("u32", "plus"), ("i32", "maximum"), ("i32", "bit_xor"), ("u64", "plus"), ("i64", "minimum"),
         ("f32", "plus"), ("f64", "plus"), ("f32", "maximum")]


def test_random_scans_against_the_oracle(pp, oracle, cuda):
    rng = np.random.default_rng(2026)
    s = cuda.cuda.current_stream().cuda_stream
    for it in range(1000):
        dtype, op = CASES[rng.integers(len(CASES))]
        n = int(np.exp(rng.uniform(0, np.log(1 << 23))))
        excl = bool(rng.integers(2))
        algo = ["decoupled", "decoupled", "decoupled", "cooperative"][rng.integers(4)]
        esz = np.dtype(NP[dtype]).itemsize
        off_in, off_out = (int(rng.integers(16 // esz)), int(rng.integers(16 // esz)))
        x = make_input(dtype, op, n, seed=1000 + it)
        d_in = to_dev(cuda, np.concatenate([np.zeros(off_in, dtype=x.dtype), x]))
        d_out = empty_dev(cuda, n, NP[dtype], pad=off_out)
        pp.scan("exclusive" if excl else "inclusive", op, d_in.data_ptr() + off_in * esz,
                d_out.data_ptr() + off_out * esz, n, dtype, stream=s, algo=algo)
        assert pp.stream_status(s) == 0, (it, dtype, op, n)
        got = from_dev(d_out, NP[dtype])[off_out:]
        tiles = (n + 1023) // 1024 + 2
        try:
            check_scan(got, x, dtype, op, excl, tiles)
        except AssertionError as e:
            raise AssertionError(f"case {it}: {dtype}/{op} n={n} excl={excl} algo={algo} "
                                 f"phases=({off_in},{off_out}): {e}") from None
