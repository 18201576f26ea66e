"""bench.py's input generator and output checks on the CPU: the device-side
splitmix64 generator gives the oracle's bytes (so the GPU arm, the CPU
baselines and the tests scan identical inputs), and the exact scan checks
accept correct outputs and reject a single wrong element."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


@pytest.mark.parametrize("seed,n,lo,hi", [(0x5CA72026, 100003, 0, 1 << 16), (0x5CA72027, 50001, 0, 1 << 32),
                                          (0x5CA72026, 1 << 16, 0, 256)])
def test_generator_gives_the_oracles_bytes(oracle, seed, n, lo, hi):
    x = bench.splitmix_u32(torch, seed, n, lo, hi, "cpu", chunk=4096)
    assert np.array_equal(x.numpy().view(np.uint32), oracle.gen_u32(seed, n, lo, hi))


def test_scan_checks_accept_correct_and_reject_wrong():
    rng = np.random.default_rng(0)
    d = torch.from_numpy(rng.integers(0, 1 << 16, 10000).astype(np.int32))
    inc = torch.cumsum(d, 0, dtype=torch.int32)
    exc = torch.cat([torch.zeros(1, dtype=torch.int32), inc[:-1]])
    assert bench.check_plus_scan(torch, d, inc, False, chunk=999)
    assert bench.check_plus_scan(torch, d, exc, True, chunk=999)
    bad = inc.clone()
    bad[5000] += 1
    assert not bench.check_plus_scan(torch, d, bad, False, chunk=999)
    assert not bench.check_plus_scan(torch, d, inc, True, chunk=999)
    m = torch.from_numpy(rng.integers(-1000, 1000, 10000).astype(np.int32))
    cm = torch.cummax(m, 0).values
    assert bench.check_max_scan(torch, m, cm, chunk=777)
    cm[3000] = -5000
    assert not bench.check_max_scan(torch, m, cm, chunk=777)


@pytest.mark.parametrize("dtype", [np.int32, np.float32])
def test_segmented_checks_against_the_oracle(oracle, dtype):
    rng = np.random.default_rng(1)
    lens = rng.integers(1, 100, 300)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    n = int(off[-1])
    x = (rng.integers(0, 1000, n) if dtype == np.int32 else rng.standard_normal(n)).astype(dtype)
    y = oracle.segmented_scan(x, off)
    t = oracle.segmented_reduce(x, off)
    tx, to = torch.from_numpy(x), torch.from_numpy(off)
    assert bench.check_segmented_scan(torch, tx, torch.from_numpy(y), to)
    assert bench.check_segmented_reduce(torch, tx, torch.from_numpy(t), to)
    y[77] += 1 if dtype == np.int32 else 0.01
    t[7] += 1 if dtype == np.int32 else 0.01
    assert not bench.check_segmented_scan(torch, tx, torch.from_numpy(y), to)
    assert not bench.check_segmented_reduce(torch, tx, torch.from_numpy(t), to)
