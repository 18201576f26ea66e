"""Helpers shared by the GPU tests: seeded inputs per (dtype, op), device
round trips through torch storage, and the floating-point error bounds the
scans are held to."""

from __future__ import annotations

import numpy as np

import pyoracle

NP = {"i32": np.int32, "u32": np.uint32, "i64": np.int64, "u64": np.uint64, "f32": np.float32,
      "f64": np.float64}
INT_DTYPES = ["i32", "u32", "i64", "u64"]
FLOAT_DTYPES = ["f32", "f64"]
INT_OPS = ["plus", "multiplies", "bit_and", "bit_or", "bit_xor", "minimum", "maximum"]
FLOAT_OPS = ["plus", "multiplies", "minimum", "maximum"]
EPS = {"f32": float(np.finfo(np.float32).eps), "f64": float(np.finfo(np.float64).eps)}


def make_input(dtype: str, op: str, n: int, seed: int) -> np.ndarray:
    """Seeded input for a (dtype, op) pair; multiplies on floats stays near 1
    so long products neither overflow nor underflow."""
    if dtype in ("u32", "i32"):
        a = pyoracle.gen_u32(seed, n)
        if op == "bit_and":  # mostly-ones words keep the running AND non-trivial
            a = a | pyoracle.gen_u32(seed + 1, n) | pyoracle.gen_u32(seed + 2, n)
        return a.view(NP[dtype])
    if dtype in ("u64", "i64"):
        lo = pyoracle.gen_u64(seed, n, 0, 1 << 32)
        hi = pyoracle.gen_u64(seed + 7, n, 0, 1 << 32)
        a = (hi << np.uint64(32)) | lo
        if op == "bit_and":
            a = a | pyoracle.gen_u64(seed + 1, n, 0, 1 << 63) | pyoracle.gen_u64(seed + 2, n, 0, 1 << 63)
        return a.view(NP[dtype])
    x = pyoracle.gen_f32_normal(seed, n)
    if op == "multiplies":
        x = (1.0 + 1e-3 * x).astype(np.float32)
    return x.astype(NP[dtype])


_SIGNED_VIEW = {np.dtype(np.uint32): np.int32, np.dtype(np.uint64): np.int64}


def to_dev(torch, a: np.ndarray):
    """numpy -> CUDA tensor holding the same bytes (unsigned viewed as signed)."""
    view = _SIGNED_VIEW.get(a.dtype, a.dtype)
    return torch.from_numpy(np.ascontiguousarray(a).view(view)).cuda()


def from_dev(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(np.dtype(dtype))


def empty_dev(torch, n: int, dtype, pad: int = 0):
    view = _SIGNED_VIEW.get(np.dtype(dtype), np.dtype(dtype))
    return torch.empty(n + pad, dtype=getattr(torch, np.dtype(view).name), device="cuda")


def float_scan_bound(x: np.ndarray, dtype: str, tiles: int) -> np.ndarray:
    """Worst-case error bound of a scan combining in a tree of depth
    <= 64 + tiles (in-tile tree + the cross-tile carry chain):
    |err_i| <= (64 + tiles) * eps * sum_{j<=i} |x_j|."""
    cabs = np.cumsum(np.abs(x.astype(np.float64)))
    return (64 + tiles) * EPS[dtype] * cabs + np.finfo(np.float64).tiny


def check_scan(got: np.ndarray, x: np.ndarray, dtype: str, op: str, exclusive: bool, tiles: int) -> None:
    if dtype in INT_DTYPES or op in ("minimum", "maximum"):
        want = pyoracle.scan(x, op, exclusive)
        if not np.array_equal(got, want):
            bad = np.nonzero(got != want)[0]
            raise AssertionError(f"{dtype}/{op}/excl={exclusive}: {bad.size} mismatches, first at {bad[0]}: "
                                 f"got {got[bad[0]]} want {want[bad[0]]}")
        return
    if op == "plus":
        want = pyoracle.scan_fp64(x, exclusive)
        bound = float_scan_bound(x, dtype, tiles)
        if exclusive:
            bound = np.concatenate([[np.finfo(np.float64).tiny], bound[:-1]])
        err = np.abs(got.astype(np.float64) - want)
        assert np.all(err <= bound), f"{dtype}/plus: max err/bound {np.max(err / bound):.3g}"
        return
    # multiplies: relative error grows with the chain length
    want = np.cumprod(x.astype(np.float64))
    if exclusive:
        want = np.concatenate([[1.0], want[:-1]])
    rel = np.abs(got.astype(np.float64) - want) / np.abs(want)
    assert np.max(rel) <= (64 + tiles) * EPS[dtype] * 8, f"{dtype}/multiplies: max rel {np.max(rel):.3g}"
