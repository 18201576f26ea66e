"""ctypes view of liboracle.so (TEST INFRASTRUCTURE ONLY: imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline legs as the checker;
never by the product library)."""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

OPS = {"plus": 0, "multiplies": 1, "bit_and": 2, "bit_or": 3, "bit_xor": 4, "minimum": 5, "maximum": 6}
DTYPES = {np.dtype(np.int32): 0, np.dtype(np.uint32): 1, np.dtype(np.int64): 2, np.dtype(np.uint64): 3,
          np.dtype(np.float32): 4, np.dtype(np.float64): 5}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        from build_oracle import build_oracle  # noqa: local recipe

        path = build_oracle()
        L = C.CDLL(str(path))
        vp, u64, i32 = C.c_void_p, C.c_uint64, C.c_int
        L.oracle_scan.argtypes = [i32, i32, i32, vp, vp, u64]
        L.oracle_reduce.argtypes = [i32, i32, vp, u64, vp]
        L.oracle_scan_fp64.argtypes = [i32, i32, vp, vp, u64]
        L.oracle_sum_fp64.argtypes = [i32, vp, u64]
        L.oracle_sum_fp64.restype = C.c_double
        L.oracle_ref_decoupled_scan.argtypes = [i32, i32, i32, vp, vp, u64, i32, u64, i32]
        L.oracle_ref_cooperative_scan.argtypes = [i32, i32, i32, vp, vp, u64, i32]
        L.oracle_ref_reduce.argtypes = [i32, i32, vp, u64, vp, i32]
        L.gen_u32_uniform.argtypes = [u64, vp, u64, C.c_uint32, u64, i32]
        L.gen_u64_uniform.argtypes = [u64, vp, u64, u64, u64, i32]
        L.gen_f32_normal.argtypes = [u64, vp, u64, i32]
        L.gen_f32_signed_lognormal.argtypes = [u64, vp, u64, C.c_double, C.c_double, i32]
        L.splitmix64.argtypes = [u64]
        L.splitmix64.restype = u64
        L.oracle_fnv1a64.argtypes = [vp, u64]
        L.oracle_fnv1a64.restype = u64
        L.oracle_num_threads.restype = i32
        L.oracle_segmented_scan.argtypes = [i32, i32, i32, vp, vp, u64, vp, u64, i32]
        L.oracle_segmented_scan_fp64.argtypes = [i32, i32, vp, vp, u64, vp, u64, i32]
        L.oracle_segmented_reduce.argtypes = [i32, i32, vp, u64, vp, u64, vp, i32]
        L.oracle_segmented_sum_fp64.argtypes = [i32, vp, u64, vp, u64, vp, i32]
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _code(a: np.ndarray) -> int:
    return DTYPES[a.dtype]


def _op(op) -> int:
    return OPS[op] if isinstance(op, str) else int(op)


def scan(a: np.ndarray, op="plus", exclusive: bool = False) -> np.ndarray:
    a = np.ascontiguousarray(a)
    out = np.empty_like(a)
    if lib().oracle_scan(_code(a), _op(op), int(exclusive), _ptr(a), _ptr(out), a.size) != 0:
        raise ValueError("unsupported dtype/op")
    return out


def reduce(a: np.ndarray, op="plus"):
    a = np.ascontiguousarray(a)
    out = np.zeros(1, dtype=a.dtype)
    if lib().oracle_reduce(_code(a), _op(op), _ptr(a), a.size, _ptr(out)) != 0:
        raise ValueError("unsupported dtype/op")
    return out[0]


def scan_fp64(a: np.ndarray, exclusive: bool = False) -> np.ndarray:
    a = np.ascontiguousarray(a)
    out = np.empty(a.size, dtype=np.float64)
    if lib().oracle_scan_fp64(_code(a), int(exclusive), _ptr(a), _ptr(out), a.size) != 0:
        raise ValueError("float inputs only")
    return out


def sum_fp64(a: np.ndarray) -> float:
    a = np.ascontiguousarray(a)
    return float(lib().oracle_sum_fp64(_code(a), _ptr(a), a.size))


def _offsets(offsets: np.ndarray, n: int) -> np.ndarray:
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    if off.size < 1 or off[0] != 0 or off[-1] != n:
        raise ValueError("offsets must start at 0 and end at n")
    return off


def segmented_scan(a: np.ndarray, offsets: np.ndarray, op="plus", exclusive: bool = False,
                   threads: int = 0) -> np.ndarray:
    """Exact scan of every segment [offsets[s], offsets[s+1]) on its own."""
    a = np.ascontiguousarray(a)
    off = _offsets(offsets, a.size)
    out = np.empty_like(a)
    if lib().oracle_segmented_scan(_code(a), _op(op), int(exclusive), _ptr(a), _ptr(out), a.size, _ptr(off),
                                   off.size - 1, threads) != 0:
        raise ValueError("unsupported dtype/op or bad offsets")
    return out


def segmented_scan_fp64(a: np.ndarray, offsets: np.ndarray, exclusive: bool = False, threads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(a)
    off = _offsets(offsets, a.size)
    out = np.empty(a.size, dtype=np.float64)
    if lib().oracle_segmented_scan_fp64(_code(a), int(exclusive), _ptr(a), _ptr(out), a.size, _ptr(off),
                                        off.size - 1, threads) != 0:
        raise ValueError("float inputs only, or bad offsets")
    return out


def segmented_reduce(a: np.ndarray, offsets: np.ndarray, op="plus", threads: int = 0) -> np.ndarray:
    """Reduction of every segment (the identity for an empty one)."""
    a = np.ascontiguousarray(a)
    off = _offsets(offsets, a.size)
    out = np.empty(off.size - 1, dtype=a.dtype)
    if lib().oracle_segmented_reduce(_code(a), _op(op), _ptr(a), a.size, _ptr(off), off.size - 1, _ptr(out),
                                     threads) != 0:
        raise ValueError("unsupported dtype/op or bad offsets")
    return out


def segmented_sum_fp64(a: np.ndarray, offsets: np.ndarray, threads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(a)
    off = _offsets(offsets, a.size)
    out = np.empty(off.size - 1, dtype=np.float64)
    if lib().oracle_segmented_sum_fp64(_code(a), _ptr(a), a.size, _ptr(off), off.size - 1, _ptr(out), threads) != 0:
        raise ValueError("float inputs only, or bad offsets")
    return out


def ref_decoupled_scan(a: np.ndarray, op="plus", exclusive=False, threads=0, local_mem_bytes=65536,
                       force_lookback=False, out: np.ndarray | None = None) -> np.ndarray:
    a = np.ascontiguousarray(a)
    out = np.empty_like(a) if out is None else out
    rc = lib().oracle_ref_decoupled_scan(_code(a), _op(op), int(exclusive), _ptr(a), _ptr(out), a.size, threads,
                                         local_mem_bytes, int(force_lookback))
    if rc != 0:
        raise ValueError("unsupported dtype/op")
    return out


def ref_cooperative_scan(a: np.ndarray, op="plus", exclusive=False, threads=0,
                         out: np.ndarray | None = None) -> np.ndarray:
    a = np.ascontiguousarray(a)
    out = np.empty_like(a) if out is None else out
    if lib().oracle_ref_cooperative_scan(_code(a), _op(op), int(exclusive), _ptr(a), _ptr(out), a.size,
                                         threads) != 0:
        raise ValueError("unsupported dtype/op")
    return out


def ref_reduce(a: np.ndarray, op="plus", threads=0):
    a = np.ascontiguousarray(a)
    out = np.zeros(1, dtype=a.dtype)
    if lib().oracle_ref_reduce(_code(a), _op(op), _ptr(a), a.size, _ptr(out), threads) != 0:
        raise ValueError("unsupported dtype/op")
    return out[0]


def gen_u32(seed: int, n: int, lo: int = 0, hi: int = 1 << 32, threads: int = 0) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().gen_u32_uniform(seed, _ptr(out), n, lo, hi, threads)
    return out


def gen_u64(seed: int, n: int, lo: int = 0, hi: int = 1 << 32, threads: int = 0) -> np.ndarray:
    out = np.empty(n, dtype=np.uint64)
    lib().gen_u64_uniform(seed, _ptr(out), n, lo, hi, threads)
    return out


def gen_i32_full(seed: int, n: int, threads: int = 0) -> np.ndarray:
    return gen_u32(seed, n, 0, 1 << 32, threads).view(np.int32)


def gen_f32_normal(seed: int, n: int, threads: int = 0) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    lib().gen_f32_normal(seed, _ptr(out), n, threads)
    return out


def gen_f32_signed_lognormal(seed: int, n: int, mu: float = 0.0, sigma: float = 2.0,
                             threads: int = 0) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    lib().gen_f32_signed_lognormal(seed, _ptr(out), n, mu, sigma, threads)
    return out


def fnv1a64(a: np.ndarray) -> int:
    a = np.ascontiguousarray(a)
    return int(lib().oracle_fnv1a64(_ptr(a), a.nbytes))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


# ---- the reference's own code on the CPU (oracle/_ref, built where the
# reference checkout exists) ---------------------------------------------------
_ref = None


def ref_lib():
    """ctypes handle of oracle/_ref/libsyclref.so, or None when it is absent."""
    global _ref
    if _ref is None:
        from build_oracle import REF_LIB, build_ref  # noqa: local recipe

        path = build_ref() or (REF_LIB if REF_LIB.exists() else None)
        if path is None:
            return None
        try:
            L = C.CDLL(str(path))
        except OSError:
            return None
        vp, u64, i32 = C.c_void_p, C.c_uint64, C.c_int
        L.ref_scan.argtypes = [i32, i32, i32, i32, vp, vp, u64]
        L.ref_reduce.argtypes = [i32, i32, vp, u64, vp]
        L.ref_funnelshift_l.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        L.ref_funnelshift_l.restype = C.c_uint32
        L.ref_funnelshift_r.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        L.ref_funnelshift_r.restype = C.c_uint32
        L.ref_brev32.argtypes = [C.c_uint32]
        L.ref_brev32.restype = C.c_uint32
        L.ref_brev64.argtypes = [C.c_uint64]
        L.ref_brev64.restype = C.c_uint64
        L.ref_upsample.argtypes = [C.c_uint8] * 4
        L.ref_upsample.restype = C.c_uint32
        L.ref_byte_bit.argtypes = [i32, i32, C.c_uint64, C.c_uint32, C.c_uint32]
        L.ref_byte_bit.restype = C.c_uint64
        L.ref_num_groups.restype = i32
        L.ref_decoupled_scan_u32_plus.argtypes = [vp, vp, u64, i32]
        L.ref_decoupled_scan_u32_plus.restype = i32
        _ref = L
    return _ref


def reference_scan(a: np.ndarray, op="plus", exclusive=False, algo="decoupled") -> np.ndarray:
    a = np.ascontiguousarray(a)
    out = np.empty_like(a)
    rc = ref_lib().ref_scan({"decoupled": 0, "cooperative": 1}[algo], _code(a), _op(op), int(exclusive), _ptr(a),
                            _ptr(out), a.size)
    if rc != 0:
        raise ValueError("unsupported dtype/op")
    return out


def reference_reduce(a: np.ndarray, op="plus"):
    a = np.ascontiguousarray(a)
    out = np.zeros(1, dtype=a.dtype)
    if ref_lib().ref_reduce(_code(a), _op(op), _ptr(a), a.size, _ptr(out)) != 0:
        raise ValueError("unsupported dtype/op")
    return out[0]
