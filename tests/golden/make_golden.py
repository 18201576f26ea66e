"""Generate tests/golden/reference_outputs.json from the reference's OWN code.

Runs the reference headers (compiled unmodified against the SYCL CPU shim,
oracle/_ref/libsyclref.so, built by oracle/build_oracle.py where the reference
checkout exists) on seeded inputs and records the results: FNV-1a-64 of every
scan output plus a few values, reduction results, and the reference's
intrinsics on the known-answer operands of tests/test_intrinsics.cpp.

Inputs are regenerated by the consumer from the recorded generator
parameters: element i of stream `seed` is mix64(seed + (i + 1) *
0x9E3779B97F4A7C15) (splitmix64), mapped to [lo, hi) by
lo + ((x >> 32) * (hi - lo) >> 32) for 32-bit values and
lo + ((x * (hi - lo)) >> 64) for 64-bit values (oracle/oracle.c).

A second file, tests/golden/intrinsics_bytes_bits.json, holds the
reference's byte / bit helpers (include/intrinsics.hpp:150-202: get_byte,
set_byte, both set_bit_in_word overloads, read_bit, flip_bit) evaluated on
words of 1, 2, 4 and 8 bytes at every byte / bit position (see
byte_bit_cases()).

Usage:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT / "oracle")]
import pyoracle  # noqa: E402

INT_OPS = ["plus", "multiplies", "bit_and", "bit_or", "bit_xor", "minimum", "maximum"]
NP = {"i32": np.int32, "u32": np.uint32, "i64": np.int64, "u64": np.uint64}


def gen(dtype: str, n: int, seed: int, lo: int, hi: int) -> np.ndarray:
    if dtype in ("u32", "i32"):
        return pyoracle.gen_u32(seed, n, lo, hi).view(NP[dtype])
    return pyoracle.gen_u64(seed, n, lo, hi).view(NP[dtype])


BYTE_VALUES = [0x00, 0x5A, 0xFF]


def byte_bit_words(width: int) -> list[int]:
    """Operand words of one width: zero, all ones, an alternating pattern and
    two splitmix64 words, truncated to the width."""
    mask = (1 << (8 * width)) - 1
    return [0, mask, 0xA5C3_0F96_5A3C_F069 & mask, pyoracle.lib().splitmix64(width) & mask,
            pyoracle.lib().splitmix64(100 + width) & mask]


def byte_bit_cases(ref) -> list[dict]:
    """Every helper at every position of every operand word; per word the
    results are lists indexed by position (bytes, or bits)."""
    out = []
    for width in (1, 2, 4, 8):
        for w in byte_bit_words(width):
            e = {"width": width, "word": w,
                 "get_byte": [int(ref.ref_byte_bit(0, width, w, p, 0)) for p in range(width)],
                 "set_byte": {str(b): [int(ref.ref_byte_bit(1, width, w, p, b)) for p in range(width)]
                              for b in BYTE_VALUES}}
            bits = range(8 * width)
            e["set_bit_true"] = [int(ref.ref_byte_bit(2, width, w, i, 1)) for i in bits]
            e["set_bit_false"] = [int(ref.ref_byte_bit(2, width, w, i, 0)) for i in bits]
            e["set_bit_runtime_true"] = [int(ref.ref_byte_bit(3, width, w, i, 1)) for i in bits]
            e["set_bit_runtime_false"] = [int(ref.ref_byte_bit(3, width, w, i, 0)) for i in bits]
            e["read_bit"] = [int(ref.ref_byte_bit(4, width, w, i, 0)) for i in bits]
            e["flip_bit"] = [int(ref.ref_byte_bit(5, width, w, i, 0)) for i in bits]
            out.append(e)
    return out


def main() -> None:
    ref = pyoracle.ref_lib()
    if ref is None:
        raise SystemExit("oracle/_ref/libsyclref.so is not available (needs the reference checkout)")
    cases, reductions = [], []
    # value ranges per dtype: full 32-bit words, and 64-bit words built from the
    # full 2^63 range so every bit position is exercised
    ranges = {"u32": (0, 1 << 32), "i32": (0, 1 << 32), "u64": (0, 1 << 63), "i64": (0, 1 << 63)}
    sizes = [1, 1000, 16385, 300007]
    seed = 0x5CA72026
    for dtype in ("i32", "u32", "i64", "u64"):
        lo, hi = ranges[dtype]
        for op in INT_OPS:
            for n in sizes:
                seed += 1
                x = gen(dtype, n, seed, lo, hi)
                for algo in ("decoupled", "cooperative"):
                    y = pyoracle.reference_scan(x, op, False, algo)
                    cases.append({"dtype": dtype, "op": op, "algo": algo, "kind": "inclusive", "n": n,
                                  "seed": seed, "lo": lo, "hi": hi, "fnv1a64": f"{pyoracle.fnv1a64(y):016x}",
                                  "head": [int(v) for v in y[:3]], "tail": [int(v) for v in y[-3:]]})
                r = pyoracle.reference_reduce(x, op)
                reductions.append({"dtype": dtype, "op": op, "n": n, "seed": seed, "lo": lo, "hi": hi,
                                   "value": int(r)})
    # the CPU-runnable headline configuration: n = 2^24 uint32 U[0, 255]
    n24 = 1 << 24
    x = gen("u32", n24, 0x5CA72026, 0, 256)
    y = pyoracle.reference_scan(x, "plus", False, "decoupled")
    headline = {"dtype": "u32", "op": "plus", "n": n24, "seed": 0x5CA72026, "lo": 0, "hi": 256,
                "scan_fnv1a64": f"{pyoracle.fnv1a64(y):016x}", "scan_last": int(y[-1]),
                "sum": int(pyoracle.reference_reduce(x, "plus"))}
    # intrinsics on the operands of tests/test_intrinsics.cpp:9-26
    hi_w, lo_w = 0xDEADBEEF, 0xCAFED00D
    intrinsics = {
        "funnelshift_l": {str(s): int(ref.ref_funnelshift_l(lo_w, hi_w, s)) for s in range(0, 31)},
        "funnelshift_r": {str(s): int(ref.ref_funnelshift_r(lo_w, hi_w, s)) for s in range(0, 31)},
        "brev32": {str(v): int(ref.ref_brev32(v)) for v in (0, 1, 2, 0xF, lo_w, hi_w)},
        "brev64": {str(v): int(ref.ref_brev64(v)) for v in (0, 1, 0xF, lo_w, 0x0123456789ABCDEF)},
        "upsample_SYCL": int(ref.ref_upsample(ord("S"), ord("Y"), ord("C"), ord("L"))),
    }
    out = {
        "generator": "splitmix64 stream: x_i = mix64(seed + (i+1)*0x9E3779B97F4A7C15); 32-bit: "
                     "lo + ((x>>32)*(hi-lo)>>32); 64-bit: lo + ((x*(hi-lo))>>64)",
        "producer": "reference headers (SYCL-Building-Blocks include/) compiled with g++ against the "
                    "oracle/sycl_shim CPU shim, -fwrapv; work-group size 1, 64 KiB local memory",
        "scans": cases,
        "reductions": reductions,
        "headline_2p24": headline,
        "intrinsics": intrinsics,
    }
    (HERE / "reference_outputs.json").write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {len(cases)} scans, {len(reductions)} reductions")
    bb = {"producer": out["producer"],
          "ops": "get_byte(word, pos); set_byte(word, byte, pos) per byte value; set_bit_in_word<true|false>(word, "
                 "idx); set_bit_in_word(word, idx, bool); read_bit(word, idx) as 0/1; flip_bit(word, idx)",
          "cases": byte_bit_cases(ref)}
    (HERE / "intrinsics_bytes_bits.json").write_text(json.dumps(bb, separators=(",", ":")) + "\n")
    print(f"wrote {len(bb['cases'])} byte/bit operand words")


if __name__ == "__main__":
    main()
