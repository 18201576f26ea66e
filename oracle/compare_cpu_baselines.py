"""Times the reference's own decoupled look-back scan (the reference headers
compiled against the SYCL CPU shim, oracle/_ref/libsyclref.so) beside the C
restatement of the same algorithm (oracle/oracle.c) and the sequential
oracle, on one input and the same host cores (TEST INFRASTRUCTURE ONLY).

The GPU machine is an Arm machine without the reference checkout, so its CPU
baseline is the C restatement; this script relates the two where both exist
(the reference checkout's machine): same input (the headline workload, n
uint32 U[0, 2^16) from the splitmix64 stream, seed 0x5CA72026), same thread
count (every core), the best of --reps runs each after one warm-up run, and
every output checked against the sequential oracle.

Usage:  python oracle/compare_cpu_baselines.py [--n N] [--reps R]
Prints one JSON object: GB/s (2n * 4 bytes per scan) of each, and the ratio
port / reference.
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import pyoracle  # noqa: E402

SEED = 0x5CA72026


def best_of(fn, reps: int) -> float:
    fn()  # warm-up
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 30)
    ap.add_argument("--reps", type=int, default=5)
    ns = ap.parse_args()
    ref = pyoracle.ref_lib()
    if ref is None:
        raise SystemExit("oracle/_ref/libsyclref.so is not available here (needs the reference checkout)")
    n = ns.n
    a = pyoracle.gen_u32(SEED, n, 0, 1 << 16)
    want = pyoracle.scan(a, "plus")
    out = np.empty_like(a)
    gb = 2 * n * 4 / 1e9

    def reference():
        if ref.ref_decoupled_scan_u32_plus(a.ctypes.data, out.ctypes.data, n, 0) != 0:
            raise RuntimeError("reference scan failed")

    def port():
        pyoracle.ref_decoupled_scan(a, "plus", False, threads=0, out=out)

    res = {"n": n, "cores": pyoracle.num_threads(), "reference_groups": int(ref.ref_num_groups()),
           "machine": platform.machine(), "cpu": platform.processor() or platform.machine()}
    t_ref = best_of(reference, ns.reps)
    res["reference_matches_oracle"] = bool(np.array_equal(out, want))
    t_port = best_of(port, ns.reps)
    res["port_matches_oracle"] = bool(np.array_equal(out, want))
    t_seq = best_of(lambda: pyoracle.scan(a, "plus"), max(1, ns.reps // 2))
    res.update({"reference_gbs": round(gb / t_ref, 2), "port_gbs": round(gb / t_port, 2),
                "sequential_oracle_gbs": round(gb / t_seq, 2), "port_over_reference": round(t_ref / t_port, 3),
                "reps": ns.reps, "timing": "best of reps after one warm-up run, wall clock"})
    print(json.dumps(res))


if __name__ == "__main__":
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    main()
