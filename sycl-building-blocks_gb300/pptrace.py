"""Per-tile timelines of the staged decoupled look-back scan and of the
batched segmented scan / reduce.

Compiles tune/tile_trace.cu (the library's own kernel configuration for one
scan policy, built with a recording trace hook), runs one traced launch on the
GPU and summarises where a tile's life goes, in nanoseconds (median, 10th and
90th percentiles over the tiles in steady state, the first and last 300 tiles
left out), plus the median tile period of a CTA:

    python sycl-building-blocks_gb300/pptrace.py u32 32            # 2^32 input bytes
    python sycl-building-blocks_gb300/pptrace.py f32_compensated 32 --keep trace.bin
    python sycl-building-blocks_gb300/pptrace.py seg_i32_reduce 30  # log-uniform segments

For the seg_* policies the ticket event holds when the producer began to wait
for a free stage, and the "scan pass" of a reduction is its totals pass.

Events per tile (16 words; %globaltimer in ns unless noted): 0 data in (seen by
the look-back warp), 1 aggregate published, 2 aggregate seen by the look-back
warp, 3 exclusive prefix known, 4 look-back rounds (value), 5 scan pass
started, 6 scan pass done, 8 CTA index (value), 9 ticket drawn, 10 bulk copy
issued, 11 compute warps start waiting for the data, 12 data at the compute
warps, 13 compute warps start waiting for the prefix, 14 first look-back poll's
round trip (value, ns; policies with pipelined polls).
"""

from __future__ import annotations

import argparse
import json
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
SLOTS = 16


def compile_tracer() -> Path:
    out = PKG / "_build" / "tile_trace"
    src = PKG / "tune" / "tile_trace.cu"
    deps = [src] + list((PKG / "csrc" / "pp").glob("*.cuh"))
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return out
    out.parent.mkdir(exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-extended-lambda",
                    "-I", str(PKG / "csrc"), "-I", str(ROOT / "include"), str(src), "-o", str(out)], check=True)
    return out


def summarise(raw: np.ndarray) -> dict:
    a = raw.reshape(-1, SLOTS).astype(np.int64)
    full, aggpub, lbdone, sstart, sdone = a[:, 0], a[:, 1], a[:, 3], a[:, 5], a[:, 6]
    cta, ticket, issue, rwait, rgot, pwait, pollrt = a[:, 8], a[:, 9], a[:, 10], a[:, 11], a[:, 12], a[:, 13], a[:, 14]
    # segmented reductions record no look-back events: their tiles are independent
    has_lb = bool((lbdone > 0).any())
    ok = (aggpub > 0) & (sdone > 0) & (issue > 0) & (rgot > 0) & (pwait > 0)
    if has_lb:
        ok &= (full > 0) & (lbdone > 0)
    ok[:300] = False
    ok[-300:] = False
    if ok.sum() < 10:
        return {"steady_tiles": int(ok.sum())}

    def q(x):
        x = x[ok]
        return {"p10": int(np.percentile(x, 10)), "p50": int(np.percentile(x, 50)), "p90": int(np.percentile(x, 90))}

    out = {
        "steady_tiles": int(ok.sum()),
        "ticket_to_issue (stage free wait)": q(issue - ticket),
        "issue_to_data_at_compute": q(rgot - issue),
        "compute_waits_for_data": q(rgot - rwait),
        "reduce_pass": q(aggpub - rgot),
        "look_back_from_data_in": q(lbdone - full) if has_lb else None,
        "prefix_known_after_own_aggregate": q(lbdone - aggpub) if has_lb else None,
        "compute_waits_for_prefix": q(sstart - pwait),
        "scan_pass": q(sdone - sstart),
        "stage_life (issue to scan done)": q(sdone - issue),
    }
    if (pollrt[ok] > 0).any():
        out["first_poll_round_trip"] = q(pollrt)
    periods = []
    for c in np.unique(cta[ok]):
        ts = np.sort(issue[ok][cta[ok] == c])
        if len(ts) > 2:
            periods.append(float(np.median(np.diff(ts))))
    out["cta_tile_period_ns"] = float(np.median(periods)) if periods else None
    return out


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("policy", choices=["u32", "f32", "u64", "f64", "f32_compensated", "f32_fp64_carry", "seg_i32",
                                       "seg_f32", "seg_i32_reduce", "seg_f32_reduce"])
    ap.add_argument("log2_bytes", type=int, help="log2 of the input size in bytes (12..34)")
    ap.add_argument("--keep", type=Path, help="also keep the raw per-tile words in this file")
    args = ap.parse_args()
    exe = compile_tracer()
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "trace.bin"
        r = subprocess.run([str(exe), args.policy, str(args.log2_bytes), str(path)], capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            return r.returncode
        head = json.loads(r.stdout.strip().splitlines()[-1])
        raw = np.fromfile(path, dtype=np.uint64)
        if args.keep:
            shutil.copyfile(path, args.keep)
    head["timeline_ns"] = summarise(raw)
    print(json.dumps(head, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
