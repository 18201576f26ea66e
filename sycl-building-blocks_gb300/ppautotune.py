"""Autotuner of the batched segmented scan.

Compiles tune/seg_autotune.cu once per payload type, in parallel (variants of
the segmented kernel: striped chunks over compute warps {4, 8, 16} = block size
{128, 256, 512} threads, items per thread {4, 8, 16, 32} and chunk vector width
{8, 16} bytes; lane rows over {12, 14, 16, 18, 20} warps with {5, 7, 9} 16-byte
chunks per lane), runs the binaries one after another on the GPU
on two length distributions ("long": 65,536 log-uniform segments in [1, 2^16];
"short": 2^21 segments of U[1, 128]) with int32, float32, int64 and float64
payloads, records every measurement in tune/seg_autotune_results.json and
writes, per payload size (4 / 8 bytes) and distribution, the variant with the
best worst-case throughput over that size's two payloads to
csrc/pp/seg_tuned.inc. The library's CSR segmented launches pick the long or
short variant from the mean segment length.

    python sycl-building-blocks_gb300/ppautotune.py
"""

from __future__ import annotations

import json
import shutil
import subprocess
import sys
import time
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent


def compile_tuners() -> list[Path]:
    """One binary per payload type (int32, float32, int64, float64), compiled in parallel."""
    (PKG / "_build").mkdir(exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    outs, procs = [], []
    for dt in range(4):
        out = PKG / "_build" / f"seg_autotune_{dt}"
        cmd = [nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-extended-lambda",
               f"-DPP_TUNE_DT={dt}", "-I", str(PKG / "csrc"), "-I", str(ROOT / "include"),
               str(PKG / "tune" / "seg_autotune.cu"), "-o", str(out)]
        procs.append(subprocess.Popen(cmd))
        outs.append(out)
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("compiling the segmented-scan autotuner failed")
    return outs


def run(exes: list[Path]) -> list[dict]:
    rows = []
    for exe in exes:
        r = subprocess.run([str(exe)], capture_output=True, text=True, check=True, timeout=2400)
        for line in r.stdout.splitlines():
            line = line.strip()
            if line.startswith("{"):
                rows.append(json.loads(line))
    return rows


SIZES = {"i32": 4, "f32": 4, "i64": 8, "f64": 8}


def choose(rows: list[dict]) -> dict:
    """Best worst-case variant per (payload size, distribution)."""
    ok = [r for r in rows if "ms" in r and r.get("err") == 0 and r.get("matches_default")]
    out = {}
    for size in (4, 8):
        for dist in ("long", "short"):
            by_key: dict[tuple, dict] = {}
            for r in ok:
                if SIZES[r["dtype"]] == size and r["dist"] == dist:
                    by_key.setdefault((r["lay"], r["nc"], r["ch"], r["vb"]), {})[r["dtype"]] = r
            best, best_score = None, -1.0
            for key, d in by_key.items():
                if len(d) < 2:
                    continue
                score = min(v["elems_per_s"] for v in d.values())
                if score > best_score:
                    best, best_score = key, score
            if best is None:
                raise RuntimeError(f"no valid variant for {size}-byte payloads, {dist} segments")
            out[f"{size}B_{dist}"] = {"lay": best[0], "nc": best[1], "ch": best[2], "vb": best[3],
                                      "worst_case_elems_per_s": best_score}
    return out


def write_inc(choice: dict, device: str) -> Path:
    inc = PKG / "csrc" / "pp" / "seg_tuned.inc"
    lines = ["// Generated by ppautotune.py: segmented-scan variants with the best worst-case",
             f"// throughput per payload size and segment-length class on {device}",
             "// (see tune/seg_autotune_results.json)."]
    for key, c in choice.items():
        size, dist = key.split("_")
        for f in ("lay", "nc", "ch", "vb"):
            lines.append(f"#define PP_SEG_{size}_{dist.upper()}_{f.upper()} {c[f]}")
    inc.write_text("\n".join(lines) + "\n")
    return inc


def main() -> None:
    exes = compile_tuners()
    t0 = time.time()
    rows = run(exes)
    choice = choose(rows)
    try:
        device = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"], capture_output=True,
                                text=True).stdout.strip().splitlines()[0]
    except Exception:
        device = "unknown GPU"
    (PKG / "tune" / "seg_autotune_results.json").write_text(
        json.dumps({"device": device, "seconds": round(time.time() - t0, 1), "choice": choice, "rows": rows},
                   indent=1) + "\n")
    print(write_inc(choice, device), choice)


if __name__ == "__main__":
    sys.exit(main())
