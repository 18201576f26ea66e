"""Autotuner of the batched segmented scan.

Compiles tune/seg_autotune.cu (every variant of the segmented kernel over
compute warps {4, 8, 16} = block size {128, 256, 512} threads, items per
thread {4, 8, 16, 32} and chunk vector width {4, 8, 16} bytes), runs it on the
GPU on the batched workload (65,536 log-uniform segments, int32 and float32
payloads), records every measurement in tune/seg_autotune_results.json and
writes the variant with the best worst-case throughput over the two payloads
to csrc/pp/seg_tuned.inc, which the library's segmented launches use for
4-byte elements.

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


def compile_tuner() -> Path:
    out = PKG / "_build" / "seg_autotune"
    out.parent.mkdir(exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-extended-lambda",
           "-I", str(PKG / "csrc"), "-I", str(ROOT / "include"), str(PKG / "tune" / "seg_autotune.cu"), "-o", str(out)]
    subprocess.run(cmd, check=True)
    return out


def run(exe: Path) -> list[dict]:
    r = subprocess.run([str(exe)], capture_output=True, text=True, check=True, timeout=1200)
    rows = []
    for line in r.stdout.splitlines():
        line = line.strip()
        if line.startswith("{"):
            rows.append(json.loads(line))
    return rows


def choose(rows: list[dict]) -> dict:
    ok = [r for r in rows if "ms" in r and r.get("err") == 0 and r.get("matches_default")]
    by_key: dict[tuple, dict] = {}
    for r in ok:
        by_key.setdefault((r["nc"], r["items"], r["vb"]), {})[r["dtype"]] = r
    best, best_score = None, -1.0
    for key, d in by_key.items():
        if len(d) < 2:
            continue
        score = min(v["elems_per_s"] for v in d.values())
        if score > best_score:
            best, best_score = key, score
    if best is None:
        raise RuntimeError("no valid variant")
    return {"nc": best[0], "items": best[1], "vb": best[2], "worst_case_elems_per_s": best_score}


def write_inc(choice: dict, device: str) -> Path:
    inc = PKG / "csrc" / "pp" / "seg_tuned.inc"
    inc.write_text(
        "// Generated by ppautotune.py: segmented-scan variant with the best worst-case\n"
        f"// throughput over int32 and float32 payloads on {device}, batched workload of\n"
        "// 65,536 log-uniform segments (see tune/seg_autotune_results.json).\n"
        f"#define PP_SEG_TUNED_4B_NC {choice['nc']}\n"
        f"#define PP_SEG_TUNED_4B_ITEMS {choice['items']}\n"
        f"#define PP_SEG_TUNED_4B_VB {choice['vb']}\n")
    return inc


def main() -> None:
    exe = compile_tuner()
    t0 = time.time()
    rows = run(exe)
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
