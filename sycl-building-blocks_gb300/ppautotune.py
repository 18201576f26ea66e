"""Autotuner of the batched segmented scan.

Compiles tune/seg_autotune.cu once per payload type, in parallel (variants of
the segmented kernel: striped chunks over compute warps {4, 8, 16} = block size
{128, 256, 512} threads, items per thread {4, 8, 16, 32} and chunk vector width
{8, 16} bytes; lane rows over {12, 14, 16, 18, 20} warps with {5, 7, 9} 16-byte
chunks per lane, look-back polls of {1, 4} windows and, with one-window polls,
an optional store warp), runs the binaries one
after another on the GPU on two length distributions ("long": 65,536
log-uniform segments in [1, 2^16]; "short": 2^21 segments of U[1, 128]) with
int32, float32, int64 and float64 payloads, records every measurement in tune/seg_autotune_results.json and
writes, per payload type and distribution, the fastest variant to
csrc/pp/seg_tuned.inc. The library's CSR segmented launches pick the long or
short variant from the mean segment length; unsigned payloads take the variant
of the signed type of their size.

    python sycl-building-blocks_gb300/ppautotune.py                  # measure and choose
    python sycl-building-blocks_gb300/ppautotune.py --from-results   # choose again from the saved run
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


DTYPES = ("i32", "f32", "i64", "f64")


def choose(rows: list[dict]) -> dict:
    """Fastest variant per (payload type, distribution)."""
    ok = [r for r in rows if "ms" in r and r.get("err") == 0 and r.get("matches_default")]
    out = {}
    for dt in DTYPES:
        for dist in ("long", "short"):
            cand = [r for r in ok if r["dtype"] == dt and r["dist"] == dist]
            if not cand:
                raise RuntimeError(f"no valid variant for {dt} payloads, {dist} segments")
            b = max(cand, key=lambda r: r["elems_per_s"])
            out[f"{dt}_{dist}"] = {"lay": b["lay"], "nc": b["nc"], "ch": b["ch"], "vb": b["vb"],
                                   "lbw": b.get("lbw", 4), "bs": b.get("bs", 0), "elems_per_s": b["elems_per_s"]}
    return out


def write_inc(choice: dict, device: str) -> Path:
    inc = PKG / "csrc" / "pp" / "seg_tuned.inc"
    lines = ["// Generated by ppautotune.py: the fastest segmented-scan variant per payload",
             f"// type and segment-length class on {device}",
             "// (see tune/seg_autotune_results.json)."]
    for key, c in choice.items():
        dt, dist = key.split("_")
        for f in ("lay", "nc", "ch", "vb", "lbw", "bs"):
            lines.append(f"#define PP_SEG_{dt.upper()}_{dist.upper()}_{f.upper()} {c[f]}")
    inc.write_text("\n".join(lines) + "\n")
    return inc


def main() -> None:
    results = PKG / "tune" / "seg_autotune_results.json"
    if "--from-results" in sys.argv:  # choose again from the committed measurements, no GPU needed
        saved = json.loads(results.read_text())
        rows, device, seconds = saved["rows"], saved["device"], saved["seconds"]
    else:
        exes = compile_tuners()
        t0 = time.time()
        rows = run(exes)
        seconds = round(time.time() - t0, 1)
        try:
            device = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"], capture_output=True,
                                    text=True).stdout.strip().splitlines()[0]
        except Exception:
            device = "unknown GPU"
    choice = choose(rows)
    # one measurement per line
    body = ",\n  ".join(json.dumps(r, separators=(",", ":")) for r in rows)
    head = json.dumps({"device": device, "seconds": seconds, "choice": choice}, indent=1)[:-2]
    results.write_text(head + ',\n "rows": [\n  ' + body + "\n ]\n}\n")
    print(write_inc(choice, device), choice)


if __name__ == "__main__":
    sys.exit(main())
