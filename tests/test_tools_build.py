"""The measurement tools that are not part of the library build still compile
for sm_103a against the current kernels (no GPU): the segmented-scan
autotuner (one payload type) and the per-tile trace harness."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "sycl-building-blocks_gb300"


def test_autotuner_and_trace_harness_compile(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    base = [nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-extended-lambda",
            "-I", str(PKG / "csrc"), "-I", str(ROOT / "include"), "-c"]
    jobs = [
        base + ["-DPP_TUNE_DT=0", str(PKG / "tune" / "seg_autotune.cu"), "-o", str(tmp_path / "seg_autotune.o")],
        base + [str(PKG / "tune" / "tile_trace.cu"), "-o", str(tmp_path / "tile_trace.o")],
    ]
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for j in jobs]
    for j, p in zip(jobs, procs):
        out, _ = p.communicate(timeout=900)
        assert p.returncode == 0, f"{Path(j[-3]).name} failed to compile:\n{out[-4000:]}"
