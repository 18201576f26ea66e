"""Builds and runs tests/cpp/test_parallel_primitives.cu: the header-only C++
drop-in API exercised like the reference's own C++ tests (reduction iota sums,
Basel / Wallis scans, fill(1) known answer, intrinsics known answers on the
device, a non-commutative user operator)."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "test_parallel_primitives.cu"
OUT = ROOT / "sycl-building-blocks_gb300" / "_build" / "test_parallel_primitives"


def _compile() -> Path:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    OUT.parent.mkdir(exist_ok=True)
    cmd = [nvcc, "-std=c++20", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-extended-lambda",
           "-I", str(ROOT / "include"), "-I", str(ROOT / "sycl-building-blocks_gb300" / "csrc"), str(SRC), "-o",
           str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return OUT


def test_cpp_api_compiles():
    """The drop-in headers compile for sm_103a (no GPU needed)."""
    if not (shutil.which("nvcc") or Path("/usr/local/cuda/bin/nvcc").exists()):
        pytest.skip("nvcc not available")
    _compile()


@pytest.mark.gpu
def test_cpp_api_runs(cuda):
    exe = _compile()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout[-3000:])
    assert r.returncode == 0 and "ALL PASSED" in r.stdout, r.stdout[-3000:] + r.stderr[-2000:]
