"""Builds and runs the C++ tests of the header-only drop-in API:

* tests/cpp/test_parallel_primitives.cu - exercised like the reference's own
  C++ tests (reduction iota sums, Basel / Wallis scans, fill(1) known answer,
  intrinsics known answers on the device, a non-commutative user operator,
  the subset grid barrier);
* tests/cpp/test_reference_call_shapes.cu - the reference's call sites
  (tests/test_reduction.cpp, benchmarks/benchmark_reduce.cpp,
  benchmarks/benchmark_scan.cpp) with only the queue and the functor's
  namespace replaced: usm_unique_ptr buffers with get_span(), spans of
  non-const T, and the trailing optimised_offload / offload_threshold
  template parameters."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
BUILD = ROOT / "sycl-building-blocks_gb300" / "_build"
PROGRAMS = ["test_parallel_primitives", "test_reference_call_shapes"]


def _nvcc() -> str | None:
    if shutil.which("nvcc"):
        return shutil.which("nvcc")
    p = Path("/usr/local/cuda/bin/nvcc")
    return str(p) if p.exists() else None


def _compile(name: str) -> Path:
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    BUILD.mkdir(exist_ok=True)
    out = BUILD / name
    cmd = [nvcc, "-std=c++20", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-extended-lambda",
           "-I", str(ROOT / "include"), "-I", str(ROOT / "sycl-building-blocks_gb300" / "csrc"),
           str(ROOT / "tests" / "cpp" / f"{name}.cu"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


@pytest.mark.parametrize("name", PROGRAMS)
def test_cpp_api_compiles(name):
    """The drop-in headers compile for sm_103a with these call sites (no GPU needed)."""
    _compile(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", PROGRAMS)
def test_cpp_api_runs(cuda, name):
    exe = _compile(name)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout[-3000:])
    assert r.returncode == 0 and "ALL PASSED" in r.stdout, r.stdout[-3000:] + r.stderr[-2000:]
