"""Build libppgb300.so: every CUDA translation unit under csrc/ compiled for
sm_103a in parallel with nvcc, linked into one shared library next to this
file. Incremental: a content hash of the sources and flags is kept in
_build/stamp and the build is skipped when nothing changed and the library is
present."""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libppgb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "--expt-extended-lambda"]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _hash_inputs(extra: list[str]) -> str:
    h = hashlib.sha256()
    files = sorted(list(CSRC.rglob("*.cu")) + list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.inc")) +
                   list((ROOT / "include").rglob("*.h")))
    for f in files:
        h.update(str(f.relative_to(ROOT)).encode())
        h.update(f.read_bytes())
    h.update(" ".join(ARCH + NVCC_FLAGS + extra).encode())
    return h.hexdigest()


def _compile(src: Path, extra: list[str]) -> tuple[Path, str]:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", str(CSRC), "-I", str(ROOT / "include"), "-c", str(src), "-o",
           str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, jobs: int | None = None, extra_flags: list[str] | None = None) -> Path:
    """Compile (if needed) and return the path of libppgb300.so."""
    extra = list(extra_flags or [])
    BUILD.mkdir(exist_ok=True)
    stamp = BUILD / "stamp"
    digest = _hash_inputs(extra)
    if LIB.exists() and stamp.exists() and stamp.read_text().strip() == digest:
        return LIB
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log, file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(digest)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
