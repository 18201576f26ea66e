"""Build recipe for the CPU checker (TEST INFRASTRUCTURE ONLY).

* oracle/liboracle.so  - the plain-C restatement (oracle.c), always built.
* oracle/_ref/libsyclref.so - the reference's own headers, compiled unmodified
  from where they lie under /root/reference/include against the project's
  SYCL-subset CPU shim (oracle/sycl_shim). Built only where the reference
  checkout exists; it is git-ignored and never shipped.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libsyclref.so"
REFERENCE_INCLUDE = Path("/root/reference/include")


def _newer(target: Path, sources: list[Path]) -> bool:
    return target.exists() and all(target.stat().st_mtime >= s.stat().st_mtime for s in sources)


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "oracle.c", HERE / "oracle.h"]
    if not force and _newer(LIB, srcs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-fPIC", "-shared", "-pthread", str(HERE / "oracle.c"), "-o",
           str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference headers in place against the SYCL shim."""
    if not REFERENCE_INCLUDE.is_dir():
        return None
    shim = HERE / "sycl_shim"
    entry = HERE / "ref_entry.cpp"
    if not entry.exists():
        return None
    srcs = [entry, *shim.rglob("*.hpp")]
    if not force and _newer(REF_LIB, srcs):
        return REF_LIB
    REF_DIR.mkdir(exist_ok=True)
    tmp = REF_LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++20", "-O2", "-fwrapv", "-fPIC", "-shared", "-pthread", "-w", "-I", str(shim), "-I",
           str(REFERENCE_INCLUDE), str(entry), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
