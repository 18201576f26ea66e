"""Build recipe for the CPU checker (TEST INFRASTRUCTURE ONLY).

* oracle/liboracle.so  - the plain-C restatement (oracle.c), always built.
* oracle/_ref/libsyclref.so - the reference's own headers, compiled unmodified
  from where they lie in the reference checkout's include/ directory against
  the project's SYCL-subset CPU shim (oracle/sycl_shim). Built only where the
  reference checkout exists; it is git-ignored and never shipped.

Where the reference checkout is: the include directory is taken from
`python oracle/build_oracle.py --reference-include DIR`, else from the
environment variable SYCL_BB_REFERENCE_INCLUDE, else from the default
checkout location /root/reference/include. No reference checkout there: only
liboracle.so is built.

Usage:  python oracle/build_oracle.py [-f] [--reference-include DIR]
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
DEFAULT_REFERENCE_INCLUDE = Path("/root/reference/include")


def reference_include() -> Path:
    """Include directory of the reference checkout (see the module docstring)."""
    env = os.environ.get("SYCL_BB_REFERENCE_INCLUDE")
    return Path(env) if env else DEFAULT_REFERENCE_INCLUDE


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


def build_ref(force: bool = False, include_dir: Path | None = None) -> Path | None:
    """Compile the reference headers in place against the SYCL shim."""
    include_dir = Path(include_dir) if include_dir else reference_include()
    if not (include_dir / "parallel_primitives").is_dir():
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
           str(include_dir), str(entry), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="build the CPU oracle and, where the reference exists, oracle/_ref")
    ap.add_argument("-f", action="store_true", help="rebuild even when the outputs are newer than the sources")
    ap.add_argument("--reference-include", type=Path, default=None,
                    help="include/ directory of the reference checkout")
    ns = ap.parse_args()
    print(build_oracle(force=ns.f))
    print(build_ref(force=ns.f, include_dir=ns.reference_include))
