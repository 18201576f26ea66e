"""The intrinsics of include/parallel_primitives/intrinsics.hpp against the
reference's own outputs (tests/golden/, produced by the reference headers on
the CPU, see tests/golden/make_golden.py):

* funnelshift_l / funnelshift_r for shifts 0..30 on the operands of the
  reference's tests/test_intrinsics.cpp:10-14 (the reference reduces the
  shift with % 31, CUDA with & 31: the two agree below 31), brev32 / brev64
  on the recorded operands and upsample("SYCL") (intrinsics.hpp:52-63,
  102-148);
* get_byte, set_byte, both set_bit_in_word overloads, read_bit and flip_bit
  (intrinsics.hpp:150-202) at every byte / bit position of 1-, 2-, 4- and
  8-byte words.

tests/cpp/intrinsics_eval.cu evaluates the requests on the host (CPU test)
and on the GPU, one thread per request (GPU test); both must reproduce the
reference bit for bit."""

from __future__ import annotations

import json
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = json.loads((ROOT / "tests" / "golden" / "reference_outputs.json").read_text())
BYTES_BITS = json.loads((ROOT / "tests" / "golden" / "intrinsics_bytes_bits.json").read_text())
EXE = ROOT / "sycl-building-blocks_gb300" / "_build" / "intrinsics_eval"
LO, HI = 0xCAFED00D, 0xDEADBEEF  # tests/test_intrinsics.cpp:9-14 operands


def _requests() -> tuple[list[tuple[int, int, int, int, int]], list[int], list[str]]:
    """(op, width, word, a, b) requests, the reference's answers, labels."""
    reqs, want, label = [], [], []

    def add(req, value, what):
        reqs.append(req)
        want.append(int(value))
        label.append(what)

    intr = GOLDEN["intrinsics"]
    word = (HI << 32) | LO
    for s, v in intr["funnelshift_l"].items():
        add((10, 8, word, int(s), 0), v, f"funnelshift_l shift {s}")
    for s, v in intr["funnelshift_r"].items():
        add((11, 8, word, int(s), 0), v, f"funnelshift_r shift {s}")
    for x, v in intr["brev32"].items():
        add((12, 4, int(x), 0, 0), v, f"brev32({x})")
    for x, v in intr["brev64"].items():
        add((13, 8, int(x), 0, 0), v, f"brev64({x})")
    sycl = (ord("S") << 24) | (ord("Y") << 16) | (ord("C") << 8) | ord("L")
    add((14, 4, sycl, 0, 0), intr["upsample_SYCL"], "upsample SYCL")
    for c in BYTES_BITS["cases"]:
        w, width = c["word"], c["width"]
        tag = f"u{8 * width} {w:#x}"
        for p, v in enumerate(c["get_byte"]):
            add((0, width, w, p, 0), v, f"get_byte {tag} pos {p}")
        for b, vals in c["set_byte"].items():
            for p, v in enumerate(vals):
                add((1, width, w, p, int(b)), v, f"set_byte {tag} byte {b} pos {p}")
        for i in range(8 * width):
            add((2, width, w, i, 1), c["set_bit_true"][i], f"set_bit_in_word<true> {tag} bit {i}")
            add((2, width, w, i, 0), c["set_bit_false"][i], f"set_bit_in_word<false> {tag} bit {i}")
            add((3, width, w, i, 1), c["set_bit_runtime_true"][i], f"set_bit_in_word(.., true) {tag} bit {i}")
            add((3, width, w, i, 0), c["set_bit_runtime_false"][i], f"set_bit_in_word(.., false) {tag} bit {i}")
            add((4, width, w, i, 0), c["read_bit"][i], f"read_bit {tag} bit {i}")
            add((5, width, w, i, 0), c["flip_bit"][i], f"flip_bit {tag} bit {i}")
    return reqs, want, label


def _compile() -> Path:
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = ROOT / "tests" / "cpp" / "intrinsics_eval.cu"
    if not (EXE.exists() and EXE.stat().st_mtime >= src.stat().st_mtime and
            EXE.stat().st_mtime >= (ROOT / "include" / "parallel_primitives" / "intrinsics.hpp").stat().st_mtime):
        EXE.parent.mkdir(exist_ok=True)
        cmd = [nvcc, "-std=c++20", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(ROOT / "include"),
               str(src), "-o", str(EXE)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
    return EXE


def _run(mode: str) -> None:
    exe = _compile()
    reqs, want, label = _requests()
    text = "".join(f"{op} {w} {word} {a} {b}\n" for op, w, word, a, b in reqs)
    r = subprocess.run([str(exe), mode], input=text, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    got = [int(x) for x in r.stdout.split()]
    assert len(got) == len(want)
    bad = [f"{label[i]}: got {got[i]:#x} want {want[i]:#x}" for i in range(len(want)) if got[i] != want[i]]
    assert not bad, f"{len(bad)} of {len(want)} differ from the reference:\n" + "\n".join(bad[:20])


def test_fixture_covers_every_helper_and_position():
    reqs, _, _ = _requests()
    ops = {r[0] for r in reqs}
    assert ops == {0, 1, 2, 3, 4, 5, 10, 11, 12, 13, 14}
    assert {c["width"] for c in BYTES_BITS["cases"]} == {1, 2, 4, 8}
    for c in BYTES_BITS["cases"]:
        assert len(c["read_bit"]) == 8 * c["width"] and len(c["get_byte"]) == c["width"]


def test_intrinsics_host_match_reference():
    """Host versions (the reference's plain C++ run of the same checks)."""
    _run("host")


@pytest.mark.gpu
def test_intrinsics_device_match_reference(cuda):
    """Device versions: the sm_103a instructions (__funnelshift_*, __brev*)
    and the byte / bit helpers compiled for the GPU."""
    _run("device")
