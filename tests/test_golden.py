"""The reference's own outputs (tests/golden/reference_outputs.json, produced
by tests/golden/make_golden.py from the reference headers compiled against
the SYCL CPU shim) pin the oracle on the CPU and the CUDA path on the GPU:
every integer scan and reduction must reproduce them bit for bit."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from helpers import NP, from_dev, to_dev

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_outputs.json").read_text())


def _input(oracle, c):
    if c["dtype"] in ("u32", "i32"):
        return oracle.gen_u32(c["seed"], c["n"], c["lo"], c["hi"]).view(NP[c["dtype"]])
    return oracle.gen_u64(c["seed"], c["n"], c["lo"], c["hi"]).view(NP[c["dtype"]])


def test_oracle_reproduces_reference_scans(oracle):
    for c in GOLDEN["scans"]:
        y = oracle.scan(_input(oracle, c), c["op"], False)
        assert f"{oracle.fnv1a64(y):016x}" == c["fnv1a64"], c
        assert [int(v) for v in y[:3]] == c["head"] and [int(v) for v in y[-3:]] == c["tail"]


def test_oracle_reproduces_reference_reductions(oracle):
    for c in GOLDEN["reductions"]:
        assert int(oracle.reduce(_input(oracle, c), c["op"])) == c["value"], c


def test_oracle_reproduces_reference_headline_case(oracle):
    h = GOLDEN["headline_2p24"]
    x = oracle.gen_u32(h["seed"], h["n"], h["lo"], h["hi"])
    y = oracle.scan(x)
    assert f"{oracle.fnv1a64(y):016x}" == h["scan_fnv1a64"]
    assert int(oracle.reduce(x)) == h["sum"] == h["scan_last"]


@pytest.mark.gpu
@pytest.mark.parametrize("algo", ["decoupled", "cooperative", "single_group"])
def test_gpu_reproduces_reference_scans(pp, oracle, cuda, algo):
    s = cuda.cuda.current_stream().cuda_stream
    for c in GOLDEN["scans"]:
        if algo == "single_group" and c["n"] > 20000:
            continue
        x = _input(oracle, c)
        d_in = to_dev(cuda, x)
        d_out = cuda.empty_like(d_in)
        pp.scan("inclusive", c["op"], d_in.data_ptr(), d_out.data_ptr(), c["n"], c["dtype"], stream=s, algo=algo)
        y = from_dev(d_out, NP[c["dtype"]])
        assert f"{oracle.fnv1a64(y):016x}" == c["fnv1a64"], (algo, c)
    assert pp.stream_status(s) == 0


@pytest.mark.gpu
def test_gpu_reproduces_reference_reductions(pp, oracle, cuda):
    s = cuda.cuda.current_stream().cuda_stream
    for c in GOLDEN["reductions"]:
        d = to_dev(cuda, _input(oracle, c))
        assert int(pp.reduce_device(c["op"], d.data_ptr(), c["n"], c["dtype"], stream=s)) == c["value"], c


@pytest.mark.gpu
def test_gpu_reproduces_reference_headline_case(pp, oracle, cuda):
    """n = 2^24 uint32 U[0,255]: inclusive plus-scan and sum reduction, bit-exact."""
    h = GOLDEN["headline_2p24"]
    x = oracle.gen_u32(h["seed"], h["n"], h["lo"], h["hi"])
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), h["n"], "u32", stream=s)
    y = from_dev(d_out, np.uint32)
    assert f"{oracle.fnv1a64(y):016x}" == h["scan_fnv1a64"]
    assert int(pp.reduce_device("plus", d_in.data_ptr(), h["n"], "u32", stream=s)) == h["sum"]
    # the blocking host-array wrappers give the same bytes
    assert f"{oracle.fnv1a64(pp.decoupled_scan('inclusive', 'plus', x)):016x}" == h["scan_fnv1a64"]
    assert int(pp.reduce_host("plus", x)) == h["sum"]
