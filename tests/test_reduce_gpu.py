"""GPU parity of the device-wide reduction against the CPU oracle, through the
C ABI, including the reference's own known answers
(tests/test_reduction.cpp:4-31: uint64 iota sums for n = 4^k)."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import EPS, FLOAT_DTYPES, FLOAT_OPS, INT_DTYPES, INT_OPS, NP, make_input, to_dev

pytestmark = pytest.mark.gpu

ALL = [(d, o) for d in INT_DTYPES for o in INT_OPS] + [(d, o) for d in FLOAT_DTYPES for o in FLOAT_OPS]


def test_reference_iota_known_answers(pp, cuda):
    """reduce_device<plus> of uint64 iota(0..n-1) == n(n-1)/2, n = 1, 4, ..., 4^9."""
    s = cuda.cuda.current_stream().cuda_stream
    n = 1
    while n < 1_000_000:
        d = cuda.arange(n, dtype=cuda.int64, device="cuda")
        assert int(pp.reduce_device("plus", d.data_ptr(), n, "u64", stream=s)) == n * (n - 1) // 2
        h = np.arange(n, dtype=np.uint64)
        assert int(pp.reduce_host("plus", h)) == n * (n - 1) // 2
        n *= 4


def test_reference_fill_one_known_answer(pp, cuda):
    """benchmarks/benchmark_reduce.cpp:9-33: fill(1) uint32 -> n."""
    n = (1 << 26) + 3
    d = cuda.ones(n, dtype=cuda.int32, device="cuda")
    assert int(pp.reduce_device("plus", d.data_ptr(), n, "u32")) == n


@pytest.mark.parametrize("dtype,op", ALL)
def test_all_ops(pp, oracle, cuda, dtype, op):
    s = cuda.cuda.current_stream().cuda_stream
    for i, n in enumerate([1, 3, 4, 17, 1000, 65536 + 5, 4_000_037]):
        x = make_input(dtype, op, n, seed=77 + i)
        d = to_dev(cuda, x)
        got = pp.reduce_device(op, d.data_ptr(), n, dtype, stream=s)
        if dtype in INT_DTYPES or op in ("minimum", "maximum"):
            assert got == oracle.reduce(x, op), (n, got, oracle.reduce(x, op))
        elif op == "plus":
            want = oracle.sum_fp64(x)
            bound = 2 * (64 + np.log2(n + 1)) * EPS[dtype] * float(np.sum(np.abs(x.astype(np.float64))))
            assert abs(float(got) - want) <= bound, (n, float(got), want)
        else:
            want = float(np.prod(x.astype(np.float64)))
            assert abs(float(got) - want) <= 8 * (64 + n // 1024) * EPS[dtype] * abs(want)


@pytest.mark.parametrize("offset", [0, 1, 2, 3])
def test_unaligned_and_empty(pp, oracle, cuda, offset):
    x = make_input("u32", "plus", 100003, seed=offset)
    d = to_dev(cuda, np.concatenate([np.zeros(offset, np.uint32), x]))
    ptr = d.data_ptr() + 4 * offset
    assert pp.reduce_device("plus", ptr, x.size, "u32") == oracle.reduce(x, "plus")
    assert pp.reduce_device("plus", ptr, 0, "u32") == 0
    assert pp.reduce_device("minimum", ptr, 0, "i32") == np.iinfo(np.int32).max
    assert pp.reduce_device("bit_and", ptr, 0, "u64") == np.iinfo(np.uint64).max


def test_async_reduce_to_device_and_determinism(pp, oracle, cuda):
    n = 10_000_019
    x = make_input("f32", "plus", n, seed=3)
    d = to_dev(cuda, x)
    res = cuda.zeros(4, dtype=cuda.float32, device="cuda")
    s = cuda.cuda.current_stream().cuda_stream
    for k in range(4):
        pp.reduce("plus", d.data_ptr(), n, "f32", res.data_ptr() + 4 * k, stream=s)
    assert pp.stream_status(s) == 0
    r = res.cpu().numpy()
    assert np.all(r == r[0]), "fixed grid must give bit-identical float sums"
