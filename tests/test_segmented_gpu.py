"""Batched segmented scans / reductions and row scans against the oracle,
applied segment by segment (no counterpart in the reference, which scans one
array per call)."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import NP, EPS, float_scan_bound, from_dev, make_input, to_dev

pytestmark = pytest.mark.gpu

DTYPES = ["i32", "u32", "i64", "u64", "f32", "f64"]
OPS = ["plus", "minimum", "maximum"]


def _lengths(rng, count, max_len, p_empty=0.1):
    """Log-uniform lengths in [1, max_len] with some empty segments."""
    lens = np.floor(np.exp(rng.uniform(0, np.log(max_len + 1), count))).astype(np.int64)
    lens = np.clip(lens, 1, max_len)
    lens[rng.uniform(size=count) < p_empty] = 0
    return lens


def _offsets(lens):
    return np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)


def _check_segment(got, x, dtype, op, excl, oracle):
    if dtype.startswith("f") and op == "plus":
        want = oracle.scan_fp64(x, excl)
        bound = float_scan_bound(x, dtype, (x.size + 1023) // 1024 + 2)
        if excl:
            bound = np.concatenate([[1e-300], bound[:-1]])
        assert np.all(np.abs(got.astype(np.float64) - want) <= bound)
    else:
        np.testing.assert_array_equal(got, oracle.scan(x, op, excl))


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("op", OPS)
def test_segmented_scan(pp, oracle, cuda, dtype, op):
    rng = np.random.default_rng(len(dtype) * 31 + len(op))
    lens = _lengths(rng, 700, 3000)
    lens[3] = 70000  # one segment spanning several tiles
    off = _offsets(lens)
    n = int(off[-1])
    x = make_input(dtype, op, n, seed=n)
    d_in, d_off = to_dev(cuda, x), cuda.from_numpy(off).cuda()
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    for excl in (False, True):
        pp.segmented_scan("exclusive" if excl else "inclusive", op, d_in.data_ptr(), d_out.data_ptr(), n,
                          d_off.data_ptr(), lens.size, dtype, stream=s)
        assert pp.stream_status(s) == 0
        got = from_dev(d_out, NP[dtype])
        for k in range(lens.size):
            a, b = off[k], off[k + 1]
            if b > a:
                _check_segment(got[a:b], x[a:b], dtype, op, excl, oracle)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("op", OPS)
# mean lengths about 30, 530 and 3,000 elements: the short-segment variant,
# the boundary of the two classes (512), and the long-segment variant whose
# warps skip the head tests on chunks without segment heads or ends
@pytest.mark.parametrize("count,max_len", [(3000, 60), (1500, 5000), (300, 30000)])
def test_segmented_reduce(pp, oracle, cuda, dtype, op, count, max_len):
    rng = np.random.default_rng(7 + len(op) + max_len)
    lens = _lengths(rng, count, max_len, p_empty=0.15)
    lens[0] = 0
    lens[-1] = 0
    lens[10] = 50000
    _reduce_and_check(pp, oracle, cuda, dtype, op, lens)


def _tile_aligned_lengths(kind):
    """Segment lengths whose starts fall on multiples of 8,064 elements: the
    tile of the 8-byte payloads' variants; every second multiple is a tile
    boundary of the 4-byte payloads' (16,128 elements). Segments end on the
    last element of a tile, start on the first of the next, are one element
    long on either side of a boundary, and empty ones sit on boundaries."""
    b = 8064
    blocks = {
        "long": [[b], [b - 1, 1], [1, b - 1], [b // 2, b // 2], [0, b, 0], [2 * b], [3, b - 3]],
        "short": [[5] * 1612 + [4], [1] * 64 + [b - 64], [b - 1, 1], [0, 1, 0, b - 1]],
    }[kind]
    lens = []
    for _ in range(3):
        for blk in blocks:
            lens += blk
    return np.array(lens, dtype=np.int64)


@pytest.mark.parametrize("dtype", ["i32", "f32", "u64", "f64"])
@pytest.mark.parametrize("op", ["plus", "maximum"])
@pytest.mark.parametrize("kind", ["long", "short"])  # mean lengths about 5,000 and 19
def test_segmented_reduce_heads_on_tile_boundaries(pp, oracle, cuda, dtype, op, kind):
    _reduce_and_check(pp, oracle, cuda, dtype, op, _tile_aligned_lengths(kind))


@pytest.mark.parametrize("dtype", ["i32", "f32", "u64", "f64"])
@pytest.mark.parametrize("kind", ["long", "short"])
def test_segmented_scan_heads_on_tile_boundaries(pp, oracle, cuda, dtype, kind):
    lens = _tile_aligned_lengths(kind)
    off = _offsets(lens)
    n = int(off[-1])
    x = make_input(dtype, "plus", n, seed=5 * n)
    d_in, d_off = to_dev(cuda, x), cuda.from_numpy(off).cuda()
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    for excl in (False, True):
        pp.segmented_scan("exclusive" if excl else "inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n,
                          d_off.data_ptr(), lens.size, dtype, stream=s)
        assert pp.stream_status(s) == 0
        got = from_dev(d_out, NP[dtype])
        for k in range(lens.size):
            a, b = off[k], off[k + 1]
            if b > a:
                _check_segment(got[a:b], x[a:b], dtype, "plus", excl, oracle)


def _reduce_and_check(pp, oracle, cuda, dtype, op, lens):
    off = _offsets(lens)
    n = int(off[-1])
    x = make_input(dtype, op, n, seed=3 * n)
    d_in, d_off = to_dev(cuda, x), cuda.from_numpy(off).cuda()
    d_res = cuda.empty(lens.size, dtype=d_in.dtype, device="cuda")
    s = cuda.cuda.current_stream().cuda_stream
    pp.segmented_reduce(op, d_in.data_ptr(), n, d_off.data_ptr(), lens.size, d_res.data_ptr(), dtype, stream=s)
    assert pp.stream_status(s) == 0
    got = from_dev(d_res, NP[dtype])
    for k in range(lens.size):
        seg = x[off[k]:off[k + 1]]
        if dtype.startswith("f") and op == "plus":
            want = oracle.sum_fp64(seg) if seg.size else 0.0
            tol = (64 + seg.size // 1024) * EPS[dtype] * float(np.sum(np.abs(seg.astype(np.float64))))
            assert abs(float(got[k]) - want) <= tol, (k, got[k], want)
        else:
            assert got[k] == oracle.reduce(seg, op), (k, seg.size, got[k], oracle.reduce(seg, op))


@pytest.mark.parametrize("dtype", ["i32", "f32", "i64", "f64"])
@pytest.mark.parametrize("op", ["plus", "maximum"])
@pytest.mark.parametrize("lens", [[40_000_003, 0, 7, 17_000_000, 1, 0], [16_515_072, 33_030_144, 5]])
def test_segmented_reduce_segments_across_chunks(pp, oracle, cuda, dtype, op, lens):
    """Segments spanning thousands of tiles: the reduction's fix-up steps over
    whole head-free chunks of 1,024 tile records. The second case puts its
    heads exactly on chunk boundaries (16,515,072 = 1,024 tiles of 16,128
    4-byte elements = 2,048 tiles of 8,064 8-byte elements)."""
    _reduce_and_check(pp, oracle, cuda, dtype, op, np.array(lens, dtype=np.int64))


@pytest.mark.parametrize("dtype", ["f32", "i32", "u64", "f64"])
# rows of >= 256 elements go one warp per row (vector steps when rows are 16-byte
# multiples, scalar otherwise); shorter rows, and few rows longer than 65536,
# are segments of the decoupled look-back kernel
@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (40, 255), (2, 16384), (7, 16385), (5, 20001), (64, 256), (33, 4096),
                                   (640, 300), (3, 70001)])
@pytest.mark.parametrize("reverse", [False, True])
def test_rows_scan(pp, oracle, cuda, dtype, shape, reverse):
    rows, cols = shape
    x = make_input(dtype, "plus", rows * cols, seed=rows * 1000 + cols)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    for excl in (False, True):
        pp.rows_scan("exclusive" if excl else "inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), rows, cols, dtype,
                     reverse=reverse, stream=s)
        assert pp.stream_status(s) == 0
        got = from_dev(d_out, NP[dtype]).reshape(rows, cols)
        xm = x.reshape(rows, cols)
        for r in range(rows):
            row = xm[r, ::-1] if reverse else xm[r]
            g = got[r, ::-1] if reverse else got[r]
            _check_segment(np.ascontiguousarray(g), np.ascontiguousarray(row), dtype, "plus", excl, oracle)


@pytest.mark.parametrize("dtype,cols", [("f32", 1024), ("i32", 2048), ("f32", 4096), ("u32", 8192), ("f32", 16384),
                                        ("f64", 512), ("i64", 2048), ("u64", 8192)])
@pytest.mark.parametrize("rows", [1, 17, 37])
@pytest.mark.parametrize("reverse", [False, True])
def test_rows_that_tile_a_stage(pp, oracle, cuda, dtype, cols, rows, reverse):
    """Row lengths that are 1, 2, 4, 8 or 16 compute-warp segments take the
    tile-of-rows kernel: whole rows per 64 KB tile, the segments of a row
    exchanging totals; row counts that leave the last tile partly empty."""
    op = "maximum" if dtype == "i32" else "plus"
    x = make_input(dtype, op, rows * cols, seed=rows * 31 + cols)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    for excl in (False, True):
        pp.rows_scan("exclusive" if excl else "inclusive", op, d_in.data_ptr(), d_out.data_ptr(), rows, cols, dtype,
                     reverse=reverse, stream=s)
        assert pp.stream_status(s) == 0
        got = from_dev(d_out, NP[dtype]).reshape(rows, cols)
        xm = x.reshape(rows, cols)
        for r in range(rows):
            row = xm[r, ::-1] if reverse else xm[r]
            g = got[r, ::-1] if reverse else got[r]
            _check_segment(np.ascontiguousarray(g), np.ascontiguousarray(row), dtype, op, excl, oracle)


def test_rows_scan_max(pp, oracle, cuda):
    rows, cols = 9, 30000
    x = make_input("i32", "maximum", rows * cols, seed=5)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    pp.rows_scan("inclusive", "maximum", d_in.data_ptr(), d_out.data_ptr(), rows, cols, "i32", reverse=True)
    got = from_dev(d_out, np.int32).reshape(rows, cols)
    for r in range(rows):
        np.testing.assert_array_equal(got[r, ::-1], oracle.scan(np.ascontiguousarray(x.reshape(rows, cols)[r, ::-1]),
                                                                "maximum"))


def test_segmented_scan_in_cuda_graph(pp, oracle, cuda):
    """The whole batched scan (pre-pass + persistent launch) is captured once
    and replayed; the workspace is sized by an ordinary call first."""
    rng = np.random.default_rng(11)
    lens = _lengths(rng, 4000, 4096, p_empty=0.05)
    off = _offsets(lens)
    n = int(off[-1])
    x = make_input("i32", "plus", n, seed=17)
    d_in, d_off = to_dev(cuda, x), cuda.from_numpy(off).cuda()
    d_out = cuda.empty_like(d_in)
    stream = cuda.cuda.Stream()
    cuda.cuda.synchronize()
    with cuda.cuda.stream(stream):
        pp.segmented_scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, d_off.data_ptr(), lens.size,
                          "i32", stream=stream.cuda_stream)
        stream.synchronize()
        g = cuda.cuda.CUDAGraph()
        with cuda.cuda.graph(g, stream=stream):
            pp.segmented_scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, d_off.data_ptr(),
                              lens.size, "i32", stream=stream.cuda_stream)
    for rep in range(3):
        d_out.zero_()
        g.replay()
        cuda.cuda.synchronize()
        got = from_dev(d_out, np.int32)
        for k in range(0, lens.size, 37):
            a, b = off[k], off[k + 1]
            np.testing.assert_array_equal(got[a:b], oracle.scan(x[a:b], "plus"))
    assert pp.stream_status(stream.cuda_stream) == 0


@pytest.mark.parametrize("warmed_stream", [True, False])
def test_rows_scan_in_cuda_graph(pp, oracle, cuda, warmed_stream):
    """Row scans captured into a CUDA graph: on the stream the warm-up sized
    the workspace on (the whole-row tile kernel), or on a fresh capture
    stream (the kernels that need no workspace)."""
    rows, cols = 96, 8192
    x = make_input("f32", "plus", rows * cols, seed=8)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    side = cuda.cuda.Stream()
    side.wait_stream(cuda.cuda.current_stream())
    with cuda.cuda.stream(side):
        pp.rows_scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), rows, cols, "f32",
                     stream=side.cuda_stream)
    cuda.cuda.current_stream().wait_stream(side)
    cuda.cuda.synchronize()
    g = cuda.cuda.CUDAGraph()
    cap = side if warmed_stream else cuda.cuda.Stream()
    with cuda.cuda.graph(g, stream=cap):
        pp.rows_scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), rows, cols, "f32",
                     stream=cap.cuda_stream)
    d_out.zero_()
    cuda.cuda.synchronize()
    g.replay()
    cuda.cuda.synchronize()
    got = from_dev(d_out, np.float32).reshape(rows, cols)
    for r in range(0, rows, 7):
        _check_segment(got[r], np.ascontiguousarray(x.reshape(rows, cols)[r]), "f32", "plus", False, oracle)
