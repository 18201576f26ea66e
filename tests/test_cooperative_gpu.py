"""The cooperative grid-barrier scan in L2-sized rounds (the staged kernel's
cooperative mode) against the CPU oracle.

The reference's cooperative scan (scan_cooperative.hpp:35-91) runs one grid
barrier over one pass; here the input streams through L2 in windows of
G x kt tiles (G co-resident CTAs, kt tiles per CTA): each window is reduced,
crosses a split window barrier and is scanned one window later. The window
geometry is forced small here (pp_set_max_ctas, pp_set_cooperative_window)
so that small inputs cross many windows and hit every edge: a last window
shorter than the grid (CTAs with empty runs), runs of one tile, a window
boundary one element away, inputs not aligned to 16 bytes (shifted tile
grid), every policy class of the staged kernel (striped 4-byte integers,
rows of 8-byte integers with the store warp, float rows, double rows,
compensated and FP64-carry floats). Also: a decoupled scan on the same
stream after a cooperative one (the tile records share the workspace with
the look-back descriptors), a caller-provided workspace of exactly
pp_workspace_size bytes, and a window barrier that never completes (the
fault-injection knob) reported as a timeout."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import NP, check_scan, empty_dev, from_dev, make_input, to_dev

pytestmark = pytest.mark.gpu

# elements per tile of the staged kernel's configuration for each type
# (compute warps x 32 lanes x 16-byte chunks per lane x elements per chunk)
TILE = {"u32": 16384, "i32": 16384, "u64": 8960, "i64": 8960, "f32": 18432, "f64": 8064}

CASES = [("u32", "plus"), ("i32", "minimum"), ("i64", "maximum"), ("u64", "bit_xor"), ("f32", "plus"),
         ("f64", "plus")]


@pytest.fixture
def windows(pp):
    def set_(ctas, kt):
        pp.set_max_ctas(ctas)
        pp.set_cooperative_window(kt)
    yield set_
    pp.set_max_ctas(0)
    pp.set_cooperative_window(0)


def _sizes(dtype, ctas, kt):
    t = TILE[dtype]
    w = ctas * kt * t  # elements per window
    return [1, t - 1, t + 1, w - 1, w, w + 1, 2 * w + 3 * t + 7, 4 * w + (w // 2) + 5]


def _run(pp, cuda, x, dtype, op, excl, offset=0, stream=None, precision="default"):
    n = x.size
    d_in = to_dev(cuda, np.concatenate([np.zeros(offset, dtype=x.dtype), x]))
    d_out = empty_dev(cuda, n, NP[dtype], pad=offset)
    esz = x.dtype.itemsize
    s = cuda.cuda.current_stream().cuda_stream if stream is None else stream
    pp.scan("exclusive" if excl else "inclusive", op, d_in.data_ptr() + offset * esz, d_out.data_ptr() + offset * esz,
            n, dtype, stream=s, algo="cooperative", precision=precision)
    assert pp.stream_status(s) == 0
    return from_dev(d_out, NP[dtype])[offset:]


@pytest.mark.parametrize("ctas,kt", [(5, 1), (3, 2), (7, 3)])
@pytest.mark.parametrize("dtype,op", CASES)
def test_window_edges(pp, oracle, cuda, windows, ctas, kt, dtype, op):
    windows(ctas, kt)
    for i, n in enumerate(_sizes(dtype, ctas, kt)):
        x = make_input(dtype, op, n, seed=97 * i + ctas + kt)
        for excl in (False, True):
            check_scan(_run(pp, cuda, x, dtype, op, excl), x, dtype, op, excl, (n + 1023) // 1024)


@pytest.mark.parametrize("dtype,op", [("u32", "plus"), ("u64", "plus"), ("f32", "plus")])
def test_unaligned_input_crosses_windows(pp, oracle, cuda, windows, dtype, op):
    """One element past a 16-byte boundary: the tile grid shifts by phantom
    elements, so the first window's first tile is partial."""
    windows(4, 1)
    n = 9 * TILE[dtype] + 11
    x = make_input(dtype, op, n, seed=5)
    for excl in (False, True):
        check_scan(_run(pp, cuda, x, dtype, op, excl, offset=1), x, dtype, op, excl, (n + 1023) // 1024)


@pytest.mark.parametrize("precision", ["compensated", "fp64_carry"])
def test_precision_modes_cross_windows(pp, oracle, cuda, windows, precision):
    windows(5, 1)
    n = 23 * 18432 + 101
    x = oracle.gen_f32_normal(31, n)
    want = oracle.scan_fp64(x)
    got = _run(pp, cuda, x, "f32", "plus", False, precision=precision)
    err = np.abs(got.astype(np.float64) - want)
    cabs = np.cumsum(np.abs(x.astype(np.float64)))
    tol = (1e-6 if precision == "compensated" else 64 * np.finfo(np.float32).eps) * cabs + 1e-30
    assert np.all(err <= tol), float(np.max(err / tol))


def test_default_windows_many_rounds(pp, oracle, cuda):
    """The library's own window size on an input of several windows and a
    partial last one."""
    n = (1 << 25) + 12345
    x = make_input("u32", "plus", n, seed=11)
    got = _run(pp, cuda, x, "u32", "plus", False)
    np.testing.assert_array_equal(got, oracle.scan(x, "plus"))


def test_decoupled_after_cooperative_on_one_stream(pp, oracle, cuda, windows):
    """The cooperative rounds keep per-tile records where the look-back
    descriptors live; they must read as invalid descriptors to the next
    decoupled scan on the stream, whatever their contents."""
    windows(6, 2)
    s = cuda.cuda.current_stream().cuda_stream
    for i, (nc, nd) in enumerate([(3_000_001, 2_500_000), (700_001, 3_100_000), (5_000_000, 65537)]):
        # all-ones words make large record words; a decoupled scan after them
        # must still publish and find every descriptor
        xc = np.full(nc, 0xFFFFFFFF, dtype=np.uint32)
        got = _run(pp, cuda, xc, "u32", "bit_or", False, stream=s)
        np.testing.assert_array_equal(got, oracle.scan(xc, "bit_or"))
        xd = make_input("u32", "plus", nd, seed=300 + i)
        d_in = to_dev(cuda, xd)
        d_out = cuda.empty_like(d_in)
        pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), nd, "u32", stream=s, algo="decoupled")
        assert pp.stream_status(s) == 0
        np.testing.assert_array_equal(from_dev(d_out, np.uint32), oracle.scan(xd, "plus"))


def test_caller_workspace(pp, oracle, cuda, windows):
    windows(5, 2)
    n = 31 * 8960 + 3
    x = make_input("u64", "plus", n, seed=8)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    need = pp.workspace_size("cooperative", "u64", d_in.data_ptr(), d_out.data_ptr(), n)
    ws = cuda.zeros(need, dtype=cuda.uint8, device="cuda")
    s = cuda.cuda.current_stream().cuda_stream
    pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u64", stream=s, algo="cooperative",
            workspace=(ws.data_ptr(), need))
    assert pp.workspace_status(s, ws.data_ptr()) == 0
    np.testing.assert_array_equal(from_dev(d_out, np.uint64), oracle.scan(x, "plus"))
    with pytest.raises(pp.PPError):
        pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u64", stream=s, algo="cooperative",
                workspace=(ws.data_ptr(), need - 16))


def test_window_barrier_timeout_is_reported(pp, oracle, cuda, windows):
    """The CTA whose run holds the skipped tile never arrives at that
    window's barrier: every CTA's bounded wait gives up, the call's status is
    a timeout, and the next call is correct again."""
    windows(5, 1)
    n = 20 * 16384
    x = make_input("u32", "plus", n, seed=13)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.set_timeout_ns(50_000_000)
    pp.debug_set_skip_tile(7)
    try:
        pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=s, algo="cooperative")
        assert pp.stream_status(s) == pp.PP_ERR_TIMEOUT
    finally:
        pp.debug_set_skip_tile(-1)
        pp.set_timeout_ns(1_000_000_000)
    pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=s, algo="cooperative")
    assert pp.stream_status(s) == 0
    np.testing.assert_array_equal(from_dev(d_out, np.uint32), oracle.scan(x, "plus"))
