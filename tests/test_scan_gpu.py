"""GPU parity of the decoupled look-back scan (and its single-group and
cooperative variants) against the CPU oracle, through the C ABI.

Integer results are compared bit for bit; float plus-scans against the FP64
oracle within the bound in helpers.float_scan_bound; min/max bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import (FLOAT_DTYPES, FLOAT_OPS, INT_DTYPES, INT_OPS, NP, check_scan, empty_dev, from_dev,
                     make_input, to_dev)

pytestmark = pytest.mark.gpu

# sizes around the tile edges of both kernels (staged tile: 64 KB = 16384 x
# 4-byte or 8192 x 8-byte elements, compute-warp segments of 1024 / 512;
# generic tile: 2048 elements), ragged tails and lengths whose byte count is
# not a multiple of 16
SIZES = [1, 2, 3, 31, 32, 33, 511, 513, 1023, 1025, 2047, 2048, 2049, 8191, 8192, 8193, 16383, 16384, 16385,
         49153, 65537, 1000003]
ALL = [(d, o) for d in INT_DTYPES for o in INT_OPS] + [(d, o) for d in FLOAT_DTYPES for o in FLOAT_OPS]


def _tiles(n):
    return (n + 1023) // 1024


def _run(pp, cuda, x, dtype, op, excl, algo="auto", offset=0, inplace=False, out_offset=None):
    n = x.size
    out_offset = offset if out_offset is None else out_offset
    d_in = to_dev(cuda, np.concatenate([np.zeros(offset, dtype=x.dtype), x]))
    if inplace:
        d_out = d_in
    else:
        d_out = empty_dev(cuda, n, NP[dtype], pad=out_offset)
    esz = x.dtype.itemsize
    stream = cuda.cuda.current_stream().cuda_stream
    pp.scan("exclusive" if excl else "inclusive", op, d_in.data_ptr() + offset * esz,
            d_out.data_ptr() + out_offset * esz, n, dtype, stream=stream, algo=algo)
    assert pp.stream_status(stream) == 0
    return from_dev(d_out, NP[dtype])[out_offset:]


@pytest.mark.parametrize("dtype,op", ALL)
@pytest.mark.parametrize("excl", [False, True])
def test_decoupled_all_ops(pp, oracle, cuda, dtype, op, excl):
    for i, n in enumerate([1, 33, 4097, 65537, 300007]):
        x = make_input(dtype, op, n, seed=1000 + 17 * i + len(op))
        got = _run(pp, cuda, x, dtype, op, excl)
        check_scan(got, x, dtype, op, excl, _tiles(n))


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dtype", ["u32", "u64", "f32"])
def test_decoupled_sizes(pp, oracle, cuda, n, dtype):
    x = make_input(dtype, "plus", n, seed=n)
    for excl in (False, True):
        check_scan(_run(pp, cuda, x, dtype, "plus", excl), x, dtype, "plus", excl, _tiles(n))


@pytest.mark.parametrize("dtype", ["u32", "i64", "f64", "f32"])
@pytest.mark.parametrize("offset,out_offset", [(1, 1), (3, 3), (1, 2), (2, 0), (0, 3)])
@pytest.mark.parametrize("n", [1, 2, 5, 16383, 70001])
def test_element_aligned_pointers_shift_the_tile_grid(pp, oracle, cuda, dtype, offset, out_offset, n):
    """Pointers aligned to the element size but not to 16 bytes stay on the
    bulk-copy kernel (tile grid shifted by the phantom elements in front of
    in[0]); an output with a different misalignment takes scalar stores."""
    x = make_input(dtype, "plus", n, seed=5 + offset + n)
    for excl in (False, True):
        got = _run(pp, cuda, x, dtype, "plus", excl, offset=offset, out_offset=out_offset)
        check_scan(got, x, dtype, "plus", excl, _tiles(n))


@pytest.mark.parametrize("dtype", ["u32", "f64"])
def test_pointers_not_aligned_to_the_element_are_rejected(pp, cuda, dtype):
    """An element cannot be loaded from an address that is not a multiple of
    its size: the call is refused on the host before anything is launched."""
    d = cuda.zeros(4096, dtype=cuda.uint8, device="cuda")
    for a, b in ((1, 0), (0, 2), (3, 3)):
        with pytest.raises(pp.PPError) as e:
            pp.scan("inclusive", "plus", d.data_ptr() + a, d.data_ptr() + 64 + b, 100, dtype)
        assert e.value.status == pp.PP_ERR_INVALID_ARG
    for a in (1, 2, 3):
        with pytest.raises(pp.PPError) as e:
            pp.reduce_device("plus", d.data_ptr() + a, 100, dtype)
        assert e.value.status == pp.PP_ERR_INVALID_ARG


@pytest.mark.parametrize("dtype", ["u32", "u64"])
def test_in_place(pp, oracle, cuda, dtype):
    n = 1 << 20
    x = make_input(dtype, "plus", n, seed=99)
    for excl in (False, True):
        check_scan(_run(pp, cuda, x, dtype, "plus", excl, inplace=True), x, dtype, "plus", excl, _tiles(n))


@pytest.mark.parametrize("algo", ["single_group", "cooperative"])
@pytest.mark.parametrize("dtype,op", [("u32", "plus"), ("i32", "maximum"), ("u64", "plus"), ("i64", "bit_xor"),
                                      ("f32", "plus"), ("f64", "minimum")])
def test_other_algorithms(pp, oracle, cuda, algo, dtype, op):
    for n in (1, 4095, 4097, 200003):
        x = make_input(dtype, op, n, seed=3 * n + 1)
        for excl in (False, True):
            check_scan(_run(pp, cuda, x, dtype, op, excl, algo=algo), x, dtype, op, excl, _tiles(n))


def test_cooperative_unaligned(pp, oracle, cuda):
    n = 123457
    x = make_input("u32", "plus", n, seed=4)
    check_scan(_run(pp, cuda, x, "u32", "plus", False, algo="cooperative", offset=1), x, "u32", "plus", False,
               _tiles(n))


def test_reference_benchmark_known_answer(pp, cuda):
    """benchmarks/benchmark_scan.cpp:32-51: fill(1) -> out[n-1] == n."""
    n = (1 << 24) + 5
    d = cuda.ones(n, dtype=cuda.int32, device="cuda")
    o = cuda.empty_like(d)
    s = cuda.cuda.current_stream().cuda_stream
    pp.decoupled_scan_device("inclusive", "plus", d.data_ptr(), o.data_ptr(), n, "u32", stream=s)
    assert int(o[-1]) == n
    assert cuda.equal(o[:1000].cpu(), cuda.arange(1, 1001, dtype=cuda.int32))


def test_many_calls_and_streams(pp, oracle, cuda):
    """Back-to-back calls re-use the per-stream workspace (epoch protocol);
    two streams get two workspaces."""
    xs = [make_input("u32", "plus", n, seed=n) for n in (5000, 300000, 17, 1 << 18)]
    want = [oracle.scan(x, "plus") for x in xs]
    streams = [cuda.cuda.Stream(), cuda.cuda.Stream()]
    dev_in = [to_dev(cuda, x) for x in xs]
    dev_out = [cuda.empty_like(d) for d in dev_in]
    cuda.cuda.synchronize()
    for rep in range(25):
        for k, (di, do) in enumerate(zip(dev_in, dev_out)):
            s = streams[(rep + k) % 2]
            with cuda.cuda.stream(s):
                do.zero_()
                pp.decoupled_scan_device("inclusive", "plus", di.data_ptr(), do.data_ptr(), di.numel(), "u32",
                                         stream=s.cuda_stream)
        cuda.cuda.synchronize()
        for k, do in enumerate(dev_out):
            assert np.array_equal(from_dev(do, np.uint32), want[k]), (rep, k)
    for s in streams:
        assert pp.stream_status(s.cuda_stream) == 0


def test_caller_workspace(pp, oracle, cuda):
    n = 777777
    x = make_input("u64", "plus", n, seed=12)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    nbytes = pp.workspace_size("decoupled", "u64", d_in.data_ptr(), d_out.data_ptr(), n)
    ws = cuda.zeros(nbytes, dtype=cuda.uint8, device="cuda")
    s = cuda.cuda.current_stream().cuda_stream
    for _ in range(3):
        pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u64", stream=s,
                workspace=(ws.data_ptr(), nbytes))
    assert pp.workspace_status(s, ws.data_ptr()) == 0
    assert np.array_equal(from_dev(d_out, np.uint64), oracle.scan(x, "plus"))
    with pytest.raises(pp.PPError) as e:
        pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u64", stream=s,
                workspace=(ws.data_ptr(), 4096))
    assert e.value.status == pp.PP_ERR_WORKSPACE


def test_lookback_timeout_is_reported_not_hung(pp, oracle, cuda):
    """A tile that never publishes its descriptor makes its successors' bounded
    look-back give up: the call returns, the stream reports PP_ERR_TIMEOUT, and
    the next call on the same stream is correct again."""
    n = 1 << 20
    x = make_input("u32", "plus", n, seed=21)
    d_in = to_dev(cuda, x)
    d_out = cuda.empty_like(d_in)
    s = cuda.cuda.current_stream().cuda_stream
    pp.set_timeout_ns(50_000_000)
    pp.debug_set_skip_tile(3)
    try:
        pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=s)
        assert pp.stream_status(s) == pp.PP_ERR_TIMEOUT
    finally:
        pp.debug_set_skip_tile(-1)
        pp.set_timeout_ns(1_000_000_000)
    pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=s)
    assert pp.stream_status(s) == 0
    assert np.array_equal(from_dev(d_out, np.uint32), oracle.scan(x, "plus"))


def test_host_wrappers(pp, oracle, cuda):
    x = make_input("i32", "plus", 300001, seed=8)
    np.testing.assert_array_equal(pp.decoupled_scan("inclusive", "plus", x), oracle.scan(x, "plus"))
    np.testing.assert_array_equal(pp.cooperative_scan("exclusive", "plus", x), oracle.scan(x, "plus", True))
    np.testing.assert_array_equal(pp.scan_host("inclusive", "maximum", x), oracle.scan(x, "maximum"))


@pytest.mark.parametrize("dtype,op,excl", [("u32", "plus", False), ("i32", "maximum", True), ("u64", "bit_xor", True),
                                           ("f64", "minimum", False)])
def test_host_wrappers_stream_several_chunks(pp, oracle, cuda, dtype, op, excl):
    """Host arrays larger than one 64 MiB chunk: chunks are scanned on their
    own and offset by the running total of the chunks before them."""
    esz = 8 if dtype in ("u64", "f64") else 4
    n = 2 * (64 << 20) // esz + 12345  # two full chunks and a ragged third
    x = make_input(dtype, op, n, seed=21)
    kind = "exclusive" if excl else "inclusive"
    np.testing.assert_array_equal(pp.decoupled_scan(kind, op, x), oracle.scan(x, op, excl))
    if dtype == "u32":
        np.testing.assert_array_equal(pp.cooperative_scan(kind, op, x), oracle.scan(x, op, excl))


def test_host_reduce_streams_several_chunks(pp, oracle, cuda):
    n = (64 << 20) // 8 * 3 + 7
    x = make_input("u64", "plus", n, seed=22)
    assert int(pp.reduce_host("plus", x)) == int(oracle.reduce(x, "plus"))
    assert int(pp.reduce_host("maximum", x)) == int(x.max())
    assert int(pp.reduce_host("plus", x[:0])) == 0


def test_bad_arguments(pp, cuda):
    d = cuda.zeros(16, dtype=cuda.float32, device="cuda")
    with pytest.raises(pp.PPError) as e:
        pp.scan("inclusive", "bit_and", d.data_ptr(), d.data_ptr(), 16, "f32")
    assert e.value.status == pp.PP_ERR_UNSUPPORTED
    with pytest.raises(pp.PPError) as e:
        pp.scan("inclusive", "plus", d.data_ptr(), d.data_ptr(), 16, "u32", precision="compensated")
    assert e.value.status == pp.PP_ERR_UNSUPPORTED


# byte offset of the epoch word in the workspace header (csrc/pp/workspace.cuh:
# ticket, descriptor high-water mark and error detail are 8 bytes each, the exit
# counter 4) and the limit after which the epoch wraps to 0
_EPOCH_OFFSET = 28
_EPOCH_LIMIT = (1 << 30) - 1


def test_epoch_wrap_clears_the_descriptors(pp, oracle, cuda):
    """A caller-owned workspace whose epoch is three launches from its limit:
    the launch that crosses it clears every descriptor word used so far and
    restarts at epoch 0, and the scans on both sides of the wrap stay exact."""
    sizes = [300000, 1 << 20, 70001, 1 << 20, 5000, 1 << 19]
    xs = [make_input("u32", "plus", n, seed=40 + i) for i, n in enumerate(sizes)]
    d_in = [to_dev(cuda, x) for x in xs]
    d_out = [cuda.empty_like(d) for d in d_in]
    nbytes = max(pp.workspace_size("decoupled", "u32", a.data_ptr(), b.data_ptr(), a.numel())
                 for a, b in zip(d_in, d_out))
    ws = cuda.zeros(nbytes, dtype=cuda.uint8, device="cuda")
    ws[_EPOCH_OFFSET:_EPOCH_OFFSET + 4] = cuda.tensor(
        list((_EPOCH_LIMIT - 3).to_bytes(4, "little")), dtype=cuda.uint8, device="cuda")
    s = cuda.cuda.current_stream().cuda_stream
    for x, a, b in zip(xs, d_in, d_out):
        pp.scan("inclusive", "plus", a.data_ptr(), b.data_ptr(), a.numel(), "u32", stream=s, algo="decoupled",
                workspace=(ws.data_ptr(), nbytes))
        assert pp.workspace_status(s, ws.data_ptr()) == 0
        assert np.array_equal(from_dev(b, np.uint32), oracle.scan(x, "plus"))
    epoch = int.from_bytes(bytes(ws[_EPOCH_OFFSET:_EPOCH_OFFSET + 4].cpu().tolist()), "little")
    assert epoch == len(sizes) - 3  # limit - 3, - 2, - 1, then 0, 1, 2 after the six launches


def _tile_elements(pp, cuda, dtype, precision="default"):
    """Elements per tile of the kernel the library picks for aligned pointers
    of this type: the first length whose workspace needs a second descriptor."""
    d = cuda.empty(16, dtype=cuda.int64, device="cuda")
    p = d.data_ptr()
    one = pp.workspace_size("decoupled", dtype, p, p, 1, precision=precision)
    lo, hi = 1, 1 << 20
    while lo < hi:  # smallest n with more workspace than n = 1
        mid = (lo + hi) // 2
        if pp.workspace_size("decoupled", dtype, p, p, mid, precision=precision) > one:
            hi = mid
        else:
            lo = mid + 1
    return lo - 1


@pytest.mark.parametrize("dtype,precision", [("u32", "default"), ("i32", "default"), ("u64", "default"),
                                             ("i64", "default"), ("f32", "default"), ("f64", "default"),
                                             ("f32", "compensated"), ("f32", "fp64_carry")])
def test_every_policy_at_its_own_tile_edges(pp, oracle, cuda, dtype, precision):
    """Lengths one below, at and above one, two and three tiles of the
    configuration each policy runs with (tile sizes differ per policy)."""
    t = _tile_elements(pp, cuda, dtype, precision)
    assert t >= 4096
    s = cuda.cuda.current_stream().cuda_stream
    for i, n in enumerate([t - 1, t, t + 1, 2 * t - 1, 2 * t + 1, 3 * t + 7]):
        x = make_input(dtype, "plus", n, seed=70 + i)
        d_in = to_dev(cuda, x)
        d_out = cuda.empty_like(d_in)
        for excl in (False, True):
            pp.scan("exclusive" if excl else "inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, dtype,
                    stream=s, algo="decoupled", precision=precision)
            assert pp.stream_status(s) == 0
            got = from_dev(d_out, NP[dtype])
            if precision == "compensated":
                want = oracle.scan_fp64(x, excl)
                m = np.abs(want) > 1e-3 * np.sqrt(np.mean(want * want))
                rel = np.abs(got.astype(np.float64)[m] - want[m]) / np.abs(want[m])
                assert rel.max() <= 1e-6, (n, excl, rel.max())
            else:
                check_scan(got, x, dtype, "plus", excl, _tiles(n))


@pytest.mark.parametrize("dtype,precision", [("u32", "default"), ("u64", "default"), ("f32", "compensated")])
def test_scan_and_reduce_replayed_from_a_cuda_graph(pp, oracle, cuda, dtype, precision):
    """A scan and a reduction captured once into a CUDA graph (the stream's
    workspace sized by ordinary calls first) and replayed with new input
    contents each time: the descriptor epochs need no reset node between
    replays."""
    n = 3 * 16384 * 152 + 12345  # several tiles per CTA
    stream = cuda.cuda.Stream()
    x0 = make_input(dtype, "plus", n, seed=90)
    d_in = to_dev(cuda, x0)
    d_out = cuda.empty_like(d_in)
    d_sum = cuda.zeros(2, dtype=cuda.float64 if dtype.startswith("f") else cuda.int64, device="cuda")
    sh = stream.cuda_stream
    cuda.cuda.synchronize()

    def body():
        pp.scan("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, dtype, stream=sh, algo="decoupled",
                precision=precision)
        pp.reduce("plus", d_in.data_ptr(), n, dtype, d_sum.data_ptr(), stream=sh)

    with cuda.cuda.stream(stream):
        body()
        stream.synchronize()
        g = cuda.cuda.CUDAGraph()
        with cuda.cuda.graph(g, stream=stream):
            body()
    for rep in range(3):
        x = make_input(dtype, "plus", n, seed=91 + rep)
        d_in.copy_(to_dev(cuda, x))
        d_out.zero_()
        cuda.cuda.synchronize()
        g.replay()
        cuda.cuda.synchronize()
        got = from_dev(d_out, NP[dtype])
        if precision == "compensated":
            want = oracle.scan_fp64(x)
            m = np.abs(want) > 1e-3 * np.sqrt(np.mean(want * want))
            assert (np.abs(got.astype(np.float64)[m] - want[m]) / np.abs(want[m])).max() <= 1e-6
        else:
            assert np.array_equal(got, oracle.scan(x, "plus"))
        if not dtype.startswith("f"):
            assert from_dev(d_sum, NP[dtype])[0] == oracle.scan(x, "plus")[-1]
    assert pp.stream_status(sh) == 0
