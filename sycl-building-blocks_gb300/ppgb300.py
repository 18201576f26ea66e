"""Python view of the C ABI (include/pp_gb300.h) over ctypes.

Mirrors the reference's entry points for the scan / reduce path with the same
names and argument meaning:

    decoupled_scan_device(kind, op, d_in, d_out, n, dtype, stream)
        parallel_primitives::decoupled_scan_device
        (include/parallel_primitives/scan_decoupled_lookback.hpp:209-217)
    cooperative_scan_device(...)   scan_cooperative.hpp:95-99
    scan_device(...), group_scan_device(...)   scan.hpp:107-130
    reduce_device(op, d_in, n, dtype, stream) -> value   reduction.hpp:113-139
    decoupled_scan / cooperative_scan / scan / reduce on host numpy arrays
        (the blocking host wrappers, :219-230, scan_cooperative.hpp:102-110,
        scan.hpp:133-140, reduction.hpp:142-151)

Device pointers are plain integers (e.g. torch.Tensor.data_ptr()); streams are
cudaStream_t handles as integers (e.g. torch.cuda.current_stream().cuda_stream).
Errors raise PPError carrying the pp_status code. There is no CPU fallback:
loading fails loudly when the shared library is missing.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libppgb300.so"

INCLUSIVE, EXCLUSIVE = 0, 1
OPS = {"plus": 0, "multiplies": 1, "bit_and": 2, "bit_or": 3, "bit_xor": 4, "minimum": 5, "maximum": 6}
DTYPES = {"i32": 0, "u32": 1, "i64": 2, "u64": 3, "f32": 4, "f64": 5}
NP_DTYPES = {np.dtype(np.int32): 0, np.dtype(np.uint32): 1, np.dtype(np.int64): 2, np.dtype(np.uint64): 3,
             np.dtype(np.float32): 4, np.dtype(np.float64): 5}
DTYPE_SIZE = {0: 4, 1: 4, 2: 8, 3: 8, 4: 4, 5: 8}
ALGOS = {"auto": 0, "decoupled": 1, "cooperative": 2, "single_group": 3}
PRECISIONS = {"default": 0, "compensated": 1, "fp64_carry": 2}

PP_OK, PP_ERR_INVALID_ARG, PP_ERR_UNSUPPORTED, PP_ERR_GRID_TOO_LARGE = 0, 1, 2, 3
PP_ERR_TIMEOUT, PP_ERR_CUDA, PP_ERR_WORKSPACE, PP_ERR_NO_DEVICE = 4, 5, 6, 7

# every symbol include/pp_gb300.h declares
EXPORTS = [
    "pp_scan", "pp_scan_ws", "pp_workspace_size", "pp_decoupled_scan_device", "pp_cooperative_scan_device",
    "pp_scan_device", "pp_group_scan_device", "pp_reduce_device", "pp_reduce", "pp_reduce_ws",
    "pp_decoupled_scan_host", "pp_cooperative_scan_host", "pp_scan_host", "pp_reduce_host", "pp_status_string",
    "pp_stream_status", "pp_workspace_status", "pp_set_timeout_ns", "pp_set_max_ctas", "pp_debug_set_skip_tile",
    "pp_version", "pp_decoupled_scan_device_noalloc", "pp_segmented_scan", "pp_segmented_reduce", "pp_rows_scan",
    "pp_debug_set_lookback_delay", "pp_debug_lookback_counters", "pp_set_cooperative_window",
]


class PPError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: pp_status {status} ({status_string(status)})")


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Load libppgb300.so (raises OSError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise OSError(f"{LIB_PATH} is missing: build it with ppbuild.build() first")
    L = C.CDLL(str(LIB_PATH))
    vp, u64, i32, sz = C.c_void_p, C.c_uint64, C.c_int, C.c_size_t
    L.pp_scan.argtypes = [vp, i32, i32, i32, vp, vp, u64, i32, i32]
    L.pp_scan_ws.argtypes = [vp, i32, i32, i32, vp, vp, u64, i32, i32, vp, sz]
    L.pp_workspace_size.argtypes = [i32, i32, i32, vp, vp, u64, C.POINTER(sz)]
    for name in ("pp_decoupled_scan_device", "pp_cooperative_scan_device", "pp_scan_device",
                 "pp_group_scan_device", "pp_decoupled_scan_device_noalloc"):
        getattr(L, name).argtypes = [vp, i32, i32, i32, vp, vp, u64]
    L.pp_reduce_device.argtypes = [vp, i32, i32, vp, u64, vp]
    L.pp_reduce.argtypes = [vp, i32, i32, vp, u64, vp]
    L.pp_reduce_ws.argtypes = [vp, i32, i32, vp, u64, vp, vp, sz]
    for name in ("pp_decoupled_scan_host", "pp_cooperative_scan_host", "pp_scan_host"):
        getattr(L, name).argtypes = [i32, i32, i32, vp, vp, u64]
    L.pp_reduce_host.argtypes = [i32, i32, vp, u64, vp]
    L.pp_segmented_scan.argtypes = [vp, i32, i32, i32, vp, vp, u64, vp, u64]
    L.pp_segmented_reduce.argtypes = [vp, i32, i32, vp, u64, vp, u64, vp]
    L.pp_rows_scan.argtypes = [vp, i32, i32, i32, vp, vp, u64, u64, i32]
    L.pp_status_string.argtypes = [i32]
    L.pp_status_string.restype = C.c_char_p
    L.pp_stream_status.argtypes = [vp]
    L.pp_workspace_status.argtypes = [vp, vp]
    L.pp_set_timeout_ns.argtypes = [u64]
    L.pp_set_max_ctas.argtypes = [i32]
    L.pp_set_cooperative_window.argtypes = [i32]
    L.pp_debug_set_skip_tile.argtypes = [C.c_longlong]
    L.pp_debug_set_lookback_delay.argtypes = [C.c_uint32, C.c_uint32]
    L.pp_debug_lookback_counters.argtypes = [vp, C.POINTER(C.c_uint64)]
    L.pp_version.restype = C.c_char_p
    for name in EXPORTS:
        if name not in ("pp_status_string", "pp_version"):
            getattr(L, name).restype = i32
    _lib = L
    return L


def status_string(status: int) -> str:
    try:
        return lib().pp_status_string(status).decode()
    except OSError:
        return "?"


def _check(status: int, what: str) -> None:
    if status != PP_OK:
        raise PPError(status, what)


def _op(op) -> int:
    return OPS[op] if isinstance(op, str) else int(op)


def _dt(dtype) -> int:
    if isinstance(dtype, str):
        return DTYPES[dtype]
    if isinstance(dtype, (np.dtype, type)):
        return NP_DTYPES[np.dtype(dtype)]
    return int(dtype)


def _kind(kind) -> int:
    if isinstance(kind, str):
        return {"inclusive": INCLUSIVE, "exclusive": EXCLUSIVE}[kind]
    return int(kind)


# ---- device-pointer API ------------------------------------------------------

def scan(kind, op, d_in: int, d_out: int, n: int, dtype, stream: int = 0, algo="auto", precision="default",
         workspace: tuple[int, int] | None = None) -> None:
    a = ALGOS[algo] if isinstance(algo, str) else int(algo)
    p = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    if workspace is None:
        st = lib().pp_scan(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n, a, p)
    else:
        st = lib().pp_scan_ws(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n, a, p, workspace[0],
                              workspace[1])
    _check(st, "pp_scan")


def workspace_size(algo, dtype, d_in: int, d_out: int, n: int, precision="default") -> int:
    a = ALGOS[algo] if isinstance(algo, str) else int(algo)
    p = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    out = C.c_size_t(0)
    _check(lib().pp_workspace_size(a, _dt(dtype), p, d_in, d_out, n, C.byref(out)), "pp_workspace_size")
    return out.value


def decoupled_scan_device(kind, op, d_in: int, d_out: int, n: int, dtype, stream: int = 0) -> None:
    _check(lib().pp_decoupled_scan_device(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n),
           "pp_decoupled_scan_device")


def decoupled_scan_device_noalloc(kind, op, d_in: int, d_out: int, n: int, dtype, stream: int = 0) -> None:
    """The decoupled scan with the library's fixed device scratch instead of an
    allocated workspace (for callers that may not allocate device memory)."""
    _check(lib().pp_decoupled_scan_device_noalloc(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n),
           "pp_decoupled_scan_device_noalloc")


def cooperative_scan_device(kind, op, d_in: int, d_out: int, n: int, dtype, stream: int = 0) -> None:
    _check(lib().pp_cooperative_scan_device(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n),
           "pp_cooperative_scan_device")


def scan_device(kind, op, d_in: int, d_out: int, n: int, dtype, stream: int = 0) -> None:
    _check(lib().pp_scan_device(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n), "pp_scan_device")


def group_scan_device(kind, op, d_in: int, d_out: int, n: int, dtype, stream: int = 0) -> None:
    _check(lib().pp_group_scan_device(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n),
           "pp_group_scan_device")


def _np_of(dtype) -> np.dtype:
    code = _dt(dtype)
    return [np.int32, np.uint32, np.int64, np.uint64, np.float32, np.float64][code]


def reduce_device(op, d_in: int, n: int, dtype, stream: int = 0):
    """Blocking device reduction returning the value on the host."""
    out = np.zeros(1, dtype=_np_of(dtype))
    _check(lib().pp_reduce_device(stream, _op(op), _dt(dtype), d_in, n, out.ctypes.data), "pp_reduce_device")
    return out[0]


def reduce(op, d_in: int, n: int, dtype, d_result: int, stream: int = 0,
           workspace: tuple[int, int] | None = None) -> None:
    """Asynchronous device reduction writing one element to d_result."""
    if workspace is None:
        st = lib().pp_reduce(stream, _op(op), _dt(dtype), d_in, n, d_result)
    else:
        st = lib().pp_reduce_ws(stream, _op(op), _dt(dtype), d_in, n, d_result, workspace[0], workspace[1])
    _check(st, "pp_reduce")


def segmented_scan(kind, op, d_in: int, d_out: int, n: int, d_offsets: int, num_segments: int, dtype,
                   stream: int = 0) -> None:
    """Scan every CSR segment [offsets[s], offsets[s+1]) of d_in independently."""
    _check(lib().pp_segmented_scan(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, n, d_offsets,
                                   num_segments), "pp_segmented_scan")


def segmented_reduce(op, d_in: int, n: int, d_offsets: int, num_segments: int, d_out: int, dtype,
                     stream: int = 0) -> None:
    _check(lib().pp_segmented_reduce(stream, _op(op), _dt(dtype), d_in, n, d_offsets, num_segments, d_out),
           "pp_segmented_reduce")


def rows_scan(kind, op, d_in: int, d_out: int, rows: int, cols: int, dtype, reverse: bool = False,
              stream: int = 0) -> None:
    _check(lib().pp_rows_scan(stream, _kind(kind), _op(op), _dt(dtype), d_in, d_out, rows, cols, int(reverse)),
           "pp_rows_scan")


# ---- host-array wrappers (blocking) --------------------------------------------

def _host_scan(fn_name: str, kind, op, h_in: np.ndarray, h_out: np.ndarray | None) -> np.ndarray:
    h_in = np.ascontiguousarray(h_in)
    out = np.empty_like(h_in) if h_out is None else h_out
    _check(getattr(lib(), fn_name)(_kind(kind), _op(op), NP_DTYPES[h_in.dtype], h_in.ctypes.data, out.ctypes.data,
                                   h_in.size), fn_name)
    return out


def decoupled_scan(kind, op, h_in: np.ndarray, h_out: np.ndarray | None = None) -> np.ndarray:
    return _host_scan("pp_decoupled_scan_host", kind, op, h_in, h_out)


def cooperative_scan(kind, op, h_in: np.ndarray, h_out: np.ndarray | None = None) -> np.ndarray:
    return _host_scan("pp_cooperative_scan_host", kind, op, h_in, h_out)


def scan_host(kind, op, h_in: np.ndarray, h_out: np.ndarray | None = None) -> np.ndarray:
    return _host_scan("pp_scan_host", kind, op, h_in, h_out)


def reduce_host(op, h_in: np.ndarray):
    h_in = np.ascontiguousarray(h_in)
    out = np.zeros(1, dtype=h_in.dtype)
    _check(lib().pp_reduce_host(_op(op), NP_DTYPES[h_in.dtype], h_in.ctypes.data, h_in.size, out.ctypes.data),
           "pp_reduce_host")
    return out[0]


# ---- status / settings ------------------------------------------------------------

def stream_status(stream: int = 0) -> int:
    """Synchronise `stream`; return (and clear) its first device-side error."""
    return int(lib().pp_stream_status(stream))


def workspace_status(stream: int, d_workspace: int) -> int:
    return int(lib().pp_workspace_status(stream, d_workspace))


def set_timeout_ns(ns: int) -> None:
    _check(lib().pp_set_timeout_ns(ns), "pp_set_timeout_ns")


def set_max_ctas(ctas: int) -> None:
    _check(lib().pp_set_max_ctas(ctas), "pp_set_max_ctas")


def set_cooperative_window(tiles_per_cta: int) -> None:
    """Tiles per CTA per window of the cooperative scan's rounds (0 = default)."""
    _check(lib().pp_set_cooperative_window(tiles_per_cta), "pp_set_cooperative_window")


def debug_set_skip_tile(tile: int) -> None:
    _check(lib().pp_debug_set_skip_tile(tile), "pp_debug_set_skip_tile")


def debug_set_lookback_delay(max_delay_ns: int, seed: int = 0) -> None:
    """Descriptor perturbation for tests (0 = off): pseudo-random delays of up
    to max_delay_ns before every descriptor publication of decoupled scans."""
    _check(lib().pp_debug_set_lookback_delay(max_delay_ns, seed), "pp_debug_set_lookback_delay")


def debug_lookback_counters(stream: int = 0) -> dict:
    """Read and clear the look-back counters gathered while the perturbation
    was on (synchronises `stream`)."""
    c = (C.c_uint64 * 4)()
    _check(lib().pp_debug_lookback_counters(stream, c), "pp_debug_lookback_counters")
    return {"reduce_then_scan": int(c[0]), "scan_then_reduce": int(c[1]), "over_32_predecessors": int(c[2]),
            "half_written_reads": int(c[3])}


def version() -> str:
    return lib().pp_version().decode()
