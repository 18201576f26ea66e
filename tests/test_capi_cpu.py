"""The C-ABI library without a GPU: it loads, exports every symbol
include/pp_gb300.h declares, and rejects bad arguments on the host before any
CUDA call."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(pp_\w+)\s*\(", text, flags=re.M))
    return names


def test_library_exports_every_declared_symbol(pp):
    declared = _declared_symbols()
    assert len(declared) >= 20
    lib = ctypes.CDLL(str(pp.LIB_PATH))
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(pp.EXPORTS) >= declared, sorted(declared - set(pp.EXPORTS))


def test_host_side_argument_checks(pp):
    L = pp.lib()
    dummy = 0x1000
    # bad enums / null pointers / unsupported combinations are rejected before any CUDA call
    assert L.pp_scan(None, 7, 0, 1, dummy, dummy, 10, 0, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_scan(None, 0, 99, 1, dummy, dummy, 10, 0, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_scan(None, 0, 0, 42, dummy, dummy, 10, 0, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_scan(None, 0, 0, 1, None, dummy, 10, 0, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_scan(None, 0, 2, 4, dummy, dummy, 10, 0, 0) == pp.PP_ERR_UNSUPPORTED  # bit_and on f32
    assert L.pp_scan(None, 0, 0, 1, dummy, dummy, 10, 0, 1) == pp.PP_ERR_UNSUPPORTED  # compensated u32
    # the descriptor perturbation knob: bounded delays only, a counters buffer required
    assert L.pp_debug_set_lookback_delay(2_000_000, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_debug_set_lookback_delay(0, 0) == pp.PP_OK
    assert L.pp_debug_lookback_counters(None, None) == pp.PP_ERR_INVALID_ARG
    assert L.pp_scan(None, 0, 1, 4, dummy, dummy, 10, 0, 2) == pp.PP_ERR_UNSUPPORTED  # fp64-carry multiplies
    assert L.pp_scan(None, 0, 0, 1, dummy, dummy, 0, 0, 0) == pp.PP_OK  # n == 0 is a no-op
    assert L.pp_scan_ws(None, 0, 0, 1, dummy, dummy, 10, 0, 0, None, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_reduce(None, 0, 1, dummy, 10, None) == pp.PP_ERR_INVALID_ARG
    assert L.pp_reduce(None, 3, 5, dummy, 10, dummy) == pp.PP_ERR_UNSUPPORTED  # bit_or on f64
    assert L.pp_reduce_device(None, 0, 1, dummy, 10, None) == pp.PP_ERR_INVALID_ARG
    assert L.pp_set_timeout_ns(0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_set_max_ctas(-1) == pp.PP_ERR_INVALID_ARG
    assert L.pp_set_cooperative_window(-1) == pp.PP_ERR_INVALID_ARG
    assert L.pp_set_cooperative_window(4097) == pp.PP_ERR_INVALID_ARG
    assert L.pp_set_cooperative_window(0) == pp.PP_OK
    assert L.pp_decoupled_scan_host(0, 0, 9, dummy, dummy, 5) == pp.PP_ERR_INVALID_ARG
    # pointers not aligned to the element size
    assert L.pp_scan(None, 0, 0, 1, dummy + 2, dummy, 10, 0, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_scan(None, 0, 0, 3, dummy, dummy + 4, 10, 0, 0) == pp.PP_ERR_INVALID_ARG
    assert L.pp_reduce(None, 0, 1, dummy + 1, 10, dummy) == pp.PP_ERR_INVALID_ARG


def test_status_strings_and_version(pp):
    for code in range(8):
        assert pp.status_string(code) not in ("", "unknown status")
    assert pp.status_string(99) == "unknown status"
    assert "sm_103a" in pp.version()


def test_workspace_size_is_host_only(pp):
    # 2^30 uint32 on the aligned (bulk-copy) path: 64 KB tiles, one descriptor word each
    a = 1 << 12
    n = 1 << 30
    size = pp.workspace_size("decoupled", "u32", a, a, n)
    assert size == 4096 + 8192 * 16 + (n // 16384) * 8
    # uint64: 70 KB tiles (8960 elements), two words each
    assert pp.workspace_size("decoupled", "u64", a, a, n) == 4096 + 8192 * 16 + -(-n // 8960) * 16
    # float: 72 KB tiles (18432 elements), one word each
    assert pp.workspace_size("decoupled", "f32", a, a, n) == 4096 + 8192 * 16 + -(-n // 18432) * 8
    # 4-byte but not 16-byte aligned input: the staged kernel's grid shifts by the phantom elements
    assert pp.workspace_size("decoupled", "u32", a + 4, a, n) == 4096 + 8192 * 16 + (n // 16384 + 1) * 8
    # not even aligned to the element size: refused
    import pytest

    with pytest.raises(pp.PPError):
        pp.workspace_size("decoupled", "u32", a + 1, a, n)
    # cooperative rounds: one record per tile, one 64-bit word per 32-bit word
    # of the tile aggregate and of the segment prefixes (one per compute warp),
    # rounded up to 16 bytes (float, uint32: 1 + 16 words; uint64: 2 + 20 * 2)
    assert pp.workspace_size("cooperative", "f32", a, a, n) == 4096 + 8192 * 16 + -(-n // 18432) * 144
    assert pp.workspace_size("cooperative", "u32", a, a, n) == 4096 + 8192 * 16 + (n // 16384) * 144
    assert pp.workspace_size("cooperative", "u64", a, a, n) == 4096 + 8192 * 16 + -(-n // 8960) * 336
    # element-aligned but not 16-byte aligned: still the staged kernel, grid shifted
    assert pp.workspace_size("cooperative", "u32", a + 4, a, n) == 4096 + 8192 * 16 + (n // 16384 + 1) * 144
