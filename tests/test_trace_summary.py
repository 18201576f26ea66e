"""The per-tile timeline summary of pptrace.py on a synthetic trace (no GPU):
every interval it reports is the difference of the right pair of events."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "sycl-building-blocks_gb300"))
import pptrace  # noqa: E402


def test_summary_of_a_synthetic_trace():
    tiles = 2000
    a = np.zeros((tiles, pptrace.SLOTS), dtype=np.uint64)
    t = np.arange(tiles, dtype=np.uint64) * 1000 + 10_000
    a[:, 9] = t  # ticket
    a[:, 10] = t + 100  # issue
    a[:, 11] = t + 1500  # compute waits for data
    a[:, 12] = t + 1700  # data at compute
    a[:, 0] = t + 1650  # data in (look-back warp)
    a[:, 1] = t + 2700  # aggregate published
    a[:, 3] = t + 4000  # prefix known
    a[:, 13] = t + 3500  # compute waits for prefix
    a[:, 5] = t + 4100  # scan pass starts
    a[:, 6] = t + 5600  # scan pass done
    a[:, 8] = np.arange(tiles) % 4  # CTA: 4 CTAs, each every 4th tile
    s = pptrace.summarise(a.reshape(-1))
    assert s["steady_tiles"] == tiles - 600
    assert s["ticket_to_issue (stage free wait)"]["p50"] == 100
    assert s["issue_to_data_at_compute"]["p50"] == 1600
    assert s["compute_waits_for_data"]["p50"] == 200
    assert s["reduce_pass"]["p50"] == 1000
    assert s["look_back_from_data_in"]["p50"] == 2350
    assert s["prefix_known_after_own_aggregate"]["p50"] == 1300
    assert s["compute_waits_for_prefix"]["p50"] == 600
    assert s["scan_pass"]["p50"] == 1500
    assert s["stage_life (issue to scan done)"]["p50"] == 5500
    assert s["cta_tile_period_ns"] == 4000.0
    assert "first_poll_round_trip" not in s
