"""Benchmark of the scan / reduce hot path on GB300.

Headline (one JSON line on rank 0): effective GB/s of the single-pass
decoupled look-back inclusive plus-scan of n = 2^30 uint32 values drawn
uniformly from [0, 2^16), counting 2n*4 bytes (read + write) per scan, with
the input resident in HBM (4 GiB in + 4 GiB out, far above the 129 MB L2, so
no flush is needed between steps). A step is one scan over the whole array.
The input is the splitmix64 stream the oracle, the tests and the CPU baselines
use (generated on the device with the same formula), and the timed scans'
output is checked exactly: on the device (neighbouring differences give back
the input) and, in the CPU-baseline leg, against the oracle's scan.

Also reported:
  roofline      achieved GB/s of the scan kernel (CUDA events around every
                launch on its stream) against the measured HBM copy peak;
  e2e           the same metric through the blocking host-pointer C-ABI call
                (pp_decoupled_scan_host): pinned host input -> device, scan,
                device -> pinned host output, every step;
  cpu_baseline  the reference's decoupled look-back algorithm restated in C
                (oracle/oracle.c) on all host cores, on the whole input;
  secondary     the other HBM-scale primitives of the same workload family,
                each output checked after its timing (`verified`).

`--impl reference` times the reference's CPU algorithm alone (the oracle
restatement, or the reference headers compiled against the SYCL CPU shim
when that library exists for this machine) and prints its own line.

Multi-GPU: the primitives do not shard in this library, so N > 1 runs N
independent replicas (one per rank) and reports the total.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "sycl-building-blocks_gb300"
ORACLE_DIR = ROOT / "oracle"
sys.path.insert(0, str(PKG))

N_HEADLINE = 1 << 30
SEED = 0x5CA72026
E2E_GUARD_BYTES = 16 << 30  # pinned guard ahead of the end-to-end leg's host buffers (see run_ours)
METRIC = "scan effective GB/s (2n bytes) vs HBM peak/memcpy; batched-segment elems/s"
UNIT = "GB/s"


def measured_peak() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel_key: str) -> float | None:
    """DRAM bytes per launch from the committed ncu summary, if present."""
    p = ROOT / "profiles" / "traffic.json"
    try:
        return float(json.loads(p.read_text())[kernel_key])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier(torch):
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        torch.distributed.barrier()


def max_over_ranks(torch, v: float) -> float:
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())
    return v


# ---------------------------------------------------------------------------------
# Inputs: the splitmix64 stream the oracle, the tests and the CPU baselines use
# (element i of stream `seed` is mix64(seed + (i + 1) * 0x9E3779B97F4A7C15),
# mapped to [lo, hi) by lo + (((x >> 32) * (hi - lo)) >> 32)), computed here
# with torch's wrapping int64 arithmetic on the benchmark's own device.
_GOLDEN = 0x9E3779B97F4A7C15
_MIX1 = 0xBF58476D1CE4E5B9
_MIX2 = 0x94D049BB133111EB


def _s64(v: int) -> int:
    """The int64 with the bits of the uint64 v."""
    return v - (1 << 64) if v >= (1 << 63) else v


def splitmix_u32(torch, seed: int, n: int, lo: int, hi: int, device, chunk: int = 1 << 25):
    """int32 tensor of n values of the splitmix64 stream `seed` in [lo, hi)."""
    out = torch.empty(n, dtype=torch.int32, device=device)
    rng = hi - lo

    def srl(z, k):  # logical shift right of int64 bit patterns
        return (z >> k) & ((1 << (64 - k)) - 1)

    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        i = torch.arange(a + 1, b + 1, dtype=torch.int64, device=device)
        z = i * _s64(_GOLDEN) + _s64(seed % (1 << 64))
        z = (z ^ srl(z, 30)) * _s64(_MIX1)
        z = (z ^ srl(z, 27)) * _s64(_MIX2)
        z = z ^ srl(z, 31)
        v = lo + ((srl(z, 32) * rng) >> 32)
        out[a:b] = v.to(torch.int32)  # the low 32 bits: uint32 values as int32
    return out


def check_plus_scan(torch, d_in, d_out, exclusive: bool, chunk: int = 1 << 27) -> bool:
    """Exact check of an integer plus-scan on the device: the first output is
    in[0] (0 when exclusive) and neighbouring outputs differ by the input
    (wrapping integer arithmetic), which determines every output."""
    n = d_in.numel()
    if n == 0:
        return True
    first = int(d_out[0]) == (0 if exclusive else int(d_in[0]))
    ok = first
    for a in range(1, n, chunk):
        b = min(n, a + chunk)
        src = d_in[a - 1:b - 1] if exclusive else d_in[a:b]
        ok &= bool(torch.equal(d_out[a:b] - d_out[a - 1:b - 1], src))
    return bool(ok)


def check_max_scan(torch, d_in, d_out, chunk: int = 1 << 27) -> bool:
    """Exact check of an inclusive max-scan on the device, chunk by chunk with
    the running maximum carried across chunks."""
    n = d_in.numel()
    carry = None
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        want = torch.cummax(d_in[a:b], 0).values
        if carry is not None:
            want = torch.maximum(want, carry)
        if not torch.equal(d_out[a:b], want):
            return False
        carry = want[-1]
    return True


def release_cached_memory(torch) -> None:
    """Return torch's cached device memory to the driver, then let the driver
    finish reclaiming it before anything is timed: on GB300 the 2^28-element
    scans that followed the release of 16 GiB ran 25-30 % slow for the next
    few milliseconds (4 GiB: about a millisecond) and at full speed after a
    pause of one second."""
    torch.cuda.synchronize()
    before = torch.cuda.memory_reserved()
    torch.cuda.empty_cache()
    freed = before - torch.cuda.memory_reserved()
    if freed > (1 << 30):
        time.sleep(min(2.0, 0.1 * freed / (1 << 30)))


def time_device(torch, fn, steps: int, warmup: int, stream) -> tuple[float, list[float]]:
    """Run fn() warmup + steps times on `stream`; return (total ms of the timed
    steps bracketed by barrier + synchronize, per-launch ms from events)."""
    release_cached_memory(torch)
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier(torch)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for a, b in evs:
        a.record(stream)
        fn()
        b.record(stream)
    end.record(stream)
    torch.cuda.synchronize()
    barrier(torch)
    torch.cuda.synchronize()
    return start.elapsed_time(end), [a.elapsed_time(b) for a, b in evs]


def run_ours(args) -> dict | None:
    import numpy as np
    import torch

    import ppbuild

    ws, rank, local = dist_info()
    if ws > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    ppbuild.build()
    import ppgb300 as pp

    pp.lib()
    n = args.n
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    # input: U[0, 2^16) uint32 from the splitmix64 stream of the oracle and the
    # CPU baselines (seed per rank), generated on the device
    d_in = splitmix_u32(torch, SEED + rank, n, 0, 1 << 16, "cuda")
    d_out = torch.empty_like(d_in)
    algo_bytes = 2 * n * 4
    # pinned host buffers of the end-to-end leg, allocated and filled now: the
    # timed host-array calls made right after pinning 8 GiB met host stalls
    # of 40-130 ms in their first steps.
    # On some GB300 machines (virtual machines) DMA over the first pinned
    # allocations of a process met periodic stalls: 30-200 ms about every
    # 0.5 s, measured with the same pipeline over buffers pinned first
    # (stalls) and second (none) in one process, alternating call by call.
    # A pinned guard allocation taken first and held through the end-to-end
    # leg keeps the timed buffers out of the first allocations.
    guard = torch.empty(E2E_GUARD_BYTES, dtype=torch.uint8, pin_memory=True)
    h_in = torch.empty(n, dtype=torch.int32, pin_memory=True)
    h_out = torch.empty(n, dtype=torch.int32, pin_memory=True)
    h_in.copy_(d_in)
    h_out.fill_(0)
    # the timed scans' output for the CPU baseline's comparison with the oracle
    h_timed = torch.empty(n, dtype=torch.int32, pin_memory=True) if (rank == 0 and not args.no_cpu_baseline) else None

    def step():
        pp.decoupled_scan_device("inclusive", "plus", d_in.data_ptr(), d_out.data_ptr(), n, "u32", stream=sh)

    step()
    if pp.stream_status(sh) != 0:
        raise RuntimeError("device error in warm-up scan")
    # sanity: last prefix == total (mod 2^32), first == in[0]
    total = int(d_in.sum(dtype=torch.int64).item()) & 0xFFFFFFFF  # no converted copy of the input
    verified = (int(d_out[-1].item()) & 0xFFFFFFFF) == total and int(d_out[0].item()) == int(d_in[0].item())
    # free torch's cached scratch of that check (a large cached but unused block slowed the timed scans by ~3%
    # on GB300), and let the driver reclaim it
    release_cached_memory(torch)

    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0]
    gpu_index = int(vis) if vis.isdigit() else local
    sampler = ClockSampler(gpu_index)
    sampler.start()
    time.sleep(0.2)
    total_ms, per_launch = time_device(torch, step, args.steps, args.warmup, stream)
    clocks = sampler.stop()
    if pp.stream_status(sh) != 0:
        raise RuntimeError("device error during the timed scans")
    # the timed scans' output, checked exactly on the device and kept for the
    # CPU baseline's comparison with the oracle
    timed_ok = check_plus_scan(torch, d_in, d_out, exclusive=False)
    if h_timed is not None:
        h_timed.copy_(d_out)
    release_cached_memory(torch)
    total_ms = max_over_ranks(torch, total_ms)
    ms_per_step = total_ms / args.steps
    value = ws * algo_bytes * args.steps / (total_ms * 1e-3) / 1e9
    launch_ms = statistics.mean(per_launch)
    achieved = algo_bytes / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()

    # device-to-device copy of the same bytes, re-measured in this run
    def copy_step():
        d_out.copy_(d_in)

    cp_ms, _ = time_device(torch, copy_step, max(3, args.steps // 4), 2, stream)
    memcpy_gbs = algo_bytes * max(3, args.steps // 4) / (cp_ms * 1e-3) / 1e9

    # end to end through the host-pointer C-ABI call
    e2e_steps = max(2, min(args.steps, args.e2e_steps))
    torch.cuda.synchronize()
    L = pp.lib()

    def e2e_step():
        st = L.pp_decoupled_scan_host(0, 0, 1, h_in.data_ptr(), h_out.data_ptr(), n)
        if st != 0:
            raise RuntimeError(f"pp_decoupled_scan_host failed: {st}")

    # The first calls through a fresh pair of pinned host buffers run up to 4x slower, for two to five calls
    # depending on the machine's state: warm up until two calls in a row agree within 5 % (at most 10 calls).
    warm_ms = []
    while len(warm_ms) < 10:
        t_w = time.perf_counter()
        e2e_step()
        warm_ms.append(round((time.perf_counter() - t_w) * 1e3, 2))
        if len(warm_ms) >= 3 and abs(warm_ms[-1] - warm_ms[-2]) <= 0.05 * warm_ms[-1]:
            break
    barrier(torch)
    t0 = time.perf_counter()
    step_ends = []
    for _ in range(e2e_steps):
        e2e_step()  # returns once the results are in the host buffer
        step_ends.append(time.perf_counter())
    torch.cuda.synchronize()
    barrier(torch)
    e2e_s = max_over_ranks(torch, time.perf_counter() - t0)
    e2e_step_ms = [round((b - a) * 1e3, 2) for a, b in zip([t0] + step_ends[:-1], step_ends)]
    e2e_value = ws * algo_bytes * e2e_steps / e2e_s / 1e9
    e2e_ok = bool(torch.equal(h_out, h_timed)) if h_timed is not None else (
        (int(h_out[-1]) & 0xFFFFFFFF) == total and int(h_out[0]) == int(h_in[0]))
    link = host_link_rates(torch, h_in, h_out, d_in, d_out)
    del h_in, h_out, guard

    secondary = {} if args.no_secondary else run_secondary(torch, pp, stream, args, d_in, d_out)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(d_in, h_timed, args)
    del h_timed

    if rank != 0:
        return None
    traffic = ncu_traffic("decoupled_scan_u32_2p30")
    return {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic: uniform [0, 2^16) uint32 from the oracle's splitmix64 stream (seed 0x5CA72026 + rank), "
                "generated on the device",
        "config": {
            "workload": "decoupled look-back inclusive plus-scan, n=2^30 uint32 U[0,2^16)",
            "n": n,
            "bytes_per_step": algo_bytes,
            "l2": "inputs (4 GiB) larger than L2 (129 MB); no flush",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "verified_last_prefix": verified,
            "verified_timed_output": {"exact_on_device": timed_ok,
                                      "matches_oracle": None if cpu is None else cpu.get("gpu_output_matches_oracle")},
        },
        "roofline": {
            "bound": "hbm",
            "achieved": round(achieved, 2),
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "peak_kind": peak_kind,
            "traffic": traffic,
            "memcpy_gbs_this_run": round(memcpy_gbs, 2),
            "frac_of_memcpy_this_run": round(achieved / memcpy_gbs, 4),
        },
        "e2e": {
            "value": round(e2e_value, 2),
            "unit": UNIT,
            "h2d_bytes_per_step": n * 4,
            "d2h_bytes_per_step": n * 4,
            "api": "pp_decoupled_scan_host (pinned host buffers; streamed in 64 MiB chunks, both copy directions overlapping the scans)",
            "verified_tail": e2e_ok,
            "host_link_gbs_this_run": link,
            "host_buffers": "torch pinned (cudaHostAlloc), allocated after a 16 GiB pinned guard: the first pinned "
                            "allocations of a process met periodic DMA stalls on some of these virtual machines",
            "step_ms": e2e_step_ms,
            "warmup_call_ms": warm_ms,
        },
        "gpu_launches": args.steps,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "secondary": secondary,
    }


def host_link_rates(torch, h_in, h_out, d_in, d_out) -> dict:
    """Plain pinned copies of the same arrays in this run (GB/s): host to device, device to host, and both at once
    on two streams (bytes of both directions counted) -- the bound of the end-to-end figure."""
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    nbytes = h_in.numel() * h_in.element_size()

    def timed(fn):  # best of three
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(3):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    def h2d():
        with torch.cuda.stream(s1):
            d_in.copy_(h_in, non_blocking=True)

    def d2h():
        with torch.cuda.stream(s2):
            h_out.copy_(d_out, non_blocking=True)

    def both():
        h2d()
        d2h()

    return {"h2d": round(nbytes / timed(h2d) / 1e9, 1), "d2h": round(nbytes / timed(d2h) / 1e9, 1),
            "both_directions": round(2 * nbytes / timed(both) / 1e9, 1)}


def run_secondary(torch, pp, stream, args, d_in32, d_out32) -> dict:
    """The other HBM-scale configurations: GB/s of each at 2n (scan) or n (reduce) bytes. Every timed output is
    checked after its timing (`verified`): integer scans exactly on the device (neighbouring differences give back
    the input; max-scans against torch.cummax), float ones against an FP64 scan within a stated bound."""
    out = {}
    verified = {}
    sh = stream.cuda_stream
    n30 = args.n
    steps = max(3, args.steps // 5)

    def rate(fn, nbytes):
        ms, per = time_device(torch, fn, steps, 5, stream)
        if pp.stream_status(sh) != 0:
            raise RuntimeError("device error in secondary benchmark")
        return round(nbytes * steps / (ms * 1e-3) / 1e9, 2)

    out["u32_exclusive_plus_2p30"] = rate(
        lambda: pp.decoupled_scan_device("exclusive", "plus", d_in32.data_ptr(), d_out32.data_ptr(), n30, "u32",
                                         stream=sh), 8 * n30)
    verified["u32_exclusive_plus_2p30"] = check_plus_scan(torch, d_in32, d_out32, exclusive=True)
    out["u32_cooperative_inclusive_plus_2p30"] = rate(
        lambda: pp.cooperative_scan_device("inclusive", "plus", d_in32.data_ptr(), d_out32.data_ptr(), n30, "u32",
                                           stream=sh), 8 * n30)
    verified["u32_cooperative_inclusive_plus_2p30"] = check_plus_scan(torch, d_in32, d_out32, exclusive=False)
    full = splitmix_u32(torch, SEED + 1, n30, 0, 1 << 32, "cuda")  # int32 over the full range
    out["i32_max_scan_2p30"] = rate(
        lambda: pp.decoupled_scan_device("inclusive", "maximum", full.data_ptr(), d_out32.data_ptr(), n30, "i32",
                                         stream=sh), 8 * n30)
    verified["i32_max_scan_2p30"] = check_max_scan(torch, full, d_out32)
    del full
    gen = torch.Generator(device="cuda")
    gen.manual_seed(SEED + 1)
    n28 = args.n // 4
    u64 = torch.randint(0, 1 << 32, (n28,), dtype=torch.int64, device="cuda", generator=gen)
    o64 = torch.empty_like(u64)
    for kind in ("inclusive", "exclusive"):
        out[f"u64_{kind}_plus_2p28"] = rate(
            lambda k=kind: pp.decoupled_scan_device(k, "plus", u64.data_ptr(), o64.data_ptr(), n28, "u64", stream=sh),
            16 * n28)
        verified[f"u64_{kind}_plus_2p28"] = check_plus_scan(torch, u64, o64, exclusive=kind == "exclusive")
    del u64, o64
    # float64: every element costs FP64 additions, whose rate on this part is far below its HBM bandwidth
    f64 = torch.randn(n28, dtype=torch.float64, device="cuda", generator=gen)
    o64 = torch.empty_like(f64)
    out["f64_inclusive_plus_2p28"] = rate(
        lambda: pp.decoupled_scan_device("inclusive", "plus", f64.data_ptr(), o64.data_ptr(), n28, "f64", stream=sh),
        16 * n28)
    # two FP64 scans of the same data differ by at most (depth) * eps * sum |x_j| per prefix
    bound64 = 256 * 2.0 ** -52 * torch.cumsum(f64.abs(), 0)
    verified["f64_inclusive_plus_2p28"] = bool(((o64 - torch.cumsum(f64, 0)).abs() <= bound64).all())
    del bound64
    out["f64_sum_reduce_2p28"] = rate(
        lambda: pp.reduce("plus", f64.data_ptr(), n28, "f64", o64.data_ptr(), stream=sh), 8 * n28)
    verified["f64_sum_reduce_2p28"] = bool(abs(float(o64[0]) - float(f64.sum())) <=
                                           1024 * 2.0 ** -52 * float(f64.abs().sum()))
    out["f64_maximum_scan_2p28"] = rate(
        lambda: pp.decoupled_scan_device("inclusive", "maximum", f64.data_ptr(), o64.data_ptr(), n28, "f64",
                                         stream=sh), 16 * n28)
    verified["f64_maximum_scan_2p28"] = check_max_scan(torch, f64, o64)
    del f64, o64
    f = torch.randn(n30, dtype=torch.float32, device="cuda", generator=gen)
    res = torch.empty(2, dtype=torch.float32, device="cuda")
    out["f32_sum_reduce_2p30"] = rate(
        lambda: pp.reduce("plus", f.data_ptr(), n30, "f32", res.data_ptr(), stream=sh), 4 * n30)
    out["f32_max_reduce_2p30"] = rate(
        lambda: pp.reduce("maximum", f.data_ptr(), n30, "f32", res.data_ptr() + 4, stream=sh), 4 * n30)
    r = res.cpu().numpy()
    ref_sum = float(f.double().sum().item())
    ref_max = float(f.max().item())
    # worst case of the reduction's combine tree: runs of at most n / (SMs * 512 threads * 4 lanes) additions,
    # then at most 64 levels
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    bound = (math.ceil(n30 / (sms * 512 * 4)) + 64) * 2.0 ** -23 * float(f.abs().double().sum().item())
    out["f32_reduce_check"] = {"sum": float(r[0]), "fp64_sum": ref_sum, "abs_err": abs(float(r[0]) - ref_sum),
                               "bound": bound, "max_exact": float(r[1]) == ref_max}
    verified["f32_sum_reduce_2p30"] = abs(float(r[0]) - ref_sum) <= bound
    verified["f32_max_reduce_2p30"] = float(r[1]) == ref_max
    del f
    out["precision_f32_2p28"] = bench_precision(torch, pp, stream, steps, gen)
    out["segmented_2p16_segments"] = bench_segmented(torch, pp, stream, steps)
    out["cumsum_4096x8192"] = bench_cumsum(torch, stream, steps)

    # last, so that its many short launches leave nothing behind in the clocks of the HBM-scale lines above
    # C1: n = 2^24 uint32 U[0, 255] (64 MiB, fits in the L2): L2 flushed (by a read) before every launch, each
    # launch timed on its own
    n24 = 1 << 24
    x24 = splitmix_u32(torch, SEED, n24, 0, 256, "cuda")  # the reference's CPU-runnable case, C1
    y24 = torch.empty_like(x24)
    r24 = torch.empty(1, dtype=torch.int64, device="cuda")
    # reading 256 MiB (twice the L2) leaves the L2 full of clean lines of another buffer: no write-back of the
    # flush itself lands in the timed launch
    flush = torch.zeros(1 << 26, dtype=torch.int32, device="cuda")

    def flushed_rate(fn, nbytes, reps=21):
        # median of `reps` launches, each timed on its own after the flush
        for _ in range(3):
            fn()
        times = []
        for _ in range(reps):
            flush.sum()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        if pp.stream_status(sh) != 0:
            raise RuntimeError("device error in the 2^24 benchmark")
        ms = sorted(times)[len(times) // 2]
        return round(nbytes / (ms * 1e-3) / 1e9, 2)

    out["u32_inclusive_plus_2p24_l2_flushed"] = flushed_rate(
        lambda: pp.decoupled_scan_device("inclusive", "plus", x24.data_ptr(), y24.data_ptr(), n24, "u32", stream=sh),
        8 * n24)
    verified["u32_inclusive_plus_2p24_l2_flushed"] = check_plus_scan(torch, x24, y24, exclusive=False)
    out["u32_sum_reduce_2p24_l2_flushed"] = flushed_rate(
        lambda: pp.reduce("plus", x24.data_ptr(), n24, "u32", r24.data_ptr(), stream=sh), 4 * n24)
    verified["u32_sum_reduce_2p24_l2_flushed"] = (int(r24[0]) & 0xFFFFFFFF) == (
        int(x24.sum(dtype=torch.int64)) & 0xFFFFFFFF)
    # the same protocol on a device copy of the same 64 MiB: what "copy speed" is at this size
    out["device_copy_64mib_l2_flushed"] = flushed_rate(lambda: y24.copy_(x24), 8 * n24)
    del x24, y24, flush
    for name in ("precision_f32_2p28", "segmented_2p16_segments", "cumsum_4096x8192"):
        verified[name] = "per line: see its own fields"
    out["verified"] = verified
    return out


def _err_stats(torch, got, ref, cabs):
    """max / RMS relative error per prefix (prefixes with |s| >= 1e-3 rms(s)),
    the normwise error max|err| / max|s|, against an FP64 scan, and for the
    prefixes left out of the relative figures (near zero crossings of the
    running sum) their largest error against the magnitude the sum was built
    from, max |err_i| / sum_{j<=i} |x_j| (`cabs`)."""
    err = (got.double() - ref).abs()
    scale = torch.sqrt(torch.mean(ref * ref))
    mask = ref.abs() >= 1e-3 * scale
    rel = err[mask] / ref.abs()[mask]
    ex = ~mask
    ex_rel = err[ex] / cabs[ex]
    return {"max_rel": float(rel.max()), "rms_rel": float(torch.sqrt(torch.mean(rel * rel))),
            "normwise": float(err.max() / ref.abs().max()), "excluded_near_zero": int(ex.sum()),
            "excluded_max_err_over_abs_prefix_sum": float(ex_rel.max()) if ex_rel.numel() else 0.0,
            "all_prefixes_max_err_over_abs_prefix_sum": float((err / cabs).max())}


def bench_precision(torch, pp, stream, steps, gen) -> dict:
    """f32 plus-scan of 2^28 N(0,1) and sign-random lognormal(0, 2) values:
    plain, compensated and FP64-carry, GB/s and errors vs an FP64 scan. The
    three modes are timed first, each into its own output, and the FP64
    references are built afterwards, so that no timing runs beside their
    temporaries."""
    sh = stream.cuda_stream
    n = 1 << 28
    res = {}
    precs = ("default", "compensated", "fp64_carry")
    outs = {p: torch.empty(n, dtype=torch.float32, device="cuda") for p in precs}
    for dist in ("normal", "lognormal"):
        x = torch.randn(n, dtype=torch.float32, device="cuda", generator=gen)
        if dist == "lognormal":
            sign = torch.randint(0, 2, (n,), device="cuda", generator=gen).float() * 2 - 1
            x = (torch.exp(2.0 * x) * sign).float()
            del sign
        d = {}
        for prec in precs:
            out = outs[prec]
            fn = lambda p=prec, o=out: pp.scan("inclusive", "plus", x.data_ptr(), o.data_ptr(), n, "f32", stream=sh,
                                               precision=p)
            ms, _ = time_device(torch, fn, steps, 2, stream)
            if pp.stream_status(sh) != 0:
                raise RuntimeError("device error in precision benchmark")
            d[prec] = {"gbs": round(8 * n * steps / (ms * 1e-3) / 1e9, 2)}
        ref = torch.cumsum(x.double(), 0)
        cabs = torch.cumsum(x.double().abs(), 0)
        for prec in precs:
            d[prec].update(_err_stats(torch, outs[prec], ref, cabs))
        d["compensated_slowdown_vs_plain"] = round(d["default"]["gbs"] / d["compensated"]["gbs"] - 1, 4)
        res[dist] = d
        del x, ref, cabs
        release_cached_memory(torch)
    del outs
    return res


def _segment_reference(torch, x, d_off):
    """Per-element inclusive sums within segments (float64, or int64 for
    integer payloads, exact there) and sum_{j<=i in the segment} |x_j|, from
    global running sums minus the running sum before each segment's start."""
    n = x.numel()
    wide = torch.float64 if x.is_floating_point() else torch.int64
    seg = torch.searchsorted(d_off[1:], torch.arange(n, device=x.device), right=True)  # segment of each element
    start = d_off[seg]
    c = torch.cumsum(x.to(wide), 0)
    ca = torch.cumsum(x.to(wide).abs(), 0)
    before = torch.where(start > 0, c[(start - 1).clamp(min=0)], torch.zeros((), dtype=wide, device=x.device))
    before_a = torch.where(start > 0, ca[(start - 1).clamp(min=0)], torch.zeros((), dtype=wide, device=x.device))
    return c - before, ca - before_a


def check_segmented_scan(torch, x, y, d_off) -> bool:
    """Every segment's inclusive plus-scan: exact for integer payloads; for
    float32 within (64 + 66) * eps * sum |x_j| (the scan tests' bound for
    segments of up to 2^16 elements) plus 1e-9 for the float64 reference's own
    rounding."""
    ref, cabs = _segment_reference(torch, x, d_off)
    if not x.is_floating_point():
        return bool(torch.equal(y.to(torch.int64), ref.to(torch.int32).to(torch.int64)))
    return bool(((y.double() - ref).abs() <= 130 * 2.0 ** -23 * cabs + 1e-9).all())


def check_segmented_reduce(torch, x, tot, d_off) -> bool:
    """Every segment's total, with the same measures as check_segmented_scan."""
    ref, cabs = _segment_reference(torch, x, d_off)
    last = d_off[1:] - 1  # every benchmark segment is non-empty
    if not x.is_floating_point():
        return bool(torch.equal(tot.to(torch.int64), ref[last].to(torch.int32).to(torch.int64)))
    return bool(((tot.double() - ref[last]).abs() <= 130 * 2.0 ** -23 * cabs[last] + 1e-9).all())


def bench_segmented(torch, pp, stream, steps) -> dict:
    """65,536 segments, lengths floor(exp(U[0, ln 2^16])) clipped to [1, 2^16]
    (about 2^28 elements), int64 offsets; int32 U[0,1000) and f32 N(0,1)
    payloads. One batched launch in a CUDA graph vs one launch per segment
    (also replayed from a CUDA graph), and the batched reduction of the same
    segments."""
    S = 65536
    g = torch.Generator(device="cpu").manual_seed(0x5EC)
    lens = torch.floor(torch.exp(torch.rand(S, generator=g, dtype=torch.float64) * math.log(2 ** 16)))
    lens = lens.clamp(1, 2 ** 16).to(torch.int64)
    offs = torch.zeros(S + 1, dtype=torch.int64)
    offs[1:] = torch.cumsum(lens, 0)
    n = int(offs[-1])
    d_off = offs.cuda()
    gd = torch.Generator(device="cuda").manual_seed(0x5EC)
    res = {"segments": S, "elements": n}
    for dt, make in (("i32", lambda: torch.randint(0, 1000, (n,), dtype=torch.int32, device="cuda", generator=gd)),
                     ("f32", lambda: torch.randn(n, dtype=torch.float32, device="cuda", generator=gd))):
        x = make()
        y = torch.empty_like(x)
        s = torch.cuda.Stream()
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            pp.segmented_scan("inclusive", "plus", x.data_ptr(), y.data_ptr(), n, d_off.data_ptr(), S, dt,
                              stream=s.cuda_stream)
            s.synchronize()
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=s):
                pp.segmented_scan("inclusive", "plus", x.data_ptr(), y.data_ptr(), n, d_off.data_ptr(), S, dt,
                                  stream=s.cuda_stream)
        ms_b, _ = time_device(torch, graph.replay, steps, 2, torch.cuda.current_stream())
        ok = check_segmented_scan(torch, x, y, d_off)
        # one plain launch per segment, captured once, replayed
        with torch.cuda.stream(s):
            big = int(lens.max())
            pp.decoupled_scan_device("inclusive", "plus", x.data_ptr(), y.data_ptr(), big, dt, stream=s.cuda_stream)
            s.synchronize()
            graph2 = torch.cuda.CUDAGraph()
            esz = x.element_size()
            offl = offs.tolist()
            with torch.cuda.graph(graph2, stream=s):
                for k in range(S):
                    a, b = offl[k], offl[k + 1]
                    pp.decoupled_scan_device("inclusive", "plus", x.data_ptr() + a * esz, y.data_ptr() + a * esz,
                                             b - a, dt, stream=s.cuda_stream)
        ms_p, _ = time_device(torch, graph2.replay, max(2, steps // 20), 1, torch.cuda.current_stream())
        # the batched reduction of the same segments (plain launches on s); n * 4 bytes read per call
        try:
            tot = torch.empty(S, dtype=x.dtype, device="cuda")
            ms_r, _ = time_device(torch, lambda: pp.segmented_reduce("plus", x.data_ptr(), n, d_off.data_ptr(), S,
                                                                      tot.data_ptr(), dt, stream=s.cuda_stream),
                                  steps, 3, s)
            ok_r = check_segmented_reduce(torch, x, tot, d_off)
            red = {"batched_ms": round(ms_r / steps, 4), "batched_gbs": round(n * 4 / (ms_r / steps * 1e-3) / 1e9, 2),
                   "verified": bool(ok_r)}
            del tot
        except Exception as e:  # the scan figures stand on their own
            red = {"error": f"{type(e).__name__}: {e}"}
        if pp.stream_status(s.cuda_stream) != 0:
            raise RuntimeError("device error in segmented benchmark")
        res[dt] = {"batched_elems_per_s": round(n * steps / (ms_b * 1e-3), 1), "batched_ms": round(ms_b / steps, 4),
                   "per_segment_launches_ms": round(ms_p / max(2, steps // 20), 3),
                   "speedup": round((ms_p / max(2, steps // 20)) / (ms_b / steps), 2),
                   "batched_gbs": round(2 * n * 4 / (ms_b / steps * 1e-3) / 1e9, 2), "verified": ok,
                   "reduce": red}
        del graph, graph2, x, y
    return res


def bench_cumsum(torch, stream, steps) -> dict:
    """Differentiable cumsum of a 4096 x 8192 f32 N(0,1) tensor through the
    libtorch binding: forward + backward GB/s (2 * B * L * 4 bytes each).

    The headline figure replays the whole step (forward, backward, gradient
    accumulation) as one CUDA graph; an eager step is bound by the host (the
    autograd engine's bookkeeping takes longer than the two scans), so it is
    reported beside it, with torch.cumsum's graph-replayed step for scale."""
    try:
        import ppcumsum

        ext = ppcumsum.load()
    except Exception as e:  # the optional binding needs a torch build toolchain
        return {"unavailable": str(e)[:200]}
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn(4096, 8192, device="cuda", generator=g).requires_grad_(True)
    up = torch.randn(4096, 8192, device="cuda", generator=g)
    nbytes = 2 * (2 * 4096 * 8192 * 4)
    cur = torch.cuda.current_stream()

    def step():
        x.grad = None
        ext.cumsum(x).backward(up)

    def torch_step():
        x.grad = None
        torch.cumsum(x, 1).backward(up)

    def graphed(fn):
        side = torch.cuda.Stream()
        side.wait_stream(cur)
        with torch.cuda.stream(side):
            for _ in range(3):
                fn()
        cur.wait_stream(side)
        gr = torch.cuda.CUDAGraph()
        x.grad = None
        with torch.cuda.graph(gr, stream=side):  # the stream the warm-up sized the library's workspace on
            fn()
        return gr

    eager_ms, _ = time_device(torch, step, steps, 2, cur)
    gr = graphed(step)
    graph_ms, _ = time_device(torch, gr.replay, steps, 2, cur)
    ref = torch.flip(torch.cumsum(torch.flip(up.double(), [1]), 1), [1])
    err = float((x.grad.double() - ref).abs().max())
    del gr
    tgr = graphed(torch_step)
    torch_ms, _ = time_device(torch, tgr.replay, steps, 2, cur)
    del tgr
    rate = lambda ms: round(nbytes * steps / (ms * 1e-3) / 1e9, 2)
    return {"fwd_bwd_gbs": rate(graph_ms), "ms_per_fwd_bwd": round(graph_ms / steps, 4), "step": "one CUDA graph replay",
            "eager_fwd_bwd_gbs": rate(eager_ms), "eager_ms_per_fwd_bwd": round(eager_ms / steps, 4),
            "torch_cumsum_fwd_bwd_gbs_graph": rate(torch_ms), "grad_max_abs_err": err}


# ---------------------------------------------------------------------------------
def load_cpu_reference():
    """The reference's CPU code: the headers compiled against the SYCL shim
    when that library exists for this machine, else the C restatement."""
    sys.path.insert(0, str(ORACLE_DIR))
    import pyoracle

    pyoracle.lib()
    ref = ORACLE_DIR / "_ref" / "libsyclref.so"
    if ref.exists():
        try:
            import ctypes

            lib = ctypes.CDLL(str(ref))
            lib.ref_decoupled_scan_u32_plus.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                                         ctypes.c_int]
            lib.ref_decoupled_scan_u32_plus.restype = ctypes.c_int
            lib.ref_num_groups.restype = ctypes.c_int

            def run(a, out):
                if lib.ref_decoupled_scan_u32_plus(a.ctypes.data, out.ctypes.data, a.size, 0) != 0:
                    raise RuntimeError("reference decoupled scan failed")

            return "reference", run, int(lib.ref_num_groups()), pyoracle
        except (OSError, AttributeError):
            pass

    def run(a, out):
        pyoracle.ref_decoupled_scan(a, "plus", False, threads=0, out=out)

    return "port", run, pyoracle.num_threads(), pyoracle


def cpu_baseline(d_in, h_timed, args) -> dict:
    """The reference's CPU algorithm on the whole headline input, on all host
    cores, repeated for about --cpu-seconds; its output and the GPU's timed
    output are both compared with the oracle's sequential scan."""
    import numpy as np

    kind, run, cores, pyoracle = load_cpu_reference()
    n = d_in.numel()
    a = pyoracle.gen_u32(SEED, n, 0, 1 << 16)
    same_input = bool(np.array_equal(a.view(np.int32), d_in.cpu().numpy()))
    out = np.empty_like(a)
    run(a, out)  # warm
    want = pyoracle.scan(a, "plus")
    ok = bool(np.array_equal(out, want))
    gpu_ok = None if h_timed is None else bool(np.array_equal(h_timed.numpy().view(np.uint32), want))
    reps, t_total = 0, 0.0
    while (t_total < args.cpu_seconds and reps < 200) or reps < 2:
        t0 = time.perf_counter()
        run(a, out)
        t_total += time.perf_counter() - t0
        reps += 1
    gbs = 2 * n * 4 * reps / t_total / 1e9
    return {"value": round(gbs, 3), "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"the whole {n}-element input, {reps} repetitions, {t_total:.1f} s",
            "matches_oracle": ok, "same_input_as_gpu": same_input, "gpu_output_matches_oracle": gpu_ok}


def run_reference(args) -> dict | None:
    import numpy as np

    ws, rank, _ = dist_info()
    if rank != 0:
        return None
    kind, run, cores, pyoracle = load_cpu_reference()
    n = args.n  # the whole workload every step: the GPU arm's configuration
    a = pyoracle.gen_u32(SEED, n, 0, 1 << 16)
    out = np.empty_like(a)
    for _ in range(args.warmup):
        run(a, out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run(a, out)
    dt = time.perf_counter() - t0
    ok = bool(np.array_equal(out, pyoracle.scan(a, "plus")))
    value = 2 * n * 4 * args.steps / dt / 1e9
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 3),
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3 / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic: seeded uniform [0, 2^16) uint32 (splitmix64)",
        "config": {
            "workload": "decoupled look-back inclusive plus-scan, n=2^30 uint32 U[0,2^16)",
            "n": n,
            "sample_per_step": n,
        },
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"the whole {n}-element input every step", "matches_oracle": ok},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_profile_cases(args) -> dict:
    """One launch of every kernel of the path on inputs larger than L2 (a few
    hundred MB each, about 3 GB in total), no timing: the command the ncu
    captures in profiles/ run. Prints the case order."""
    import torch

    import ppbuild

    ppbuild.build()
    import ppgb300 as pp

    pp.lib()
    sh = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda").manual_seed(SEED)
    n = 1 << 26  # 256 MiB of 4-byte elements
    u = torch.randint(0, 1 << 16, (n,), dtype=torch.int32, device="cuda", generator=g)
    f = torch.randn(n, dtype=torch.float32, device="cuda", generator=g)
    o = torch.empty_like(u)
    w = torch.randint(0, 1 << 32, (n // 2,), dtype=torch.int64, device="cuda", generator=g)
    ow = torch.empty_like(w)
    res = torch.empty(4, dtype=torch.float64, device="cuda")
    cases = []

    def case(name, fn):
        fn()
        torch.cuda.synchronize()
        if pp.stream_status(sh) != 0:
            raise RuntimeError(f"device error in profile case {name}")
        cases.append(name)

    case("u32 inclusive plus 2^26", lambda: pp.decoupled_scan_device("inclusive", "plus", u.data_ptr(), o.data_ptr(),
                                                                       n, "u32", stream=sh))
    case("u32 exclusive plus 2^26", lambda: pp.decoupled_scan_device("exclusive", "plus", u.data_ptr(), o.data_ptr(),
                                                                       n, "u32", stream=sh))
    case("i32 inclusive maximum 2^26", lambda: pp.decoupled_scan_device("inclusive", "maximum", u.data_ptr(),
                                                                          o.data_ptr(), n, "i32", stream=sh))
    case("u64 inclusive plus 2^25", lambda: pp.decoupled_scan_device("inclusive", "plus", w.data_ptr(), ow.data_ptr(),
                                                                       n // 2, "u64", stream=sh))
    for prec in ("default", "compensated", "fp64_carry"):
        case(f"f32 inclusive plus {prec} 2^26",
             lambda p=prec: pp.scan("inclusive", "plus", f.data_ptr(), o.data_ptr(), n, "f32", stream=sh, precision=p))
    case("u32 cooperative inclusive plus 2^26", lambda: pp.cooperative_scan_device("inclusive", "plus", u.data_ptr(),
                                                                                   o.data_ptr(), n, "u32", stream=sh))
    case("f32 sum reduce 2^26", lambda: pp.reduce("plus", f.data_ptr(), n, "f32", res.data_ptr(), stream=sh))
    case("u64 sum reduce 2^25", lambda: pp.reduce("plus", w.data_ptr(), n // 2, "u64", res.data_ptr(), stream=sh))
    segs = 65536  # log-uniform lengths in [1, 2^13]: about 60 M elements (240 MB), twice the L2
    gc = torch.Generator(device="cpu").manual_seed(0x5EC)
    lens = torch.floor(torch.exp(torch.rand(segs, generator=gc, dtype=torch.float64) * math.log(2 ** 13)))
    offs = torch.zeros(segs + 1, dtype=torch.int64)
    offs[1:] = torch.cumsum(lens.clamp(1, 2 ** 13).to(torch.int64), 0)
    ns = int(offs[-1])
    d_off = offs.cuda()
    case(f"i32 segmented plus scan {segs} segments {ns} elements",
         lambda: pp.segmented_scan("inclusive", "plus", u.data_ptr(), o.data_ptr(), ns, d_off.data_ptr(), segs, "i32",
                                   stream=sh))
    seg_out = torch.empty(segs, dtype=torch.int32, device="cuda")
    case(f"i32 segmented plus reduce {segs} segments",
         lambda: pp.segmented_reduce("plus", u.data_ptr(), ns, d_off.data_ptr(), segs, seg_out.data_ptr(), "i32",
                                     stream=sh))
    case("f32 row scans 8192 x 8192 forward", lambda: pp.rows_scan("inclusive", "plus", f.data_ptr(), o.data_ptr(),
                                                                     8192, 8192, "f32", stream=sh))
    case("f32 row scans 8192 x 8192 reverse", lambda: pp.rows_scan("inclusive", "plus", f.data_ptr(), o.data_ptr(),
                                                                     8192, 8192, "f32", reverse=True, stream=sh))
    case("device copy 256 MiB (torch, reference point)", lambda: o.copy_(u))
    return {"profile_cases": cases}


def run_profile_segmented(args) -> dict:
    """The batched benchmark's segments (65,536 log-uniform lengths, 385 M
    int32 elements): three segmented reductions, then three segmented scans,
    no timing: the command of the launch-list capture in profiles/."""
    import torch

    import ppbuild

    ppbuild.build()
    import ppgb300 as pp

    pp.lib()
    sh = torch.cuda.current_stream().cuda_stream
    S = 65536
    g = torch.Generator(device="cpu").manual_seed(0x5EC)
    lens = torch.floor(torch.exp(torch.rand(S, generator=g, dtype=torch.float64) * math.log(2 ** 16)))
    offs = torch.zeros(S + 1, dtype=torch.int64)
    offs[1:] = torch.cumsum(lens.clamp(1, 2 ** 16).to(torch.int64), 0)
    n = int(offs[-1])
    d_off = offs.cuda()
    x = splitmix_u32(torch, SEED + 4, n, 0, 1000, "cuda")
    y = torch.empty_like(x)
    tot = torch.empty(S, dtype=torch.int32, device="cuda")
    for _ in range(3):
        pp.segmented_reduce("plus", x.data_ptr(), n, d_off.data_ptr(), S, tot.data_ptr(), "i32", stream=sh)
    for _ in range(3):
        pp.segmented_scan("inclusive", "plus", x.data_ptr(), y.data_ptr(), n, d_off.data_ptr(), S, "i32", stream=sh)
    torch.cuda.synchronize()
    if pp.stream_status(sh) != 0:
        raise RuntimeError("device error in the segmented profile case")
    ok = check_segmented_reduce(torch, x, tot, d_off) and check_segmented_scan(torch, x, y, d_off)
    return {"profile_segmented": {"segments": S, "elements": n, "verified": bool(ok)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_HEADLINE)
    ap.add_argument("--e2e-steps", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-cases", action="store_true",
                    help="run each kernel of the path once on a small case (the ncu capture command)")
    ap.add_argument("--profile-segmented", action="store_true",
                    help="three segmented reductions and scans of the batched benchmark's segments, untimed")
    args = ap.parse_args()
    if args.profile_cases:
        print(json.dumps(run_profile_cases(args)), flush=True)
        return
    if args.profile_segmented:
        print(json.dumps(run_profile_segmented(args)), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    res = run_reference(args) if args.impl == "reference" else run_ours(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
