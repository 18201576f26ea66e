// Cooperative grid-barrier scan for sm_103a.
//
// Re-design of parallel_primitives::internal::scan_cooperative_device
// (include/parallel_primitives/scan_cooperative.hpp:35-91) and of its software
// grid barrier nd_range_barrier (include/cooperative_groups.hpp:26-147).
//
// The reference scans each group's chunk into the output, crosses a grid
// barrier, lets every group fold the tails of all earlier chunks serially
// (an O(G) fan per group), crosses a second barrier and re-reads and
// re-writes the whole output to add the carry: about 4n memory traffic and a
// 64-group limit (cooperative_groups.hpp:66-68).
//
// Element types whose size divides 16 bytes take the staged kernel of
// decoupled_scan.cuh in cooperative rounds (CO = 1): the input streams
// through L2 in windows of about 20 MB; each CTA reduces its run of window w
// (first read, from HBM), publishes the run aggregate at window barrier w,
// and scans its run of window w - 1 (second read, from L2) with the prefix of
// all earlier runs: 2n HBM traffic, one split-phase grid barrier per window.
//
// This file holds the register-tile kernel for the other element types: one
// cooperative launch (all blocks co-resident, checked with the occupancy
// calculator before the launch) runs:
//   1. each block reduces its contiguous run of tiles in sequence order and
//      publishes the run aggregate;
//   2. a bounded-spin grid barrier;
//   3. each block folds the aggregates of the blocks before it (32 per warp
//      step, ordered shuffle reduction);
//   4. each block re-reads its run tile by tile and scans it in registers
//      (thread-serial 16-byte chunks + shuffle Kogge-Stone across lanes +
//      shared-memory scan across warps, the radix-N Kogge-Stone structure of
//      the reference's group scans) carrying the running prefix, and writes the
//      output once.
// Traffic is 3n instead of 4n, and any grid the device can hold co-resident
// is allowed.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "decoupled_scan.cuh"
#include "workspace.cuh"

namespace pp {

// Bounded-spin grid barrier over all blocks of a co-resident launch. Thread 0
// of each block arrives; the last arrival re-arms the counter and advances the
// generation. Returns false (in every thread of the block) if the wait timed
// out or another block aborted.
__device__ __forceinline__ bool grid_barrier(WsHeader* h, uint64_t timeout_ns) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    const uint32_t gen = ptx::ld_acquire(reinterpret_cast<const uint32_t*>(&h->bar_gen));
    __threadfence();
    const unsigned arrived = atomicAdd(&h->bar_count, 1u) + 1u;
    if (arrived == gridDim.x) {
      h->bar_count = 0u;
      __threadfence();
      ptx::st_release(reinterpret_cast<uint32_t*>(&h->bar_gen), gen + 1u);
    } else {
      const uint64_t t0 = ptx::globaltimer_ns();
      uint32_t it = 0;
      while (ptx::ld_acquire(reinterpret_cast<const uint32_t*>(&h->bar_gen)) == gen) {
        if ((++it & 15u) == 0u) {
          const uint64_t waited = ptx::globaltimer_ns() - t0;
          if (waited > kAbortCheckAfterNs && aborted(h)) {
            ok = 0;
            break;
          }
          if (waited > timeout_ns) {
            raise_error(h, kDevTimeout, ~0ull);
            ok = 0;
            break;
          }
        }
      }
    }
  }
  return __syncthreads_and(ok) != 0;
}

struct CoopArgs {
  ScanArgs s;
  void* block_aggs;  // gridDim.x carries (16-byte slots)
};

template <class Pol, int NC, int CH>
struct CoopCfg {
  using in_t = typename Pol::in_t;
  static constexpr int V = (16 % sizeof(in_t) == 0) ? int(16 / sizeof(in_t)) : 1;
  static constexpr int WARP_ELEMS = 32 * CH * V;
  static constexpr int TILE = NC * WARP_ELEMS;
  static constexpr int THREADS = NC * 32;
};

template <class Pol, int NC, int CH, int V>
__device__ __forceinline__ void coop_load_tile(const Pol& pol, const typename Pol::in_t* gin, uint64_t base,
                                               int valid, int cw, int lane, bool vec_ok,
                                               typename Pol::acc_t (&a)[CH][V]) {
  using in_t = typename Pol::in_t;
  constexpr int WARP_ELEMS = 32 * CH * V;
#pragma unroll
  for (int c = 0; c < CH; ++c) {
    const int e0 = cw * WARP_ELEMS + (c * 32 + lane) * V;
    if (vec_ok && e0 + V <= valid) {
      union {
        uint4 u;
        in_t x[V];
      } buf;
      buf.u = ptx::ld_stream_v4(gin + base + e0);
#pragma unroll
      for (int j = 0; j < V; ++j) a[c][j] = pol.load(buf.x[j]);
    } else {
#pragma unroll
      for (int j = 0; j < V; ++j) a[c][j] = (e0 + j < valid) ? pol.load(gin[base + e0 + j]) : pol.aid();
    }
  }
}

template <class Pol, int NC, int CH>
__global__ void __launch_bounds__(NC * 32) cooperative_scan_kernel(const CoopArgs cargs) {
  using Cfg = CoopCfg<Pol, NC, CH>;
  using in_t = typename Pol::in_t;
  using out_t = typename Pol::out_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  using pre_t = typename Pol::pre_t;
  constexpr int V = Cfg::V;
  constexpr int TILE = Cfg::TILE;
  using TS = TileScan<Pol, NC, CH, V>;
  static_assert(sizeof(carry_t) <= 16, "carry slots hold at most 16 bytes");

  __shared__ acc_t s_wtot[2][NC];
  __shared__ carry_t s_carry;

  const ScanArgs& args = cargs.s;
  // the workspace epoch at the start, for the exit re-arm (read early, used last)
  const uint32_t epoch0 = ptx::ld_relaxed(reinterpret_cast<const uint32_t*>(&args.hdr->epoch));
  const Pol pol{};
  const int cw = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t n = args.n;
  const in_t* gin = static_cast<const in_t*>(args.in);
  out_t* gout = static_cast<out_t*>(args.out);
  const bool vec_in = V > 1 && (reinterpret_cast<uintptr_t>(gin) & 15u) == 0;
  const bool vec_out = V > 1 && (reinterpret_cast<uintptr_t>(gout) & 15u) == 0;
  auto aop = [&](const acc_t& x, const acc_t& y) { return pol.aop(x, y); };
  auto cop = [&](const carry_t& x, const carry_t& y) { return pol.cop(x, y); };

  // contiguous run of tiles for this block (first ntiles % G blocks get one more,
  // as get_group_work_size / get_cumulative_work_size, internal/common.h:74-86)
  const uint64_t ntiles = (n + TILE - 1) / TILE;
  const uint64_t G = gridDim.x, b = blockIdx.x;
  const uint64_t q = ntiles / G, r = ntiles % G;
  const uint64_t t_begin = b * q + (b < r ? b : r);
  const uint64_t t_end = t_begin + q + (b < r ? 1 : 0);

  // ---- phase 1: ordered aggregate of the run --------------------------------
  carry_t run = pol.cid();
  for (uint64_t t = t_begin; t < t_end; ++t) {
    const uint64_t base = t * TILE;
    const int valid = (n - base < uint64_t(TILE)) ? int(n - base) : TILE;
    acc_t a[CH][V];
    coop_load_tile<Pol, NC, CH, V>(pol, gin, base, valid, cw, lane, vec_in, a);
    acc_t pre_lane[CH];
    const acc_t wagg = TS::warp_part(pol, a, pre_lane, lane);
    if (lane == 0) s_wtot[t & 1][cw] = wagg;
    __syncthreads();
    acc_t x = lane < NC ? s_wtot[t & 1][lane] : pol.aid();
    x = warp_inclusive_scan(x, aop, lane);
    run = pol.cop(run, pol.to_carry(shfl_idx(x, NC - 1)));
  }
  carry_t* aggs = static_cast<carry_t*>(cargs.block_aggs);
  constexpr int CSTRIDE = int(16 / sizeof(carry_t)) > 0 ? int(16 / sizeof(carry_t)) : 1;
  if (threadIdx.x == 0) aggs[b * CSTRIDE] = run;
  __threadfence();

  // ---- phase 2: grid barrier ------------------------------------------------
  const bool ok = grid_barrier(args.hdr, args.timeout_ns);

  if (ok) {
    // ---- phase 3: fold the aggregates of earlier blocks (warp 0) -----------
    if (cw == 0) {
      carry_t pref = pol.cid();
      for (uint64_t b0 = 0; b0 < b; b0 += 32) {
        const uint64_t i = b0 + lane;
        carry_t v = pol.cid();
        if (i < b) {
          words<carry_t> w;
          const volatile uint32_t* p = reinterpret_cast<const volatile uint32_t*>(aggs + i * CSTRIDE);
#pragma unroll
          for (int k = 0; k < words<carry_t>::W; ++k) w.w[k] = p[k];
          v = from_words<carry_t>(w);
        }
        pref = pol.cop(pref, warp_reduce(v, cop, lane));
      }
      if (lane == 0) s_carry = pref;
    }
    __syncthreads();
    carry_t carry = s_carry;

    // ---- phase 4: scan the run with the carried prefix ----------------------
    const bool excl = args.exclusive != 0;
    for (uint64_t t = t_begin; t < t_end; ++t) {
      const uint64_t base = t * TILE;
      const int valid = (n - base < uint64_t(TILE)) ? int(n - base) : TILE;
      acc_t a[CH][V];
      coop_load_tile<Pol, NC, CH, V>(pol, gin, base, valid, cw, lane, vec_in, a);
      acc_t pre_lane[CH];
      const acc_t wagg = TS::warp_part(pol, a, pre_lane, lane);
      if (lane == 0) s_wtot[t & 1][cw] = wagg;
      __syncthreads();
      // every warp scans the warp totals itself: no second barrier
      acc_t x = lane < NC ? s_wtot[t & 1][lane] : pol.aid();
      x = warp_inclusive_scan(x, aop, lane);
      acc_t wex = shfl_up(x, 1);
      if (lane == 0) wex = pol.aid();
      const acc_t my_wex = shfl_idx(wex, cw);
      const acc_t tagg = shfl_idx(x, NC - 1);
      const pre_t pw = pol.prepare(pol.cop(carry, pol.to_carry(my_wex)));
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int e0 = cw * Cfg::WARP_ELEMS + (c * 32 + lane) * V;
        const pre_t pc = pol.extend(pw, pre_lane[c]);
        union {
          uint4 u;
          out_t x[V];
        } o;
        TS::finish_chunk(pol, pc, a[c], excl, o.x);
        if constexpr (V > 1) {
          if (vec_out && e0 + V <= valid) {
            ptx::st_stream_v4(gout + base + e0, o.u);
            continue;
          }
        }
#pragma unroll
        for (int j = 0; j < V; ++j)
          if (e0 + j < valid) gout[base + e0 + j] = o.x[j];
      }
      carry = pol.cop(carry, pol.to_carry(tagg));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) cta_exit_rearm(args.hdr, args.desc, 0, epoch0);
}

}  // namespace pp
