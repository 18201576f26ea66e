// Single-pass decoupled look-back prefix scan for sm_103a.
//
// Re-design of parallel_primitives::internal::scan_decoupled_device and its
// kernel (include/parallel_primitives/scan_decoupled_lookback.hpp:106-182):
//
//  * Tiles are handed out by an atomic ticket counter (not by block id), so
//    every predecessor of a tile belongs to a CTA that is already running:
//    forward progress holds for any grid size and residency.
//  * DecoupledTmaKernel: a persistent, warp-specialised kernel. Warp 0 is the
//    producer: one lane takes tickets and streams whole tiles into a ring of
//    shared-memory stages with cp.async.bulk (TMA, completion on mbarriers).
//    The other NC warps consume: 16-byte conflict-free shared loads, a
//    register scan (thread-serial inside each 16-byte chunk, shuffle
//    Kogge-Stone across lanes, shared-memory scan across warps), then
//    coalesced 16-byte streaming stores.
//  * DecoupledGenericKernel: the same algorithm with plain element loads for
//    any alignment and any element type (user functors, packed structs).
//  * Strategy choice of the reference (:143-174): consumer warp 0 peeks at the
//    predecessor's descriptor when the tile arrives. If the predecessor's
//    inclusive prefix is already there ("reduce-then-scan"), the tile
//    publishes its own inclusive prefix straight away and skips the
//    look-back. Otherwise ("scan-then-reduce") it publishes its aggregate,
//    runs the look-back and then publishes the prefix.
//  * The look-back is warp-wide: 32 predecessors per step, the nearest
//    inclusive prefix found with a ballot, the window folded with an ordered
//    shuffle reduction (the reference walks one predecessor at a time on one
//    work-item, partition_descriptor.h:115-130).
//  * Every wait is bounded by %globaltimer; a timeout records an error in the
//    workspace header and makes every CTA leave its loop.
//  * Combine order is prefix op local everywhere, so associative operators
//    that are not commutative scan correctly (the reference combines
//    op(aggregate, prefix), :157,170, and op(local, prefix), :98).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "scan_policy.cuh"
#include "workspace.cuh"

namespace pp {

struct ScanArgs {
  const void* in;
  void* out;
  uint64_t n;
  WsHeader* hdr;
  uint64_t* desc;
  uint64_t timeout_ns;
  long long debug_skip_tile;  // a tile that never publishes (timeout tests); -1 = off
  int exclusive;
};

__host__ __device__ constexpr size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Warp-wide look-back for `tile`. On success writes the combination of the
// aggregates/prefix of all tiles before `tile` (in sequence order) to `out`.
template <class Pol>
__device__ __forceinline__ bool lookback_warp(const Pol& pol, const uint64_t* desc, long long tile,
                                              uint32_t etag, WsHeader* hdr, uint64_t timeout_ns, int lane,
                                              typename Pol::carry_t& out) {
  using C = typename Pol::carry_t;
  using codec = desc_codec<C>;
  C acc = pol.cid();
  long long base = tile - 1;
  uint32_t spins = 0;
  uint64_t t0 = 0;
  while (true) {
    const long long t = base - lane;
    C v = pol.cid();
    uint32_t st = kPrefix;  // before tile 0: the identity prefix
    if (t >= 0) st = codec::read(desc + t * codec::W, etag, v);
    const uint32_t pm = __ballot_sync(kFullMask, st == kPrefix);
    const uint32_t xm = __ballot_sync(kFullMask, st == kInvalid);
    const int p = pm ? (__ffs(pm) - 1) : 32;
    const uint32_t need = (p >= 31) ? kFullMask : ((2u << p) - 1u);
    if (xm & need) {
      // some predecessor up to the nearest prefix has not published yet
      if (spins == 0) t0 = ptx::globaltimer_ns();
      ++spins;
      if ((spins & 7u) == 0u) {
        bool give_up = false;
        if (lane == 0) {
          if (aborted(hdr)) {
            give_up = true;
          } else if (ptx::globaltimer_ns() - t0 > timeout_ns) {
            raise_error(hdr, kDevTimeout, (unsigned long long)tile);
            give_up = true;
          }
        }
        if (__shfl_sync(kFullMask, give_up, 0)) return false;
      }
      continue;
    }
    spins = 0;
    C w = (lane <= p) ? v : pol.cid();
    w = warp_reduce_reversed(w, [&](const C& x, const C& y) { return pol.cop(x, y); }, lane);
    acc = pol.cop(w, acc);
    if (p < 32) break;
    base -= 32;
  }
  out = acc;
  return true;
}

// Shared per-tile machinery of both kernels. `a[c][j]` holds the loaded
// accumulators of chunk c (V consecutive elements). Computes the in-warp
// prefixes, then consumer warp 0 resolves the tile prefix.
template <class Pol, int NC, int CH, int V>
struct TileScan {
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  using pre_t = typename Pol::pre_t;
  using codec = desc_codec<carry_t>;

  // Thread-serial scan of each chunk, then Kogge-Stone across lanes.
  // pre_lane[c] = warp-local exclusive prefix of chunk c of this lane.
  __device__ __forceinline__ static acc_t warp_part(const Pol& pol, acc_t (&a)[CH][V], acc_t (&pre_lane)[CH],
                                                    int lane) {
    auto aop = [&](const acc_t& x, const acc_t& y) { return pol.aop(x, y); };
    acc_t inc[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) {
#pragma unroll
      for (int j = 1; j < V; ++j) a[c][j] = pol.aop(a[c][j - 1], a[c][j]);
      inc[c] = a[c][V - 1];
    }
#pragma unroll
    for (int c = 0; c < CH; ++c) inc[c] = warp_inclusive_scan(inc[c], aop, lane);
    acc_t X = pol.aid();
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      acc_t ex = shfl_up(inc[c], 1);
      if (lane == 0) ex = pol.aid();
      pre_lane[c] = (c == 0) ? ex : pol.aop(X, ex);
      const acc_t ct = shfl_idx(inc[c], 31);
      X = (c == 0) ? ct : pol.aop(X, ct);
    }
    return X;
  }

  // Consumer warp 0: scan the warp totals, publish, look back. Writes the
  // per-warp carried prefixes to s_wpref and the abort flag to *s_flag.
  __device__ __forceinline__ static void resolve(const Pol& pol, const ScanArgs& args, long long tile,
                                                 uint32_t etag, const acc_t* s_wtot, carry_t* s_wpref,
                                                 int* s_flag, uint32_t peek_st, const carry_t& peek_v,
                                                 int lane) {
    auto aop = [&](const acc_t& x, const acc_t& y) { return pol.aop(x, y); };
    acc_t wt = (lane < NC) ? s_wtot[lane] : pol.aid();
    acc_t winc = warp_inclusive_scan(wt, aop, lane);
    acc_t wex = shfl_up(winc, 1);
    if (lane == 0) wex = pol.aid();
    const carry_t agg = pol.to_carry(shfl_idx(winc, NC - 1));
    uint64_t* d = args.desc + tile * codec::W;
    const bool publish = tile != args.debug_skip_tile;
    carry_t excl = pol.cid();
    bool ok = true;
    if (tile == 0) {
      if (lane == 0 && publish) codec::publish(d, agg, make_tag(etag, kPrefix));
    } else if (__shfl_sync(kFullMask, peek_st, 0) == kPrefix) {
      // reduce-then-scan: predecessor prefix known on arrival
      excl = shfl_idx(peek_v, 0);
      if (lane == 0 && publish) codec::publish(d, pol.cop(excl, agg), make_tag(etag, kPrefix));
    } else {
      // scan-then-reduce: publish the aggregate, then look back
      if (lane == 0 && publish) codec::publish(d, agg, make_tag(etag, kAggregate));
      ok = lookback_warp(pol, args.desc, tile, etag, args.hdr, args.timeout_ns, lane, excl);
      if (ok && lane == 0 && publish) codec::publish(d, pol.cop(excl, agg), make_tag(etag, kPrefix));
    }
    if (lane < NC) s_wpref[lane] = pol.cop(excl, pol.to_carry(wex));
    if (lane == 0) *s_flag = ok ? 0 : 1;
  }

  // Finishes chunk c of this thread into V outputs.
  __device__ __forceinline__ static void finish_chunk(const Pol& pol, const pre_t& pc, const acc_t (&ac)[V],
                                                      bool exclusive, typename Pol::out_t (&o)[V]) {
    if (exclusive) {
      o[0] = pol.finish_first(pc);
#pragma unroll
      for (int j = 1; j < V; ++j) o[j] = pol.finish(pc, ac[j - 1]);
    } else {
#pragma unroll
      for (int j = 0; j < V; ++j) o[j] = pol.finish(pc, ac[j]);
    }
  }
};

template <class Pol, int NC_, int CH_, int STAGES_>
struct DecoupledTmaCfg {
  using in_t = typename Pol::in_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  static constexpr int NC = NC_;
  static constexpr int CH = CH_;
  static constexpr int STAGES = STAGES_;
  static_assert(16 % sizeof(in_t) == 0, "TMA path needs element sizes dividing 16 bytes");
  static constexpr int V = 16 / sizeof(in_t);
  static constexpr int WARP_ELEMS = 32 * CH * V;
  static constexpr int TILE = NC * WARP_ELEMS;
  static constexpr int TILE_BYTES = TILE * int(sizeof(in_t));
  static constexpr int THREADS = (NC + 1) * 32;
  static constexpr size_t OFF_BAR = size_t(STAGES) * TILE_BYTES;
  static constexpr size_t OFF_TILE = OFF_BAR + 2 * STAGES * 8;
  static constexpr size_t OFF_WTOT = align_up(OFF_TILE + STAGES * 8, 16);
  static constexpr size_t OFF_WPREF = align_up(OFF_WTOT + NC * sizeof(acc_t), 16);
  static constexpr size_t OFF_FLAG = align_up(OFF_WPREF + NC * sizeof(carry_t), 16);
  static constexpr size_t SMEM = OFF_FLAG + 16;
  static_assert(NC <= 32, "at most 32 consumer warps");
};

template <class Pol, int NC, int CH, int STAGES>
__global__ void __launch_bounds__((NC + 1) * 32)
    decoupled_tma_kernel(const ScanArgs args) {
  using Cfg = DecoupledTmaCfg<Pol, NC, CH, STAGES>;
  using in_t = typename Pol::in_t;
  using out_t = typename Pol::out_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  using pre_t = typename Pol::pre_t;
  using TS = TileScan<Pol, NC, CH, Cfg::V>;
  constexpr int V = Cfg::V;
  constexpr int TILE = Cfg::TILE;
  static_assert(sizeof(out_t) == sizeof(in_t), "in/out element sizes must match");

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Cfg::OFF_BAR);
  uint64_t* empty = full + STAGES;
  long long* s_tile = reinterpret_cast<long long*>(smem + Cfg::OFF_TILE);
  acc_t* s_wtot = reinterpret_cast<acc_t*>(smem + Cfg::OFF_WTOT);
  carry_t* s_wpref = reinterpret_cast<carry_t*>(smem + Cfg::OFF_WPREF);
  int* s_flag = reinterpret_cast<int*>(smem + Cfg::OFF_FLAG);

  const Pol pol{};
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t n = args.n;
  const long long ntiles = (long long)((n + TILE - 1) / TILE);
  WsHeader* hdr = args.hdr;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], NC);
    }
    ptx::fence_mbar_init();
  }
  __syncthreads();

  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      const uint64_t pol_l2 = ptx::policy_evict_first();
      const unsigned char* in = static_cast<const unsigned char*>(args.in);
      uint32_t pending = 0;  // stages whose last copy may still be in flight
      uint32_t pend_par = 0;
      long long t = (long long)atomicAdd(&hdr->ticket, 1ull);
      for (int k = 0;; ++k) {
        const int s = k % STAGES;
        if (k >= STAGES) {
          if (!mbar_wait_bounded(&empty[s], ((k / STAGES) - 1) & 1, hdr, args.timeout_ns, (unsigned long long)t))
            break;
          pending &= ~(1u << s);
        }
        s_tile[s] = t;
        if (t < ntiles) {
          const uint64_t base = uint64_t(t) * TILE;
          const uint64_t valid = (n - base < uint64_t(TILE)) ? (n - base) : uint64_t(TILE);
          const uint32_t bytes = uint32_t(valid * sizeof(in_t)) & ~15u;
          if (bytes) {
            ptx::mbar_arrive_expect_tx(&full[s], bytes);
            ptx::bulk_g2s(smem + size_t(s) * Cfg::TILE_BYTES, in + base * sizeof(in_t), bytes, &full[s], pol_l2);
            pending |= 1u << s;
            pend_par = (pend_par & ~(1u << s)) | ((uint32_t(k / STAGES) & 1u) << s);
          } else {
            ptx::mbar_arrive(&full[s]);
          }
          t = (long long)atomicAdd(&hdr->ticket, 1ull);
        } else {
          ptx::mbar_arrive(&full[s]);
          break;
        }
      }
      // never leave with a bulk copy still writing into this CTA's shared memory
      for (int s = 0; s < STAGES; ++s)
        if (pending & (1u << s)) mbar_wait_bounded(&full[s], (pend_par >> s) & 1u, hdr, args.timeout_ns, 0ull);
    }
    __syncwarp();
  } else {
    // ---------------- consumers ----------------
    const int cw = warp - 1;
    const uint32_t etag = ptx::ld_relaxed(reinterpret_cast<const uint32_t*>(&hdr->epoch)) + 1u;
    const in_t* gin = static_cast<const in_t*>(args.in);
    out_t* gout = static_cast<out_t*>(args.out);
    for (int k = 0;; ++k) {
      const int s = k % STAGES;
      // A warp whose wait gave up (timeout / abort) and the end-of-work
      // sentinel both make the warp inactive; the OR-vote at the first named
      // barrier lets every consumer warp leave the loop together.
      const bool got = mbar_wait_bounded(&full[s], (k / STAGES) & 1, hdr, args.timeout_ns, 0ull);
      const long long tile = got ? s_tile[s] : ntiles;
      const bool active = tile < ntiles;

      uint32_t peek_st = kInvalid;
      carry_t peek_v = pol.cid();
      const uint64_t base = uint64_t(active ? tile : 0) * TILE;
      const uint64_t rem = n - base;
      const int valid = rem < uint64_t(TILE) ? int(rem) : TILE;
      acc_t a[CH][V];
      acc_t pre_lane[CH];
      if (active) {
        if (cw == 0 && lane == 0 && tile > 0)
          peek_st = TS::codec::read(args.desc + (tile - 1) * TS::codec::W, etag, peek_v);
        const int bulk_elems = int((uint32_t(valid * sizeof(in_t)) & ~15u) / sizeof(in_t));
        const unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
#pragma unroll
        for (int c = 0; c < CH; ++c) {
          const int e0 = cw * Cfg::WARP_ELEMS + (c * 32 + lane) * V;
          if (e0 + V <= bulk_elems) {
            union {
              uint4 u;
              in_t x[V];
            } buf;
            buf.u = *reinterpret_cast<const uint4*>(stage + size_t(e0) * sizeof(in_t));
#pragma unroll
            for (int j = 0; j < V; ++j) a[c][j] = pol.load(buf.x[j]);
          } else {
#pragma unroll
            for (int j = 0; j < V; ++j) {
              const int e = e0 + j;
              if (e < bulk_elems)
                a[c][j] = pol.load(reinterpret_cast<const in_t*>(stage)[e]);
              else if (e < valid)
                a[c][j] = pol.load(gin[base + e]);
              else
                a[c][j] = pol.aid();
            }
          }
        }
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&empty[s]);  // stage may be refilled

        const acc_t wagg = TS::warp_part(pol, a, pre_lane, lane);
        if (lane == 0) s_wtot[cw] = wagg;
      }
      if (ptx::named_sync_or(1, NC * 32, !active)) break;
      if (cw == 0) TS::resolve(pol, args, tile, etag, s_wtot, s_wpref, s_flag, peek_st, peek_v, lane);
      ptx::named_sync(1, NC * 32);
      if (*s_flag) break;

      const pre_t pw = pol.prepare(s_wpref[cw]);
      const bool excl = args.exclusive != 0;
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int e0 = cw * Cfg::WARP_ELEMS + (c * 32 + lane) * V;
        const pre_t pc = pol.extend(pw, pre_lane[c]);
        union {
          uint4 u;
          out_t x[V];
        } o;
        TS::finish_chunk(pol, pc, a[c], excl, o.x);
        if (e0 + V <= valid) {
          ptx::st_stream_v4(gout + base + e0, o.u);
        } else {
#pragma unroll
          for (int j = 0; j < V; ++j)
            if (e0 + j < valid) gout[base + e0 + j] = o.x[j];
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) cta_exit_rearm(hdr, args.desc, uint64_t(ntiles) * TS::codec::W);
}

// ---------------------------------------------------------------------------
// Generic variant: element loads from global memory (any alignment, any T).
template <class Pol, int NC_, int IPT_>
struct DecoupledGenericCfg {
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  static constexpr int NC = NC_;
  static constexpr int CH = IPT_;
  static constexpr int V = 1;
  static constexpr int WARP_ELEMS = 32 * CH;
  static constexpr int TILE = NC * WARP_ELEMS;
  static constexpr int THREADS = NC * 32;
  static constexpr size_t OFF_WTOT = 16;
  static constexpr size_t OFF_WPREF = align_up(OFF_WTOT + NC * sizeof(acc_t), 16);
  static constexpr size_t OFF_FLAG = align_up(OFF_WPREF + NC * sizeof(carry_t), 16);
  static constexpr size_t SMEM = OFF_FLAG + 16;
};

template <class Pol, int NC, int IPT>
__global__ void __launch_bounds__(NC * 32) decoupled_generic_kernel(const ScanArgs args) {
  using Cfg = DecoupledGenericCfg<Pol, NC, IPT>;
  using in_t = typename Pol::in_t;
  using out_t = typename Pol::out_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  using pre_t = typename Pol::pre_t;
  constexpr int CH = IPT;
  constexpr int TILE = Cfg::TILE;
  using TS = TileScan<Pol, NC, CH, 1>;

  __shared__ __align__(16) unsigned char smem[Cfg::SMEM];
  long long* s_tile = reinterpret_cast<long long*>(smem);  // two ticket slots
  acc_t* s_wtot = reinterpret_cast<acc_t*>(smem + Cfg::OFF_WTOT);
  carry_t* s_wpref = reinterpret_cast<carry_t*>(smem + Cfg::OFF_WPREF);
  int* s_flag = reinterpret_cast<int*>(smem + Cfg::OFF_FLAG);

  const Pol pol{};
  const int cw = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t n = args.n;
  const long long ntiles = (long long)((n + TILE - 1) / TILE);
  WsHeader* hdr = args.hdr;
  const in_t* gin = static_cast<const in_t*>(args.in);
  out_t* gout = static_cast<out_t*>(args.out);

  if (threadIdx.x == 0) s_tile[0] = (long long)atomicAdd(&hdr->ticket, 1ull);
  __syncthreads();
  const uint32_t etag = ptx::ld_relaxed(reinterpret_cast<const uint32_t*>(&hdr->epoch)) + 1u;

  for (int k = 0;; ++k) {
    const long long tile = s_tile[k & 1];
    if (tile >= ntiles) break;
    long long next = 0;
    uint32_t peek_st = kInvalid;
    carry_t peek_v = pol.cid();
    if (cw == 0 && lane == 0) {
      next = (long long)atomicAdd(&hdr->ticket, 1ull);
      if (tile > 0) peek_st = TS::codec::read(args.desc + (tile - 1) * TS::codec::W, etag, peek_v);
    }
    const uint64_t base = uint64_t(tile) * TILE;
    const uint64_t rem = n - base;
    const int valid = rem < uint64_t(TILE) ? int(rem) : TILE;

    acc_t a[CH][1];
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int e = cw * Cfg::WARP_ELEMS + c * 32 + lane;
      a[c][0] = (e < valid) ? pol.load(gin[base + e]) : pol.aid();
    }
    acc_t pre_lane[CH];
    const acc_t wagg = TS::warp_part(pol, a, pre_lane, lane);
    if (lane == 0) s_wtot[cw] = wagg;
    ptx::named_sync(1, NC * 32);
    if (cw == 0) {
      TS::resolve(pol, args, tile, etag, s_wtot, s_wpref, s_flag, peek_st, peek_v, lane);
      if (lane == 0) s_tile[(k + 1) & 1] = *s_flag ? ntiles : next;
    }
    ptx::named_sync(1, NC * 32);
    if (*s_flag) break;

    const pre_t pw = pol.prepare(s_wpref[cw]);
    const bool excl = args.exclusive != 0;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      const int e = cw * Cfg::WARP_ELEMS + c * 32 + lane;
      const pre_t pc = pol.extend(pw, pre_lane[c]);
      out_t o[1];
      TS::finish_chunk(pol, pc, a[c], excl, o);
      if (e < valid) gout[base + e] = o[0];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) cta_exit_rearm(hdr, args.desc, uint64_t(ntiles) * TS::codec::W);
}

}  // namespace pp
