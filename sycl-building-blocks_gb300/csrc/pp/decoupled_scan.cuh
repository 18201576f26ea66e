// Single-pass decoupled look-back prefix scan for sm_103a.
//
// Re-design of parallel_primitives::internal::scan_decoupled_device and its
// kernel (include/parallel_primitives/scan_decoupled_lookback.hpp:106-182):
//
//  * Tiles are handed out by an atomic ticket counter (not by block id), so
//    every predecessor of a tile belongs to a CTA that is already running:
//    forward progress holds for any grid size and residency.
//  * decoupled_staged_kernel (element-aligned data, element sizes dividing 16
//    bytes): a persistent, warp-specialised kernel with one CTA per SM. Warp 0
//    is the producer: one lane takes tickets and streams whole tiles (64-72
//    KB) into a ring of shared-memory stages with cp.async.bulk (completion on
//    mbarriers). Warp 1 runs the look-back and publishes the inclusive
//    prefix. The NC compute warps reduce tile k+1 out of shared memory while
//    the look-back of tile k is in flight (the last of them publishes the tile
//    aggregate at once), then scan tile k and write it with coalesced 16-byte
//    streaming stores. Large tiles keep the number of tiles, and so the
//    length of the look-back chain, small.
//  * decoupled_generic_kernel: register tiles with plain element loads for
//    element types whose size does not divide 16 bytes (user functors, packed
//    structs).
//  * Strategy choice of the reference (:143-174), decided by the predecessor
//    descriptors: when the nearest predecessor's inclusive prefix is already
//    published the look-back ends after one read ("reduce-then-scan");
//    otherwise the published aggregates are folded back to the nearest
//    prefix ("scan-then-reduce"). In the staged kernel the look-back does
//    not wait for the tile's own aggregate (published separately, as soon as
//    the reduce pass ends), so both overlap.
//  * The look-back is warp-wide: LBW windows of 32 predecessors per memory
//    round trip, the nearest inclusive prefix found with ballots, the windows
//    folded with ordered shuffle reductions (the reference walks one
//    predecessor at a time on one work-item, partition_descriptor.h:115-130).
//  * Every wait is bounded by %globaltimer; a timeout records an error in the
//    workspace header and makes every CTA leave its loop.
//  * Combine order is prefix op local everywhere, so associative operators
//    that are not commutative scan correctly (the reference combines
//    op(aggregate, prefix), :157,170, and op(local, prefix), :98).
#pragma once

#include <cstdint>
#include <type_traits>
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
  int head;  // staged kernel: elements between the previous 16-byte boundary and in[0]
  // Descriptor perturbation knob of the staged kernel (tests; 0 = off): every
  // tile delays the publication of its aggregate and of its inclusive prefix
  // by a pseudo-random time in [0, debug_delay_ns] ns drawn from
  // (debug_seed, tile), spaces the words of a multi-word descriptor by up to a
  // quarter of that, and counts look-back outcomes in WsHeader::dbg.
  uint32_t debug_delay_ns = 0;
  uint32_t debug_seed = 0;
  // Cooperative rounds of the staged kernel (CO = 1): tiles per CTA per
  // window, the window aggregate slots (4 x gridDim.x slots of 16 bytes) and
  // the L2 priority of the first read of a window (0: evict_normal,
  // 1: evict_last).
  int coop_kt = 0;
  int coop_l2 = 0;
  void* coop_aggs = nullptr;
};

// Pseudo-random delay in [0, max_ns] for event `ev` of `tile` (a 32-bit
// integer hash of seed, tile and event).
__device__ __forceinline__ uint32_t debug_delay(uint32_t seed, long long tile, uint32_t ev, uint32_t max_ns) {
  uint32_t h = seed ^ (uint32_t(tile) * 0x9E3779B1u) ^ (uint32_t(uint64_t(tile) >> 32) * 0x85EBCA77u) ^
               (ev * 0xC2B2AE3Du);
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return max_ns ? h % (max_ns + 1u) : 0u;
}

// Publishes descriptor `d` of `tile`; with the perturbation knob on, after a
// pseudo-random delay and with its words spaced apart (event 0: aggregate,
// 1: inclusive prefix).
template <class C>
__device__ __forceinline__ void publish_desc(const ScanArgs& args, uint64_t* d, const C& v, uint32_t tag,
                                             long long tile, uint32_t ev) {
  if (args.debug_delay_ns == 0u) {
    desc_codec<C>::publish(d, v, tag);
    return;
  }
  ptx::nanosleep(debug_delay(args.debug_seed, tile, ev, args.debug_delay_ns));
  desc_codec<C>::publish_spaced(d, v, tag, debug_delay(args.debug_seed, tile, ev + 2u, args.debug_delay_ns / 4u));
}

__host__ __device__ constexpr size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Instrumentation hook of the staged kernel: called at fixed points of a
// tile's life with an event id, the tile index and a value. The default does
// nothing and compiles away.
struct NoTrace {
  static constexpr bool kOn = false;
  __device__ __forceinline__ void operator()(int, long long, unsigned long long) const {}
};
enum TraceEvent : int {
  kTrFull = 0,     // look-back warp sees the tile in shared memory
  kTrAggPub = 1,   // last compute warp published the tile aggregate
  kTrAgg = 2,      // look-back warp has the tile aggregate (publishes the prefix)
  kTrLbDone = 3,   // look-back warp has the exclusive prefix
  kTrLbRounds = 4, // look-back rounds (value), spins in the upper half
  kTrSStart = 5,   // compute warp 0 starts the scan pass
  kTrSDone = 6,    // compute warp 0 finished the scan pass
  kTrTicket = 9,   // producer drew the tile's ticket
  kTrIssue = 10,   // producer issued the tile's bulk copy (its stage was free)
  kTrRWait = 11,   // compute warp 0 starts waiting for the tile's data
  kTrRGot = 12,    // compute warp 0 has the tile's data (reduce pass begins)
  kTrPWait = 13,   // compute warp 0 starts waiting for the tile's prefix
  kTrPollRt = 14,  // duration of the first look-back poll (ns)
};

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
          const uint64_t waited = ptx::globaltimer_ns() - t0;
          if (waited > kAbortCheckAfterNs && aborted(hdr)) {
            give_up = true;
          } else if (waited > timeout_ns) {
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

// ---------------------------------------------------------------------------
// Staged (bulk-copy) variant: large tiles live in a ring of shared-memory
// stages; the tile is reduced from shared memory, its aggregate published,
// and it is scanned from shared memory once its prefix is known. Roles:
//   warp 0          producer: tickets + cp.async.bulk of whole tiles;
//   warp 1          look-back: tile aggregate, publish, look-back, prefix;
//   warps 2..NC+1   compute: reduce pass of tile k+1 while the look-back of
//                   tile k is in flight, then the scan pass of tile k with
//                   coalesced 16-byte streaming stores.
// Hand-offs use mbarriers only (no CTA-wide barrier inside the loop), and
// every wait is bounded, so a timeout anywhere lets every warp leave.
template <class Pol>
struct pol_commutative : std::false_type {};
template <class T, class Op>
struct pol_commutative<PlainScan<T, Op>>
    : std::bool_constant<std::is_same_v<Op, plus> || std::is_same_v<Op, multiplies> ||
                         std::is_same_v<Op, bit_and> || std::is_same_v<Op, bit_or> ||
                         std::is_same_v<Op, bit_xor> || std::is_same_v<Op, minimum> ||
                         std::is_same_v<Op, maximum>> {};
template <>
struct pol_commutative<CompensatedF32> : std::true_type {};
template <>
struct pol_commutative<F64CarryF32> : std::true_type {};

// LAY selects the layout of the passes over a tile:
//   0 striped: chunk c of a warp's segment is 32 consecutive 16-byte chunks,
//     one per lane; every chunk needs its own warp scan;
//   2 rows: each lane owns a row of CH consecutive chunks; the reduce pass
//     walks the row in order and leaves the row's prefix inside its segment
//     in shared memory, so the scan pass is one thread-serial chain along the
//     row (Pol::row_incl / row_excl: one combine per element).
// CH odd in the rows layout: rows of CH * 16 bytes then start in 8 different
// 16-byte bank groups for any 8 consecutive lanes, so row reads are free of
// bank conflicts; results go back into the row and leave striped or by bulk
// copy.
template <class Pol, int NC_, int CH_, int STAGES_, int LBW_, int LAY_ = 0, int SW_ = 0, int CO_ = 0>
struct StagedCfg {
  using in_t = typename Pol::in_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  static constexpr int LAY = LAY_;
  static_assert(LAY_ == 0 || LAY_ == 2, "striped (0) or rows (2) layout");
  static_assert(LAY_ == 0 || (CH_ % 2) == 1, "rows need an odd chunk count");
  static constexpr int NC = NC_;            // compute warps
  static constexpr int CH = CH_;            // 16-byte chunks per lane per segment
  static constexpr int STAGES = STAGES_;    // shared-memory ring depth
  static constexpr int LBW = LBW_;          // look-back windows (of 32 tiles) per round trip
  static_assert(16 % sizeof(in_t) == 0, "staged path needs element sizes dividing 16 bytes");
  static constexpr int V = 16 / sizeof(in_t);
  static constexpr int SEG = 32 * CH * V;   // elements per compute warp
  static constexpr int TILE = NC * SEG;
  static constexpr int TILE_BYTES = TILE * int(sizeof(in_t));
  static constexpr int SW = SW_;            // store warps (1: a warp writes finished tiles back by bulk copy)
  static constexpr int CO = CO_;            // cooperative rounds: one more warp (window barriers and folds)
  static constexpr int THREADS = (NC + 2 + SW + (CO_ != 0 ? 1 : 0)) * 32;
  // per-stage metadata
  static constexpr size_t META_AGG = 0;  // acc_t[NC] segment aggregates, then their exclusive prefixes
  static constexpr size_t META_PREF = align_up(NC * sizeof(acc_t), 16);   // carry_t tile exclusive prefix
  static constexpr size_t META_TAGG = META_PREF + align_up(sizeof(carry_t), 16);  // carry_t tile aggregate
  static constexpr size_t META_TILE = META_TAGG + align_up(sizeof(carry_t), 8);   // long long tile index
  static constexpr size_t META_CNT = META_TILE + 8;                                // unsigned arrivals
  static constexpr size_t META_JOB = META_CNT + 4;  // unsigned: 1 = a scan job of the cooperative rounds
  static constexpr size_t META_ROWS = align_up(META_JOB + 4, 16);  // acc_t[NC*32] row prefixes in the segment
  static constexpr size_t META_BYTES = align_up(META_ROWS + (LAY_ == 2 ? NC_ * 32 * sizeof(acc_t) : 0), 16);
  // cooperative rounds: per-tile record of REC_WORDS 64-bit words, the
  // 32-bit words of the tile aggregate (carry_t) and of the NC segment
  // exclusive prefixes (acc_t) in their low halves. The high halves stay 0:
  // the records live where look-back descriptors live, and a word with a 0
  // tag reads as an invalid descriptor that any later publication overwrites.
  static constexpr int REC_CW = words<carry_t>::W;
  static constexpr int REC_AW = words<acc_t>::W;
  static constexpr int REC_WORDS = REC_CW + NC * REC_AW;
  static constexpr size_t REC_BYTES = align_up(size_t(REC_WORDS) * 8, 16);
  static constexpr size_t OFF_META = size_t(STAGES) * TILE_BYTES;
  static constexpr size_t OFF_BAR = align_up(OFF_META + STAGES * META_BYTES, 8);  // 5 barriers / stage
  // cooperative rounds: carry_t run aggregates by window parity, carry_t
  // window prefixes by window parity, two counters, two mbarriers, then the
  // ring that hands scan jobs their prefixes: RING slots of {carry_t tile
  // prefix in 16 bytes, acc_t[NC] segment prefixes} with a full and a free
  // mbarrier each
  static constexpr int RING = 2;
  static constexpr size_t RING_SLOT = 16 + align_up(NC * sizeof(acc_t), 16);
  static constexpr size_t OFF_CO = align_up(OFF_BAR + 5 * STAGES * 8, 16);
  static constexpr size_t CO_WAGG = OFF_CO;
  static constexpr size_t CO_WIN = OFF_CO + 32;
  static constexpr size_t CO_CNT = OFF_CO + 64;  // unsigned reduce jobs done, unsigned windows taken
  static constexpr size_t CO_BAR = OFF_CO + 80;  // 2 window mbarriers, then RING full and RING free
  static constexpr size_t CO_RING = align_up(CO_BAR + (2 + 2 * RING) * 8, 16);
  static constexpr size_t SMEM = CO_ != 0 ? CO_RING + RING * RING_SLOT : OFF_BAR + 5 * STAGES * 8;
};

// Geometry of tile t in the staged kernel. The tile grid is shifted by `head`
// phantom elements so that every tile starts on a 16-byte boundary of the
// input: tile t covers global indices [t*TILE - head, (t+1)*TILE - head).
// Positions [lo, valid) of the tile hold data; positions [blo, bhi) arrive by
// bulk copy, the rest of the valid ones (the first partial chunk of tile 0 and
// the last < 16 bytes of the array) are read from global memory directly.
struct StagedGeom {
  long long gbase;  // global index of tile position 0
  int lo, valid, blo, bhi;
};
template <int TILE, int V, int ESZ>
__device__ __forceinline__ StagedGeom staged_geom(long long t, uint64_t n, int head) {
  StagedGeom g;
  g.gbase = t * TILE - head;
  g.lo = t == 0 ? head : 0;
  const long long end = (long long)n - g.gbase;
  g.valid = end < TILE ? int(end) : TILE;
  g.blo = (t == 0 && head > 0) ? V : 0;
  const int span = g.valid > g.blo ? g.valid - g.blo : 0;
  g.bhi = g.blo + int((uint32_t(span * ESZ) & ~15u) / ESZ);
  return g;
}

// V elements of a tile at offset e0 next to a ragged edge: bulk-copied ones
// from the stage, the rest of the valid range from global memory, the
// identity outside it.
template <class T, int V>
struct EdgeChunk {
  T x[V];
};
template <class T, int V>
__device__ __noinline__ EdgeChunk<T, V> load_edge_chunk(const unsigned char* stage, const T* gin, StagedGeom g,
                                                         int e0, T id) {
  EdgeChunk<T, V> c;
#pragma unroll
  for (int j = 0; j < V; ++j) {
    const int e = e0 + j;
    if (e < g.lo || e >= g.valid)
      c.x[j] = id;
    else if (e >= g.blo && e < g.bhi)
      c.x[j] = reinterpret_cast<const T*>(stage)[e];
    else
      c.x[j] = gin[g.gbase + e];
  }
  return c;
}

// Warp-wide look-back reading LBW windows of 32 descriptors per round trip.
// depth_out (optional): tile minus the index of the predecessor whose
// inclusive prefix ended the look-back (-1 for the identity before tile 0);
// torn_out (optional): incremented for every poll that met a half-written
// multi-word descriptor.
template <class Pol, int LBW>
__device__ __forceinline__ bool lookback_multi(const Pol& pol, const uint64_t* desc, long long tile,
                                               uint32_t etag, WsHeader* hdr, uint64_t timeout_ns, int lane,
                                               typename Pol::carry_t& out, unsigned long long& stats,
                                               long long* depth_out = nullptr, unsigned* torn_out = nullptr) {
  unsigned rounds = 0, spin_total = 0;
  using C = typename Pol::carry_t;
  using codec = desc_codec<C>;
  auto cop = [&](const C& x, const C& y) { return pol.cop(x, y); };
  C acc = pol.cid();
  long long base = tile - 1;
  uint32_t spins = 0;
  uint64_t t0 = 0;
  while (true) {
    C v[LBW];
    uint32_t st[LBW];
    bool torn = false;
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      const long long t = base - lane - 32 * j;
      v[j] = pol.cid();
      st[j] = kPrefix;
      if (t >= 0) {
        uint64_t raw[codec::W];
        codec::load_raw(desc + t * codec::W, raw);
        st[j] = codec::decode(raw, etag, v[j]);
        if (torn_out) torn |= codec::torn(raw, etag);
      }
    }
    if (torn_out && __ballot_sync(kFullMask, torn)) ++*torn_out;
    // nearest inclusive prefix: first window with one, lowest lane in it
    int pj = LBW, pl = 32;
    bool blocked = false;
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      const uint32_t pm = __ballot_sync(kFullMask, st[j] == kPrefix);
      const uint32_t xm = __ballot_sync(kFullMask, st[j] == kInvalid);
      if (pj == LBW) {
        if (pm) {
          const int p = __ffs(pm) - 1;
          const uint32_t need = (p >= 31) ? kFullMask : ((2u << p) - 1u);
          blocked |= (xm & need) != 0u;
          pj = j;
          pl = p;
        } else {
          blocked |= xm != 0u;
        }
      }
    }
    if (blocked) {
      if (spins == 0) t0 = ptx::globaltimer_ns();
      ++spins;
      ++spin_total;
      if ((spins & 7u) == 0u) {
        bool give_up = false;
        if (lane == 0) {
          const uint64_t waited = ptx::globaltimer_ns() - t0;
          if (waited > kAbortCheckAfterNs && aborted(hdr)) {
            give_up = true;
          } else if (waited > timeout_ns) {
            raise_error(hdr, kDevTimeout, (unsigned long long)tile);
            give_up = true;
          }
        }
        if (__shfl_sync(kFullMask, give_up, 0)) return false;
      }
      continue;
    }
    spins = 0;
    ++rounds;
    // fold windows newest -> oldest: acc = older op acc
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      if (j <= pj) {
        C w = (j < pj || lane <= pl) ? v[j] : pol.cid();
        w = warp_reduce_reversed(w, cop, lane);
        acc = pol.cop(w, acc);
      }
    }
    if (pj < LBW) {
      if (depth_out) *depth_out = tile - (base - pl - 32 * pj);
      break;
    }
    base -= 32 * LBW;
  }
  out = acc;
  stats = (unsigned long long)rounds | ((unsigned long long)spin_total << 32);
  return true;
}

// Look-back with two polls in flight. Descriptors become visible one L2
// round trip (about a microsecond while HBM streams at full rate) after they
// are published; a poll that just misses a publication would add another
// round trip. Here a second poll is issued GAP_NS after the first and each
// evaluated poll is re-issued at once, so successive samples of the window
// are about half a round trip apart.
// depth_out / torn_out as for lookback_multi.
template <class Pol, int LBW, unsigned GAP_NS, bool TIMED = false>
__device__ __forceinline__ bool lookback_pipelined(const Pol& pol, const uint64_t* desc, long long tile,
                                                   uint32_t etag, WsHeader* hdr, uint64_t timeout_ns, int lane,
                                                   typename Pol::carry_t& out, unsigned long long& stats,
                                                   unsigned long long* first_rt = nullptr,
                                                   long long* depth_out = nullptr, unsigned* torn_out = nullptr) {
  using C = typename Pol::carry_t;
  using codec = desc_codec<C>;
  constexpr int W = codec::W;
  auto cop = [&](const C& x, const C& y) { return pol.cop(x, y); };
  C acc = pol.cid();
  long long base = tile - 1;
  unsigned rounds = 0, spin_total = 0, spins = 0;
  uint64_t t0 = 0;
  uint64_t ra[LBW][W], rb[LBW][W];
  auto issue = [&](uint64_t (&r)[LBW][W]) {
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      const long long t = base - lane - 32 * j;
      if (t >= 0) codec::load_raw(desc + t * W, r[j]);
    }
  };
  // 0: blocked (an unpublished predecessor before the nearest prefix),
  // 1: done (acc holds the exclusive prefix), 2: folded all windows, go on
  auto step = [&](const uint64_t (&r)[LBW][W]) -> int {
    C v[LBW];
    uint32_t st[LBW];
    bool torn = false;
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      const long long t = base - lane - 32 * j;
      v[j] = pol.cid();
      st[j] = kPrefix;
      if (t >= 0) {
        st[j] = codec::decode(r[j], etag, v[j]);
        if (torn_out) torn |= codec::torn(r[j], etag);
      }
    }
    if (torn_out && __ballot_sync(kFullMask, torn)) ++*torn_out;
    int pj = LBW, pl = 32;
    bool blocked = false;
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      const uint32_t pm = __ballot_sync(kFullMask, st[j] == kPrefix);
      const uint32_t xm = __ballot_sync(kFullMask, st[j] == kInvalid);
      if (pj == LBW) {
        if (pm) {
          const int p = __ffs(pm) - 1;
          const uint32_t need = (p >= 31) ? kFullMask : ((2u << p) - 1u);
          blocked |= (xm & need) != 0u;
          pj = j;
          pl = p;
        } else {
          blocked |= xm != 0u;
        }
      }
    }
    if (blocked) return 0;
    ++rounds;
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      if (j <= pj) {
        C x = (j < pj || lane <= pl) ? v[j] : pol.cid();
        x = warp_reduce_reversed(x, cop, lane);
        acc = pol.cop(x, acc);
      }
    }
    if (pj < LBW) {
      if (depth_out) *depth_out = tile - (base - pl - 32 * pj);
      return 1;
    }
    base -= 32 * LBW;
    return 2;
  };
  // bounded spinning: false when the wait timed out or another CTA aborted
  auto spin_ok = [&]() -> bool {
    if (spins == 0) t0 = ptx::globaltimer_ns();
    ++spins;
    ++spin_total;
    if ((spins & 7u) != 0u) return true;
    bool give_up = false;
    if (lane == 0) {
      const uint64_t waited = ptx::globaltimer_ns() - t0;
      if (waited > kAbortCheckAfterNs && aborted(hdr)) {
        give_up = true;
      } else if (waited > timeout_ns) {
        raise_error(hdr, kDevTimeout, (unsigned long long)tile);
        give_up = true;
      }
    }
    return !__shfl_sync(kFullMask, give_up, 0);
  };
  const uint64_t t_first = TIMED ? ptx::globaltimer_ns() : 0ull;
  issue(ra);
  bool first = true;
  while (true) {
    ptx::nanosleep(GAP_NS);
    issue(rb);
    int x = step(ra);
    if (TIMED && first) {
      *first_rt = ptx::globaltimer_ns() - t_first;
      first = false;
    }
    if (x == 1) break;
    if (x == 2) {
      spins = 0;
      issue(ra);
      continue;
    }
    if (!spin_ok()) return false;
    issue(ra);
    x = step(rb);
    if (x == 1) break;
    if (x == 2) {
      spins = 0;
      issue(ra);
      continue;
    }
    if (!spin_ok()) return false;
  }
  out = acc;
  stats = (unsigned long long)rounds | ((unsigned long long)spin_total << 32);
  return true;
}

// ---------------------------------------------------------------------------
// Cooperative rounds (CO = 1): the grid-barrier scan of scan_cooperative.hpp
// with the input streamed through L2 in windows. The tiles are cut into
// windows of gridDim.x * coop_kt tiles; window w is split into one contiguous
// run per CTA, in block order. Round r of a CTA reduces its run of window r
// (a first read from HBM, which leaves the window in L2) and publishes the run
// aggregate at window barrier r, then scans its run of window r - 1 (a second
// read, served by L2) with the prefix of all earlier runs. The barrier is
// split: arriving never waits, and the wait for barrier r - 1 comes a whole
// window of reduce work after this CTA's own arrival there, so CTAs only stall
// when one falls a round behind. HBM sees each element read once and written
// once (2n) instead of the 3n of reduce, barrier, re-read.
struct CoopRuns {
  long long ntiles, G, b, kt, R;  // R windows
  __device__ __forceinline__ CoopRuns(long long ntiles_, long long G_, long long b_, long long kt_)
      : ntiles(ntiles_), G(G_), b(b_), kt(kt_), R((ntiles_ + G_ * kt_ - 1) / (G_ * kt_)) {}
  // tiles [t0, t1) of this CTA in window w (the last window may be partial:
  // its runs differ by at most one tile)
  __device__ __forceinline__ void run(long long w, long long& t0, long long& t1) const {
    const long long base = w * G * kt;
    const long long rem = (ntiles - base < G * kt) ? ntiles - base : G * kt;
    const long long q = rem / G, r = rem % G;
    t0 = base + b * q + (b < r ? b : r);
    t1 = t0 + q + (b < r ? 1 : 0);
  }
};

// The job sequence of one CTA: (tile, scan?) pairs, round by round.
struct CoopCursor {
  CoopRuns runs;
  long long r = 0, t = 0, e = 0;
  int part = 0;  // 0: reduce jobs of window r, 1: scan jobs of window r - 1
  __device__ __forceinline__ explicit CoopCursor(const CoopRuns& rr) : runs(rr) { runs.run(0, t, e); }
  __device__ __forceinline__ bool next(long long& tile, bool& scan) {
    while (t >= e) {
      if (part == 0) {
        part = 1;
        if (r >= 1) {
          runs.run(r - 1, t, e);
        } else {
          t = e = 0;
        }
      } else {
        ++r;
        part = 0;
        if (r > runs.R) return false;
        if (r < runs.R) {
          runs.run(r, t, e);
        } else {
          t = e = 0;
        }
      }
    }
    tile = t++;
    scan = part == 1;
    return true;
  }
};

// Window aggregate slots: 16 bytes each, written by lane 0 with plain stores
// before the fence and the arrival, read with volatile word loads after an
// acquire of the arrival counter.
template <class C>
__device__ __forceinline__ void coop_store_slot(C* slot, const C& v) {
  const words<C> w = to_words(v);
  volatile uint32_t* p = reinterpret_cast<volatile uint32_t*>(slot);
#pragma unroll
  for (int i = 0; i < words<C>::W; ++i) p[i] = w.w[i];
}
template <class C>
__device__ __forceinline__ C coop_load_slot(const C* slot) {
  words<C> w;
  const volatile uint32_t* p = reinterpret_cast<const volatile uint32_t*>(slot);
#pragma unroll
  for (int i = 0; i < words<C>::W; ++i) w.w[i] = p[i];
  return from_words<C>(w);
}

// Whole-warp bounded wait until *ctr >= target (every lane acquires the
// counter itself). False after a timeout (recorded, detail = the window) or
// when another CTA aborted.
__device__ __forceinline__ bool coop_wait_arrivals(WsHeader* h, const unsigned long long* ctr,
                                                   unsigned long long target, uint64_t timeout_ns,
                                                   unsigned long long detail, int lane) {
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    const unsigned long long v = ptx::ld_acquire(reinterpret_cast<const uint64_t*>(ctr));
    if (__all_sync(kFullMask, v >= target)) return true;
    if (it == 0) t0 = ptx::globaltimer_ns();
    if ((it & 15u) == 15u) {
      int stop = 0;
      if (lane == 0) {
        const uint64_t waited = ptx::globaltimer_ns() - t0;
        if (waited > kAbortCheckAfterNs && aborted(h)) {
          stop = 1;
        } else if (waited > timeout_ns) {
          raise_error(h, kDevTimeout, detail);
          stop = 1;
        }
      }
      if (__shfl_sync(kFullMask, stop, 0)) return false;
    }
  }
}

// Whole-warp bounded wait until the shared counter *cnt >= target (then an
// acquire fence at CTA scope). False after a timeout (recorded) or when
// another CTA aborted.
__device__ __forceinline__ bool coop_wait_smem_count(WsHeader* h, const unsigned* cnt, unsigned target,
                                                     uint64_t timeout_ns, unsigned long long detail, int lane) {
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    const unsigned v = *reinterpret_cast<const volatile unsigned*>(cnt);
    if (__all_sync(kFullMask, v >= target)) {
      __threadfence_block();
      return true;
    }
    if (it == 0) t0 = ptx::globaltimer_ns();
    if (it >= 4) ptx::nanosleep(64);
    if ((it & 15u) == 15u) {
      int stop = 0;
      if (lane == 0) {
        const uint64_t waited = ptx::globaltimer_ns() - t0;
        if (waited > kAbortCheckAfterNs && aborted(h)) {
          stop = 1;
        } else if (waited > timeout_ns) {
          raise_error(h, kDevTimeout, detail);
          stop = 1;
        }
      }
      if (__shfl_sync(kFullMask, stop, 0)) return false;
    }
  }
}

// Every compute warp runs the reduce pass of tile k+1 before the scan pass of
// tile k, so the next aggregate is published before this CTA waits for a
// prefix.
// PG: 0 = one look-back poll in flight; > 0 = two, the second PG ns later.
// BS: 0 = the compute warps store their results; 2 = one extra store warp
// writes each finished tile of the rows layout back with one bulk copy and
// frees the stage, so the compute warps never wait for stores.
// TK: when the producer draws the ticket of the next tile for a stage.
//   0: right after issuing the previous copy (a full stage life ahead);
//   2: once the stage is free.
// Later tickets make the order of tickets follow the order in which tiles
// reach their reduce pass more closely, so predecessors' aggregates arrive
// closer together; earlier ones hide the latency of the ticket atomic.
// CO: 0 = decoupled look-back (tickets, descriptors); 1 = cooperative rounds
// (a cooperative launch; warp 1 runs the window barriers and the carry chain
// of this CTA's tiles instead of the look-back).
template <class Pol, int NC, int CH, int STAGES, int LBW, int LAY = 0, int TK = 0, unsigned PG = 0, int BS = 0,
          class Trace = NoTrace, int CO = 0>
__global__ void __launch_bounds__((NC + 2 + (BS == 2 ? 1 : 0) + (CO != 0 ? 1 : 0)) * 32, 1)
    decoupled_staged_kernel(const ScanArgs args) {
  using Cfg = StagedCfg<Pol, NC, CH, STAGES, LBW, LAY, (BS == 2 ? 1 : 0), CO>;
  static_assert(TK == 0 || TK == 2, "tickets a stage life ahead (0) or once the stage is free (2)");
  static_assert(BS == 0 || (BS == 2 && LAY == 2), "the store warp serves the rows layout");
  using in_t = typename Pol::in_t;
  using out_t = typename Pol::out_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  using pre_t = typename Pol::pre_t;
  using codec = desc_codec<carry_t>;
  constexpr int V = Cfg::V;
  constexpr int TILE = Cfg::TILE;
  static_assert(sizeof(out_t) == sizeof(in_t), "in/out element sizes must match");

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + Cfg::OFF_BAR);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* aggb = bars + 2 * STAGES;
  uint64_t* prefb = bars + 3 * STAGES;
  uint64_t* scanned = bars + 4 * STAGES;  // the compute warps' results are in the stage (BS == 2)
  auto meta = [&](int s) { return smem + Cfg::OFF_META + size_t(s) * Cfg::META_BYTES; };
  auto s_aggs = [&](int s) { return reinterpret_cast<acc_t*>(meta(s) + Cfg::META_AGG); };
  auto s_pref = [&](int s) { return reinterpret_cast<carry_t*>(meta(s) + Cfg::META_PREF); };
  auto s_tagg = [&](int s) { return reinterpret_cast<carry_t*>(meta(s) + Cfg::META_TAGG); };
  auto s_tile = [&](int s) { return reinterpret_cast<long long*>(meta(s) + Cfg::META_TILE); };
  auto s_cnt = [&](int s) { return reinterpret_cast<unsigned*>(meta(s) + Cfg::META_CNT); };
  auto s_job = [&](int s) { return reinterpret_cast<unsigned*>(meta(s) + Cfg::META_JOB); };
  // cooperative rounds (unused otherwise): run aggregates and window prefixes
  // by window parity; co_cnt[0] = reduce jobs done, co_cnt[1] = windows whose
  // prefix warp 1 has taken; co_winb[p]: the prefix of a window of parity p
  // is in co_win[p]
  carry_t* co_wagg = reinterpret_cast<carry_t*>(smem + Cfg::CO_WAGG);
  carry_t* co_win = reinterpret_cast<carry_t*>(smem + Cfg::CO_WIN);
  unsigned* co_cnt = reinterpret_cast<unsigned*>(smem + Cfg::CO_CNT);
  uint64_t* co_winb = reinterpret_cast<uint64_t*>(smem + Cfg::CO_BAR);
  uint64_t* co_rfull = co_winb + 2;
  uint64_t* co_rfree = co_winb + 2 + Cfg::RING;
  auto co_slot = [&](int d) { return smem + Cfg::CO_RING + size_t(d) * Cfg::RING_SLOT; };
  auto s_rows = [&](int s) { return reinterpret_cast<acc_t*>(meta(s) + Cfg::META_ROWS); };

  const Pol pol{};
  const Trace trace{};
  // timestamps are read only when a recording Trace is compiled in
  auto trace_now = [&](int ev, long long tile) {
    if constexpr (Trace::kOn) trace(ev, tile, ptx::globaltimer_ns());
  };
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint64_t n = args.n;
  const int head = args.head;
  const long long ntiles = (long long)((n + head + TILE - 1) / TILE);
  WsHeader* hdr = args.hdr;
  const uint64_t tmo = args.timeout_ns;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], BS == 2 ? 1 : NC);
      ptx::mbar_init(&scanned[s], NC);
      ptx::mbar_init(&aggb[s], NC);
      ptx::mbar_init(&prefb[s], 1);
      *s_cnt(s) = 0u;
    }
    if constexpr (CO != 0) {
      for (int p = 0; p < 2; ++p) {
        ptx::mbar_init(&co_winb[p], 1);
        co_wagg[p] = Pol{}.cid();
      }
      for (int d = 0; d < Cfg::RING; ++d) {
        ptx::mbar_init(&co_rfull[d], 1);
        ptx::mbar_init(&co_rfree[d], NC);
      }
      co_cnt[0] = 0u;
      co_cnt[1] = 0u;
    }
    ptx::fence_mbar_init();
  }
  __syncthreads();
  const uint32_t etag = ptx::ld_relaxed(reinterpret_cast<const uint32_t*>(&hdr->epoch)) + 1u;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      const uint64_t pol_l2 = ptx::policy_evict_first();
      const unsigned char* in = static_cast<const unsigned char*>(args.in);
      uint32_t pending = 0, pend_par = 0;
      // bulk copy of tile t into stage s (use k)
      auto issue = [&](int s, int k, long long t, uint64_t l2) {
        trace_now(kTrIssue, t);
        const StagedGeom g = staged_geom<TILE, V, int(sizeof(in_t))>(t, n, head);
        const uint32_t bytes = uint32_t(g.bhi - g.blo) * uint32_t(sizeof(in_t));
        if (bytes) {
          ptx::mbar_arrive_expect_tx(&full[s], bytes);
          ptx::bulk_g2s(smem + size_t(s) * Cfg::TILE_BYTES + size_t(g.blo) * sizeof(in_t),
                        in + (g.gbase + g.blo) * (long long)sizeof(in_t), bytes, &full[s], l2);
          pending |= 1u << s;
          pend_par = (pend_par & ~(1u << s)) | ((uint32_t(k / STAGES) & 1u) << s);
        } else {
          ptx::mbar_arrive(&full[s]);
        }
      };
      if constexpr (CO != 0) {
        // the first read of a window stays in L2 for the second (scan) read,
        // which is its last use
        const uint64_t pol_keep = args.coop_l2 ? ptx::policy_evict_last() : ptx::policy_evict_normal();
        CoopCursor cur(CoopRuns(ntiles, gridDim.x, blockIdx.x, args.coop_kt));
        for (int k = 0;; ++k) {
          const int s = k % STAGES;
          if (k >= STAGES) {
            const uint32_t par = ((k / STAGES) - 1) & 1;
            if (!mbar_wait_bounded(&empty[s], par, hdr, tmo, 0ull)) break;
            pending &= ~(1u << s);
          }
          long long t = 0;
          bool scan = false;
          const bool more = cur.next(t, scan);
          *s_tile(s) = more ? t : ntiles;
          *s_job(s) = scan ? 1u : 0u;
          if (!more) {
            ptx::mbar_arrive(&full[s]);
            break;
          }
          issue(s, k, t, scan ? pol_l2 : pol_keep);
        }
      } else {
        auto draw = [&]() {
          const long long x = (long long)atomicAdd(&hdr->ticket, 1ull);
          if (x < ntiles) trace_now(kTrTicket, x);
          return x;
        };
        long long t = TK == 0 ? draw() : 0;
        for (int k = 0;; ++k) {
          const int s = k % STAGES;
          if (k >= STAGES) {
            const uint32_t par = ((k / STAGES) - 1) & 1;
            if (!mbar_wait_bounded(&empty[s], par, hdr, tmo, (unsigned long long)t)) break;
            if constexpr (TK == 2) t = draw();
            pending &= ~(1u << s);
          } else if constexpr (TK != 0) {
            t = draw();
          }
          *s_tile(s) = t;
          if (t < ntiles) {
            issue(s, k, t, pol_l2);
            if constexpr (TK == 0) t = draw();
          } else {
            ptx::mbar_arrive(&full[s]);
            break;
          }
        }
      }
      for (int s = 0; s < STAGES; ++s)
        if (pending & (1u << s)) mbar_wait_drain(&full[s], (pend_par >> s) & 1u, hdr, tmo);
    }
    __syncwarp();
  } else if (CO != 0 && warp == 1) {
    // ------------------------------------------------------------ carry chain
    // Scan jobs only; it never touches the stages (a reduce job never waits
    // for this warp). For the scan jobs of window w: takes the prefix of this
    // CTA's run from the fold warp, then, tile by tile, fills the next slot of
    // the ring with the tile's exclusive prefix (the carry chain of the run)
    // and the segment prefixes of its record. The record of window w's tiles
    // is complete once the fold warp posts window w's prefix; records are
    // loaded one tile ahead. Every window is taken (also with an empty run)
    // so that the fold warp can reuse the window's parity slot.
    const CoopRuns runs(ntiles, gridDim.x, blockIdx.x, args.coop_kt);
    const uint64_t* recs = args.desc;
    constexpr int RW = Cfg::REC_WORDS;
    constexpr int RCW = Cfg::REC_CW;
    constexpr size_t RSTRIDE = Cfg::REC_BYTES / 8;
    constexpr int RL = (RW + 31) / 32;  // this lane's record words: lane, lane + 32, ...
    auto load_rec = [&](long long t, uint32_t (&rw)[RL]) {
#pragma unroll
      for (int q = 0; q < RL; ++q) {
        const int i = q * 32 + lane;
        rw[q] = i < RW ? uint32_t(recs[size_t(t) * RSTRIDE + i]) : 0u;
      }
    };
    long long q = 0;  // scan jobs handed out
    for (long long w = 0; w < runs.R; ++w) {
      if (!mbar_wait_bounded(&co_winb[w & 1], uint32_t(w >> 1) & 1u, hdr, tmo, 0ull)) break;
      carry_t carry = co_win[w & 1];
      __threadfence_block();
      __syncwarp();
      if (lane == 0) atomicAdd(&co_cnt[1], 1u);
      long long t0, t1;
      runs.run(w, t0, t1);
      uint32_t rw[RL];
      if (t0 < t1) load_rec(t0, rw);
      bool ok = true;
      for (long long t = t0; t < t1; ++t, ++q) {
        const int d = int(q % Cfg::RING);
        if (q >= Cfg::RING &&
            !mbar_wait_bounded(&co_rfree[d], uint32_t(q / Cfg::RING - 1) & 1u, hdr, tmo, 0ull)) {
          ok = false;
          break;
        }
        unsigned char* slot = co_slot(d);
        uint32_t* sa = reinterpret_cast<uint32_t*>(slot + 16);
        words<carry_t> tw;
#pragma unroll
        for (int qq = 0; qq < RL; ++qq) {
          const int i = qq * 32 + lane;
          if (i >= RCW && i < RW) sa[i - RCW] = rw[qq];
        }
#pragma unroll
        for (int i = 0; i < RCW; ++i) tw.w[i] = __shfl_sync(kFullMask, rw[0], i);
        if (lane == 0) *reinterpret_cast<carry_t*>(slot) = carry;
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&co_rfull[d]);
        carry = pol.cop(carry, from_words<carry_t>(tw));
        if (t + 1 < t1) load_rec(t + 1, rw);
      }
      if (!ok) break;
    }
  } else if (CO != 0 && warp == NC + 2 + (BS == 2 ? 1 : 0)) {
    // ------------------------------------------------------------ window barriers
    // Window w in turn: first the prefix of window w - 1 (wait for barrier
    // w - 1, fold the run aggregates of window w - 1 in block order: this
    // CTA's run prefix for warp 1), then the run aggregate of window w (once
    // this CTA's reduce jobs of window w are done): published in slot w % 4,
    // arrival at barrier w. Slot reuse: a CTA overwrites slot w % 4 with
    // window w + 4 only after barrier w + 3, which every CTA reaches after its
    // fold of window w.
    const CoopRuns runs(ntiles, gridDim.x, blockIdx.x, args.coop_kt);
    const long long G = gridDim.x, b = blockIdx.x;
    carry_t* slots = static_cast<carry_t*>(args.coop_aggs);
    constexpr int CST = int(16 / sizeof(carry_t)) > 0 ? int(16 / sizeof(carry_t)) : 1;
    auto cop = [&](const carry_t& x, const carry_t& y) { return pol.cop(x, y); };
    carry_t wcarry = pol.cid();  // all windows before the next one to fold
    unsigned nred = 0;           // this CTA's reduce jobs up to the current window
    for (long long w = 0; w <= runs.R; ++w) {
      if (w >= 1) {
        const long long v = w - 1;
        if (!coop_wait_arrivals(hdr, &hdr->coop_arrive[v & 1], (unsigned long long)(v / 2 + 1) * G, tmo,
                                (unsigned long long)v, lane))
          break;
        // all slots of the window at once, FU per lane per round trip
        constexpr int FU = 8;
        carry_t pref = pol.cid(), tot = pol.cid();
        for (long long cc = 0; cc < G; cc += 32 * FU) {
          carry_t vv[FU];
#pragma unroll
          for (int u = 0; u < FU; ++u) {
            const long long i = cc + u * 32 + lane;
            vv[u] = i < G ? coop_load_slot(slots + ((v & 3) * G + i) * CST) : pol.cid();
          }
#pragma unroll
          for (int u = 0; u < FU; ++u) {
            const carry_t inc = warp_inclusive_scan(vv[u], cop, lane);
            const long long j = b - (cc + u * 32);  // warp-uniform
            const carry_t before = shfl_idx(inc, (j >= 1 && j < 32) ? int(j - 1) : 0);
            if (j >= 1 && j < 32) pref = pol.cop(tot, before);
            if (j == 0) pref = tot;
            tot = pol.cop(tot, shfl_idx(inc, 31));
          }
        }
        // the parity slot of window v - 2 is free once warp 1 has taken it
        if (v >= 2 && !coop_wait_smem_count(hdr, &co_cnt[1], unsigned(v - 1), tmo, (unsigned long long)v, lane))
          break;
        if (lane == 0) {
          co_win[v & 1] = pol.cop(wcarry, pref);
          ptx::mbar_arrive(&co_winb[v & 1]);
        }
        wcarry = pol.cop(wcarry, tot);
        __syncwarp();
      }
      if (w < runs.R) {
        long long t0, t1;
        runs.run(w, t0, t1);
        nred += unsigned(t1 - t0);
        if (!coop_wait_smem_count(hdr, &co_cnt[0], nred, tmo, (unsigned long long)w, lane)) break;
        // fault injection for tests: the CTA whose run holds the skipped tile
        // never arrives at this window's barrier, so every CTA's wait for it
        // times out
        const bool skip = args.debug_skip_tile >= t0 && args.debug_skip_tile < t1;
        if (lane == 0 && !skip) {
          coop_store_slot(slots + ((w & 3) * G + b) * CST, co_wagg[w & 1]);
          co_wagg[w & 1] = pol.cid();
          __threadfence();
          atomicAdd(&hdr->coop_arrive[w & 1], 1ull);
        }
        __syncwarp();
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ look-back
    for (int k = 0;; ++k) {
      const int s = k % STAGES;
      const uint32_t par = (k / STAGES) & 1;
      if (!mbar_wait_bounded(&full[s], par, hdr, tmo, 0ull)) break;
      const long long tile = *s_tile(s);
      if (tile >= ntiles) break;
      trace_now(kTrFull, tile);
      // The exclusive prefix depends on the predecessors' descriptors only, so
      // it is looked up while the compute warps still reduce this tile. The
      // nearest predecessors decide the path: a published inclusive prefix
      // ends the look-back at once (reduce-then-scan); published aggregates
      // are combined back to the nearest prefix (scan-then-reduce).
      carry_t excl = pol.cid();
      unsigned long long stats = 0;
      if (tile > 0) {
        bool ok;
        unsigned long long rt = 0;
        const bool dbg = args.debug_delay_ns != 0u;
        long long depth = 0;
        unsigned torn = 0;
        if constexpr (PG > 0)
          ok = lookback_pipelined<Pol, LBW, PG, Trace::kOn>(pol, args.desc, tile, etag, hdr, tmo, lane, excl, stats,
                                                           &rt, dbg ? &depth : nullptr, dbg ? &torn : nullptr);
        else
          ok = lookback_multi<Pol, LBW>(pol, args.desc, tile, etag, hdr, tmo, lane, excl, stats,
                                        dbg ? &depth : nullptr, dbg ? &torn : nullptr);
        if (!ok) break;
        trace(kTrPollRt, tile, rt);
        if (dbg && lane == 0) {
          atomicAdd(&hdr->dbg[depth == 1 ? 0 : 1], 1ull);
          if (depth > 32) atomicAdd(&hdr->dbg[2], 1ull);
          if (torn) atomicAdd(&hdr->dbg[3], (unsigned long long)torn);
        }
      }
      trace_now(kTrLbDone, tile);
      trace(kTrLbRounds, tile, stats);
      if (!mbar_wait_bounded(&aggb[s], par, hdr, tmo, 0ull)) break;
      trace_now(kTrAgg, tile);
      // the tile aggregate was published by the last compute warp of the
      // reduce pass (tile 0: as its inclusive prefix)
      if (tile > 0 && lane == 0 && tile != args.debug_skip_tile)
        publish_desc(args, args.desc + tile * codec::W, pol.cop(excl, *s_tagg(s)), make_tag(etag, kPrefix), tile, 1u);
      if (lane == 0) {
        *s_pref(s) = excl;
        ptx::mbar_arrive(&prefb[s]);
      }
      __syncwarp();
    }
  } else if (BS == 2 && warp == NC + 2) {
    // ------------------------------------------------------------ store
    // Each finished full tile leaves as one bulk copy; the stage is freed as
    // soon as the copy has read it. Partial tiles and outputs that are not
    // 16-byte aligned are stored by the compute warps themselves.
    out_t* gout = static_cast<out_t*>(args.out);
    const bool out_vec = ((reinterpret_cast<uintptr_t>(gout) - uintptr_t(head) * sizeof(out_t)) & 15u) == 0;
    const uint64_t pol_l2 = ptx::policy_evict_first();
    for (int k = 0;; ++k) {
      const int s = k % STAGES;
      const uint32_t par = (k / STAGES) & 1;
      if (!mbar_wait_bounded(&full[s], par, hdr, tmo, 0ull)) break;
      const long long tile = *s_tile(s);
      if (tile >= ntiles) break;
      if (!mbar_wait_bounded(&scanned[s], par, hdr, tmo, 0ull)) break;
      const StagedGeom g = staged_geom<TILE, V, int(sizeof(in_t))>(tile, n, head);
      if (lane == 0) {
        if ((CO == 0 || *s_job(s) != 0u) && out_vec && g.lo == 0 && g.valid == TILE) {
          ptx::bulk_s2g_hint(gout + g.gbase, smem + size_t(s) * Cfg::TILE_BYTES, uint32_t(Cfg::TILE_BYTES), pol_l2);
          ptx::bulk_commit();
          ptx::bulk_wait_read<0>();
        }
        ptx::mbar_arrive(&empty[s]);
      }
      __syncwarp();
    }
  } else {
    // ------------------------------------------------------------ compute
    const int w = warp - 2;
    const in_t* gin = static_cast<const in_t*>(args.in);
    out_t* gout = static_cast<out_t*>(args.out);
    const bool excl_kind = args.exclusive != 0;
    auto aop = [&](const acc_t& x, const acc_t& y) { return pol.aop(x, y); };

    const bool out_vec = ((reinterpret_cast<uintptr_t>(gout) - uintptr_t(head) * sizeof(out_t)) & 15u) == 0;
    // V elements at tile offset e0 (a 16-byte chunk of the stage)
    auto load_at = [&](int s, int e0, const StagedGeom& g, acc_t (&a)[V]) {
      const unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
      if (e0 >= g.blo && e0 + V <= g.bhi) {
        union {
          uint4 u;
          in_t x[V];
        } buf;
        buf.u = *reinterpret_cast<const uint4*>(stage + size_t(e0) * sizeof(in_t));
#pragma unroll
        for (int j = 0; j < V; ++j) a[j] = pol.load(buf.x[j]);
      } else {
#pragma unroll
        for (int j = 0; j < V; ++j) {
          const int e = e0 + j;
          if (e < g.lo || e >= g.valid)
            a[j] = pol.aid();
          else if (e >= g.blo && e < g.bhi)
            a[j] = pol.load(reinterpret_cast<const in_t*>(stage)[e]);
          else
            a[j] = pol.load(gin[g.gbase + e]);
        }
      }
    };
    // V raw elements at tile offset e0, the identity outside the valid range
    // (the ragged edges of the array take an out-of-line path: it keeps the
    // unrolled loops of interior tiles small)
    auto load_raw_at = [&](int s, int e0, const StagedGeom& g, bool interior, in_t (&x)[V]) {
      const unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
      if (interior || (e0 >= g.blo && e0 + V <= g.bhi)) {
        union {
          uint4 u;
          in_t x[V];
        } buf;
        buf.u = *reinterpret_cast<const uint4*>(stage + size_t(e0) * sizeof(in_t));
#pragma unroll
        for (int j = 0; j < V; ++j) x[j] = buf.x[j];
      } else {
        const EdgeChunk<in_t, V> c = load_edge_chunk<in_t, V>(stage, gin, g, e0, pol.in_id());
#pragma unroll
        for (int j = 0; j < V; ++j) x[j] = c.x[j];
      }
    };
    // striped chunk c of this lane in segment seg: tile offset seg*SEG + (c*32 + lane)*V
    auto load_chunk = [&](int s, int seg, int c, const StagedGeom& g, acc_t (&a)[V]) {
      load_at(s, seg * Cfg::SEG + (c * 32 + lane) * V, g, a);
    };
    // Writes this warp's finished segment (already in the stage, in order):
    // with a store warp, a full tile with an aligned output leaves by its bulk
    // copy; else striped 16-byte stores. Returns once the stage may be reused.
    auto store_segment = [&](const unsigned char* stage, const StagedGeom& g) {
      const int s0 = w * Cfg::SEG;
      if (BS == 2 && out_vec && g.lo == 0 && g.valid == TILE) {
        // the store warp writes the whole tile once every segment is in
        ptx::fence_proxy_async_smem();
        return;
      }
      __syncwarp();
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int e0 = s0 + (c * 32 + lane) * V;
        union {
          uint4 u;
          out_t x[V];
        } o;
        o.u = *reinterpret_cast<const uint4*>(stage + size_t(e0) * sizeof(in_t));
        if (out_vec && e0 >= g.lo && e0 + V <= g.valid) {
          ptx::st_stream_v4(gout + (g.gbase + e0), o.u);
        } else {
#pragma unroll
          for (int j = 0; j < V; ++j)
            if (e0 + j >= g.lo && e0 + j < g.valid) gout[g.gbase + e0 + j] = o.x[j];
        }
      }
      // the stage was written through the generic proxy; the next bulk copy
      // into it is an async-proxy write
      ptx::fence_proxy_async_smem();
    };
    // aggregate of segment seg of stage s (a warp-wide value); rows layout:
    // `info` gets the policy's statistic of this lane's row (fast rows)
    using RF = row_fast_traits<Pol>;
    using row_info_t = typename RF::info_t;
    auto reduce_segment = [&](int s, int seg, const StagedGeom& g, row_info_t& info) -> acc_t {
      acc_t r = pol.aid();
      if constexpr (LAY == 2) {
        // this lane's row, in order; the scan of the row totals over the
        // segment is done here, off the scan pass's critical path, and the
        // row's exclusive prefix stays for the scan pass
        const int r0 = seg * Cfg::SEG + lane * (CH * V);
        const bool interior = g.lo == 0 && g.blo == 0 && g.bhi == TILE;
        row_info_t m = RF::id(pol);
        if constexpr (RF::value) {
          // the row's statistic first, then its total: from an offset that
          // dominates every partial sum, with the policy's cheaper exact
          // additions (compensated sums: FastTwoSum instead of TwoSum); the
          // row's elements stay in registers between the two
          in_t xs[CH][V];
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            load_raw_at(s, r0 + c * V, g, interior, xs[c]);
#pragma unroll
            for (int j = 0; j < V; ++j) m = RF::add(pol, m, xs[c][j]);
          }
          const float off = pol.row_offset(m);
          if (off != 0.0f) {
            acc_t t{off, 0.0f};
#pragma unroll
            for (int c = 0; c < CH; ++c)
#pragma unroll
              for (int j = 0; j < V; ++j) pol.row_offset_add(t, xs[c][j]);
            r = pol.row_offset_total(t, off);
          } else {
#pragma unroll
            for (int c = 0; c < CH; ++c)
#pragma unroll
              for (int j = 0; j < V; ++j) r = pol.aop_in(r, xs[c][j]);
          }
        } else {
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            in_t x[V];
            load_raw_at(s, r0 + c * V, g, interior, x);
#pragma unroll
            for (int j = 0; j < V; ++j) r = pol.aop_in(r, x[j]);
          }
        }
        info = m;
        const acc_t inc = warp_inclusive_scan(r, aop, lane);
        const acc_t ex = shfl_up(inc, 1);
        s_rows(s)[seg * 32 + lane] = lane == 0 ? pol.aid() : ex;
        r = shfl_idx(inc, 31);
      } else if constexpr (pol_commutative<Pol>::value) {
        // V independent accumulators: short dependency chains
        acc_t rv[V];
#pragma unroll
        for (int j = 0; j < V; ++j) rv[j] = pol.aid();
#pragma unroll 4
        for (int c = 0; c < CH; ++c) {
          acc_t a[V];
          load_chunk(s, seg, c, g, a);
#pragma unroll
          for (int j = 0; j < V; ++j) rv[j] = pol.aop(rv[j], a[j]);
        }
#pragma unroll
        for (int j = 0; j < V; ++j) r = pol.aop(r, rv[j]);
        r = warp_reduce(r, aop, lane);
      } else {
        for (int c = 0; c < CH; ++c) {
          acc_t a[V];
          load_chunk(s, seg, c, g, a);
          acc_t t = a[0];
#pragma unroll
          for (int j = 1; j < V; ++j) t = pol.aop(t, a[j]);
          r = pol.aop(r, warp_reduce(t, aop, lane));
        }
      }
      return r;
    };
    // Records the aggregate of segment seg. The warp that records the last
    // segment of the tile combines them and publishes the tile aggregate at
    // once (tile 0: its inclusive prefix), so successors never wait for this
    // CTA's look-back of an earlier tile; it leaves each segment's exclusive
    // prefix inside the tile in place of its aggregate for the scan pass.
    auto record_segment = [&](int s, int seg, long long tile, const acc_t& r) {
      unsigned last = 0;
      if (lane == 0) {
        s_aggs(s)[seg] = r;
        __threadfence_block();
        last = atomicAdd(s_cnt(s), 1u) == unsigned(NC - 1);
      }
      if (__shfl_sync(kFullMask, last, 0)) {
        __threadfence_block();
        acc_t x = lane < NC ? s_aggs(s)[lane] : pol.aid();
        x = warp_inclusive_scan(x, aop, lane);
        const acc_t xe = shfl_up(x, 1);
        if (lane < NC) s_aggs(s)[lane] = lane == 0 ? pol.aid() : xe;
        const carry_t agg = pol.to_carry(shfl_idx(x, NC - 1));
        if constexpr (CO != 0) {
          // cooperative rounds: the tile's record (segment prefixes, then the
          // aggregate), the run aggregate of the tile's window, then one more
          // reduce job done
          uint64_t* rec = args.desc + size_t(tile) * (Cfg::REC_BYTES / 8);
          if (lane < NC) {
            const words<acc_t> aw = to_words(lane == 0 ? pol.aid() : xe);
#pragma unroll
            for (int i = 0; i < Cfg::REC_AW; ++i) rec[Cfg::REC_CW + lane * Cfg::REC_AW + i] = aw.w[i];
          }
          __syncwarp();
          if (lane == 0) {
            const words<carry_t> cw = to_words(agg);
#pragma unroll
            for (int i = 0; i < Cfg::REC_CW; ++i) rec[i] = cw.w[i];
            const int p = int((tile / ((long long)gridDim.x * args.coop_kt)) & 1);
            co_wagg[p] = pol.cop(co_wagg[p], agg);
            *s_cnt(s) = 0u;
            __threadfence_block();
            atomicAdd(&co_cnt[0], 1u);
          }
        } else if (lane == 0) {
          *s_tagg(s) = agg;
          *s_cnt(s) = 0u;
          if (tile != args.debug_skip_tile)
            publish_desc(args, args.desc + tile * codec::W, agg, make_tag(etag, tile == 0 ? kPrefix : kAggregate),
                         tile, 0u);
          trace_now(kTrAggPub, tile);
        }
      }
      __syncwarp();
    };
    // reduce pass of use k over the segments of this warp: returns false at
    // the end of work or on a failed wait
    auto reduce_pass = [&](int k, row_info_t& info) -> bool {
      const int s = k % STAGES;
      const unsigned long long tw = Trace::kOn ? ptx::globaltimer_ns() : 0ull;
      if (!mbar_wait_bounded(&full[s], (k / STAGES) & 1, hdr, tmo, 0ull)) return false;
      const long long tile = *s_tile(s);
      if (tile >= ntiles) return false;
      if (w == 0 && lane == 0) {
        trace(kTrRWait, tile, tw);
        trace_now(kTrRGot, tile);
      }
      const StagedGeom g = staged_geom<TILE, V, int(sizeof(in_t))>(tile, n, head);
      record_segment(s, w, tile, reduce_segment(s, w, g, info));
      if (lane == 0) ptx::mbar_arrive(&aggb[s]);
      __syncwarp();
      return true;
    };

    // Exclusive prefix of this warp's segment: the tile prefix combined with
    // the segment's exclusive prefix inside the tile.
    auto segment_prefix = [&](const carry_t& tile_pref, const acc_t& sx) -> pre_t {
      return pol.prepare(w == 0 ? tile_pref : pol.cop(tile_pref, pol.to_carry(sx)));
    };
    // Scan pass of the tile in stage s (geometry g) with this warp's segment
    // prefix pw; rows: this warp's row prefixes are in the stage's metadata,
    // `info_cur` their statistic.
    auto scan_pass = [&](int s, const StagedGeom& g, const row_info_t& info_cur, const pre_t& pw) {
      if constexpr (LAY == 2) {
        // rows: each row's prefix inside the segment comes from the reduce
        // pass; a thread-serial chain along the row
        unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
        const int r0 = w * Cfg::SEG + lane * (CH * V);
        const bool interior = g.lo == 0 && g.blo == 0 && g.bhi == TILE;
        const acc_t ex = s_rows(s)[w * 32 + lane];
        typename Pol::row_t row = pol.row_start(pol.extend(pw, ex));
        auto chain = [&](auto excl_c, auto fast_c) {
          constexpr bool kEx = decltype(excl_c)::value;
          constexpr bool kFast = decltype(fast_c)::value;
          union Out {
            uint4 u;
            out_t x[V];
          };
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            in_t x[V];
            load_raw_at(s, r0 + c * V, g, interior, x);
            Out o;
#pragma unroll
            for (int j = 0; j < V; ++j) {
              if constexpr (kFast)
                o.x[j] = kEx ? RF::excl(pol, row, x[j]) : RF::incl(pol, row, x[j]);
              else
                o.x[j] = kEx ? pol.row_excl(row, x[j]) : pol.row_incl(row, x[j]);
            }
            *reinterpret_cast<uint4*>(stage + size_t(r0 + c * V) * sizeof(in_t)) = o.u;
          }
        };
        // fast rows when every lane's row qualifies (a warp-uniform choice)
        bool fast = false;
        if constexpr (RF::value) fast = __all_sync(kFullMask, RF::ok(pol, row, info_cur, CH * V));
        if constexpr (RF::value) {
          if (fast) {
            if (excl_kind)
              chain(std::true_type{}, std::true_type{});
            else
              chain(std::false_type{}, std::true_type{});
          }
        }
        if (!fast) {
          if (excl_kind)
            chain(std::true_type{}, std::false_type{});
          else
            chain(std::false_type{}, std::false_type{});
        }
        store_segment(stage, g);
      } else {
      acc_t X = pol.aid();
      // chunks in groups of SG: the SG warp scans of a group are independent
      // and interleave, hiding shuffle and arithmetic latency
      constexpr int SG = CH < 4 ? CH : 4;
#pragma unroll 1
      for (int c0 = 0; c0 < CH; c0 += SG) {
        acc_t a[SG][V];
        acc_t inc[SG];
#pragma unroll
        for (int q = 0; q < SG; ++q) {
          load_chunk(s, w, c0 + q, g, a[q]);
#pragma unroll
          for (int j = 1; j < V; ++j) a[q][j] = pol.aop(a[q][j - 1], a[q][j]);
          inc[q] = a[q][V - 1];
        }
#pragma unroll
        for (int q = 0; q < SG; ++q) inc[q] = warp_inclusive_scan(inc[q], aop, lane);
#pragma unroll
        for (int q = 0; q < SG; ++q) {
          const int c = c0 + q;
          acc_t ex = shfl_up(inc[q], 1);
          if (lane == 0) ex = pol.aid();
          const pre_t pc = pol.extend(pw, c == 0 ? ex : pol.aop(X, ex));
          X = (c == 0) ? shfl_idx(inc[q], 31) : pol.aop(X, shfl_idx(inc[q], 31));
          union {
            uint4 u;
            out_t x[V];
          } o;
          TileScan<Pol, NC, CH, V>::finish_chunk(pol, pc, a[q], excl_kind, o.x);
          const int e0 = w * Cfg::SEG + (c * 32 + lane) * V;
          if (out_vec && e0 >= g.lo && e0 + V <= g.valid) {
            ptx::st_stream_v4(gout + (g.gbase + e0), o.u);
          } else {
#pragma unroll
            for (int j = 0; j < V; ++j)
              if (e0 + j >= g.lo && e0 + j < g.valid) gout[g.gbase + e0 + j] = o.x[j];
          }
        }
      }
      }
    };

    if constexpr (CO != 0) {
      // Cooperative rounds: a reduce job leaves its tile's record and frees
      // the stage at once; a scan job takes its tile prefix and this warp's
      // segment prefix from the next slot of warp 1's ring, then runs the scan
      // pass alone (rows: after this warp's own row totals).
      long long q = 0;  // scan jobs taken
      for (int k = 0;; ++k) {
        const int s = k % STAGES;
        if (!mbar_wait_bounded(&full[s], (k / STAGES) & 1, hdr, tmo, 0ull)) break;
        const long long tile = *s_tile(s);
        if (tile >= ntiles) break;
        const StagedGeom g = staged_geom<TILE, V, int(sizeof(in_t))>(tile, n, head);
        row_info_t info = RF::id(pol);
        if (*s_job(s) == 0u) {
          record_segment(s, w, tile, reduce_segment(s, w, g, info));
          if (lane == 0) ptx::mbar_arrive(BS == 2 ? &scanned[s] : &empty[s]);
          __syncwarp();
          continue;
        }
        if constexpr (LAY == 2) {
          (void)reduce_segment(s, w, g, info);  // this warp's row prefixes and statistic
          __syncwarp();
        }
        const int d = int(q % Cfg::RING);
        if (!mbar_wait_bounded(&co_rfull[d], uint32_t(q / Cfg::RING) & 1u, hdr, tmo, 0ull)) break;
        const unsigned char* slot = co_slot(d);
        const pre_t pw = segment_prefix(*reinterpret_cast<const carry_t*>(slot),
                                        reinterpret_cast<const acc_t*>(slot + 16)[w]);
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&co_rfree[d]);
        ++q;
        scan_pass(s, g, info, pw);
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(BS == 2 ? &scanned[s] : &empty[s]);
      }
    } else {
    // the reduce pass runs one tile ahead of the scan pass (row statistics:
    // info_cur of tile k, info_next of tile k + 1)
    row_info_t info_cur = RF::id(pol), info_next = RF::id(pol);
    bool have = reduce_pass(0, info_cur);
    for (int k = 0; have; ++k) {
      const bool have_next = reduce_pass(k + 1, info_next);
      const int s = k % STAGES;
      // scan pass of use k
      if constexpr (Trace::kOn)
        if (w == 0 && lane == 0) trace_now(kTrPWait, *s_tile(s));
      if (!mbar_wait_bounded(&prefb[s], (k / STAGES) & 1, hdr, tmo, 0ull)) break;
      const long long tile = *s_tile(s);
      if (w == 0 && lane == 0) trace_now(kTrSStart, tile);
      // the tile prefix from warp 1, this segment's prefix inside the tile
      // from the reduce pass
      scan_pass(s, staged_geom<TILE, V, int(sizeof(in_t))>(tile, n, head), info_cur,
                segment_prefix(*s_pref(s), s_aggs(s)[w]));
      __syncwarp();
      if (lane == 0) {
        if (w == 0) trace_now(kTrSDone, tile);
        ptx::mbar_arrive(BS == 2 ? &scanned[s] : &empty[s]);
      }
      have = have_next;
      info_cur = info_next;
    }
    }
  }
  if constexpr (BS != 0) ptx::bulk_wait<0>();  // this thread's bulk stores are complete
  __syncthreads();
  if (threadIdx.x == 0) cta_exit_rearm(hdr, args.desc, CO != 0 ? 0ull : uint64_t(ntiles) * codec::W, etag - 1u);
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
  if (threadIdx.x == 0) cta_exit_rearm(hdr, args.desc, uint64_t(ntiles) * TS::codec::W, etag - 1u);
}

}  // namespace pp
