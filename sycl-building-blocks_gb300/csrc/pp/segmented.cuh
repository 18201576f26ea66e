// Batched segmented scan / reduce for sm_103a: many independent segments of
// uneven length, laid out back to back (CSR: int64 offsets, S + 1 entries,
// offsets[0] = 0, offsets[S] = n), in ONE persistent launch of the staged
// decoupled look-back pipeline (decoupled_scan.cuh) instead of one launch per
// segment. No counterpart in the reference, which scans one array per call.
//
// Segments become a segmented operator on (value, count) pairs:
//     (a, c) op (b, d) = (d ? b : a op b, c + d)
// where d counts the segment heads inside the right operand. It is
// associative, so tiles may cross segment boundaries freely and the look-back
// stops contributing at the nearest head. The count also ranks every element:
// the inclusive count at element e is the number of distinct segment starts
// at or before e.
//
// Head flags come from a bitmap of n bits (one per element): a pre-pass
// scatters the start of every non-empty segment into it, and the producer warp
// bulk-copies each tile's 2 KB slice of the bitmap into shared memory next to
// the tile's data. Uniform segments (rows of equal length, as for a batched
// cumsum) need no bitmap: heads are computed from the index.
//
// Reverse scans (suffix sums, the adjoint of a prefix sum) walk the tiles from
// the last to the first and mirror the element order inside each tile; they
// are provided for uniform segments.
//
// Segmented reduce writes no scanned array and needs no look-back: every
// tile reduces on its own, with tile-local prefixes only. The element that
// ends a non-empty segment whose head lies in the same tile writes the
// segment's total to rank_out[base + count - 1] (base: the non-empty segments
// that start before the tile, written by the rank pre-pass; count: the heads
// of the tile up to the element). The one segment per tile that was open
// where the tile begins and ends inside it leaves its piece in the tile's
// record, beside the tile's aggregate; segment_fixup_kernel scans the records in tile order and
// completes those segments, and segment_gather_kernel moves the totals from
// rank order to their segments (empty segments get the identity from the
// pre-pass). In the rows layout the data is read once: the reduce pass
// leaves each row's running value at the row's segment ends and keeps the
// row's head and end bits, and the totals pass reads only the end elements.
// A stage is free as soon as its tile's totals are written.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "decoupled_scan.cuh"

namespace pp {

template <class T>
struct seg_pair {
  T v;
  uint32_t c;  // segment heads covered by this partial
};

// Segmented plain policy over (value, head-count) pairs.
template <class T, class Op>
struct SegPlainScan {
  using in_t = T;
  using out_t = T;
  using acc_t = seg_pair<T>;
  using carry_t = seg_pair<T>;
  using pre_t = seg_pair<T>;
  Op op;

  __device__ __forceinline__ acc_t aop(const acc_t& a, const acc_t& b) const {
    return acc_t{b.c ? b.v : op(a.v, b.v), a.c + b.c};
  }
  __device__ __forceinline__ acc_t aid() const { return acc_t{identity<Op, T>(), 0u}; }
  __device__ __forceinline__ carry_t cop(const carry_t& a, const carry_t& b) const { return aop(a, b); }
  __device__ __forceinline__ carry_t cid() const { return aid(); }
  __device__ __forceinline__ carry_t to_carry(const acc_t& a) const { return a; }
  __device__ __forceinline__ acc_t load(const T& x, bool head) const { return acc_t{x, head ? 1u : 0u}; }
};

// Where segment heads are.
struct CsrHeads {
  static constexpr bool kBitmap = true;
  uint64_t len = 0;  // unused
};
struct UniformHeads {
  static constexpr bool kBitmap = false;
  uint64_t len = 1;  // segment (row) length
};

struct SegArgs {
  ScanArgs s;
  const uint32_t* heads;         // CSR: n-bit head bitmap (tile-padded), else null
  uint64_t seg_len;              // uniform: row length
  void* rank_out;                // reduce: total of each non-empty segment, by rank
  const uint32_t* tile_base;     // reduce: non-empty segments that start before each tile
  void* tile_rec;                // reduce: SegTileRec<T> per tile (zero-filled before the launch)
};

// Per-tile record of a segmented reduce: the tile's aggregate pair and the
// piece of the segment that was open where the tile begins and ends inside
// it (its value from the tile's start to its end; flag 1 when there is one).
// segment_fixup_kernel completes those segments in tile order.
template <class T>
struct SegTileRec {
  T agg_v;
  uint32_t agg_c;
  T piece_v;
  uint32_t piece_flag;
};

// NC compute warps, CH chunks per lane, VB bytes per chunk (the vector width
// of shared-memory loads and global stores: 4, 8 or 16), STAGES-deep ring.
// LAY 0: striped chunks (a warp scan per chunk); LAY 2: lane rows of CH
// consecutive 16-byte chunks (CH odd: conflict-free), the reduce pass leaves
// each row's (value, count) total in shared memory and the scan pass is one
// thread-serial chain per row (forward scans and reductions with CSR heads).
template <class Pol, int NC_, int CH_, int STAGES_, int LBW_, int VB_ = 16, int LAY_ = 0, int SW_ = 0>
struct SegCfg {
  using in_t = typename Pol::in_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  static constexpr int NC = NC_;
  static constexpr int CH = CH_;
  static constexpr int STAGES = STAGES_;
  static constexpr int LBW = LBW_;
  static constexpr int VB = VB_;
  static_assert(VB == 4 || VB == 8 || VB == 16, "chunk width of 4, 8 or 16 bytes");
  static_assert(VB % sizeof(in_t) == 0, "element size must divide the chunk width");
  static constexpr int V = VB / int(sizeof(in_t));
  static constexpr int SEG = 32 * CH * V;
  static constexpr int TILE = NC * SEG;
  static_assert(TILE % 128 == 0, "tile must cover whole 16-byte bitmap words");
  static constexpr int TILE_BYTES = TILE * int(sizeof(in_t));
  static constexpr int MAP_BYTES = TILE / 8;  // head bits of one tile
  // a stage's map slot: the tile's head bits and, for reductions, the first
  // 16 bytes of the next tile's (whether the tile's last element ends its
  // segment is then known from shared memory)
  static constexpr int MAP_STRIDE = MAP_BYTES + 16;
  static constexpr int SW = SW_;  // store warps (1: finished tiles leave by one bulk copy, rows scans only)
  static_assert(SW == 0 || (SW == 1 && LAY_ == 2), "the store warp serves the rows layout");
  static constexpr int THREADS = (NC + 2 + SW) * 32;
  static constexpr size_t META_AGG = 0;
  static constexpr size_t META_PREF = align_up(NC * sizeof(acc_t), 16);
  static constexpr size_t META_TAGG = META_PREF + align_up(sizeof(carry_t), 16);
  static constexpr size_t META_TILE = META_TAGG + align_up(sizeof(carry_t), 8);
  static constexpr size_t META_CNT = META_TILE + 8;
  static constexpr int LAY = LAY_;
  static_assert(LAY_ == 0 || (LAY_ == 2 && VB_ == 16 && (CH_ % 2) == 1), "rows need odd counts of 16-byte chunks");
  static constexpr size_t META_ROWS = align_up(META_CNT + 4, 16);  // acc_t[NC * 32] row prefixes (LAY 2)
  static constexpr size_t META_BYTES = align_up(META_ROWS + (LAY_ == 2 ? NC_ * 32 * sizeof(acc_t) : 0), 16);
  static constexpr size_t OFF_MAP = size_t(STAGES) * TILE_BYTES;
  static constexpr size_t OFF_META = OFF_MAP + size_t(STAGES) * MAP_STRIDE;
  static constexpr size_t OFF_BAR = align_up(OFF_META + STAGES * META_BYTES, 8);
  static constexpr size_t SMEM = OFF_BAR + 5 * STAGES * 8;  // full, empty, aggb, prefb, scanned
};

// REDUCE: write only segment totals (by rank) instead of the scan.
// BS: 2 = a store warp writes each finished full tile of a rows-layout scan
// back with one bulk copy and frees the stage (the compute warps go on to the
// next tile); 0 = the compute warps store.
// SKIP (rows layout): a warp whose chunks hold no segment head (and, in the
// second pass of a reduction, no segment end) combines them without the
// per-element head tests; it pays off when segments are long.
// Trace: instrumentation hook with the events of the plain staged kernel
// (kTr*); the default records nothing and compiles away.
template <class Pol, int NC, int CH, int STAGES, int LBW, class Heads, bool REVERSE, bool REDUCE, int VB = 16,
          int LAY = 0, int BS = 0, bool SKIP = false, class Trace = NoTrace>
__global__ void __launch_bounds__((NC + 2 + (BS == 2 ? 1 : 0)) * 32, 1) segmented_staged_kernel(const SegArgs sargs) {
  using Cfg = SegCfg<Pol, NC, CH, STAGES, LBW, VB, LAY, (BS == 2 ? 1 : 0)>;
  static_assert(LAY == 0 || (!REVERSE && Heads::kBitmap), "rows: forward scans over CSR heads");
  static_assert(BS == 0 || (BS == 2 && LAY == 2 && !REDUCE), "the store warp serves rows-layout scans");
  using vec_t = std::conditional_t<VB == 16, uint4, std::conditional_t<VB == 8, uint2, uint32_t>>;
  using in_t = typename Pol::in_t;
  using out_t = typename Pol::out_t;
  using acc_t = typename Pol::acc_t;
  using carry_t = typename Pol::carry_t;
  using codec = desc_codec<carry_t>;
  constexpr int V = Cfg::V;
  constexpr int TILE = Cfg::TILE;
  static_assert(!(REVERSE && Heads::kBitmap), "reverse scans are provided for uniform segments");
  static_assert(!(REVERSE && REDUCE), "reverse segmented reduce is not provided");
  static_assert(!(REDUCE && LAY == 2) || CH * V <= 32, "a lane row's head and end bits fit one word");

  const ScanArgs& args = sargs.s;
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
  auto s_map = [&](int s) { return reinterpret_cast<const uint32_t*>(smem + Cfg::OFF_MAP + size_t(s) * Cfg::MAP_STRIDE); };
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
  const long long ntiles = (long long)((n + TILE - 1) / TILE);
  WsHeader* hdr = args.hdr;
  const uint64_t tmo = args.timeout_ns;
  // ticket k (sequence position) -> physical tile
  auto phys = [&](long long k) { return REVERSE ? ntiles - 1 - k : k; };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], BS == 2 ? 1 : NC);
      ptx::mbar_init(&aggb[s], NC);
      ptx::mbar_init(&prefb[s], 1);
      ptx::mbar_init(&scanned[s], NC);
      *s_cnt(s) = 0u;
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
      // tickets are drawn once a stage is free, so ticket order follows the
      // order in which tiles reach their reduce pass
      for (int k = 0;; ++k) {
        const int s = k % STAGES;
        // traced: the ticket slot holds when the wait for a free stage began
        const unsigned long long tfree = Trace::kOn ? ptx::globaltimer_ns() : 0ull;
        if (k >= STAGES) {
          if (!mbar_wait_bounded(&empty[s], ((k / STAGES) - 1) & 1, hdr, tmo, 0ull)) break;
          pending &= ~(1u << s);
        }
        const long long t = (long long)atomicAdd(&hdr->ticket, 1ull);
        *s_tile(s) = t;
        if (t < ntiles) {
          trace(kTrTicket, t, tfree);
          trace_now(kTrIssue, t);
          const uint64_t base = uint64_t(phys(t)) * TILE;
          const uint64_t valid = (n - base < uint64_t(TILE)) ? (n - base) : uint64_t(TILE);
          const uint32_t bytes = uint32_t(valid * sizeof(in_t)) & ~15u;
          uint32_t map_bytes = 0;
          if constexpr (Heads::kBitmap) {
            map_bytes = uint32_t((valid + 127) / 128) * 16u;
            // reductions: a full tile that is not the array's last brings the
            // next tile's first head bits along (the bitmap is padded past n)
            if (REDUCE && valid == uint64_t(TILE) && base + TILE < n) map_bytes += 16u;
          }
          if (bytes + map_bytes) {
            ptx::mbar_arrive_expect_tx(&full[s], bytes + map_bytes);
            if (bytes)
              ptx::bulk_g2s(smem + size_t(s) * Cfg::TILE_BYTES, in + base * sizeof(in_t), bytes, &full[s], pol_l2);
            if (map_bytes)
              ptx::bulk_g2s(smem + Cfg::OFF_MAP + size_t(s) * Cfg::MAP_STRIDE,
                            reinterpret_cast<const unsigned char*>(sargs.heads) + base / 8, map_bytes, &full[s],
                            pol_l2);
            pending |= 1u << s;
            pend_par = (pend_par & ~(1u << s)) | ((uint32_t(k / STAGES) & 1u) << s);
          } else {
            ptx::mbar_arrive(&full[s]);
          }
        } else {
          ptx::mbar_arrive(&full[s]);
          break;
        }
      }
      for (int s = 0; s < STAGES; ++s)
        if (pending & (1u << s)) mbar_wait_drain(&full[s], (pend_par >> s) & 1u, hdr, tmo);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ look-back
    // (a reduction needs none: its tiles are independent)
    for (int k = 0; !REDUCE; ++k) {
      const int s = k % STAGES;
      const uint32_t par = (k / STAGES) & 1;
      if (!mbar_wait_bounded(&full[s], par, hdr, tmo, 0ull)) break;
      const long long tile = *s_tile(s);
      if (tile >= ntiles) break;
      if (lane == 0) trace_now(kTrFull, tile);
      // exclusive prefix from the predecessors' descriptors while the compute
      // warps still reduce this tile (two polls in flight, 250 ns apart)
      carry_t excl = pol.cid();
      unsigned long long stats = 0;
      if (tile > 0 && !lookback_pipelined<Pol, LBW, 250u>(pol, args.desc, tile, etag, hdr, tmo, lane, excl, stats))
        break;
      if (lane == 0) {
        trace_now(kTrLbDone, tile);
        trace(kTrLbRounds, tile, stats);
      }
      if (!mbar_wait_bounded(&aggb[s], par, hdr, tmo, 0ull)) break;
      if (lane == 0) trace_now(kTrAgg, tile);
      if (tile > 0 && lane == 0)
        codec::publish(args.desc + tile * codec::W, pol.cop(excl, *s_tagg(s)), make_tag(etag, kPrefix));
      if (lane == 0) {
        *s_pref(s) = excl;
        ptx::mbar_arrive(&prefb[s]);
      }
      __syncwarp();
    }
  } else if (BS == 2 && warp == NC + 2) {
    // ------------------------------------------------------------ store
    // Each finished full tile leaves as one bulk copy; the stage is freed as
    // soon as the copy has read it. A partial tile (or an output that is not
    // 16-byte aligned) is stored by the compute warps themselves.
    out_t* gout = static_cast<out_t*>(args.out);
    const bool out_vec = (reinterpret_cast<uintptr_t>(gout) & 15u) == 0;
    const uint64_t pol_l2 = ptx::policy_evict_first();
    for (int k = 0;; ++k) {
      const int s = k % STAGES;
      const uint32_t par = (k / STAGES) & 1;
      if (!mbar_wait_bounded(&full[s], par, hdr, tmo, 0ull)) break;
      const long long tile = *s_tile(s);
      if (tile >= ntiles) break;
      if (!mbar_wait_bounded(&scanned[s], par, hdr, tmo, 0ull)) break;
      const uint64_t base = uint64_t(phys(tile)) * TILE;
      if (lane == 0) {
        if (out_vec && n - base >= uint64_t(TILE)) {
          ptx::bulk_s2g_hint(gout + base, smem + size_t(s) * Cfg::TILE_BYTES, uint32_t(Cfg::TILE_BYTES), pol_l2);
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
    const uint64_t seg_len = sargs.seg_len;

    // Loads logical chunk c of this lane (V consecutive sequence positions).
    // Returns the head bits of the V elements (bit j for element j).
    auto load_chunk = [&](int s, int c, uint64_t base, int valid, int bulk, uint64_t mt, in_t (&x)[V]) -> uint32_t {
      const unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
      const int e0 = w * Cfg::SEG + (c * 32 + lane) * V;  // logical tile offset
      uint32_t hb = 0;
      if (!REVERSE || valid == TILE) {
        // physical positions p_j = e0 + j (forward) or TILE - 1 - (e0 + j) (reverse)
        const int p0 = REVERSE ? TILE - V - e0 : e0;
        if (p0 + V <= bulk) {
          union {
            vec_t u;
            in_t v[V];
          } buf;
          buf.u = *reinterpret_cast<const vec_t*>(stage + size_t(p0) * sizeof(in_t));
#pragma unroll
          for (int j = 0; j < V; ++j) x[j] = buf.v[REVERSE ? V - 1 - j : j];
        } else {
#pragma unroll
          for (int j = 0; j < V; ++j) {
            const int p = REVERSE ? TILE - 1 - (e0 + j) : e0 + j;
            if (p < bulk)
              x[j] = reinterpret_cast<const in_t*>(stage)[p];
            else if (p < valid)
              x[j] = gin[base + p];
            else
              x[j] = identity<decltype(pol.op), in_t>();
          }
        }
      } else {
        // partial tile of a reverse scan: logical e -> physical valid - 1 - e
#pragma unroll
        for (int j = 0; j < V; ++j) {
          const int e = e0 + j;
          const int p = valid - 1 - e;
          if (e < valid)
            x[j] = p < bulk ? reinterpret_cast<const in_t*>(stage)[p] : gin[base + p];
          else
            x[j] = identity<decltype(pol.op), in_t>();
        }
      }
      if constexpr (Heads::kBitmap) {
        const uint32_t word = s_map(s)[e0 >> 5];
        hb = (word >> (e0 & 31)) & ((1u << V) - 1u);
        if (e0 + V > valid) hb &= (e0 >= valid) ? 0u : ((1u << (valid - e0)) - 1u);
      } else {
        // rows of seg_len elements; mt = base % seg_len (one 64-bit modulo per tile)
        const uint64_t len = seg_len;
        // distance D(j) from the tile's base to the element's row boundary:
        // forward  phys = base + e0 + j,          head iff (phys) % len == 0
        // reverse  phys = base + span - 1 - e0 - j, head iff (phys + 1) % len == 0
        //          (span = TILE for full tiles, valid for the partial one)
        const uint64_t span = uint64_t(valid == TILE ? TILE : valid);
#pragma unroll
        for (int j = 0; j < V; ++j) {
          const int e = e0 + j;
          if (e < valid) {
            const uint64_t off = REVERSE ? span - uint64_t(e) : uint64_t(e);  // < 2 * TILE
            const uint64_t r = len > uint64_t(2 * TILE) ? (mt + off >= len ? mt + off - len : mt + off)
                                                        : uint64_t(uint32_t(mt + off) % uint32_t(len));
            hb |= uint32_t(r == 0) << j;
          }
        }
      }
      return hb;
    };
    auto tile_geom = [&](int s, long long& tile, uint64_t& base, int& valid, int& bulk, uint64_t& mt) {
      tile = *s_tile(s);
      base = uint64_t(phys(tile)) * TILE;
      const uint64_t rem = n - base;
      valid = rem < uint64_t(TILE) ? int(rem) : TILE;
      bulk = int((uint32_t(valid * sizeof(in_t)) & ~15u) / sizeof(in_t));
      mt = Heads::kBitmap ? 0 : base % seg_len;
    };
    // rows (LAY 2): V raw elements at tile offset e0 (no head bits)
    auto load_row_vals = [&](int s, int e0, uint64_t base, int valid, int bulk, in_t (&x)[V]) {
      const unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
      if (e0 + V <= bulk) {
        union {
          vec_t u;
          in_t v[V];
        } buf;
        buf.u = *reinterpret_cast<const vec_t*>(stage + size_t(e0) * sizeof(in_t));
#pragma unroll
        for (int j = 0; j < V; ++j) x[j] = buf.v[j];
      } else {
#pragma unroll
        for (int j = 0; j < V; ++j) {
          const int p = e0 + j;
          x[j] = p < bulk ? reinterpret_cast<const in_t*>(stage)[p]
                          : (p < valid ? gin[base + p] : identity<decltype(pol.op), in_t>());
        }
      }
    };
    // rows (LAY 2): head bits of the lane row starting at tile offset r0
    // (bit i for element r0 + i, i < CH * V <= 32) from one 64-bit window of
    // the stage's map, and in `ends` the elements that end their segment: the
    // next element is a head, or the element is the array's last. The element
    // after a full tile that is not the array's last is the next tile's first,
    // whose head bit the map slot holds for reductions.
    auto row_bits = [&](int s, int r0, uint64_t base, int valid, uint32_t& ends) -> uint32_t {
      constexpr int CNT = CH * V;
      auto low = [](int k) -> uint32_t { return k >= 32 ? 0xFFFFFFFFu : ((1u << k) - 1u); };
      const uint32_t w0 = uint32_t(r0) >> 5;
      const uint64_t win = ((uint64_t(s_map(s)[w0 + 1]) << 32) | s_map(s)[w0]) >> (r0 & 31);
      const int nv = valid - r0;  // valid elements of this row
      if (nv >= CNT) {
        const uint32_t h = uint32_t(win) & low(CNT);
        const uint32_t next =
            (nv == CNT && base + uint64_t(valid) >= n) ? 1u : uint32_t(win >> CNT) & 1u;
        ends = (h >> 1) | (next << (CNT - 1));
        return h;
      }
      if (nv > 0) {  // the array's last tile: its last element ends its segment
        const uint32_t h = uint32_t(win) & low(nv);
        ends = ((h >> 1) & low(nv - 1)) | (1u << (nv - 1));
        return h;
      }
      ends = 0u;
      return 0u;
    };
    // reduce: head and end bits of this lane's row in the tile of the last
    // reduce pass (bit c * V + j for element j of chunk c)
    uint32_t row_heads = 0, row_ends = 0;
    auto reduce_pass = [&](int k) -> bool {
      const int s = k % STAGES;
      const unsigned long long tw = Trace::kOn ? ptx::globaltimer_ns() : 0ull;
      if (!mbar_wait_bounded(&full[s], (k / STAGES) & 1, hdr, tmo, 0ull)) return false;
      long long tile;
      uint64_t base, mt;
      int valid, bulk;
      tile_geom(s, tile, base, valid, bulk, mt);
      if (tile >= ntiles) return false;
      if (w == 0 && lane == 0) {
        trace(kTrRWait, tile, tw);
        trace_now(kTrRGot, tile);
      }
      acc_t r = pol.aid();
      if constexpr (LAY == 2) {
        // this lane's row in order; the scan of the (value, count) row totals
        // over the segment is done here, and each row's exclusive prefix stays
        // for the scan pass
        const int r0 = w * Cfg::SEG + lane * (CH * V);
        bool plain_rows = false;  // no lane's row holds a head: every count is zero
        if constexpr (REDUCE) {
          // the only pass over the data: a chunk holding segment ends leaves
          // the row's running value in place of its elements (the stage is
          // not read again but for those), and the row's head and end bits
          // are kept for the totals
          unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
          uint32_t epk = 0;
          const uint32_t hpk = row_bits(s, r0, base, valid, epk);
          // no head and no end in any lane's whole row (one vote instead of
          // one per chunk): plain combines, and nothing to leave in the stage
          if (SKIP && !__any_sync(kFullMask, (hpk | epk) != 0u)) {
            plain_rows = true;
#pragma unroll
            for (int c = 0; c < CH; ++c) {
              in_t x[V];
              load_row_vals(s, r0 + c * V, base, valid, bulk, x);
#pragma unroll
              for (int j = 0; j < V; ++j) r = pol.aop(r, pol.load(x[j], false));
            }
          } else {
#pragma unroll
            for (int c = 0; c < CH; ++c) {
              const int e0 = r0 + c * V;
              in_t x[V];
              load_row_vals(s, e0, base, valid, bulk, x);
              const uint32_t hb = (hpk >> (c * V)) & ((1u << V) - 1u);
              const uint32_t en = (epk >> (c * V)) & ((1u << V) - 1u);
              if (!SKIP || __any_sync(kFullMask, (hb | en) != 0u)) {
                union {
                  vec_t u;
                  out_t v[V];
                } o;
#pragma unroll
                for (int j = 0; j < V; ++j) {
                  r = pol.aop(r, pol.load(x[j], (hb >> j) & 1u));
                  o.v[j] = r.v;
                }
                if (en) *reinterpret_cast<vec_t*>(stage + size_t(e0) * sizeof(in_t)) = o.u;
              } else {
                // no head and no end in any of the warp's chunks: the same
                // combines with those bits known to be zero
#pragma unroll
                for (int j = 0; j < V; ++j) r = pol.aop(r, pol.load(x[j], false));
              }
            }
          }
          row_heads = hpk;
          row_ends = epk;
        } else {
          uint32_t unused_ends;
          const uint32_t hrow = row_bits(s, r0, base, valid, unused_ends);
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            in_t x[V];
            load_row_vals(s, r0 + c * V, base, valid, bulk, x);
            const uint32_t hb = (hrow >> (c * V)) & ((1u << V) - 1u);
#pragma unroll
            for (int j = 0; j < V; ++j) r = pol.aop(r, pol.load(x[j], (hb >> j) & 1u));
          }
        }
        const acc_t inc = plain_rows ? acc_t{warp_inclusive_scan(r.v, pol.op, lane), 0u}
                                     : warp_inclusive_scan(r, aop, lane);
        const acc_t ex = shfl_up(inc, 1);
        s_rows(s)[w * 32 + lane] = lane == 0 ? pol.aid() : ex;
        r = shfl_idx(inc, 31);
      } else {
        for (int c = 0; c < CH; ++c) {
          in_t x[V];
          const uint32_t hb = load_chunk(s, c, base, valid, bulk, mt, x);
          acc_t t = pol.load(x[0], hb & 1u);
#pragma unroll
          for (int j = 1; j < V; ++j) t = pol.aop(t, pol.load(x[j], (hb >> j) & 1u));
          r = pol.aop(r, warp_reduce(t, aop, lane));
        }
      }
      unsigned last = 0;
      if (lane == 0) {
        s_aggs(s)[w] = r;
        __threadfence_block();
        last = atomicAdd(s_cnt(s), 1u) == unsigned(NC - 1);
      }
      if (__shfl_sync(kFullMask, last, 0)) {
        __threadfence_block();
        acc_t x = lane < NC ? s_aggs(s)[lane] : pol.aid();
        x = warp_inclusive_scan(x, aop, lane);
        // each segment's exclusive prefix inside the tile replaces its aggregate
        const acc_t xe = shfl_up(x, 1);
        if (lane < NC) s_aggs(s)[lane] = lane == 0 ? pol.aid() : xe;
        const carry_t agg = pol.to_carry(shfl_idx(x, NC - 1));
        if (lane == 0) {
          *s_tagg(s) = agg;
          *s_cnt(s) = 0u;
          if constexpr (REDUCE) {
            // no look-back: the totals pass works from the tile's start
            SegTileRec<out_t>* rec = static_cast<SegTileRec<out_t>*>(sargs.tile_rec) + tile;
            rec->agg_v = agg.v;
            rec->agg_c = agg.c;
            *s_pref(s) = pol.cid();
            trace_now(kTrAggPub, tile);
            ptx::mbar_arrive(&prefb[s]);
          } else {
            codec::publish(args.desc + tile * codec::W, agg, make_tag(etag, tile == 0 ? kPrefix : kAggregate));
            trace_now(kTrAggPub, tile);
          }
        }
      }
      __syncwarp();
      if (!REDUCE && lane == 0) ptx::mbar_arrive(&aggb[s]);
      __syncwarp();
      return true;
    };

    // scans: the reduce pass runs one tile ahead of the scan pass; reductions
    // finish each tile (totals from tile-local prefixes) before the next
    bool have = reduce_pass(0);
    for (int k = 0; have; ++k) {
      const uint32_t cur_heads = row_heads, cur_ends = row_ends;  // tile k
      const bool have_next = REDUCE ? true : reduce_pass(k + 1);
      const int s = k % STAGES;
      if constexpr (Trace::kOn)
        if (w == 0 && lane == 0) trace_now(kTrPWait, *s_tile(s));
      if (!mbar_wait_bounded(&prefb[s], (k / STAGES) & 1, hdr, tmo, 0ull)) break;
      long long tile;
      uint64_t base, mt;
      int valid, bulk;
      tile_geom(s, tile, base, valid, bulk, mt);
      if (w == 0 && lane == 0) trace_now(kTrSStart, tile);
      const acc_t pw = w == 0 ? *s_pref(s) : pol.aop(*s_pref(s), s_aggs(s)[w]);
      if constexpr (LAY == 2) {
        unsigned char* stage = smem + size_t(s) * Cfg::TILE_BYTES;
        const int r0 = w * Cfg::SEG + lane * (CH * V);
        // the row's prefix inside the segment comes from the reduce pass
        acc_t p = pol.aop(pw, s_rows(s)[w * 32 + lane]);
        if constexpr (REDUCE) {
          // totals of the segments that end in this row, from the running
          // values the reduce pass left at their last elements; the segment
          // that is open where the row begins (no head in the row up to its
          // end) adds the row's prefix
          const uint32_t tbase = cur_ends ? __ldg(sargs.tile_base + tile) : 0u;
          for (uint32_t m = cur_ends; m != 0u; m &= m - 1u) {
            const int i = __ffs(m) - 1;
            const uint32_t h = __popc(cur_heads & (0xFFFFFFFFu >> (31 - i)));  // heads up to element i
            acc_t t = pol.load(reinterpret_cast<const out_t*>(stage)[r0 + i], false);
            if (h == 0) t = pol.aop(p, t);
            const uint32_t cnt = p.c + h;  // heads of the tile up to element i
            if (cnt > 0) {
              static_cast<out_t*>(sargs.rank_out)[tbase + cnt - 1] = t.v;
            } else {
              // the segment open where the tile begins ends here
              SegTileRec<out_t>* rec = static_cast<SegTileRec<out_t>*>(sargs.tile_rec) + tile;
              rec->piece_v = t.v;
              rec->piece_flag = 1u;
            }
          }
          // the stage was written through the generic proxy; the producer's
          // next bulk copy into it is an async-proxy write
          ptx::fence_proxy_async_smem();
        } else {
          // a thread-serial chain per row
          uint32_t unused_ends;
          const uint32_t hrow = row_bits(s, r0, base, valid, unused_ends);
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            in_t x[V];
            load_row_vals(s, r0 + c * V, base, valid, bulk, x);
            const uint32_t hb = (hrow >> (c * V)) & ((1u << V) - 1u);
            const int e0 = r0 + c * V;
            union {
              vec_t u;
              out_t v[V];
            } o;
#pragma unroll
            for (int j = 0; j < V; ++j) {
              const bool head = (hb >> j) & 1u;
              const acc_t before = p;
              p = pol.aop(p, pol.load(x[j], head));
              o.v[j] = excl_kind ? (head ? pol.aid().v : before.v) : p.v;
            }
            *reinterpret_cast<vec_t*>(stage + size_t(e0) * sizeof(in_t)) = o.u;
          }
          if (BS == 2 && (reinterpret_cast<uintptr_t>(gout) & 15u) == 0 && valid == TILE) {
            // a full tile with an aligned output leaves by the store warp's bulk copy
            ptx::fence_proxy_async_smem();
          } else {
            __syncwarp();
#pragma unroll
            for (int c = 0; c < CH; ++c) {
              const int e0 = w * Cfg::SEG + (c * 32 + lane) * V;
              union {
                vec_t u;
                out_t v[V];
              } o;
              o.u = *reinterpret_cast<const vec_t*>(stage + size_t(e0) * sizeof(in_t));
              if (e0 + V <= valid) {
                ptx::st_stream<VB>(gout + base + e0, &o.u);
              } else {
#pragma unroll
                for (int j = 0; j < V; ++j)
                  if (e0 + j < valid) gout[base + e0 + j] = o.v[j];
              }
            }
            // the stage was written through the generic proxy; the next bulk
            // copy into it is an async-proxy write
            ptx::fence_proxy_async_smem();
          }
        }
      } else {
      acc_t X = pol.aid();
      for (int c = 0; c < CH; ++c) {
        in_t x[V];
        const uint32_t hb = load_chunk(s, c, base, valid, bulk, mt, x);
        acc_t a[V];
        a[0] = pol.load(x[0], hb & 1u);
#pragma unroll
        for (int j = 1; j < V; ++j) a[j] = pol.aop(a[j - 1], pol.load(x[j], (hb >> j) & 1u));
        const acc_t inc = warp_inclusive_scan(a[V - 1], aop, lane);
        acc_t ex = shfl_up(inc, 1);
        if (lane == 0) ex = pol.aid();
        const acc_t pc = pol.aop(pw, c == 0 ? ex : pol.aop(X, ex));  // everything before this chunk
        X = (c == 0) ? shfl_idx(inc, 31) : pol.aop(X, shfl_idx(inc, 31));
        const int e0 = w * Cfg::SEG + (c * 32 + lane) * V;
        if constexpr (!REDUCE) {
          union {
            vec_t u;
            out_t v[V];
          } o;
#pragma unroll
          for (int j = 0; j < V; ++j) {
            if (excl_kind) {
              // exclusive: identity at a head, else the inclusive value before
              const acc_t before = j == 0 ? pc : pol.aop(pc, a[j - 1]);
              o.v[j] = ((hb >> j) & 1u) ? pol.aid().v : before.v;
            } else {
              o.v[j] = pol.aop(pc, a[j]).v;
            }
          }
          if (!REVERSE || valid == TILE) {
            const int p0 = REVERSE ? TILE - V - e0 : e0;
            if (p0 + V <= valid) {
              if constexpr (REVERSE) {
                union {
                  vec_t u;
                  out_t v[V];
                } r;
#pragma unroll
                for (int j = 0; j < V; ++j) r.v[j] = o.v[V - 1 - j];
                ptx::st_stream<VB>(gout + base + p0, &r.u);
              } else {
                ptx::st_stream<VB>(gout + base + p0, &o.u);
              }
            } else {
#pragma unroll
              for (int j = 0; j < V; ++j) {
                const int p = REVERSE ? TILE - 1 - (e0 + j) : e0 + j;
                if (p < valid) gout[base + p] = o.v[j];
              }
            }
          } else {
#pragma unroll
            for (int j = 0; j < V; ++j)
              if (e0 + j < valid) gout[base + (valid - 1 - (e0 + j))] = o.v[j];
          }
        } else {
          // segment totals: element e ends a non-empty segment when e + 1 is a
          // head or e is the last element
#pragma unroll
          for (int j = 0; j < V; ++j) {
            const int e = e0 + j;
            if (e >= valid) break;
            bool end;
            const int e1 = e + 1;
            if (base + uint64_t(e1) >= n) {
              end = true;  // the last element of the array ends its segment
            } else if (j + 1 < V) {
              end = (hb >> (j + 1)) & 1u;
            } else {
              // in this tile, or the first element of the next (this tile is
              // full and not the last: its map slot holds that head bit)
              end = (s_map(s)[e1 >> 5] >> (e1 & 31)) & 1u;
            }
            if (end) {
              const acc_t v = pol.aop(pc, a[j]);  // tile-local
              if (v.c > 0) {
                static_cast<out_t*>(sargs.rank_out)[__ldg(sargs.tile_base + tile) + v.c - 1] = v.v;
              } else {
                SegTileRec<out_t>* rec = static_cast<SegTileRec<out_t>*>(sargs.tile_rec) + tile;
                rec->piece_v = v.v;
                rec->piece_flag = 1u;
              }
            }
          }
        }
      }
      }
      __syncwarp();
      if (lane == 0) {
        if (w == 0) trace_now(kTrSDone, tile);
        ptx::mbar_arrive(BS == 2 ? &scanned[s] : &empty[s]);
      }
      have = REDUCE ? reduce_pass(k + 1) : have_next;
    }
  }
  if constexpr (BS == 2) ptx::bulk_wait<0>();  // this thread's bulk stores are complete
  __syncthreads();
  if (threadIdx.x == 0) cta_exit_rearm(hdr, args.desc, uint64_t(ntiles) * codec::W, etag - 1u);
}

// ---------------------------------------------------------------------------
// Pre-pass for CSR segments: head bitmap, empty segments, ranks.
//   heads: bit offsets[s] set for every non-empty segment s (bitmap cleared
//          by the caller);
//   nonempty[s] = 1 for a non-empty segment (input of the rank scan);
//   reduce only: out[s] = identity for every empty segment.
template <class T, class Op>
__global__ void segment_heads_kernel(const int64_t* offsets, uint64_t num_segments, uint64_t n, uint32_t* heads,
                                     uint32_t* nonempty, T* reduce_out) {
  for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < num_segments;
       s += uint64_t(gridDim.x) * blockDim.x) {
    int64_t b = offsets[s], e = offsets[s + 1];
    if (b < 0) b = 0;
    if (e > int64_t(n)) e = int64_t(n);
    const bool ne = e > b;
    if (nonempty) nonempty[s] = ne ? 1u : 0u;
    if (ne) atomicOr(heads + (uint64_t(b) >> 5), 1u << (uint64_t(b) & 31));
    if (reduce_out && !ne) reduce_out[s] = identity<Op, T>();
  }
}

// Segmented reduce, first pass (segment_heads_kernel for reductions): block b
// of the grid takes the contiguous segments [b * 256 * per_thread, (b + 1) *
// 256 * per_thread), each thread `per_thread` consecutive ones; it writes the
// head bitmap, the non-empty flags and the identity of every empty segment,
// and the block's count of non-empty segments to block_count[b].
template <class T, class Op>
__global__ void __launch_bounds__(256) segment_heads_count_kernel(const int64_t* offsets, uint64_t num_segments,
                                                                  uint64_t n, uint64_t per_thread, uint32_t* heads,
                                                                  uint32_t* nonempty, T* reduce_out,
                                                                  uint32_t* block_count) {
  __shared__ uint32_t s_w[8];
  const uint64_t s0 = (uint64_t(blockIdx.x) * 256 + threadIdx.x) * per_thread;
  uint32_t cnt = 0;
  for (uint64_t s = s0; s < s0 + per_thread && s < num_segments; ++s) {
    int64_t b = offsets[s], e = offsets[s + 1];
    if (b < 0) b = 0;
    if (e > int64_t(n)) e = int64_t(n);
    const bool ne = e > b;
    nonempty[s] = ne ? 1u : 0u;
    cnt += ne ? 1u : 0u;
    if (ne) atomicOr(heads + (uint64_t(b) >> 5), 1u << (uint64_t(b) & 31));
    if (!ne) reduce_out[s] = identity<Op, T>();
  }
  const int lane = threadIdx.x & 31;
  cnt = warp_reduce(cnt, plus{}, lane);
  if (lane == 0) s_w[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int i = 0; i < 8; ++i) t += s_w[i];
    block_count[blockIdx.x] = t;
  }
}

// Segmented reduce, second pass: rank[s] = the non-empty segments before s
// (the exclusive scan of the flags), over the blocks of
// segment_heads_count_kernel: a block adds up the counts of the blocks before
// it (at most 1,024) and scans its own flags in order. It also writes base[t],
// the non-empty segments that start before tile t: the non-empty segments
// cover [0, n) without gaps, so every tile start t * tile lies in exactly one
// of them, [a, b), and base[t] is that segment's rank, plus one when the
// segment starts before the tile. A segment covering more than 32 tile starts
// has them written by its whole warp. (A template only so that every
// translation unit including this header may instantiate it.)
template <class Index = int64_t>
__global__ void __launch_bounds__(256) segment_rank_kernel(const Index* offsets, const uint32_t* nonempty,
                                                           uint64_t num_segments, uint64_t n, uint64_t per_thread,
                                                           const uint32_t* block_count, uint64_t tile,
                                                           uint32_t* rank, uint32_t* base) {
  __shared__ uint32_t s_w[8];
  __shared__ uint32_t s_base;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t before = 0;
  for (uint32_t bk = threadIdx.x; bk < blockIdx.x; bk += 256) before += block_count[bk];
  before = warp_reduce(before, plus{}, lane);
  if (lane == 0) s_w[w] = before;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int i = 0; i < 8; ++i) t += s_w[i];
    s_base = t;
  }
  __syncthreads();
  const uint64_t s0 = (uint64_t(blockIdx.x) * 256 + threadIdx.x) * per_thread;
  uint32_t cnt = 0;
  for (uint64_t s = s0; s < s0 + per_thread && s < num_segments; ++s) cnt += nonempty[s];
  const uint32_t inc = warp_inclusive_scan(cnt, plus{}, lane);
  if (lane == 31) s_w[w] = inc;
  __syncthreads();
  uint32_t r = s_base + inc - cnt;
  for (int i = 0; i < w; ++i) r += s_w[i];
  for (uint64_t i = 0; i < per_thread; ++i) {  // the same trip count in every lane
    const uint64_t s = s0 + i;
    uint64_t t0 = 0, t1 = 0;  // tile starts in [t0, t1) lie in this segment
    int64_t a = 0;
    if (s < num_segments) {
      rank[s] = r;
      if (nonempty[s]) {
        a = int64_t(offsets[s]) < 0 ? 0 : int64_t(offsets[s]);
        const int64_t e = int64_t(offsets[s + 1]) > int64_t(n) ? int64_t(n) : int64_t(offsets[s + 1]);
        t0 = (uint64_t(a) + tile - 1) / tile;
        t1 = (uint64_t(e) + tile - 1) / tile;
      }
    }
    const bool long_run = t1 > t0 + 32;
    if (!long_run)
      for (uint64_t t = t0; t < t1; ++t) base[t] = r + (t * tile > uint64_t(a) ? 1u : 0u);
    for (uint32_t m = __ballot_sync(kFullMask, long_run); m != 0u; m &= m - 1u) {
      const int src = __ffs(m) - 1;
      const uint64_t u0 = __shfl_sync(kFullMask, t0, src), u1 = __shfl_sync(kFullMask, t1, src);
      const int64_t ua = __shfl_sync(kFullMask, a, src);
      const uint32_t ur = __shfl_sync(kFullMask, r, src);
      for (uint64_t t = u0 + lane; t < u1; t += 32) base[t] = ur + (t * tile > uint64_t(ua) ? 1u : 0u);
    }
    if (s < num_segments) r += nonempty[s];
  }
}

// Segmented reduce, after the main kernel: per chunk of kSegChunk tiles, the
// heads it holds and the reduction of its tiles' aggregates (used by the
// fix-up to step over long head-free runs of tiles in one go).
constexpr int kSegChunk = 1024;
template <class T, class Op>
__global__ void __launch_bounds__(256) segment_chunk_kernel(const SegTileRec<T>* rec, uint64_t ntiles, T* chunk_v,
                                                            uint32_t* chunk_c) {
  const Op op{};
  __shared__ T s_v[8];
  __shared__ uint32_t s_c[8];
  const uint64_t b = uint64_t(blockIdx.x) * kSegChunk;
  T v = identity<Op, T>();
  uint32_t c = 0;
  for (uint64_t t = b + threadIdx.x; t < b + kSegChunk && t < ntiles; t += 256) {
    v = op(v, rec[t].agg_v);
    c += rec[t].agg_c;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_reduce(v, op, lane);
  c = warp_reduce(c, plus{}, lane);
  if (lane == 0) {
    s_v[w] = v;
    s_c[w] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < 8; ++i) {
      v = op(v, s_v[i]);
      c += s_c[i];
    }
    chunk_v[blockIdx.x] = v;
    chunk_c[blockIdx.x] = c;
  }
}

// Segmented reduce, last: every tile whose record holds a piece (the segment
// open where the tile begins ends inside it) gets the rest of that segment by
// a warp-wide look-back over the earlier tiles' records: 32 tiles per step
// back to the nearest tile with a head, whose aggregate is the segment's value
// from its head; runs of kSegChunk head-free tiles are stepped over with their
// chunk's reduction. The total goes to rank tile_base[t] - 1. Deterministic.
template <class T, class Op>
__global__ void __launch_bounds__(256) segment_fixup_kernel(const SegTileRec<T>* rec, uint64_t ntiles,
                                                            const T* chunk_v, const uint32_t* chunk_c,
                                                            const uint32_t* tile_base, T* rank_out) {
  const Op op{};
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t t = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5; t < ntiles; t += warps) {
    if (!rec[t].piece_flag) continue;  // warp-uniform
    T acc = rec[t].piece_v;            // the piece, then earlier tiles folded in front of it
    long long hi = (long long)t;       // tiles [0, hi) remain
    bool done = false;
    while (!done && hi > 0) {
      if (hi % kSegChunk == 0) {
        const long long ch = hi / kSegChunk - 1;
        if (chunk_c[ch] == 0) {  // a whole head-free chunk
          acc = op(chunk_v[ch], acc);
          hi -= kSegChunk;
          continue;
        }
      }
      const long long u = hi - 1 - lane;  // lane i reads tile hi - 1 - i
      const bool ok = u >= 0 && u >= (hi - 1) / kSegChunk * kSegChunk;  // within this chunk
      T v = identity<Op, T>();
      uint32_t c = 0;
      if (ok) {
        v = rec[u].agg_v;
        c = rec[u].agg_c;
      }
      const uint32_t hm = __ballot_sync(kFullMask, ok && c > 0);
      const uint32_t okm = __ballot_sync(kFullMask, ok);
      const int last = hm ? __ffs(hm) - 1 : 31 - __clz(okm);  // nearest head, else the chunk's first tile
      if (lane > last) v = identity<Op, T>();
      v = warp_reduce_reversed(v, [&](const T& x, const T& y) { return op(x, y); }, lane);  // lanes last .. 0
      acc = op(v, acc);
      if (hm) done = true;
      hi -= last + 1;
    }
    if (lane == 0 && tile_base[t] > 0) rank_out[tile_base[t] - 1] = acc;
  }
}

// out[s] = rank_out[rank[s]] for every non-empty segment (rank = exclusive
// scan of nonempty).
template <class T>
__global__ void segment_gather_kernel(const uint32_t* nonempty, const uint32_t* rank, const T* rank_out,
                                      uint64_t num_segments, T* out) {
  for (uint64_t s = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; s < num_segments;
       s += uint64_t(gridDim.x) * blockDim.x)
    if (nonempty[s]) out[s] = rank_out[rank[s]];
}

}  // namespace pp
