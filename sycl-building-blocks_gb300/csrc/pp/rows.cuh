// Independent scans of the rows of a row-major matrix.
//
// rows_warp_kernel: one warp per row. A row of a few hundred or more elements
// is long enough to keep a warp streaming, and a matrix with many rows has
// enough of them to fill the GPU, so no row needs to wait for another: each
// warp walks its row front to back (or back to front for reverse scans) in
// steps of 32 lanes x V elements, carrying the running prefix in a register.
// Loads for U steps are issued before the first of them is scanned, which
// keeps U x 512 bytes per warp in flight.
// rows_tile_kernel (below): rows whose length tiles a 64 KB shared-memory
// stage stream through a ring of stages as contiguous whole-row tiles.
// Short rows or few long rows take the segmented decoupled-look-back kernel
// instead (the host picks).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ops.cuh"
#include "ptx.cuh"
#include "warp.cuh"
#include "workspace.cuh"

namespace pp {

template <class T>
__device__ __forceinline__ uint4 ld_stream_u4(const T* p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

// V elements per lane per step (V * sizeof(T) == 16 for the vector path,
// V == 1 for rows that are not 16-byte aligned), U steps in flight.
template <class T, class Op, bool REVERSE, int V, int U>
__global__ void __launch_bounds__(256) rows_warp_kernel(const T* __restrict__ in, T* __restrict__ out, uint64_t rows,
                                                        uint64_t cols, int exclusive) {
  static_assert(V == 1 || V * sizeof(T) == 16, "vector steps are 16 bytes");
  const Op op{};
  const T id = identity<Op, T>();
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  const uint64_t nvec = cols / V;  // whole steps of V elements (cols % V == 0 on the vector path)
  auto opf = [&](const T& a, const T& b) { return op(a, b); };
  for (uint64_t row = warp; row < rows; row += nwarps) {
    const T* rin = in + row * cols;
    T* rout = out + row * cols;
    T carry = id;
    for (uint64_t q0 = 0; q0 < nvec; q0 += uint64_t(32) * U) {
      union Vec {
        uint4 u;
        T x[V];
      };
      Vec buf[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint64_t q = q0 + uint64_t(u) * 32 + lane;  // step index along the scan direction
        if (q < nvec) {
          const uint64_t qp = REVERSE ? nvec - 1 - q : q;
          if constexpr (V == 1) {
            buf[u].x[0] = __ldg(rin + qp);
          } else {
            buf[u].u = ld_stream_u4(rin + qp * V);
          }
        } else {
#pragma unroll
          for (int j = 0; j < V; ++j) buf[u].x[j] = id;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (q0 + uint64_t(u) * 32 >= nvec) break;  // warp-uniform
        const uint64_t q = q0 + uint64_t(u) * 32 + lane;
        // elements of this step in scan order
        T a[V];
#pragma unroll
        for (int j = 0; j < V; ++j) a[j] = buf[u].x[REVERSE ? V - 1 - j : j];
        T loc[V];
        loc[0] = a[0];
#pragma unroll
        for (int j = 1; j < V; ++j) loc[j] = op(loc[j - 1], a[j]);
        const T inc = warp_inclusive_scan(loc[V - 1], opf, lane);
        T ex = shfl_up(inc, 1);
        if (lane == 0) ex = id;
        const T pre = op(carry, ex);  // everything before this lane's first element
        Vec o;
#pragma unroll
        for (int j = 0; j < V; ++j) {
          const T v = exclusive ? (j == 0 ? pre : op(pre, loc[j - 1])) : op(pre, loc[j]);
          o.x[REVERSE ? V - 1 - j : j] = v;
        }
        if (q < nvec) {
          const uint64_t qp = REVERSE ? nvec - 1 - q : q;
          if constexpr (V == 1) {
            rout[qp] = o.x[0];
          } else {
            ptx::st_stream_v4(rout + qp * V, o.u);
          }
        }
        carry = op(carry, shfl_idx(inc, 31));
      }
    }
  }
}


// ---------------------------------------------------------------------------
// Rows whose length is a multiple of one compute warp's segment and divides a
// 64 KB tile: the matrix streams through a ring of shared-memory stages as
// contiguous tiles of whole rows (one bulk copy per tile, like a flat copy,
// instead of one DRAM stream per warp), and no row crosses a tile, so tiles
// need no look-back. Each row spans P = cols / SEG compute warps: every warp
// reduces its segment, the warps of a row exchange their totals through
// shared memory, and each scans its segment with the total of the segments
// before it (after it, for suffix scans). Persistent CTAs take tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...; every wait is bounded.
template <class T, int NC_, int CH_, int STAGES_>
struct RowsTileCfg {
  static constexpr int NC = NC_;          // compute warps
  static constexpr int CH = CH_;          // 16-byte chunks per lane per segment
  static constexpr int STAGES = STAGES_;  // shared-memory ring depth
  static constexpr int V = 16 / int(sizeof(T));
  static constexpr int SEG = 32 * CH * V;  // elements per compute warp
  static constexpr int TILE = NC * SEG;
  static constexpr int TILE_BYTES = TILE * int(sizeof(T));
  static constexpr int THREADS = (NC + 1) * 32;  // producer warp + compute warps
  static constexpr size_t OFF_TOT = size_t(STAGES) * TILE_BYTES;  // T[STAGES][NC] segment totals
  static constexpr size_t OFF_BAR = (OFF_TOT + size_t(STAGES) * NC * sizeof(T) + 15) / 16 * 16;
  static constexpr size_t SMEM = OFF_BAR + 3 * size_t(STAGES) * 8;  // full, empty, totals-ready
  // the tile kernel takes rows of P segments, P dividing NC
  static bool fits(uint64_t cols) {
    if (cols == 0 || cols % SEG != 0) return false;
    const uint64_t p = cols / SEG;
    return p <= uint64_t(NC) && NC % p == 0;
  }
};

template <class T, class Op, bool REVERSE, int NC, int CH, int STAGES>
__global__ void __launch_bounds__((NC + 1) * 32, 1) rows_tile_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                                     uint64_t rows, uint64_t cols, int exclusive,
                                                                     WsHeader* hdr, uint64_t tmo) {
  using Cfg = RowsTileCfg<T, NC, CH, STAGES>;
  constexpr int V = Cfg::V;
  constexpr int SEG = Cfg::SEG;
  extern __shared__ __align__(128) unsigned char smem[];
  T* s_tot = reinterpret_cast<T*>(smem + Cfg::OFF_TOT);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Cfg::OFF_BAR);
  uint64_t* empty = full + STAGES;
  uint64_t* totb = full + 2 * STAGES;
  const Op op{};
  const T id = identity<Op, T>();
  auto opf = [&](const T& a, const T& b) { return op(a, b); };
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int P = int(cols / SEG);  // warps per row
  const int R = NC / P;           // rows per tile
  const long long ntiles = (long long)((rows + R - 1) / R);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], NC);
      ptx::mbar_init(&totb[s], NC);
    }
    ptx::fence_mbar_init();
  }
  __syncthreads();

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      const uint64_t pol_l2 = ptx::policy_evict_first();
      int k = 0;
      for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
        const int s = k % STAGES;
        if (k >= STAGES && !mbar_wait_bounded(&empty[s], uint32_t((k / STAGES) - 1) & 1u, hdr, tmo, 0ull)) break;
        const uint64_t r0 = uint64_t(t) * R;
        const uint64_t nr = rows - r0 < uint64_t(R) ? rows - r0 : uint64_t(R);
        const uint32_t bytes = uint32_t(nr * cols * sizeof(T));
        ptx::mbar_arrive_expect_tx(&full[s], bytes);
        ptx::bulk_g2s(smem + size_t(s) * Cfg::TILE_BYTES, in + r0 * cols, bytes, &full[s], pol_l2);
      }
      // copies still in flight land before the CTA may exit
      for (int s = 0; s < STAGES; ++s) {
        const int last = s + ((k - 1 - s) / STAGES) * STAGES;
        if (last >= 0 && last < k) mbar_wait_bounded(&full[s], uint32_t(last / STAGES) & 1u, hdr, tmo, 0ull);
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ compute
    const int w = warp - 1;
    const int rit = w / P;   // row of this warp inside the tile
    const int pos = w % P;   // segment of this warp inside its row
    int k = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int s = k % STAGES;
      const uint32_t par = uint32_t(k / STAGES) & 1u;
      if (!mbar_wait_bounded(&full[s], par, hdr, tmo, 0ull)) break;
      const uint64_t r0 = uint64_t(t) * R;
      const bool active = r0 + rit < rows;
      const T* seg = reinterpret_cast<const T*>(smem + size_t(s) * Cfg::TILE_BYTES) + size_t(w) * SEG;
      union Vec {
        uint4 u;
        T x[V];
      };
      // pass 1: the total of this warp's segment
      T tot = id;
      if (active) {
        T acc[V];
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = id;
#pragma unroll 4
        for (int c = 0; c < CH; ++c) {
          Vec b;
          b.u = reinterpret_cast<const uint4*>(seg)[c * 32 + lane];
#pragma unroll
          for (int j = 0; j < V; ++j) acc[j] = op(acc[j], b.x[j]);
        }
#pragma unroll
        for (int j = 0; j < V; ++j) tot = op(tot, acc[j]);
        tot = warp_reduce(tot, opf, lane);
      }
      if (lane == 0) {
        s_tot[s * NC + w] = tot;
        ptx::mbar_arrive(&totb[s]);
      }
      if (!mbar_wait_bounded(&totb[s], par, hdr, tmo, 0ull)) break;
      // pass 2: this segment's scan, carried in from the row's other segments
      if (active) {
        T carry = id;
        // lanes fold the totals of the row's segments before (after) this one
        T other = id;
        if (lane < P && (REVERSE ? lane > pos : lane < pos)) other = s_tot[s * NC + rit * P + lane];
        carry = warp_reduce(other, opf, lane);
        T* gout = out + (r0 + rit) * cols + size_t(pos) * SEG;
        if constexpr (!REVERSE) {
#pragma unroll 2
          for (int c = 0; c < CH; ++c) {
            Vec b;
            b.u = reinterpret_cast<const uint4*>(seg)[c * 32 + lane];
            T loc[V];
            loc[0] = b.x[0];
#pragma unroll
            for (int j = 1; j < V; ++j) loc[j] = op(loc[j - 1], b.x[j]);
            const T inc = warp_inclusive_scan(loc[V - 1], opf, lane);
            T ex = shfl_up(inc, 1);
            if (lane == 0) ex = id;
            const T pre = op(carry, ex);
            Vec o;
#pragma unroll
            for (int j = 0; j < V; ++j) o.x[j] = exclusive ? (j == 0 ? pre : op(pre, loc[j - 1])) : op(pre, loc[j]);
            ptx::st_stream_v4(gout + size_t(c * 32 + lane) * V, o.u);
            carry = op(carry, shfl_idx(inc, 31));
          }
        } else {
#pragma unroll 2
          for (int c = CH - 1; c >= 0; --c) {
            Vec b;
            b.u = reinterpret_cast<const uint4*>(seg)[c * 32 + lane];
            T suf[V];  // suffix inside the lane's V elements
            suf[V - 1] = b.x[V - 1];
#pragma unroll
            for (int j = V - 2; j >= 0; --j) suf[j] = op(b.x[j], suf[j + 1]);
            T inc = suf[0];  // suffix scan over lanes: lane l holds lanes l..31
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
              const T o2 = shfl_down(inc, d);
              if (lane + d < 32) inc = op(inc, o2);
            }
            T ex = shfl_down(inc, 1);
            if (lane == 31) ex = id;
            const T pre = op(carry, ex);
            Vec o;
#pragma unroll
            for (int j = 0; j < V; ++j)
              o.x[j] = exclusive ? (j == V - 1 ? pre : op(pre, suf[j + 1])) : op(pre, suf[j]);
            ptx::st_stream_v4(gout + size_t(c * 32 + lane) * V, o.u);
            carry = op(carry, shfl_idx(inc, 0));
          }
        }
      }
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&empty[s]);
    }
  }
}

}  // namespace pp
