// Independent scans of the rows of a row-major matrix, one warp per row.
//
// A row of a few hundred or more elements is long enough to keep a warp
// streaming, and a matrix with many rows has enough of them to fill the GPU,
// so no row needs to wait for another: each warp walks its row front to back
// (or back to front for reverse scans) in steps of 32 lanes x V elements,
// carrying the running prefix in a register. Loads for U steps are issued
// before the first of them is scanned, which keeps U x 512 bytes per warp in
// flight; with 48 warps per SM that is enough to stream at HBM speed. Short
// rows or few long rows take the segmented decoupled-look-back kernel
// instead (the host picks).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ops.cuh"
#include "ptx.cuh"
#include "warp.cuh"

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

}  // namespace pp
