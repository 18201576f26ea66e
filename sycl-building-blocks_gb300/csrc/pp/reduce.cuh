// Device-wide reduction for sm_103a.
//
// Re-design of parallel_primitives::reduce_device / dispatch_kernel_call /
// reduce_device_impl (include/parallel_primitives/reduction.hpp:35-139). The
// reference launches one blocking kernel per unroll level (64 -> 4 -> 1), cuts
// the input into INT32_MAX chunks and finishes through sycl::reduction. Here a
// single persistent launch streams the input with 16-byte non-allocating
// loads (UNROLL independent loads in flight per thread, V accumulators per
// thread to break dependency chains), reduces warps with shuffles and blocks
// through shared memory, and the last block to finish folds the per-block
// partials (all its threads, then a block reduction) and writes the result to
// device memory. For a
// fixed grid the combine order is fixed, so floating-point results are
// reproducible run to run. As with sycl::reduction, the operator must be
// associative and commutative.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "ops.cuh"
#include "warp.cuh"
#include "workspace.cuh"

namespace pp {

struct ReduceArgs {
  const void* in;
  uint64_t n;
  void* result;  // device pointer to one T
  WsHeader* hdr;
  void* partials;  // kMaxPartials slots of 16 bytes
};

// L1-bypassing load of a value another block wrote (after its fence).
template <class T>
__device__ __forceinline__ T ld_cg(const T* p) {
  if constexpr (std::is_arithmetic_v<T> && (sizeof(T) == 4 || sizeof(T) == 8)) {
    return __ldcg(p);
  } else {
    words<T> w;
    const volatile uint32_t* q = reinterpret_cast<const volatile uint32_t*>(p);
#pragma unroll
    for (int i = 0; i < words<T>::W; ++i) w.w[i] = q[i];
    return from_words<T>(w);
  }
}

template <class T, class Op, int BLOCK>
__device__ __forceinline__ T block_reduce(T v, const Op& op, T* s_warp) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  v = warp_reduce(v, op, lane);
  if (lane == 0) s_warp[warp] = v;
  __syncthreads();
  constexpr int NW = BLOCK / 32;
  T r = identity<Op, T>();
  if (warp == 0) {
    T x = lane < NW ? s_warp[lane] : identity<Op, T>();
    r = warp_reduce(x, op, lane);
  }
  return r;  // valid in warp 0
}

template <class T, class Op, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) reduce_kernel(const ReduceArgs args) {
  __shared__ T s_warp[BLOCK / 32];
  __shared__ bool s_last;
  const Op op{};
  const T* in = static_cast<const T*>(args.in);
  const uint64_t n = args.n;
  constexpr int V = (16 % sizeof(T) == 0) ? int(16 / sizeof(T)) : 1;

  T acc[V];
#pragma unroll
  for (int j = 0; j < V; ++j) acc[j] = identity<Op, T>();

  const uint64_t gtid = uint64_t(blockIdx.x) * BLOCK + threadIdx.x;
  const uint64_t gstride = uint64_t(gridDim.x) * BLOCK;

  uint64_t head = 0, nv = 0;
  if constexpr (V > 1) {
    const uintptr_t addr = reinterpret_cast<uintptr_t>(in);
    head = ((16u - (addr & 15u)) & 15u) / sizeof(T);  // the host guarantees addr % sizeof(T) == 0
    if (head > n) head = n;
    nv = (n - head) / V;
    const uint4* vin = reinterpret_cast<const uint4*>(in + head);
    union U {
      uint4 u;
      T x[V];
    };
    uint64_t i = gtid;
    for (; i + uint64_t(UNROLL - 1) * gstride < nv; i += uint64_t(UNROLL) * gstride) {
      U v[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) v[u].u = ptx::ld_stream_v4(vin + i + u * gstride);
#pragma unroll
      for (int u = 0; u < UNROLL; ++u)
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = op(acc[j], v[u].x[j]);
    }
    for (; i < nv; i += gstride) {
      U v;
      v.u = ptx::ld_stream_v4(vin + i);
#pragma unroll
      for (int j = 0; j < V; ++j) acc[j] = op(acc[j], v.x[j]);
    }
  }
  // head (before the first 16-byte boundary) and tail (after the last full vector)
  const uint64_t tail = head + nv * V;
  for (uint64_t i = gtid; i < head; i += gstride) acc[0] = op(acc[0], in[i]);
  for (uint64_t i = tail + gtid; i < n; i += gstride) acc[0] = op(acc[0], in[i]);

  T t = acc[0];
#pragma unroll
  for (int j = 1; j < V; ++j) t = op(t, acc[j]);
  t = block_reduce<T, Op, BLOCK>(t, op, s_warp);

  static_assert(sizeof(T) <= 16, "partial slots hold at most 16 bytes");
  constexpr int STRIDE = int(16 / sizeof(T));
  T* partials = static_cast<T*>(args.partials);
  if (threadIdx.x == 0) {
    if (gridDim.x == 1) {
      *static_cast<T*>(args.result) = t;
      s_last = false;
    } else {
      partials[size_t(blockIdx.x) * STRIDE] = t;
      __threadfence();
      const unsigned prev = atomicAdd(&args.hdr->done, 1u);
      s_last = (prev == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!s_last) return;
  // last block: every thread folds its share of the partials (one round trip
  // to the L2 instead of one per 32 blocks), then one block reduction; the
  // order is fixed for a fixed grid
  __threadfence();
  T r = identity<Op, T>();
  for (unsigned b = threadIdx.x; b < gridDim.x; b += BLOCK) r = op(r, ld_cg(partials + size_t(b) * STRIDE));
  r = block_reduce<T, Op, BLOCK>(r, op, s_warp);
  if (threadIdx.x == 0) {
    *static_cast<T*>(args.result) = r;
    args.hdr->done = 0u;
  }
}

}  // namespace pp
