// Carry propagation between consecutive chunks of one long scan: the host
// entry points stream an array through the GPU in chunks (copy in, scan,
// copy out on three streams), so chunk i is scanned on its own and then
// offset by everything before it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ops.cuh"

namespace pp {

// carry_next <- total of everything up to and including the last element of
// this chunk, from the chunk's (already offset) output: the last inclusive
// output, or for an exclusive scan the last output combined with the last
// input.
template <class T, class Op>
__device__ __forceinline__ T chunk_total(const T& out_last, const T& in_last, bool exclusive) {
  const Op op{};
  return exclusive ? op(out_last, in_last) : out_last;
}

// First chunk: nothing to offset, only the running total to record.
template <class T, class Op>
__global__ void carry_first_kernel(const T* out, const T* in, uint64_t n, T* carry_next, int exclusive) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && n > 0) *carry_next = chunk_total<T, Op>(out[n - 1], in[n - 1], exclusive != 0);
}

// out[i] = carry_prev op out[i] over the chunk (16-byte vectors; the chunk
// buffers are allocated by the library, so `out` is 256-byte aligned); the
// thread that offsets the last element records the new running total.
template <class T, class Op>
__global__ void __launch_bounds__(256) carry_apply_kernel(T* out, const T* in, uint64_t n, const T* carry_prev,
                                                          T* carry_next, int exclusive) {
  constexpr int V = 16 / sizeof(T);
  const Op op{};
  const T c = *carry_prev;
  const uint64_t nv = n / V;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < nv; i += stride) {
    union {
      uint4 u;
      T x[V];
    } b;
    b.u = reinterpret_cast<const uint4*>(out)[i];
#pragma unroll
    for (int j = 0; j < V; ++j) b.x[j] = op(c, b.x[j]);
    reinterpret_cast<uint4*>(out)[i] = b.u;
    if (i * V + V == n) *carry_next = chunk_total<T, Op>(b.x[V - 1], in[n - 1], exclusive != 0);
  }
  if (blockIdx.x == 0 && threadIdx.x < n - nv * V) {
    const uint64_t k = nv * V + threadIdx.x;
    const T y = op(c, out[k]);
    out[k] = y;
    if (k == n - 1) *carry_next = chunk_total<T, Op>(y, in[n - 1], exclusive != 0);
  }
}

}  // namespace pp
