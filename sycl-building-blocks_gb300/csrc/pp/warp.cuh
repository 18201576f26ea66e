// Warp-level building blocks: shuffles of any trivially-copyable type,
// Kogge-Stone inclusive scan over the 32 lanes and an order-preserving
// reduction. All of them keep the combine order of the sequence (older
// operand on the left), so they are correct for associative operators that
// are not commutative.
#pragma once

#include <cstdint>
#include <cstring>
#include <type_traits>
#include <cuda_runtime.h>

namespace pp {

constexpr uint32_t kFullMask = 0xffffffffu;

template <class T>
struct words {
  static constexpr int W = (sizeof(T) + 3) / 4;
  uint32_t w[W];
};

template <class T>
__device__ __forceinline__ words<T> to_words(const T& v) {
  words<T> r;
  if constexpr (sizeof(T) % 4 != 0) r.w[words<T>::W - 1] = 0;
  memcpy(&r, &v, sizeof(T));
  return r;
}
template <class T>
__device__ __forceinline__ T from_words(const words<T>& r) {
  T v;
  memcpy(&v, &r, sizeof(T));
  return v;
}

template <class T>
__device__ __forceinline__ T shfl_idx(const T& v, int src) {
  if constexpr ((sizeof(T) == 4 || sizeof(T) == 8) && std::is_arithmetic_v<T>) {
    return __shfl_sync(kFullMask, v, src);
  } else {
    words<T> r = to_words(v);
#pragma unroll
    for (int i = 0; i < words<T>::W; ++i) r.w[i] = __shfl_sync(kFullMask, r.w[i], src);
    return from_words<T>(r);
  }
}

template <class T>
__device__ __forceinline__ T shfl_up(const T& v, int d) {
  if constexpr ((sizeof(T) == 4 || sizeof(T) == 8) && std::is_arithmetic_v<T>) {
    return __shfl_up_sync(kFullMask, v, d);
  } else {
    words<T> r = to_words(v);
#pragma unroll
    for (int i = 0; i < words<T>::W; ++i) r.w[i] = __shfl_up_sync(kFullMask, r.w[i], d);
    return from_words<T>(r);
  }
}

template <class T>
__device__ __forceinline__ T shfl_down(const T& v, int d) {
  if constexpr ((sizeof(T) == 4 || sizeof(T) == 8) && std::is_arithmetic_v<T>) {
    return __shfl_down_sync(kFullMask, v, d);
  } else {
    words<T> r = to_words(v);
#pragma unroll
    for (int i = 0; i < words<T>::W; ++i) r.w[i] = __shfl_down_sync(kFullMask, r.w[i], d);
    return from_words<T>(r);
  }
}

// Inclusive Kogge-Stone scan across the warp: lane l returns v_0 op ... op v_l.
template <class T, class Op>
__device__ __forceinline__ T warp_inclusive_scan(T v, const Op& op, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = shfl_up(v, d);
    if (lane >= d) v = op(o, v);
  }
  return v;
}

// Inclusive scan over the first `width` lanes (width a power of two <= 32).
template <class T, class Op, int WIDTH>
__device__ __forceinline__ T warp_inclusive_scan_w(T v, const Op& op, int lane) {
#pragma unroll
  for (int d = 1; d < WIDTH; d <<= 1) {
    T o = shfl_up(v, d);
    if ((lane & (WIDTH - 1)) >= d) v = op(o, v);
  }
  return v;
}

// Reduction in lane order: every lane returns v_0 op v_1 op ... op v_31.
template <class T, class Op>
__device__ __forceinline__ T warp_reduce(T v, const Op& op, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = shfl_down(v, d);
    if (lane + d < 32) v = op(v, o);
  }
  return shfl_idx(v, 0);
}

// Reduction where lane 0 holds the NEWEST element and lane 31 the oldest
// (the look-back window): returns v_31 op ... op v_1 op v_0 on every lane.
template <class T, class Op>
__device__ __forceinline__ T warp_reduce_reversed(T v, const Op& op, int lane) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    T o = shfl_down(v, d);
    if (lane + d < 32) v = op(o, v);
  }
  return shfl_idx(v, 0);
}

}  // namespace pp
