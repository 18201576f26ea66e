// parallel_primitives/intrinsics.hpp - native CUDA versions of the
// reference's SYCL intrinsics (include/intrinsics.hpp, namespace sycl::ext).
//
// Bit intrinsics map to the sm_103a instructions (__brev, __funnelshift_*,
// __popc, __byte_perm); warp-level ones (the reference's sub-group functions)
// act on the calling warp and must be called by all 32 lanes.
//
// One deliberate divergence: funnelshift_l / funnelshift_r follow CUDA's
// wrap semantics (shift & 31). The reference reduces the shift with
// `shift % 31` (include/intrinsics.hpp:52-63), which agrees for shifts 0..30
// and differs from 31 on (its shift of 31 even shifts a 32-bit value by 32).
#pragma once

#include <cstdint>
#include <type_traits>

#include <cuda_runtime.h>

#if defined(__CUDACC__)
#define PP_INTR_HD __host__ __device__ __forceinline__
#else
#define PP_INTR_HD inline
#endif

namespace parallel_primitives::ext {

// (lo, hi) funnel shifts: the upper / lower 32 bits of (hi:lo) << / >> (shift & 31)
PP_INTR_HD uint32_t funnelshift_l(uint32_t lo, uint32_t hi, uint32_t shift) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, shift);
#else
  const uint64_t v = (uint64_t(hi) << 32) | lo;
  return uint32_t((v << (shift & 31u)) >> 32);
#endif
}

PP_INTR_HD uint32_t funnelshift_r(uint32_t lo, uint32_t hi, uint32_t shift) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(lo, hi, shift);
#else
  const uint64_t v = (uint64_t(hi) << 32) | lo;
  return uint32_t(v >> (shift & 31u));
#endif
}

PP_INTR_HD uint32_t brev32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __brev(x);
#else
  uint32_t r = 0;
  for (int i = 0; i < 32; ++i) r |= ((x >> i) & 1u) << (31 - i);
  return r;
#endif
}

PP_INTR_HD uint64_t brev64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __brevll(x);
#else
  uint64_t r = 0;
  for (int i = 0; i < 64; ++i) r |= ((x >> i) & 1ull) << (63 - i);
  return r;
#endif
}

PP_INTR_HD uint32_t popcount(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return uint32_t(__popc(x));
#else
  return uint32_t(__builtin_popcount(x));
#endif
}

PP_INTR_HD uint32_t upsample(uint16_t hi, uint16_t lo) { return (uint32_t(hi) << 16) | lo; }

// Four bytes, most significant first (reference :138-148).
PP_INTR_HD uint32_t upsample(uint8_t hi_hi, uint8_t hi, uint8_t lo, uint8_t lo_lo) {
  return (uint32_t(hi_hi) << 24) | (uint32_t(hi) << 16) | (uint32_t(lo) << 8) | uint32_t(lo_lo);
}

template <class T>
PP_INTR_HD uint8_t get_byte(T word, uint32_t position) {
  static_assert(std::is_unsigned_v<T>, "unsigned words only");
  return uint8_t((word >> (8 * position)) & 0xFFu);
}

template <class T>
PP_INTR_HD T set_byte(T word, uint8_t byte, uint32_t position) {
  static_assert(std::is_unsigned_v<T>, "unsigned words only");
  const T mask = static_cast<T>(~(T(0xFF) << (8 * position)));
  return static_cast<T>((word & mask) | (T(byte) << (8 * position)));
}

template <bool Bit, class T>
PP_INTR_HD T set_bit_in_word(T word, uint32_t idx) {
  static_assert(std::is_unsigned_v<T>, "unsigned words only");
  if constexpr (Bit) return static_cast<T>(word | (T(1) << idx));
  else return static_cast<T>(word & ~(T(1) << idx));
}

template <class T>
PP_INTR_HD T set_bit_in_word(T word, uint32_t idx, bool bit) {
  return bit ? set_bit_in_word<true>(word, idx) : set_bit_in_word<false>(word, idx);
}

template <class T>
PP_INTR_HD bool read_bit(T word, uint32_t idx) {
  static_assert(std::is_unsigned_v<T>, "unsigned words only");
  return ((word >> idx) & T(1)) != 0;
}

template <class T>
PP_INTR_HD T flip_bit(T word, uint32_t idx) {
  static_assert(std::is_unsigned_v<T>, "unsigned words only");
  return static_cast<T>(word ^ (T(1) << idx));
}

#if defined(__CUDACC__)

// L1 prefetch of a global address (hand-written PTX, as the reference).
template <class T>
__device__ __forceinline__ void prefetch(const T* ptr) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(ptr));
}
// Uniform (constant-cache) prefetch.
template <class T>
__device__ __forceinline__ void prefetch_constant(const T* ptr) {
  asm volatile("prefetchu.L1 [%0];" ::"l"(ptr));
}

// Bit i set when pred(i) holds, i over the 32 lanes (reference :204-212).
template <class F>
__device__ __forceinline__ uint32_t predicate_to_mask(F&& pred) {
  uint32_t m = 0;
#pragma unroll
  for (int i = 0; i < 32; ++i) m |= uint32_t(pred(i) ? 1u : 0u) << i;
  return m;
}

__device__ __forceinline__ uint32_t ballot(int predicate) { return __ballot_sync(0xffffffffu, predicate != 0); }

// Lanes holding the same value as this lane (reference :221-230).
template <class T>
__device__ __forceinline__ uint32_t match_any(T val) {
  if constexpr (sizeof(T) == 4 || sizeof(T) == 8) {
    return __match_any_sync(0xffffffffu, val);
  } else {
    return __match_any_sync(0xffffffffu, static_cast<unsigned long long>(val));
  }
}

// True when every lane in `mask` holds the value of the lowest lane of
// `mask` (reference :233-240); false for an empty mask.
template <class T>
__device__ __forceinline__ bool match_all(uint32_t mask, T val) {
  if (mask == 0) return false;
  const int leader = __ffs(mask) - 1;
  const T lv = __shfl_sync(0xffffffffu, val, leader);
  return mask == (__ballot_sync(0xffffffffu, val == lv) & mask);
}

template <class T>
__device__ __forceinline__ T broadcast_leader(T val) {
  return __shfl_sync(0xffffffffu, val, 0);
}

#endif  // __CUDACC__

}  // namespace parallel_primitives::ext
