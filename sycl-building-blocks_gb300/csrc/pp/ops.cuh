// Associative operators and their identities.
//
// Mirrors the functor set the reference scans and reduces with (sycl::plus,
// multiplies, bit_and, bit_or, bit_xor, minimum, maximum) and the identity
// table of parallel_primitives::internal::get_init
// (include/parallel_primitives/internal/common.h:41-68):
//   plus -> 0, multiplies -> 1, bit_or / bit_xor -> 0, bit_and -> ~0,
//   minimum -> +inf (floating point) or max(), maximum -> -inf or lowest().
//
// Signed integer plus / multiplies are evaluated in the unsigned type of the
// same width, so overflow wraps (two's complement) instead of being undefined.
// minimum / maximum follow sycl::minimum / sycl::maximum: (a < b) ? a : b and
// (a > b) ? a : b. For floating point, NaN inputs and the sign of a tie between
// -0 and +0 depend on the evaluation order, as they do in the reference.
#pragma once

#include <cstdint>
#include <limits>
#include <type_traits>

#if defined(__CUDACC__)
#define PP_HD __host__ __device__ __forceinline__
#else
#define PP_HD inline
#endif

namespace pp {

struct plus {
  template <class T>
  PP_HD T operator()(const T& a, const T& b) const {
    if constexpr (std::is_integral_v<T> && std::is_signed_v<T>) {
      using U = std::make_unsigned_t<T>;
      return static_cast<T>(static_cast<U>(a) + static_cast<U>(b));
    } else {
      return a + b;
    }
  }
};

struct multiplies {
  template <class T>
  PP_HD T operator()(const T& a, const T& b) const {
    if constexpr (std::is_integral_v<T>) {
      // unsigned short-width types would promote to int; widen explicitly
      using U = std::conditional_t<(sizeof(T) < 4), uint32_t, std::make_unsigned_t<T>>;
      return static_cast<T>(static_cast<U>(a) * static_cast<U>(b));
    } else {
      return a * b;
    }
  }
};

struct bit_and {
  template <class T>
  PP_HD T operator()(const T& a, const T& b) const { return static_cast<T>(a & b); }
};
struct bit_or {
  template <class T>
  PP_HD T operator()(const T& a, const T& b) const { return static_cast<T>(a | b); }
};
struct bit_xor {
  template <class T>
  PP_HD T operator()(const T& a, const T& b) const { return static_cast<T>(a ^ b); }
};
struct minimum {
  template <class T>
  PP_HD T operator()(const T& a, const T& b) const { return (a < b) ? a : b; }
};
struct maximum {
  template <class T>
  PP_HD T operator()(const T& a, const T& b) const { return (a > b) ? a : b; }
};

// Identity element of Op over T. A user-defined functor provides its own by
// specialising op_traits (or by defining a static member `identity<T>()`).
template <class Op, class T, class Enable = void>
struct op_traits {
  static_assert(sizeof(T) == 0, "no known identity for this operator/type: specialise pp::op_traits");
};

template <class T>
struct op_traits<plus, T> {
  PP_HD static T identity() { return T(0); }
};
template <class T>
struct op_traits<multiplies, T> {
  PP_HD static T identity() { return T(1); }
};
template <class T>
struct op_traits<bit_or, T, std::enable_if_t<std::is_integral_v<T>>> {
  PP_HD static T identity() { return T(0); }
};
template <class T>
struct op_traits<bit_xor, T, std::enable_if_t<std::is_integral_v<T>>> {
  PP_HD static T identity() { return T(0); }
};
template <class T>
struct op_traits<bit_and, T, std::enable_if_t<std::is_integral_v<T>>> {
  PP_HD static T identity() { return static_cast<T>(~T(0)); }
};
// Largest / lowest finite-or-infinite value of T, usable in device code
// (std::numeric_limits members are host-only constexpr functions).
template <class T>
PP_HD T max_value() {
  if constexpr (std::is_same_v<T, float>) return __builtin_huge_valf();
  else if constexpr (std::is_same_v<T, double>) return __builtin_huge_val();
  else if constexpr (std::is_unsigned_v<T>) return static_cast<T>(~T(0));
  else return static_cast<T>(static_cast<std::make_unsigned_t<T>>(~std::make_unsigned_t<T>(0)) >> 1);
}
template <class T>
PP_HD T lowest_value() {
  if constexpr (std::is_floating_point_v<T>) return -max_value<T>();
  else if constexpr (std::is_unsigned_v<T>) return T(0);
  else return static_cast<T>(-max_value<T>() - 1);
}

template <class T>
struct op_traits<minimum, T> {
  PP_HD static T identity() { return max_value<T>(); }
};
template <class T>
struct op_traits<maximum, T> {
  PP_HD static T identity() { return lowest_value<T>(); }
};

template <class Op, class T>
PP_HD T identity() { return op_traits<Op, T>::identity(); }

}  // namespace pp
