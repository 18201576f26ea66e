// Scan policies: how an input element becomes an in-tile accumulator, how
// the cross-tile carry (look-back descriptor payload) is represented, and how
// an output element is formed from the carry and the in-tile prefix.
//
//   acc_t    in-tile accumulator (thread / warp / block scans)
//   carry_t  tile aggregate and look-back carry (descriptor payload)
//   pre_t    per-thread prepared carry used to finish outputs
//   row_t    running state of a thread-serial scan along a row of elements
//            (row_start from a prepared carry, then row_incl / row_excl per
//            element, returning the output)
//
// PlainScan is the reference's semantics (one type, one operator).
// CompensatedF32 keeps float-float (hi, lo) pairs everywhere: TwoSum
// accumulation for the tile aggregates, the carries and the in-tile prefixes.
// F64CarryF32 keeps the in-tile work in FP32 and only the cross-tile carry
// chain in FP64.
#pragma once

#include <type_traits>

#include <cuda_runtime.h>

#include "ops.cuh"

namespace pp {

template <class T, class Op>
struct PlainScan {
  using in_t = T;
  using out_t = T;
  using acc_t = T;
  using carry_t = T;
  using pre_t = T;
  Op op;

  __device__ __forceinline__ acc_t load(const in_t& x) const { return x; }
  __device__ __forceinline__ acc_t aop(const acc_t& a, const acc_t& b) const { return op(a, b); }
  __device__ __forceinline__ acc_t aid() const { return identity<Op, T>(); }
  __device__ __forceinline__ carry_t to_carry(const acc_t& a) const { return a; }
  __device__ __forceinline__ carry_t cop(const carry_t& a, const carry_t& b) const { return op(a, b); }
  __device__ __forceinline__ carry_t cid() const { return identity<Op, T>(); }
  __device__ __forceinline__ pre_t prepare(const carry_t& c) const { return c; }
  __device__ __forceinline__ pre_t extend(const pre_t& p, const acc_t& a) const { return op(p, a); }
  __device__ __forceinline__ out_t finish(const pre_t& p, const acc_t& a) const { return op(p, a); }
  __device__ __forceinline__ out_t finish_first(const pre_t& p) const { return p; }
  __device__ __forceinline__ acc_t aop_in(const acc_t& a, const in_t& x) const { return op(a, x); }
  __device__ __forceinline__ in_t in_id() const { return identity<Op, T>(); }
  using row_t = T;
  __device__ __forceinline__ row_t row_start(const pre_t& p) const { return p; }
  __device__ __forceinline__ out_t row_incl(row_t& r, const in_t& x) const {
    r = op(r, x);
    return r;
  }
  __device__ __forceinline__ out_t row_excl(row_t& r, const in_t& x) const {
    const out_t o = r;
    r = op(r, x);
    return o;
  }
};

// float-float pair: value = hi + lo, |lo| <= ulp(hi)/2.
struct ff32 {
  float hi, lo;
};

// Knuth TwoSum: s + e == a + b exactly (round-to-nearest, no FMA involved).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// Dekker FastTwoSum, exact when |a| >= |b| (or a == 0).
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
// Pair + pair without renormalisation: hi carries the rounded sum of the high
// parts, lo collects the low parts and the exact rounding error of hi. The
// pair stays an exact-up-to-u*|lo| representation; |lo| grows by at most half
// an ulp of hi per addition, so chains of a few dozen additions (tile scans)
// stay far from overflowing lo's significance. Renormalise with ff_norm.
__device__ __forceinline__ ff32 ff_add_lazy(const ff32& x, const ff32& y) {
  float s, e;
  two_sum(x.hi, y.hi, s, e);
  return ff32{s, __fadd_rn(e, __fadd_rn(x.lo, y.lo))};
}
__device__ __forceinline__ ff32 ff_norm(const ff32& x) {
  ff32 r;
  fast_two_sum(x.hi, x.lo, r.hi, r.lo);
  return r;
}
// Pair + pair ("sloppy" double-word addition): absolute error O(u^2 (|x|+|y|)).
__device__ __forceinline__ ff32 ff_add(const ff32& x, const ff32& y) {
  float s, e;
  two_sum(x.hi, y.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
  ff32 r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}
// Pair + float.
__device__ __forceinline__ ff32 ff_add_f(const ff32& x, float y) {
  float s, e;
  two_sum(x.hi, y, s, e);
  e = __fadd_rn(e, x.lo);
  ff32 r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}

// In-tile pairs are added lazily (no renormalisation, ff_add_lazy); pairs are
// renormalised when they become carries (descriptors, prefixes).
struct CompensatedF32 {
  using in_t = float;
  using out_t = float;
  using acc_t = ff32;
  using carry_t = ff32;
  using pre_t = ff32;

  __device__ __forceinline__ acc_t load(const float& x) const { return ff32{x, 0.0f}; }
  __device__ __forceinline__ acc_t aop(const acc_t& a, const acc_t& b) const { return ff_add_lazy(a, b); }
  __device__ __forceinline__ acc_t aid() const { return ff32{0.0f, 0.0f}; }
  __device__ __forceinline__ carry_t to_carry(const acc_t& a) const { return ff_norm(a); }
  __device__ __forceinline__ carry_t cop(const carry_t& a, const carry_t& b) const { return ff_add(a, b); }
  __device__ __forceinline__ carry_t cid() const { return ff32{0.0f, 0.0f}; }
  __device__ __forceinline__ pre_t prepare(const carry_t& c) const { return c; }
  __device__ __forceinline__ pre_t extend(const pre_t& p, const acc_t& a) const { return ff_norm(ff_add_lazy(p, a)); }
  __device__ __forceinline__ out_t finish(const pre_t& p, const acc_t& a) const {
    float s, e;
    two_sum(p.hi, a.hi, s, e);
    return __fadd_rn(s, __fadd_rn(e, __fadd_rn(p.lo, a.lo)));
  }
  __device__ __forceinline__ out_t finish_first(const pre_t& p) const { return __fadd_rn(p.hi, p.lo); }
  __device__ __forceinline__ in_t in_id() const { return 0.0f; }
  // pair + element: TwoSum of the high parts, the error joins lo (lazily)
  __device__ __forceinline__ acc_t aop_in(const acc_t& a, float x) const {
    float s, e;
    two_sum(a.hi, x, s, e);
    return ff32{s, __fadd_rn(a.lo, e)};
  }
  // The running prefix is a lazy pair: every element is added with TwoSum,
  // the output is the pair rounded to FP32.
  using row_t = ff32;
  __device__ __forceinline__ row_t row_start(const pre_t& p) const { return p; }
  __device__ __forceinline__ out_t row_incl(row_t& r, float x) const {
    r = aop_in(r, x);
    return __fadd_rn(r.hi, r.lo);
  }
  __device__ __forceinline__ out_t row_excl(row_t& r, float x) const {
    const float o = __fadd_rn(r.hi, r.lo);
    r = aop_in(r, x);
    return o;
  }
  // Fast rows (scan pass): the reduce pass also records max |x| of each row.
  // When the row's starting prefix satisfies |hi| >= (k + 3) * max|x| for a
  // row of k elements, every running hi of the row stays at least max|x| in
  // magnitude, so Dekker's FastTwoSum (3 operations) gives exactly the sum
  // and error TwoSum (6) would: the outputs are the same bit for bit.
  static constexpr bool kRowFast = true;
  using row_info_t = float;
  __device__ __forceinline__ row_info_t row_info_id() const { return 0.0f; }
  __device__ __forceinline__ row_info_t row_info_add(row_info_t m, float x) const { return fmaxf(m, fabsf(x)); }
  __device__ __forceinline__ bool row_fast_ok(const row_t& r, row_info_t m, int k) const {
    return fabsf(r.hi) >= __fmul_rn(float(k + 3), m);
  }
  __device__ __forceinline__ out_t row_incl_fast(row_t& r, float x) const {
    float s, e;
    fast_two_sum(r.hi, x, s, e);
    r = ff32{s, __fadd_rn(r.lo, e)};
    return __fadd_rn(r.hi, r.lo);
  }
  __device__ __forceinline__ out_t row_excl_fast(row_t& r, float x) const {
    const float o = __fadd_rn(r.hi, r.lo);
    float s, e;
    fast_two_sum(r.hi, x, s, e);
    r = ff32{s, __fadd_rn(r.lo, e)};
    return o;
  }
  // Row totals (reduce pass) from the row's max|x| = m: starting the chain at
  // P, a power of two with P >= 64 m, every running sum stays in [P/2, 2P]
  // for rows of up to 31 elements, so each element enters with FastTwoSum
  // (exact) and the total (s - P, lo) is exact too (s - P by Sterbenz's
  // lemma). row_offset returns 0 where that cannot be used (m infinite, NaN
  // or at least 2^120): those rows keep TwoSum.
  __device__ __forceinline__ float row_offset(float m) const {
    const uint32_t ex = (__float_as_uint(m) >> 23) & 0xFFu;  // m < 2^(ex - 126)
    if (!(m < 0x1.0p120f)) return 0.0f;
    return __uint_as_float((ex + 7u) << 23);  // 2^(ex - 120) >= 64 * 2^(ex - 126) > 64 m
  }
  __device__ __forceinline__ void row_offset_add(ff32& r, float x) const {
    float s, e;
    fast_two_sum(r.hi, x, s, e);
    r = ff32{s, __fadd_rn(r.lo, e)};
  }
  __device__ __forceinline__ ff32 row_offset_total(const ff32& r, float p) const {
    return ff32{__fsub_rn(r.hi, p), r.lo};
  }
};

// Policies without a fast row path (kRowFast absent) see these defaults.
template <class Pol, class = void>
struct row_fast_traits {
  static constexpr bool value = false;
  using info_t = int;
  using row_t = typename Pol::row_t;
  using in_t = typename Pol::in_t;
  using out_t = typename Pol::out_t;
  __device__ __forceinline__ static info_t id(const Pol&) { return 0; }
  __device__ __forceinline__ static info_t add(const Pol&, info_t m, const in_t&) { return m; }
  __device__ __forceinline__ static bool ok(const Pol&, const row_t&, info_t, int) { return false; }
  __device__ __forceinline__ static out_t incl(const Pol& p, row_t& r, const in_t& x) { return p.row_incl(r, x); }
  __device__ __forceinline__ static out_t excl(const Pol& p, row_t& r, const in_t& x) { return p.row_excl(r, x); }
};
template <class Pol>
struct row_fast_traits<Pol, std::void_t<decltype(Pol::kRowFast)>> {
  static constexpr bool value = Pol::kRowFast;
  using info_t = typename Pol::row_info_t;
  using row_t = typename Pol::row_t;
  using in_t = typename Pol::in_t;
  using out_t = typename Pol::out_t;
  __device__ __forceinline__ static info_t id(const Pol& p) { return p.row_info_id(); }
  __device__ __forceinline__ static info_t add(const Pol& p, info_t m, const in_t& x) { return p.row_info_add(m, x); }
  __device__ __forceinline__ static bool ok(const Pol& p, const row_t& r, info_t m, int k) {
    return p.row_fast_ok(r, m, k);
  }
  __device__ __forceinline__ static out_t incl(const Pol& p, row_t& r, const in_t& x) { return p.row_incl_fast(r, x); }
  __device__ __forceinline__ static out_t excl(const Pol& p, row_t& r, const in_t& x) { return p.row_excl_fast(r, x); }
};

struct F64CarryF32 {
  using in_t = float;
  using out_t = float;
  using acc_t = float;
  using carry_t = double;
  using pre_t = ff32;

  __device__ __forceinline__ acc_t load(const float& x) const { return x; }
  __device__ __forceinline__ acc_t aop(const acc_t& a, const acc_t& b) const { return __fadd_rn(a, b); }
  __device__ __forceinline__ acc_t aid() const { return 0.0f; }
  __device__ __forceinline__ carry_t to_carry(const acc_t& a) const { return double(a); }
  __device__ __forceinline__ carry_t cop(const carry_t& a, const carry_t& b) const { return __dadd_rn(a, b); }
  __device__ __forceinline__ carry_t cid() const { return 0.0; }
  __device__ __forceinline__ pre_t prepare(const carry_t& c) const {
    const float hi = __double2float_rn(c);
    return ff32{hi, __double2float_rn(__dsub_rn(c, double(hi)))};
  }
  __device__ __forceinline__ pre_t extend(const pre_t& p, const acc_t& a) const { return ff_add_f(p, a); }
  __device__ __forceinline__ out_t finish(const pre_t& p, const acc_t& a) const {
    return __fadd_rn(p.hi, __fadd_rn(p.lo, a));
  }
  __device__ __forceinline__ out_t finish_first(const pre_t& p) const { return __fadd_rn(p.hi, p.lo); }
  __device__ __forceinline__ acc_t aop_in(float a, float x) const { return __fadd_rn(a, x); }
  __device__ __forceinline__ in_t in_id() const { return 0.0f; }
  // FP32 running sum inside the row, added to the prepared carry per output
  struct row_t {
    ff32 p;
    float a;
  };
  __device__ __forceinline__ row_t row_start(const pre_t& p) const { return row_t{p, 0.0f}; }
  __device__ __forceinline__ out_t row_incl(row_t& r, float x) const {
    r.a = __fadd_rn(r.a, x);
    return finish(r.p, r.a);
  }
  __device__ __forceinline__ out_t row_excl(row_t& r, float x) const {
    const float o = finish(r.p, r.a);
    r.a = __fadd_rn(r.a, x);
    return o;
  }
};

}  // namespace pp
