// Definitions of the typed dispatch functions declared in dispatch.cuh.
#pragma once

#include <type_traits>

#include "dispatch.cuh"
#include "pp/carry.cuh"

namespace pp {
namespace capi {

template <class Pol>
Status scan_policy(const ScanReq& r) {
  switch (r.algo) {
    case PP_ALGO_AUTO:
    case PP_ALGO_DECOUPLED:
      return host::decoupled_scan<Pol>(r.s, r.in, r.out, r.n, r.exclusive, r.ws, r.ws_bytes, 0);
    case PP_ALGO_SINGLE_GROUP:
      return host::decoupled_scan<Pol>(r.s, r.in, r.out, r.n, r.exclusive, r.ws, r.ws_bytes, 1);
    case PP_ALGO_COOPERATIVE:
      return host::cooperative_scan<Pol>(r.s, r.in, r.out, r.n, r.exclusive, r.ws, r.ws_bytes, 0);
  }
  return Status::invalid_arg;
}

template <class Pol>
size_t workspace_policy(pp_scan_algo algo, const void* in, const void* out, uint64_t n) {
  if (algo == PP_ALGO_COOPERATIVE) return host::cooperative_workspace_bytes<Pol>(n, in, out);
  return host::decoupled_workspace_bytes<Pol>(n, in, out);
}

template <class T>
Status scan_typed(const ScanReq& r) {
  switch (r.op) {
    case PP_OP_PLUS:
      return scan_policy<PlainScan<T, plus>>(r);
    case PP_OP_MULTIPLIES:
      return scan_policy<PlainScan<T, multiplies>>(r);
    case PP_OP_MINIMUM:
      return scan_policy<PlainScan<T, minimum>>(r);
    case PP_OP_MAXIMUM:
      return scan_policy<PlainScan<T, maximum>>(r);
    case PP_OP_BIT_AND:
    case PP_OP_BIT_OR:
    case PP_OP_BIT_XOR:
      if constexpr (std::is_integral_v<T>) {
        if (r.op == PP_OP_BIT_AND) return scan_policy<PlainScan<T, bit_and>>(r);
        if (r.op == PP_OP_BIT_OR) return scan_policy<PlainScan<T, bit_or>>(r);
        return scan_policy<PlainScan<T, bit_xor>>(r);
      } else {
        return Status::unsupported;
      }
  }
  return Status::invalid_arg;
}

template <class T>
Status reduce_typed(cudaStream_t s, pp_op op, const void* in, uint64_t n, void* d_result, void* ws,
                    size_t ws_bytes) {
  const T* p = static_cast<const T*>(in);
  T* res = static_cast<T*>(d_result);
  switch (op) {
    case PP_OP_PLUS:
      return host::reduce<T, plus>(s, p, n, res, ws, ws_bytes);
    case PP_OP_MULTIPLIES:
      return host::reduce<T, multiplies>(s, p, n, res, ws, ws_bytes);
    case PP_OP_MINIMUM:
      return host::reduce<T, minimum>(s, p, n, res, ws, ws_bytes);
    case PP_OP_MAXIMUM:
      return host::reduce<T, maximum>(s, p, n, res, ws, ws_bytes);
    case PP_OP_BIT_AND:
    case PP_OP_BIT_OR:
    case PP_OP_BIT_XOR:
      if constexpr (std::is_integral_v<T>) {
        if (op == PP_OP_BIT_AND) return host::reduce<T, bit_and>(s, p, n, res, ws, ws_bytes);
        if (op == PP_OP_BIT_OR) return host::reduce<T, bit_or>(s, p, n, res, ws, ws_bytes);
        return host::reduce<T, bit_xor>(s, p, n, res, ws, ws_bytes);
      } else {
        return Status::unsupported;
      }
  }
  return Status::invalid_arg;
}

template <class T>
size_t workspace_typed(pp_scan_algo algo, const void* in, const void* out, uint64_t n) {
  return workspace_policy<PlainScan<T, plus>>(algo, in, out, n);
}

template <class T, class Op>
Status carry_op(cudaStream_t s, void* out, const void* in, uint64_t n, const void* carry_prev, void* carry_next,
                bool exclusive, bool first) {
  if (n == 0) return Status::ok;
  T* o = static_cast<T*>(out);
  const T* i = static_cast<const T*>(in);
  if (first) {
    carry_first_kernel<T, Op><<<1, 32, 0, s>>>(o, i, n, static_cast<T*>(carry_next), exclusive ? 1 : 0);
  } else {
    host::DeviceInfo di;
    const Status st = host::device_info(di);
    if (st != Status::ok) return st;
    const uint64_t vecs = n / (16 / sizeof(T));
    uint64_t grid = (vecs + 255) / 256;
    if (grid > uint64_t(di.sm_count) * 8) grid = uint64_t(di.sm_count) * 8;
    if (grid == 0) grid = 1;
    carry_apply_kernel<T, Op><<<unsigned(grid), 256, 0, s>>>(o, i, n, static_cast<const T*>(carry_prev),
                                                            static_cast<T*>(carry_next), exclusive ? 1 : 0);
  }
  return host::from_cuda(cudaGetLastError());
}

template <class T>
Status carry_typed(cudaStream_t s, pp_op op, void* out, const void* in, uint64_t n, const void* carry_prev,
                   void* carry_next, bool exclusive, bool first) {
  switch (op) {
    case PP_OP_PLUS:
      return carry_op<T, plus>(s, out, in, n, carry_prev, carry_next, exclusive, first);
    case PP_OP_MULTIPLIES:
      return carry_op<T, multiplies>(s, out, in, n, carry_prev, carry_next, exclusive, first);
    case PP_OP_MINIMUM:
      return carry_op<T, minimum>(s, out, in, n, carry_prev, carry_next, exclusive, first);
    case PP_OP_MAXIMUM:
      return carry_op<T, maximum>(s, out, in, n, carry_prev, carry_next, exclusive, first);
    case PP_OP_BIT_AND:
    case PP_OP_BIT_OR:
    case PP_OP_BIT_XOR:
      if constexpr (std::is_integral_v<T>) {
        if (op == PP_OP_BIT_AND) return carry_op<T, bit_and>(s, out, in, n, carry_prev, carry_next, exclusive, first);
        if (op == PP_OP_BIT_OR) return carry_op<T, bit_or>(s, out, in, n, carry_prev, carry_next, exclusive, first);
        return carry_op<T, bit_xor>(s, out, in, n, carry_prev, carry_next, exclusive, first);
      } else {
        return Status::unsupported;
      }
  }
  return Status::invalid_arg;
}

// Segmented operators: plus, minimum, maximum.
template <class T, class F>
Status with_seg_op(pp_op op, F&& f) {
  switch (op) {
    case PP_OP_PLUS:
      return f(plus{});
    case PP_OP_MINIMUM:
      return f(minimum{});
    case PP_OP_MAXIMUM:
      return f(maximum{});
    default:
      return Status::unsupported;
  }
}

template <class T>
Status seg_scan_typed(const SegReq& r) {
  return with_seg_op<T>(r.op, [&](auto op) {
    using Op = decltype(op);
    return host::segmented_scan<T, Op>(r.s, static_cast<const T*>(r.in), static_cast<T*>(r.out), r.n, r.offsets,
                                       r.num_segments, r.exclusive);
  });
}

template <class T>
Status seg_reduce_typed(const SegReq& r) {
  return with_seg_op<T>(r.op, [&](auto op) {
    using Op = decltype(op);
    return host::segmented_reduce<T, Op>(r.s, static_cast<const T*>(r.in), r.n, r.offsets, r.num_segments,
                                         static_cast<T*>(r.out));
  });
}

template <class T>
Status rows_scan_typed(const SegReq& r) {
  return with_seg_op<T>(r.op, [&](auto op) {
    using Op = decltype(op);
    return host::rows_scan<T, Op>(r.s, static_cast<const T*>(r.in), static_cast<T*>(r.out), r.rows, r.cols,
                                  r.exclusive, r.reverse);
  });
}

#define PP_INSTANTIATE_SEG(T)                     \
  template Status seg_scan_typed<T>(const SegReq&);   \
  template Status seg_reduce_typed<T>(const SegReq&); \
  template Status rows_scan_typed<T>(const SegReq&);

#define PP_INSTANTIATE_DISPATCH(T)                                                                     \
  template Status scan_typed<T>(const ScanReq&);                                                       \
  template Status reduce_typed<T>(cudaStream_t, pp_op, const void*, uint64_t, void*, void*, size_t); \
  template size_t workspace_typed<T>(pp_scan_algo, const void*, const void*, uint64_t);                \
  template Status carry_typed<T>(cudaStream_t, pp_op, void*, const void*, uint64_t, const void*, void*, bool, bool);

}  // namespace capi
}  // namespace pp
