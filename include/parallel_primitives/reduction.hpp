// parallel_primitives/reduction.hpp - C++ drop-in for the reference's
// device-wide reduction (include/parallel_primitives/reduction.hpp:113-151).
// As with sycl::reduction, `func` must be associative and commutative.
//
// Signatures follow the reference:
//   template <typename func, typename T, bool optimised_offload = true,
//             size_t offload_threshold = 16384>
//   T reduce_device(stream, const span<T>&)          (reference :113-139)
//   T reduce(stream, const span<T>&)                 (reference :142-151)
// with sycl::queue& -> cudaStream_t and sycl::span -> std::span. T is deduced
// from a span of T or of const T, so the reference's call sites
// `reduce_device<plus<>>(q, buf.get_span())` and
// `reduce<plus<>>(q, std::span<T>{vec})` compile unchanged apart from the
// queue. The reference moves chunks shorter than offload_threshold to the
// host CPU when the device is a GPU (:129-133, :144-146); this library has no
// CPU fallback, so every length reduces on the GPU and the two trailing
// parameters are accepted for source compatibility only.
#pragma once

#include <cstddef>
#include <span>
#include <type_traits>

#include "common.hpp"
#include "../usm_smart_ptr.hpp"

// The reference's headers bring usm_unique_ptr / alloc into the global
// namespace for their callers (reduction.hpp:27, scan.hpp:27,
// scan_cooperative.hpp:27); callers written against it rely on that.
using namespace usm_smart_ptr;

namespace parallel_primitives {

// Asynchronous: the result goes to device memory d_result.
template <typename func, typename T>
void reduce_device_async(cudaStream_t stream, const T* input, index_t length, T* d_result) {
  internal::check(pp::host::reduce<T, func>(stream, input, length, d_result), "reduce_device_async");
}

namespace internal {
template <typename func, typename T>
T reduce_device_blocking(cudaStream_t stream, const T* input, index_t length) {
  internal::device_buffer<T> d_res(1);
  reduce_device_async<func, T>(stream, input, length, d_res.ptr);
  T out{};
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(&out, d_res.ptr, sizeof(T), cudaMemcpyDeviceToHost, stream)),
                  "copy result");
  internal::sync_and_check(stream);
  return out;
}

template <typename func, typename T>
T reduce_host_blocking(cudaStream_t stream, const T* input, index_t length) {
  if (length == 0) return pp::identity<func, T>();
  internal::device_buffer<T> d_in(length);
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(d_in.ptr, input, length * sizeof(T),
                                                      cudaMemcpyHostToDevice, stream)),
                  "copy in");
  return reduce_device_blocking<func, T>(stream, d_in.ptr, length);
}
}  // namespace internal

// reduce_device<func, T> (reference :113-139): the span views device (or
// managed) memory; blocking, returns the value.
template <typename func, typename T, bool optimised_offload = true, size_t offload_threshold = 16384>
std::remove_cv_t<T> reduce_device(cudaStream_t stream, const std::span<T>& input) {
  using V = std::remove_cv_t<T>;
  return internal::reduce_device_blocking<func, V>(stream, input.data(), input.size());
}

// Same for a span of const T with T named explicitly.
template <typename func, typename T, bool optimised_offload = true, size_t offload_threshold = 16384>
T reduce_device(cudaStream_t stream, const std::span<const T>& input) {
  return internal::reduce_device_blocking<func, T>(stream, input.data(), input.size());
}

// reduce<func, T> (reference :142-151): the span views host memory; copied to
// the device, reduced there; blocking.
template <typename func, typename T, bool optimised_offload = true, size_t offload_threshold = 16384>
std::remove_cv_t<T> reduce(cudaStream_t stream, const std::span<T>& input) {
  using V = std::remove_cv_t<T>;
  return internal::reduce_host_blocking<func, V>(stream, input.data(), input.size());
}

template <typename func, typename T, bool optimised_offload = true, size_t offload_threshold = 16384>
T reduce(cudaStream_t stream, const std::span<const T>& input) {
  return internal::reduce_host_blocking<func, T>(stream, input.data(), input.size());
}

}  // namespace parallel_primitives
