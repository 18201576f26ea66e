// parallel_primitives/reduction.hpp - C++ drop-in for the reference's
// device-wide reduction (include/parallel_primitives/reduction.hpp:113-151).
// As with sycl::reduction, `func` must be associative and commutative.
#pragma once

#include <span>

#include "common.hpp"

namespace parallel_primitives {

// Asynchronous: the result goes to device memory d_result.
template <typename func, typename T>
void reduce_device_async(cudaStream_t stream, const T* input, index_t length, T* d_result) {
  internal::check(pp::host::reduce<T, func>(stream, input, length, d_result), "reduce_device_async");
}

// reduce_device<func, T> (reference :113-139): blocking, returns the value.
template <typename func, typename T>
T reduce_device(cudaStream_t stream, std::span<const T> input) {
  internal::device_buffer<T> d_res(1);
  reduce_device_async<func, T>(stream, input.data(), input.size(), d_res.ptr);
  T out{};
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(&out, d_res.ptr, sizeof(T), cudaMemcpyDeviceToHost, stream)),
                  "copy result");
  internal::sync_and_check(stream);
  return out;
}

// reduce<func, T> (reference :142-151): host array, blocking.
template <typename func, typename T>
T reduce(cudaStream_t stream, std::span<const T> input) {
  if (input.empty()) return pp::identity<func, T>();
  internal::device_buffer<T> d_in(input.size());
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(d_in.ptr, input.data(), input.size_bytes(),
                                                      cudaMemcpyHostToDevice, stream)),
                  "copy in");
  return reduce_device<func, T>(stream, std::span<const T>(d_in.ptr, input.size()));
}

}  // namespace parallel_primitives
