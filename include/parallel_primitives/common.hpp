// parallel_primitives/common.hpp - shared names of the C++ drop-in API.
//
// Mirrors include/parallel_primitives/internal/common.h of the reference:
// index_t (:25), scan_type (:27-30) and the functor set whose identities
// get_init provides (:41-68). `sycl::queue&` becomes a `cudaStream_t`;
// `sycl::plus<>` becomes `parallel_primitives::plus<>` (any functor with a
// __device__ operator() works once pp::op_traits<Op, T> gives its identity).
//
// Compile user code that includes these headers with nvcc for sm_103a and
// add both `include/` and `sycl-building-blocks_gb300/csrc/` to the include
// path. Calls are stream-ordered and asynchronous unless documented
// otherwise; errors throw parallel_primitives::error.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>

#include "pp/host.cuh"

namespace parallel_primitives {

using index_t = uint64_t;

enum class scan_type { inclusive, exclusive };

template <class T = void>
using plus = pp::plus;
template <class T = void>
using multiplies = pp::multiplies;
template <class T = void>
using bit_and = pp::bit_and;
template <class T = void>
using bit_or = pp::bit_or;
template <class T = void>
using bit_xor = pp::bit_xor;
template <class T = void>
using minimum = pp::minimum;
template <class T = void>
using maximum = pp::maximum;

class error : public std::runtime_error {
 public:
  explicit error(pp::host::Status s, const char* what)
      : std::runtime_error(std::string(what) + ": status " + std::to_string(static_cast<int>(s))), status(s) {}
  pp::host::Status status;
};

namespace internal {
inline void check(pp::host::Status s, const char* what) {
  if (s != pp::host::Status::ok) throw error(s, what);
}
// Blocking copy helpers of the host-array wrappers.
template <class T>
struct device_buffer {
  T* ptr = nullptr;
  explicit device_buffer(index_t n) {
    if (n && cudaMalloc(&ptr, n * sizeof(T)) != cudaSuccess) throw error(pp::host::Status::cuda, "cudaMalloc");
  }
  ~device_buffer() {
    if (ptr) cudaFree(ptr);
  }
  device_buffer(const device_buffer&) = delete;
  device_buffer& operator=(const device_buffer&) = delete;
};
inline void sync_and_check(cudaStream_t s) {
  check(pp::host::read_device_error(s, nullptr), "device-side error");
}
}  // namespace internal

}  // namespace parallel_primitives
