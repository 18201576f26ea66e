// usm_smart_ptr.hpp - owning device / managed / pinned-host buffers with a
// span view, the ownership model of the reference's host wrappers and tests.
//
// Mirrors include/usm_smart_ptr.hpp of the reference:
//   usm_unique_ptr<T, alloc> (:48-72): a std::unique_ptr that frees with the
//     allocator it came from and remembers its element count; get_span()
//     (:69-71) hands (pointer, count) to the device API, e.g.
//     reduce_device<plus<>>(stream, buf.get_span());
//   usm_shared_ptr<T, alloc> (:80-105): the same over std::shared_ptr.
// `sycl::usm::alloc` becomes `usm_smart_ptr::alloc` with the same three
// kinds, backed by CUDA allocations:
//   alloc::device  cudaMalloc         (device memory only)
//   alloc::shared  cudaMallocManaged  (migrates between host and device;
//                                      the host may fill it, as the reference's
//                                      tests fill shared USM with std::iota)
//   alloc::host    cudaMallocHost     (pinned host memory the device can read)
// `sycl::queue` becomes a cudaStream_t; allocation is not stream-ordered (as
// sycl::malloc is not), and the stream is kept only so the deleter can finish
// the stream's work on the buffer before it is freed. A failed allocation
// throws parallel_primitives::error with status cuda. Sizes are element
// counts; a count of 0 holds no allocation.
#pragma once

#include <cstddef>
#include <memory>
#include <span>

#include <cuda_runtime.h>

#include "parallel_primitives/common.hpp"

namespace usm_smart_ptr {

enum class alloc { host, device, shared };

template <typename T>
struct usm_deleter {
  cudaStream_t stream = nullptr;
  alloc kind = alloc::device;

  void operator()(T* ptr) const noexcept {
    if (!ptr) return;
    // pending work on the stream may still use the buffer
    cudaStreamSynchronize(stream);
    if (kind == alloc::host)
      cudaFreeHost(ptr);
    else
      cudaFree(ptr);
  }
};

namespace detail {
template <typename T>
T* allocate(size_t count, alloc kind) {
  if (count == 0) return nullptr;
  void* p = nullptr;
  cudaError_t e = cudaSuccess;
  switch (kind) {
    case alloc::device:
      e = cudaMalloc(&p, count * sizeof(T));
      break;
    case alloc::shared:
      e = cudaMallocManaged(&p, count * sizeof(T));
      break;
    case alloc::host:
      e = cudaMallocHost(&p, count * sizeof(T));
      break;
  }
  if (e != cudaSuccess || !p) throw parallel_primitives::error(pp::host::Status::cuda, "usm allocation");
  return static_cast<T*>(p);
}
}  // namespace detail

template <typename T, alloc location>
class usm_unique_ptr : public std::unique_ptr<T, usm_deleter<T>> {
  using base = std::unique_ptr<T, usm_deleter<T>>;
  size_t count_{};

 public:
  [[nodiscard]] usm_unique_ptr(size_t count, cudaStream_t stream)
      : base(detail::allocate<T>(count, location), usm_deleter<T>{stream, location}), count_(count) {}

  [[nodiscard]] explicit usm_unique_ptr(cudaStream_t stream) : usm_unique_ptr(1, stream) {}

  [[nodiscard]] size_t size_bytes() const noexcept { return count_ * sizeof(T); }
  [[nodiscard]] size_t size() const noexcept { return count_; }
  [[nodiscard]] std::span<T> get_span() const noexcept { return {base::get(), count_}; }
};

template <typename T, alloc location>
class usm_shared_ptr : public std::shared_ptr<T> {
  using base = std::shared_ptr<T>;
  size_t count_{};

 public:
  [[nodiscard]] usm_shared_ptr(size_t count, cudaStream_t stream)
      : base(detail::allocate<T>(count, location), usm_deleter<T>{stream, location}), count_(count) {}

  [[nodiscard]] explicit usm_shared_ptr(cudaStream_t stream) : usm_shared_ptr(1, stream) {}

  [[nodiscard]] size_t size_bytes() const noexcept { return count_ * sizeof(T); }
  [[nodiscard]] size_t size() const noexcept { return count_; }
  [[nodiscard]] std::span<T> get_span() const noexcept { return {base::get(), count_}; }
};

}  // namespace usm_smart_ptr
