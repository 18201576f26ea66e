// parallel_primitives/scan_cooperative.hpp - C++ drop-in for the reference's
// cooperative grid-barrier scan (include/parallel_primitives/
// scan_cooperative.hpp:95-110).
#pragma once

#include "common.hpp"
#include "../usm_smart_ptr.hpp"

// as the reference's scan_cooperative.hpp:27: usm_unique_ptr / alloc for its
// callers
using namespace usm_smart_ptr;

namespace parallel_primitives {

// cooperative_scan_device<type, func, T> (reference :95-99). `ctas` = 0 uses
// every block the device holds co-resident; a larger request throws with
// status grid_too_large, as the reference's perform_check throws
// (include/cooperative_groups.hpp:65-76).
template <scan_type type, typename func, typename T>
void cooperative_scan_device(cudaStream_t stream, const T* input, T* output, index_t length, int ctas = 0) {
  internal::check(pp::host::cooperative_scan<pp::PlainScan<T, func>>(stream, input, output, length,
                                                                      type == scan_type::exclusive, nullptr, 0, ctas),
                  "cooperative_scan_device");
}

// cooperative_scan<type, func, T> (reference :102-110): host arrays, blocking.
template <scan_type type, typename func, typename T>
void cooperative_scan(cudaStream_t stream, const T* input, T* output, index_t length) {
  if (length == 0) return;
  internal::device_buffer<T> d_in(length), d_out(length);
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(d_in.ptr, input, length * sizeof(T),
                                                      cudaMemcpyHostToDevice, stream)),
                  "copy in");
  cooperative_scan_device<type, func, T>(stream, d_in.ptr, d_out.ptr, length);
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(output, d_out.ptr, length * sizeof(T),
                                                      cudaMemcpyDeviceToHost, stream)),
                  "copy out");
  internal::sync_and_check(stream);
}

}  // namespace parallel_primitives
