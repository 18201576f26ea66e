// parallel_primitives/scan_decoupled_lookback.hpp - single-pass decoupled
// look-back scan, C++ drop-in for the reference header of the same name
// (include/parallel_primitives/scan_decoupled_lookback.hpp).
//
// Template shape as the reference:
//   decoupled_scan_device<scan_type, func, T, bool optimised_offload = true>
//     (reference :209-217);
//   decoupled_scan<scan_type, func, T, bool optimised_offload = true,
//                  size_t offload_threshold = 131072> (reference :219-230),
// with sycl::queue& -> cudaStream_t. The reference sends short inputs
// elsewhere when the device is a GPU: decoupled_scan_device below 65,536
// elements to its two-kernel scan_device (:211-213), decoupled_scan below
// offload_threshold to a sequential scan on the host CPU (:221-224). Here
// every length runs on the GPU's single-pass kernel (this library has no CPU
// fallback, and its scan_device is served by the same kernel), so
// `optimised_offload` and `offload_threshold` are accepted for source
// compatibility and select nothing; the results are the same either way.
#pragma once

#include <cstddef>

#include "common.hpp"
#include "cooperative_groups.hpp"

namespace parallel_primitives {

// decoupled_scan_device (reference :209-217). Asynchronous on `stream`;
// device-side errors surface at the next synchronising call or through
// pp_stream_status().
template <scan_type type, typename func, typename T, bool optimised_offload = true>
void decoupled_scan_device(cudaStream_t stream, const T* input, T* output, index_t length) {
  internal::check(pp::host::decoupled_scan<pp::PlainScan<T, func>>(stream, input, output, length,
                                                                    type == scan_type::exclusive),
                  "decoupled_scan_device");
}

// decoupled_scan (reference :219-230): host arrays in and out, blocking. The
// device scan is called with optimised_offload = false, as the reference does
// (:227).
template <scan_type type, typename func, typename T, bool optimised_offload = true,
          size_t offload_threshold = 131072>
void decoupled_scan(cudaStream_t stream, const T* input, T* output, index_t length) {
  if (length == 0) return;
  internal::device_buffer<T> d_in(length), d_out(length);
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(d_in.ptr, input, length * sizeof(T),
                                                      cudaMemcpyHostToDevice, stream)),
                  "copy in");
  decoupled_scan_device<type, func, T, false>(stream, d_in.ptr, d_out.ptr, length);
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(output, d_out.ptr, length * sizeof(T),
                                                      cudaMemcpyDeviceToHost, stream)),
                  "copy out");
  internal::sync_and_check(stream);
}

}  // namespace parallel_primitives

// The reference's header also provides the two-kernel entry points
// (scan_device, group_scan_device, scan) to its callers.
#include "scan.hpp"
