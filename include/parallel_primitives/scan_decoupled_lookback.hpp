// parallel_primitives/scan_decoupled_lookback.hpp - single-pass decoupled
// look-back scan, C++ drop-in for the reference header of the same name
// (include/parallel_primitives/scan_decoupled_lookback.hpp).
#pragma once

#include "common.hpp"

namespace parallel_primitives {

// decoupled_scan_device<type, func, T> (reference :209-217). Asynchronous on
// `stream`; device-side errors surface at the next synchronising call or
// through pp_stream_status(). There is no small-input host offload: every
// length runs on the GPU.
template <scan_type type, typename func, typename T>
void decoupled_scan_device(cudaStream_t stream, const T* input, T* output, index_t length) {
  internal::check(pp::host::decoupled_scan<pp::PlainScan<T, func>>(stream, input, output, length,
                                                                    type == scan_type::exclusive),
                  "decoupled_scan_device");
}

// decoupled_scan<type, func, T> (reference :219-230): host arrays in and out,
// blocking.
template <scan_type type, typename func, typename T>
void decoupled_scan(cudaStream_t stream, const T* input, T* output, index_t length) {
  if (length == 0) return;
  internal::device_buffer<T> d_in(length), d_out(length);
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(d_in.ptr, input, length * sizeof(T),
                                                      cudaMemcpyHostToDevice, stream)),
                  "copy in");
  decoupled_scan_device<type, func, T>(stream, d_in.ptr, d_out.ptr, length);
  internal::check(pp::host::from_cuda(cudaMemcpyAsync(output, d_out.ptr, length * sizeof(T),
                                                      cudaMemcpyDeviceToHost, stream)),
                  "copy out");
  internal::sync_and_check(stream);
}

}  // namespace parallel_primitives
