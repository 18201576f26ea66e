// parallel_primitives/scan.hpp - C++ drop-in for the reference's two-kernel
// scan entry points (include/parallel_primitives/scan.hpp:107-140). Both are
// served by the single-pass decoupled look-back kernel: scan_device with the
// persistent grid, group_scan_device with one CTA walking every tile (one
// work-group, as in the reference).
#pragma once

#include "scan_decoupled_lookback.hpp"
#include "../usm_smart_ptr.hpp"

// as the reference's scan.hpp:27: usm_unique_ptr / alloc for its callers
using namespace usm_smart_ptr;

namespace parallel_primitives {

template <scan_type type, typename func, typename T>
void scan_device(cudaStream_t stream, const T* input, T* output, index_t length) {
  decoupled_scan_device<type, func, T>(stream, input, output, length);
}

template <scan_type type, typename func, typename T>
void group_scan_device(cudaStream_t stream, const T* input, T* output, index_t length) {
  internal::check(pp::host::decoupled_scan<pp::PlainScan<T, func>>(stream, input, output, length,
                                                                    type == scan_type::exclusive, nullptr, 0, 1),
                  "group_scan_device");
}

template <scan_type type, typename func, typename T>
void scan(cudaStream_t stream, const T* input, T* output, index_t length) {
  decoupled_scan<type, func, T>(stream, input, output, length);
}

}  // namespace parallel_primitives
