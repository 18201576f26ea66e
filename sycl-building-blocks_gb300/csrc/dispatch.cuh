// Run-time dispatch from the C ABI enums to the kernel templates. The typed
// entry points are defined in dispatch_impl.cuh and explicitly instantiated
// once per element type in capi_<type>.cu, so the instantiations compile in
// parallel translation units.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "pp/host.cuh"
#include "pp_gb300.h"

namespace pp {
namespace capi {

using host::Status;

struct ScanReq {
  cudaStream_t s = nullptr;
  bool exclusive = false;
  pp_op op = PP_OP_PLUS;
  const void* in = nullptr;
  void* out = nullptr;
  uint64_t n = 0;
  pp_scan_algo algo = PP_ALGO_AUTO;
  void* ws = nullptr;
  size_t ws_bytes = 0;
};

template <class T>
Status scan_typed(const ScanReq& r);
template <class T>
Status reduce_typed(cudaStream_t s, pp_op op, const void* in, uint64_t n, void* d_result, void* ws,
                    size_t ws_bytes);
template <class T>
size_t workspace_typed(pp_scan_algo algo, const void* in, const void* out, uint64_t n);
// Offsets chunk `out` (n elements, scanned on its own) by *carry_prev and
// records the running total in *carry_next; the first chunk only records.
template <class T>
Status carry_typed(cudaStream_t s, pp_op op, void* out, const void* in, uint64_t n, const void* carry_prev,
                   void* carry_next, bool exclusive, bool first);

// Batched segmented scan / reduce and row scans (capi_seg_<type>.cu).
struct SegReq {
  cudaStream_t s = nullptr;
  bool exclusive = false;
  pp_op op = PP_OP_PLUS;
  const void* in = nullptr;
  void* out = nullptr;
  uint64_t n = 0;
  const int64_t* offsets = nullptr;
  uint64_t num_segments = 0;
  uint64_t rows = 0, cols = 0;
  bool reverse = false;
};
template <class T>
Status seg_scan_typed(const SegReq& r);
template <class T>
Status seg_reduce_typed(const SegReq& r);
template <class T>
Status rows_scan_typed(const SegReq& r);

// F32 plus-scan with a precision mode (capi_precision.cu).
Status scan_f32_precision(const ScanReq& r, pp_precision prec);
size_t workspace_f32_precision(pp_scan_algo algo, pp_precision prec, const void* in, const void* out, uint64_t n);

// Scratch array of the allocation-free scan on the current device, or null
// when that entry point has not run there (capi_noalloc.cu).
void* noalloc_scratch_used_on_current_device();

}  // namespace capi
}  // namespace pp
