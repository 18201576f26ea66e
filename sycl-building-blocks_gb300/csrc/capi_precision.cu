// F32 plus-scans with a precision mode: compensated float-float accumulation
// and the FP64 cross-tile carry chain (no counterpart in the reference, whose
// float scans accumulate in plain FP32).
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {

Status scan_f32_precision(const ScanReq& r, pp_precision prec) {
  if (r.op != PP_OP_PLUS) return Status::unsupported;
  switch (prec) {
    case PP_PREC_DEFAULT:
      return scan_policy<PlainScan<float, plus>>(r);
    case PP_PREC_COMPENSATED:
      return scan_policy<CompensatedF32>(r);
    case PP_PREC_FP64_CARRY:
      return scan_policy<F64CarryF32>(r);
  }
  return Status::invalid_arg;
}

size_t workspace_f32_precision(pp_scan_algo algo, pp_precision prec, const void* in, const void* out, uint64_t n) {
  switch (prec) {
    case PP_PREC_COMPENSATED:
      return workspace_policy<CompensatedF32>(algo, in, out, n);
    case PP_PREC_FP64_CARRY:
      return workspace_policy<F64CarryF32>(algo, in, out, n);
    default:
      return workspace_policy<PlainScan<float, plus>>(algo, in, out, n);
  }
}

}  // namespace capi
}  // namespace pp
