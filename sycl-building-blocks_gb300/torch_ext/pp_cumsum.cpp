// Optional libtorch binding over the C ABI: a differentiable float32 cumsum
// along the last dimension.
//
// forward : y[r, :] = inclusive plus-scan of x[r, :]        (pp_rows_scan)
// backward: dx[r, :] = reverse inclusive scan of dy[r, :]   (pp_rows_scan, reverse)
// The adjoint of a prefix sum is the suffix sum of the upstream gradient, so
// the backward needs nothing saved from the forward.
#include <ATen/cuda/CUDAContext.h>
#include <c10/cuda/CUDAGuard.h>
#include <torch/extension.h>

#include <cstdint>

#include "pp_gb300.h"

namespace {

torch::Tensor rows_scan(const torch::Tensor& x, bool reverse) {
  TORCH_CHECK(x.is_cuda(), "pp cumsum: CUDA tensor expected");
  TORCH_CHECK(x.scalar_type() == torch::kFloat32, "pp cumsum: float32 expected");
  torch::Tensor xc = x.contiguous();
  // the scan kernels want 16-byte aligned rows; views with an offset are copied
  if (reinterpret_cast<uintptr_t>(xc.data_ptr()) % 16 != 0) xc = xc.clone();
  torch::Tensor y = torch::empty_like(xc);
  if (xc.numel() == 0) return y;
  const int64_t cols = xc.dim() == 0 ? 1 : xc.size(-1);
  const int64_t rows = xc.numel() / cols;
  const c10::cuda::CUDAGuard guard(xc.device());
  cudaStream_t stream = at::cuda::getCurrentCUDAStream(xc.device().index()).stream();
  const pp_status st = pp_rows_scan(stream, PP_SCAN_INCLUSIVE, PP_OP_PLUS, PP_F32, xc.data_ptr(), y.data_ptr(),
                                    uint64_t(rows), uint64_t(cols), reverse ? 1 : 0);
  TORCH_CHECK(st == PP_OK, "pp_rows_scan failed: ", pp_status_string(st));
  return y;
}

class CumsumFunction : public torch::autograd::Function<CumsumFunction> {
 public:
  static torch::Tensor forward(torch::autograd::AutogradContext*, const torch::Tensor& x) {
    return rows_scan(x, false);
  }
  static torch::autograd::tensor_list backward(torch::autograd::AutogradContext*,
                                               torch::autograd::tensor_list grad_out) {
    return {rows_scan(grad_out[0], true)};
  }
};

torch::Tensor cumsum(const torch::Tensor& x) { return CumsumFunction::apply(x); }
torch::Tensor reverse_cumsum(const torch::Tensor& x) { return rows_scan(x, true); }

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
  m.def("cumsum", &cumsum, "differentiable float32 cumsum along the last dimension (GB300 decoupled scan)");
  m.def("reverse_cumsum", &reverse_cumsum, "float32 suffix sums along the last dimension");
}
