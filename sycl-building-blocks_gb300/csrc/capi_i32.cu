// Kernel instantiations for int32_t elements (every operator, every algorithm).
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_DISPATCH(int32_t)
}  // namespace capi
}  // namespace pp
