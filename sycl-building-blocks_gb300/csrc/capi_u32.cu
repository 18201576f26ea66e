// Kernel instantiations for uint32_t elements (every operator, every algorithm).
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_DISPATCH(uint32_t)
}  // namespace capi
}  // namespace pp
