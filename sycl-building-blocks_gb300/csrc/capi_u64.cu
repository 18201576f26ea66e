// Kernel instantiations for uint64_t elements (every operator, every algorithm).
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_DISPATCH(uint64_t)
}  // namespace capi
}  // namespace pp
