// Kernel instantiations for double elements (every operator, every algorithm).
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_DISPATCH(double)
}  // namespace capi
}  // namespace pp
