// Kernel instantiations for float elements (every operator, every algorithm).
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_DISPATCH(float)
}  // namespace capi
}  // namespace pp
