// Kernel instantiations for int64_t elements (every operator, every algorithm).
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_DISPATCH(int64_t)
}  // namespace capi
}  // namespace pp
