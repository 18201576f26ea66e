// Segmented scan / reduce and row-scan instantiations for int32_t elements.
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_SEG(int32_t)
}  // namespace capi
}  // namespace pp
