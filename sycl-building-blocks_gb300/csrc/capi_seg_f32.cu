// Segmented scan / reduce and row-scan instantiations for float elements.
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_SEG(float)
}  // namespace capi
}  // namespace pp
