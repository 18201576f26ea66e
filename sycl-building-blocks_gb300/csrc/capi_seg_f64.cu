// Segmented scan / reduce and row-scan instantiations for double elements.
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_SEG(double)
}  // namespace capi
}  // namespace pp
