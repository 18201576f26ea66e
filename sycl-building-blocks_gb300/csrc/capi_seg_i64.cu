// Segmented scan / reduce and row-scan instantiations for int64_t elements.
#include "dispatch_impl.cuh"

namespace pp {
namespace capi {
PP_INSTANTIATE_SEG(int64_t)
}  // namespace capi
}  // namespace pp
