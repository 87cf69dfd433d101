// The robust-predicate instantiation of the clip passes (clip_kernels.cuh):
// its own translation unit, so it compiles beside the float one.
#include "clip_kernels.cuh"

namespace vgb {

template struct ClipPasses<true>;

}  // namespace vgb
