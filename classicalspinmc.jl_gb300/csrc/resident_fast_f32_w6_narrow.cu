// resident_fast_f32_w6_narrow.cu -- the specialised resident kernel (resident.cuh)
// in single precision for 6 bilinear partners per site with scalar couplings
// and no or diagonal onsite terms, bound to at most kNarrowThreads threads per
// CTA (more registers per thread than the 896-thread build), for each cluster
// size.
#include "resident.cuh"

namespace csmc {

template <> const void *resident_kernel_fast_narrow<float, 6>(int bil, int ons, int cl) {
    if (bil != 0 || ons > 1) return nullptr;
    return ons == 0 ? resident_fast_narrow_for<float, 6, 0>(cl) : resident_fast_narrow_for<float, 6, 1>(cl);
}

} // namespace csmc
