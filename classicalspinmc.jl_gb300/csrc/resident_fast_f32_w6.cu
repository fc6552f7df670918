// resident_fast_f32_w6.cu -- instantiations of the specialised resident kernel (resident.cuh)
// in single precision for 6 bilinear partners per site: every bilinear class
// (scalar / general 3x3), onsite class (none / diagonal / general) and cluster
// size (1, 2 or 4 CTAs per replica).
#include "resident.cuh"

namespace csmc {

template <> const void *resident_kernel_fast<float, 6>(int bil, int ons, int cl) {
    return resident_fast_table<float, 6>(bil, ons, cl);
}

} // namespace csmc
