// resident_fast_f64.cu -- instantiations of the specialised resident kernel
// (resident.cuh) in double precision, one per bilinear class (scalar /
// general 3x3), onsite class (none / diagonal / general) and block size.
#include "resident.cuh"

namespace csmc {

template <int BIL, int ONS> static const void *fast_for(int block) {
    return block == 1024 ? (const void *)k_resident<ResidentFast<double, BIL, ONS, 1024>, double, 1024>
                         : (const void *)k_resident<ResidentFast<double, BIL, ONS, 512>, double, 512>;
}

const void *resident_kernel_fast_f64(int block, int bil, int ons) {
    if (bil == 0) return ons == 0 ? fast_for<0, 0>(block) : ons == 1 ? fast_for<0, 1>(block) : fast_for<0, 2>(block);
    return ons == 0 ? fast_for<1, 0>(block) : ons == 1 ? fast_for<1, 1>(block) : fast_for<1, 2>(block);
}

} // namespace csmc
