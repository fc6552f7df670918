// resident_fast_f64.cu -- instantiations of the specialised resident kernel
// (resident.cuh) in double precision: per bilinear class (scalar /
// general 3x3), onsite class (none / diagonal / general) and cluster size
// (1, 2 or 4 CTAs per replica), 1024 threads per CTA.
#include "resident.cuh"

namespace csmc {

template <int BIL, int ONS> static const void *fast_for(int cl) {
    if (cl == 4) return (const void *)k_resident<ResidentFast<double, BIL, ONS, 1024, 4>, double, 1024, 4>;
    if (cl == 2) return (const void *)k_resident<ResidentFast<double, BIL, ONS, 1024, 2>, double, 1024, 2>;
    return (const void *)k_resident<ResidentFast<double, BIL, ONS, 1024, 1>, double, 1024, 1>;
}

const void *resident_kernel_fast_f64(int, int bil, int ons, int cl) {
    if (bil == 0) return ons == 0 ? fast_for<0, 0>(cl) : ons == 1 ? fast_for<0, 1>(cl) : fast_for<0, 2>(cl);
    return ons == 0 ? fast_for<1, 0>(cl) : ons == 1 ? fast_for<1, 1>(cl) : fast_for<1, 2>(cl);
}

} // namespace csmc
