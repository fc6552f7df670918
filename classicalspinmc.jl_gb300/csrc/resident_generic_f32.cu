// resident_generic_f32.cu -- instantiations of the generic resident kernel (resident.cuh) in
// single precision: with and without cubic / quartic terms, one CTA per
// replica or a cluster of 2 or 4.
#include "resident.cuh"

namespace csmc {

template <> const void *resident_kernel_generic<float>(bool cub, bool qua, int cl) {
    if (cub && qua) return resident_generic_for<float, true, true>(cl);
    if (cub) return resident_generic_for<float, true, false>(cl);
    if (qua) return resident_generic_for<float, false, true>(cl);
    return resident_generic_for<float, false, false>(cl);
}

} // namespace csmc
