// resident_generic.cu -- instantiations of the generic resident kernel and the
// host launcher that picks a resident kernel (resident.cuh).
#include "launch.hpp"
#include "resident.cuh"

namespace csmc {

template <typename R, int NT> static const void *generic_for(bool cub, bool qua) {
    if (cub && qua) return (const void *)k_resident<ResidentGeneric<R, true, true, NT>, R, NT>;
    if (cub) return (const void *)k_resident<ResidentGeneric<R, true, false, NT>, R, NT>;
    if (qua) return (const void *)k_resident<ResidentGeneric<R, false, true, NT>, R, NT>;
    return (const void *)k_resident<ResidentGeneric<R, false, false, NT>, R, NT>;
}

template <typename R> const void *resident_kernel_generic(int block, bool cub, bool qua) {
    return block == 1024 ? generic_for<R, 1024>(cub, qua) : generic_for<R, 512>(cub, qua);
}

const void *resident_kernel_fast_f32(int block, int bil, int ons);
const void *resident_kernel_fast_f64(int block, int bil, int ons);

template <typename R> static const void *pick(int block, const ResidentSel &sel) {
    if (!sel.fast) return resident_kernel_generic<R>(block, sel.cub, sel.qua);
    return sizeof(R) == 4 ? resident_kernel_fast_f32(block, sel.bil, sel.ons)
                          : resident_kernel_fast_f64(block, sel.bil, sel.ons);
}

template <typename R>
cudaError_t launch_resident(const ResSys<R> *d_sys, const int2 *items, int n_items, int *work_ctr,
                            const ChainState &cs, const RunDesc &rd, int grid, int block, size_t smem,
                            const ResidentSel &sel, cudaStream_t st) {
    // work_ctr must be zero when the kernel starts (the caller resets it on `st`)
    const void *fn = pick<R>(block, sel);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    ChainState csv = cs;
    RunDesc rdv = rd;
    void *args[] = {(void *)&d_sys, (void *)&items, (void *)&n_items, (void *)&work_ctr, (void *)&csv, (void *)&rdv};
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, st);
}

template <typename R> int resident_max_blocks_per_sm(int block, size_t smem, const ResidentSel &sel) {
    const void *fn = pick<R>(block, sel);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem) != cudaSuccess) return 0;
    return n;
}

template const void *resident_kernel_generic<float>(int, bool, bool);
template const void *resident_kernel_generic<double>(int, bool, bool);
template cudaError_t launch_resident<float>(const ResSys<float> *, const int2 *, int, int *, const ChainState &,
                                            const RunDesc &, int, int, size_t, const ResidentSel &, cudaStream_t);
template cudaError_t launch_resident<double>(const ResSys<double> *, const int2 *, int, int *, const ChainState &,
                                             const RunDesc &, int, int, size_t, const ResidentSel &, cudaStream_t);
template int resident_max_blocks_per_sm<float>(int, size_t, const ResidentSel &);
template int resident_max_blocks_per_sm<double>(int, size_t, const ResidentSel &);

} // namespace csmc
