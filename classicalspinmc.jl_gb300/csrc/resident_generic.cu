// resident_generic.cu -- instantiations of the generic resident kernel and the
// host launcher that picks a resident kernel (resident.cuh).
#include "launch.hpp"
#include "resident.cuh"

namespace csmc {

template <typename R, int NT> static const void *generic_for(bool cub, bool qua) {
    if (cub && qua) return (const void *)k_resident<ResidentGeneric<R, true, true, NT, 1>, R, NT, 1>;
    if (cub) return (const void *)k_resident<ResidentGeneric<R, true, false, NT, 1>, R, NT, 1>;
    if (qua) return (const void *)k_resident<ResidentGeneric<R, false, true, NT, 1>, R, NT, 1>;
    return (const void *)k_resident<ResidentGeneric<R, false, false, NT, 1>, R, NT, 1>;
}

template <typename R> const void *resident_kernel_generic(int block, bool cub, bool qua) {
    return block == 1024 ? generic_for<R, 1024>(cub, qua) : generic_for<R, 512>(cub, qua);
}

const void *resident_kernel_fast_f32(int block, int bil, int ons, int cl);
const void *resident_kernel_fast_f64(int block, int bil, int ons, int cl);

template <typename R> static const void *pick(int block, const ResidentSel &sel) {
    if (!sel.fast) return resident_kernel_generic<R>(block, sel.cub, sel.qua);
    return sizeof(R) == 4 ? resident_kernel_fast_f32(block, sel.bil, sel.ons, sel.cl)
                          : resident_kernel_fast_f64(block, sel.bil, sel.ons, sel.cl);
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
    if (sel.cl <= 1) return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, st);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = sel.cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

// Resident CTAs (cl = 1) or clusters (cl > 1) that fit on the device at once.
template <typename R> int resident_capacity(int block, size_t smem, const ResidentSel &sel, int n_sms) {
    const void *fn = pick<R>(block, sel);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (sel.cl <= 1) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem) != cudaSuccess) return 0;
        return n * n_sms;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sel.cl * n_sms);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = sel.cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) return 0;
    return n;
}

template const void *resident_kernel_generic<float>(int, bool, bool);
template const void *resident_kernel_generic<double>(int, bool, bool);
template cudaError_t launch_resident<float>(const ResSys<float> *, const int2 *, int, int *, const ChainState &,
                                            const RunDesc &, int, int, size_t, const ResidentSel &, cudaStream_t);
template cudaError_t launch_resident<double>(const ResSys<double> *, const int2 *, int, int *, const ChainState &,
                                             const RunDesc &, int, int, size_t, const ResidentSel &, cudaStream_t);
template int resident_capacity<float>(int, size_t, const ResidentSel &, int);
template int resident_capacity<double>(int, size_t, const ResidentSel &, int);

} // namespace csmc
