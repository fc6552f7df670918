// resident_generic.cu -- the host launcher that picks a resident kernel
// (resident.cuh) and queries its occupancy and shared memory.
#include "launch.hpp"
#include "resident.cuh"

#include <map>
#include <mutex>
#include <tuple>

namespace csmc {

// The host-side attributes a launch needs, looked up once: the dynamic
// shared memory a kernel is allowed (set per device and kernel, raised when a
// launch needs more) and the resident capacity of a (kernel, block, shared
// memory, cluster) shape.  The driver's occupancy queries cost microseconds
// per call, paid on every run otherwise.
namespace {
std::mutex g_attr_mu;
std::map<std::pair<int, const void *>, size_t> g_smem_allowed;
std::map<std::tuple<int, const void *, int, size_t, int, int>, int> g_capacity;

cudaError_t allow_smem(const void *fn, size_t smem) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_attr_mu);
    auto it = g_smem_allowed.find({dev, fn});
    if (it != g_smem_allowed.end() && it->second >= smem) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) g_smem_allowed[{dev, fn}] = smem;
    return e;
}
} // namespace

// The kernel of a selection; `block` > 0: the threads per CTA of the launch,
// which may take a build bound to fewer threads (more registers per thread).
template <typename R> static const void *pick(const ResidentSel &sel, int block = 0) {
    if (!sel.fast) return resident_kernel_generic<R>(sel.cub, sel.qua, sel.cl);
    if constexpr (sizeof(R) == 4) {
        if (block > 0 && block <= kNarrowThreads && sel.width > 4 && sel.width <= 6)
            if (const void *fn = resident_kernel_fast_narrow<float, 6>(sel.bil, sel.ons, sel.cl)) return fn;
    }
    if (sel.width <= 4) return resident_kernel_fast<R, 4>(sel.bil, sel.ons, sel.cl);
    if (sel.width <= 6) return resident_kernel_fast<R, 6>(sel.bil, sel.ons, sel.cl);
    return resident_kernel_fast<R, 8>(sel.bil, sel.ons, sel.cl);
}

template <typename R>
cudaError_t launch_resident(const ResSys<R> *d_sys, const int2 *items, int n_items, int *work_ctr,
                            const ChainState &cs, const RunDesc &rd, int grid, int block, size_t smem,
                            const ResidentSel &sel, bool cooperative, cudaStream_t st) {
    // work_ctr must be zero when the kernel starts (the caller resets it on `st`)
    if (block < 32 || block > resident_max_threads(sel.fast, sel.bil, sel.ons) || block % 32 != 0)
        return cudaErrorInvalidValue;
    const void *fn = pick<R>(sel, block);
    cudaError_t e = allow_smem(fn, smem);
    if (e != cudaSuccess) return e;
    ChainState csv = cs;
    RunDesc rdv = rd;
    void *args[] = {(void *)&d_sys, (void *)&items, (void *)&n_items, (void *)&work_ctr, (void *)&csv, (void *)&rdv};
    if (sel.cl <= 1 && !cooperative) return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, st);
    // clusters and/or a cooperative launch (every CTA co-resident, for the
    // persistent kernel's grid barriers)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    int na = 0;
    if (sel.cl > 1) {
        attr[na].id = cudaLaunchAttributeClusterDimension;
        attr[na].val.clusterDim.x = sel.cl;
        attr[na].val.clusterDim.y = 1;
        attr[na].val.clusterDim.z = 1;
        na++;
    }
    if (cooperative) {
        attr[na].id = cudaLaunchAttributeCooperative;
        attr[na].val.cooperative = 1;
        na++;
    }
    cfg.attrs = attr;
    cfg.numAttrs = na;
    return cudaLaunchKernelExC(&cfg, fn, args);
}

// Resident CTAs (cl = 1) or clusters (cl > 1) that fit on the device at once.
template <typename R> static int resident_capacity_query(const void *fn, int block, size_t smem,
                                                          const ResidentSel &sel, int n_sms) {
    if (allow_smem(fn, smem) != cudaSuccess) return 0;
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

template <typename R> int resident_capacity(int block, size_t smem, const ResidentSel &sel, int n_sms) {
    const void *fn = pick<R>(sel, block);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    const auto key = std::make_tuple(dev, fn, block, smem, sel.cl, n_sms);
    {
        std::lock_guard<std::mutex> lock(g_attr_mu);
        auto it = g_capacity.find(key);
        if (it != g_capacity.end()) return it->second;
    }
    const int n = resident_capacity_query<R>(fn, block, smem, sel, n_sms);
    if (n > 0) {
        std::lock_guard<std::mutex> lock(g_attr_mu);
        g_capacity[key] = n;
    }
    return n;
}

// Static shared memory of the selected kernel (its descriptor copy, reduction
// scratch and staged couplings), or -1.
template <typename R> int resident_static_smem(const ResidentSel &sel) {
    cudaFuncAttributes at{};
    if (cudaFuncGetAttributes(&at, pick<R>(sel)) != cudaSuccess) return -1;
    return (int)at.sharedSizeBytes;
}

// Self-test of the bounded waits: a wait that can never complete must give
// up, set the error flag and return.  which = 0: an mbarrier phase that
// expects 16 bytes no copy delivers (one CTA); which = 1: a grid barrier that
// expects one more CTA than the launch has (two co-resident CTAs).
__global__ void k_wait_selftest(int which, unsigned int *ctr, int *error_flag, uint64_t budget) {
    __shared__ uint64_t bar;
    __shared__ int s_ok;
    if (which == 0) {
        if (threadIdx.x == 0) {
            mbar_init(&bar, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);
        mbar_wait_bounded(&bar, 0, error_flag, budget);
        __syncthreads();
    } else {
        unsigned int epoch = 0;
        grid_barrier(ctr, gridDim.x + 1, epoch, error_flag, &s_ok, budget);
    }
}

cudaError_t launch_wait_selftest(int which, unsigned int *ctr, int *error_flag, cudaStream_t st) {
    uint64_t budget = 20000000ull; // 20 ms
    void *args[] = {(void *)&which, (void *)&ctr, (void *)&error_flag, (void *)&budget};
    if (which == 0) return cudaLaunchKernel((const void *)k_wait_selftest, dim3(1), dim3(64), args, 0, st);
    return cudaLaunchCooperativeKernel((const void *)k_wait_selftest, dim3(2), dim3(64), args, 0, st);
}

template cudaError_t launch_resident<float>(const ResSys<float> *, const int2 *, int, int *, const ChainState &,
                                            const RunDesc &, int, int, size_t, const ResidentSel &, bool, cudaStream_t);
template cudaError_t launch_resident<double>(const ResSys<double> *, const int2 *, int, int *, const ChainState &,
                                             const RunDesc &, int, int, size_t, const ResidentSel &, bool,
                                             cudaStream_t);
template int resident_capacity<float>(int, size_t, const ResidentSel &, int);
template int resident_capacity<double>(int, size_t, const ResidentSel &, int);
template int resident_static_smem<float>(const ResidentSel &);
template int resident_static_smem<double>(const ResidentSel &);

} // namespace csmc
