// noalloc.cu -- csmc_energy_diff_static: the energy differences of
// csmc_energy_diff computed without any device allocation.
//
// Who needs it: csmc_energy_diff stages its inputs and outputs in three
// device buffers that it allocates and frees on every call.  Some callers
// cannot allow that: a host program whose own memory pool has already
// reserved the GPU's memory (a Julia or PyTorch process with a caching
// allocator), or a proposal-evaluation loop where each cudaFree would
// synchronise the device and stall the work queued around it.  This entry
// point uses instead a fixed array compiled into the library.
//
// The array is CSMC_ENERGY_DIFF_STATIC_MAX * 40 bytes (2.5 MiB) of static
// device memory; every GPU on which the library is loaded holds it until the
// process exits.  Its address is looked up once per device, on the first call
// made with a context on that device, with that device current; make that
// first call before any stream capture.  All calls share the array, which
// keeps the contents of the last call.  Nothing in it has to start at zero:
// each call writes the sites, the new spins and all n results before reading
// them.  Calls whose GPU work overlaps (two host threads, or contexts on two
// streams) race on the array and must be serialised by the caller.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/csmc.h"

namespace csmc {
void set_last_error(const char *msg);
int context_device(void *c, int *device);
int energy_diff_staged(void *c, int32_t slot, int64_t n, const int64_t *sites, const double *ns, double *dE,
                       void *scratch, int64_t n_max);
} // namespace csmc

namespace {

constexpr int64_t kMax = CSMC_ENERGY_DIFF_STATIC_MAX;
// per proposal: one int64 site, three doubles of new spin, one double result
constexpr size_t kBytes = (size_t)kMax * (sizeof(int64_t) + 4 * sizeof(double));

static __device__ __align__(256) unsigned char g_scratch[kBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

// Device address of g_scratch on `device`, looked up once with that device current.
int scratch_address(int device, void **out) {
    if (device < 0 || device >= kMaxDevices) {
        csmc::set_last_error("csmc_energy_diff_static: device ordinal out of range");
        return CSMC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[device]) {
        int prev = -1;
        cudaError_t e = cudaGetDevice(&prev);
        if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
        void *p = nullptr;
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_scratch);
        if (prev >= 0 && prev != device) cudaSetDevice(prev);
        if (e != cudaSuccess) {
            csmc::set_last_error(cudaGetErrorString(e));
            return CSMC_ERR_CUDA;
        }
        g_addr[device] = p;
    }
    *out = g_addr[device];
    return CSMC_OK;
}

} // namespace

extern "C" int csmc_energy_diff_static(void *ctx, int32_t slot, int64_t n, const int64_t *sites,
                                       const double *new_spins, double *dE) {
    if (n < 0 || n > kMax) {
        csmc::set_last_error("csmc_energy_diff_static: n must be between 0 and CSMC_ENERGY_DIFF_STATIC_MAX "
                             "(65536) proposals per call");
        return CSMC_ERR_INVALID;
    }
    int device = 0;
    int rc = csmc::context_device(ctx, &device);
    if (rc != CSMC_OK) return rc;
    void *scratch = nullptr;
    rc = scratch_address(device, &scratch);
    if (rc != CSMC_OK) return rc;
    return csmc::energy_diff_staged(ctx, slot, n, sites, new_spins, dE, scratch, kMax);
}
