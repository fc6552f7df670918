// kernels.cuh -- launch-side declarations of the sweep kernels (kernels.cu)
// and the replay kernel (exact.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"

namespace csmc {

// Per-replica state, context-wide device arrays.  Slots are temperature
// slots (MPI ranks of the reference); chains are physical replicas.
struct ChainState {
    int32_t *slot_of;  // chain -> slot
    int32_t *chain_of; // slot -> chain
    double *T_slot, *sigma_slot;
    double *acc_slot, *exch_slot;
    double *E_chain, *M_chain;
    unsigned long long *sweep_acc; // accepted proposals of the current sweep, per chain
    unsigned int *drift_bits;      // max relative |S| error, float bits
    int *error_flag;               // nonzero: a bounded wait gave up
};

// One lattice for the global-memory kernels.
template <typename R> struct SysArgs {
    Tab<uint32_t> tb;
    Coef<R> cf;
    R *spins; // replica r at spins + r * 3 * Np (x, y, z blocks of Np)
    const int32_t *dev2ref;
    const int64_t *ref2dev;
    int32_t chain_base, n_rep;
    int64_t n_real; // real sites
    R S;
    uint32_t k0, k1; // Philox key (seed)
    int cub, qua;
};

// One lattice for the resident kernel (lives in device memory).
template <typename R> struct ResSys {
    Tab<uint16_t> tb;
    Coef<R> cf;
    R *spins;
    int32_t chain_base, n_rep;
    int32_t n_colours, nb;
    int64_t col_start[CSMC_MAX_COLOURS + 1];
    int64_t col_count[CSMC_MAX_COLOURS];
    int32_t col_pattern[CSMC_MAX_COLOURS]; // the one basis of each colour class, or -1
    int64_t n_real;
    R S;
    uint32_t k0, k1;
    // split over a cluster of `cl` CTAs (cl > 1): per rank and colour class,
    // the local start, the site count and the device index of the first site
    int32_t cl, Npl;
    int32_t loc_start[4][CSMC_MAX_COLOURS], loc_count[4][CSMC_MAX_COLOURS], src_start[4][CSMC_MAX_COLOURS];
    // the bilinear partners of each site packed in one 16-byte word (up to 8
    // 16-bit partners, sentinel-padded): p2v[i] (device index) for one CTA
    // per replica; q2v[rank][i] for clusters, each entry
    // (owner rank - rank mod cl) << 14 | owner-local index, so partners in the
    // reading CTA's own shared memory have the top two bits clear; used by
    // the specialised kernel
    const uint4 *p2v, *q2v;
    // nonzero: the specialised kernel stages the CTA's partner words in
    // shared memory too (they fit beside the spins)
    int32_t pv_stage;
};
constexpr int RESIDENT_CLUSTER_MAX = 4;

// Which resident kernel: the generic one (per-site pattern, cubic and
// quartic terms) or the specialised one for lattices without cubic/quartic
// terms whose colour classes each hold a single basis; for the latter the
// bilinear class (0: every coupling c*I, 1: general 3x3) and the onsite class
// (0: none, 1: diagonal, 2: general) of 2O+P.
struct ResidentSel {
    bool fast;
    int bil, ons;
    int width; // specialised kernel: bilinear partners per site (4, 6 or 8)
    bool cub, qua;
    int cl; // CTAs per replica (thread-block cluster size; 1 = no cluster)
};
constexpr int RESIDENT_WMAX = 8; // bilinear slots per site of the specialised kernel
// Threads per CTA at most of a resident kernel (its launch bound): 1024 for
// the specialised kernel with scalar couplings and at most diagonal onsite
// terms (64 registers per thread suffice), else 512.
__host__ __device__ constexpr int resident_max_threads(bool fast, int bil, int ons) {
    return fast && bil == 0 && ons < 2 ? 896 : 512;
}

// The sweep schedule of one resident launch (see csmc_run_params).
struct RunDesc {
    int64_t it0, it1;         // iterations [it0, it1)
    int64_t t_therm;
    int64_t probe_first;      // iteration of probe record 0
    int64_t probe_cap;
    double *rec_E, *rec_M;    // [probe_cap][n_slots]
    double T_override;        // > 0: this temperature for every replica (annealing)
    double sigma0;
    uint32_t msweep0;         // Metropolis sweep counter at the first Metropolis sweep
    int32_t or_rate, swap_rate, probe_rate, kind;
    int32_t reset_sigma;      // sigma <- sigma0 before the first sweep
    int32_t n_slots;
    int32_t renorm_every;     // single precision: renormalise every k sweeps
    uint64_t sweeps0;         // the context's sweeps (all kinds) before this launch
    int32_t swap_enabled;
};

} // namespace csmc
