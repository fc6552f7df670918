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
    float *invT_slot;  // (float)(1 / T) per slot, formed on the host
    const double *invT64_slot; // 1 / T per slot in FP64, formed on the host (the same bits as a division here)
    double *acc_slot, *exch_slot;
    double *E_chain, *M_chain;
    unsigned long long *sweep_acc; // accepted proposals of the current sweep, per chain
    unsigned int *drift_bits;      // max relative |S| error, float bits
    int *error_flag;               // nonzero: a bounded wait gave up
    const uint32_t *chain_id;      // per chain: the key of its Philox streams (default: the chain index)
    double *E_win; // persistent windows: each window's last energy by slot, two buffers alternating
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

// The closed-form constraint of one lattice (csmc_constraint) for the
// constrained Metropolis kinds: c = g.V + q |V|^2 + p |V| + c0 with
// V = sum_d w[d] s_d over device positions (w zero at padding; w == nullptr:
// weight 1 everywhere, padding spins being zero).
struct ConsArgs {
    const double *w;
    double g[3], q, p, c0, weight;
    double *lambda_slot; // mc.lambda of every slot
};

// c(V) with explicit rounding (the sequential and the batched constrained
// kernels evaluate it bit for bit alike)
template <typename T> __device__ __forceinline__ T constraint_value(const ConsArgs &k, T vx, T vy, T vz) {
    using F = Fp<T>;
    T c = F::fma((T)k.g[2], vz, F::fma((T)k.g[1], vy, F::mul((T)k.g[0], vx)));
    // a zero q or p adds nothing (fma(0, x, c) = c for finite x, up to the
    // sign of a zero c, which the + c0 below makes +0 either way); skipping
    // them takes |V|^2 and the square root off the chain of the sequential
    // decisions
    if (k.q != 0.0 || k.p != 0.0) {
        const T vv = F::fma(vz, vz, F::fma(vy, vy, F::mul(vx, vx)));
        c = F::fma((T)k.q, vv, c);
        c = F::fma((T)k.p, sqrt(vv), c);
    }
    return F::add(c, (T)k.c0);
}

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
    // generic kernel on a cluster: each rank's partner tables (cubic and
    // quartic too, same encoding) and the pattern of its local sites
    const uint16_t *q2c, *q3c, *q4c;
    const uint8_t *patc;
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
// Threads per CTA at most of a resident kernel (its launch bound): 896 for
// the specialised kernel with scalar couplings and at most diagonal onsite
// terms (72 registers per thread), else 512.
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
    // persistent mode: the launch covers every window of [it0, it1) (a window
    // ends at an exchange iteration, a multiple of swap_period); between
    // windows all CTAs meet at one grid barrier, then each replica takes the
    // exchange of its own pair (exchange_partner) and writes its own records
    int32_t persistent;
    int32_t n_lattices;
    int64_t swap_period;      // lcm(swap_rate, max(or_rate, 1)): iterations that exchange
    const int2 *lattices;     // per lattice {first slot, replicas}
    uint32_t k0, k1;          // the context's Philox key (exchange streams)
    unsigned int *grid_bar;   // grid barrier arrival counter, zero at launch
    uint32_t n_blocks;        // CTAs in the launch
};

// Replica exchange of one lattice's slots at iteration `it`
// (monte_carlo.jl:308-349), by all threads of one block: pairs
// (a, a+1) with a = (it/swap_rate) % 2 + 2m are disjoint and decided in
// parallel; the even slot of a pair accepts with probability
// min(1, exp((1/T_odd - 1/T_even)(E_odd - E_even))) from the Philox SWAP
// stream; an accepted exchange swaps which replica sits in the two slots.
// Loads bypass L1: in the persistent kernel other blocks wrote these values.
__device__ __forceinline__ void exchange_slots(const ChainState &cs, int sys, int slot_base, int n_rep, int64_t it,
                                               int swap_rate, uint32_t k0, uint32_t k1) {
    if (n_rep < 2) return;
    const int phase = (int)((it / swap_rate) % 2);
    for (int m = threadIdx.x; phase + 2 * m + 1 < n_rep; m += blockDim.x) {
        const int a = phase + 2 * m, b = a + 1;
        const int ev = (a % 2 == 0) ? a : b, od = (ev == a) ? b : a;
        const int sa = slot_base + a, sb = slot_base + b;
        const int se = slot_base + ev, so = slot_base + od;
        const double Te = __ldcg(cs.T_slot + se), To = __ldcg(cs.T_slot + so);
        const double Ee = __ldcg(cs.E_chain + __ldcg(cs.chain_of + se));
        const double Eo = __ldcg(cs.E_chain + __ldcg(cs.chain_of + so));
        const double x = exp((1 / To - 1 / Te) * (Eo - Ee));
        const U4 w = philox4x32_10((uint32_t)a, (uint32_t)it, (uint32_t)sys ^ (uint32_t)(it >> 32), PURPOSE_SWAP, k0, k1);
        if (u53(w.x, w.y) < (x < 1.0 ? x : 1.0)) {
            const int ca = __ldcg(cs.chain_of + sa), cb = __ldcg(cs.chain_of + sb);
            cs.chain_of[sa] = cb;
            cs.chain_of[sb] = ca;
            cs.slot_of[cb] = sa;
            cs.slot_of[ca] = sb;
            cs.exch_slot[sa] = __ldcg(cs.exch_slot + sa) + 1;
            cs.exch_slot[sb] = __ldcg(cs.exch_slot + sb) + 1;
        }
    }
}

// The same exchange seen from one replica, in slot `slot` of a lattice of
// slots [slot_base, slot_base + n_rep): the pair of this iteration that holds
// the slot (pairs start at relative slot `phase`), the decision of
// exchange_slots for it -- the same formula, draw and operands, with the
// energies of the pair's slots taken from E_slot (the energy of the chain in
// each slot) -- and the slot the replica holds afterwards.  Both replicas of
// a pair reach the same decision, each on its own.  *swapped: the pair was
// exchanged.
// The slot paired with `slot` at exchange iteration `it` (pairs of relative
// slots (phase + 2m, phase + 2m + 1)), or -1.
__device__ __forceinline__ int exchange_pair_slot(int slot_base, int n_rep, int slot, int64_t it, int swap_rate) {
    const int rel = slot - slot_base;
    const int phase = (int)((it / swap_rate) % 2);
    if (rel < phase) return -1;
    const int a = phase + 2 * ((rel - phase) / 2), b = a + 1;
    if (b >= n_rep) return -1;
    return slot_base + (rel == a ? b : a);
}
__device__ __forceinline__ int exchange_partner(const ChainState &cs, const double *E_slot, int sys, int slot_base,
                                                int n_rep, int slot, int64_t it, int swap_rate, uint32_t k0,
                                                uint32_t k1, bool *swapped) {
    *swapped = false;
    const int ps = exchange_pair_slot(slot_base, n_rep, slot, it, swap_rate);
    if (ps < 0) return slot;
    const int a = (slot < ps ? slot : ps) - slot_base, b = a + 1;
    const int ev = (a % 2 == 0) ? a : b, od = (ev == a) ? b : a;
    const int se = slot_base + ev, so = slot_base + od;
    // 1/To - 1/Te from reciprocals formed on the host: the bits of the divisions
    const double iTe = __ldcg(cs.invT64_slot + se), iTo = __ldcg(cs.invT64_slot + so);
    const double Ee = __ldcg(E_slot + se), Eo = __ldcg(E_slot + so);
    const double x = exp((iTo - iTe) * (Eo - Ee));
    const U4 w = philox4x32_10((uint32_t)a, (uint32_t)it, (uint32_t)sys ^ (uint32_t)(it >> 32), PURPOSE_SWAP, k0, k1);
    if (!(u53(w.x, w.y) < (x < 1.0 ? x : 1.0))) return slot;
    *swapped = true;
    return ps;
}

// Probe record kq of one lattice's slots (monte_carlo.jl:368-370): the energy
// of the last Metropolis sweep and |M| of the replica in each slot.
__device__ __forceinline__ void record_slots(const ChainState &cs, int slot_base, int n_rep, double *rec_E,
                                             double *rec_M, int64_t kq, int n_slots) {
    for (int q = threadIdx.x; q < n_rep; q += blockDim.x) {
        const int slot = slot_base + q, c = __ldcg(cs.chain_of + slot);
        if (rec_E) rec_E[kq * n_slots + slot] = __ldcg(cs.E_chain + c);
        if (rec_M) rec_M[kq * n_slots + slot] = __ldcg(cs.M_chain + c);
    }
}

} // namespace csmc
