// launch.hpp -- host launchers of the kernels in kernels.cu and exact.cu.
#pragma once

#include "kernels.cuh"

namespace csmc {

template <typename R>
void launch_metro_colour(const SysArgs<R> &a, const ChainState &cs, int64_t start, int64_t count, int chain_lo,
                         int n_chains, int kind, uint32_t msweep, double T_override, cudaStream_t st);
template <typename R>
void launch_or_colour(const SysArgs<R> &a, int64_t start, int64_t count, int chain_lo, int n_chains,
                      cudaStream_t st);
template <typename R>
void launch_det_colour(const SysArgs<R> &a, int64_t start, int64_t count, int chain_lo, int n_chains,
                       cudaStream_t st);
int64_t partial_blocks(int64_t Np);
// total_energy of replicas [chain_lo, chain_lo+n) into cs.E_chain; part needs
// n * partial_blocks(Np) doubles
template <typename R>
void launch_energy(const SysArgs<R> &a, const ChainState &cs, int chain_lo, int n_chains, double *part,
                   cudaStream_t st);
// |M| into cs.M_chain; part needs 3 * n * partial_blocks(Np) doubles
template <typename R>
void launch_magnet(const SysArgs<R> &a, const ChainState &cs, int chain_lo, int n_chains, double *part,
                   cudaStream_t st);
void launch_after_metro(const ChainState &cs, int chain_first, int n, int kind, int64_t n_sites, double sigma0,
                        double *last_acc, cudaStream_t st);
// one constrained Metropolis sweep (kind 3 or 4) of every replica of a lattice
template <typename R>
void launch_metro_constraint(const SysArgs<R> &a, const ChainState &cs, const ConsArgs &k, int kind, uint32_t msweep,
                             double T_override, cudaStream_t st);
// Exchange of every lattice (lattices[k] = {first slot, replicas}) at
// iteration `it`, then, if kq >= 0, probe record kq of every slot.
void launch_exchange(const ChainState &cs, const int2 *lattices, int n_lattices, int64_t it, int swap_rate, uint32_t k0,
                     uint32_t k1, bool do_swap, double *rec_E, double *rec_M, int64_t kq, int n_slots, cudaStream_t st);
// FP64 reference layout <-> device order for slots [slot_first, +n_slots) of
// one lattice (the replica of each slot looked up in chain_of on the device);
// buf holds n_slots consecutive 3 x N arrays.
template <typename R>
void launch_scatter(const SysArgs<R> &a, const int32_t *chain_of, int slot_first, int n_slots, const double *src,
                    cudaStream_t st);
template <typename R>
void launch_gather(const SysArgs<R> &a, const int32_t *chain_of, int slot_first, int n_slots, double *dst,
                   cudaStream_t st);
// uniform spins from the INIT stream of each replica's chain id
template <typename R>
void launch_random_spins(const SysArgs<R> &a, const uint32_t *chain_id, uint32_t k0, uint32_t k1, cudaStream_t st);
template <typename R> void launch_local_field(const SysArgs<R> &a, int r, double *out, cudaStream_t st);
// energy differences on the replica in `slot` (looked up in chain_of on the device)
template <typename R>
void launch_energy_diff(const SysArgs<R> &a, const int32_t *chain_of, int slot, int64_t n, const int64_t *sites,
                        const double *ns, double *dE, cudaStream_t st);
template <typename R> void launch_renorm(const SysArgs<R> &a, int chain_lo, int n_chains, cudaStream_t st);
template <typename R> void launch_drift(const SysArgs<R> &a, unsigned int *bits, cudaStream_t st);
template <typename R>
cudaError_t launch_resident(const ResSys<R> *d_sys, const int2 *items, int n_items, int *work_ctr,
                            const ChainState &cs, const RunDesc &rd, int grid, int block, size_t smem,
                            const ResidentSel &sel, bool cooperative, cudaStream_t st);
// CTAs (cl = 1) or clusters (cl > 1) of the selected resident kernel that fit on the device at once
template <typename R> int resident_capacity(int block, size_t smem, const ResidentSel &sel, int n_sms);
// compute_equal_time_correlations of every replica of one lattice (correlations.cu):
// pos 3 per device site, ks 3 per wavevector, out [slot - slot_base][n_k][9]
template <typename R>
void launch_structure_factor(const SysArgs<R> &a, const R *pos, const R *ks, int64_t n_k, const int32_t *slot_of,
                             int slot_base, double *out, cudaStream_t st);
// Philox4x32-10 of n counters (4 words each) under n keys (2 words each)
void launch_philox(const uint32_t *ctr, const uint32_t *key, int64_t n, uint32_t *out, cudaStream_t st);
// the same on the tensor cores for a single-precision lattice (correlations_tc.cu):
// pos 3 per device site for sf_tc_sites(Np) sites (zero-padded), packed
// sf_tc_packed_floats(Np, n_rep) floats of scratch for the split spins
// scratch for the split spins, and (splits > 1: the sites of a tile split over
// several CTAs to fill the SMs) sf_tc_partial_floats of partial sums
int64_t sf_tc_sites(int64_t Np);
int64_t sf_tc_packed_floats(int64_t Np, int n_rep);
int sf_tc_splits(int64_t n_k, int n_rep, int64_t Np, int n_sms);
int64_t sf_tc_partial_floats(int64_t n_k, int n_rep, int splits);
cudaError_t launch_structure_factor_tc(const SysArgs<float> &a, const float *pos, const float *ks, int64_t n_k,
                                       const int32_t *slot_of, int slot_base, double *out, float *packed,
                                       float *partial, int splits, int *error_flag, cudaStream_t st);
// a kernel whose bounded wait cannot complete (see csmc_selftest_timeout)
cudaError_t launch_wait_selftest(int which, unsigned int *ctr, int *error_flag, cudaStream_t st);
// static shared memory of the selected resident kernel in bytes (-1: query failed)
template <typename R> int resident_static_smem(const ResidentSel &sel);

// Reference-layout tables of one lattice for the replay kernel (exact.cu):
// per reference site, N2/N3/N4 term entries with 0-based partners (-1 absent).
struct ExactTables {
    int64_t N;
    int N2, N3, N4;
    const int64_t *bs, *cs, *qs;
    const double *bm, *ct, *qt, *field, *onsite;
    const int64_t *ref2dev;
    int64_t Np;
    double S;
};
// The constraint of the replayed slot for the constrained kinds: weights in
// reference site order (nullptr: all 1), the slot's lambda (updated in
// place) and sigma0 of the adaptive rule.
struct ExactCons {
    const double *w;
    double g[3], q, p, c0, weight;
    double *lambda;
    double sigma0;
};
// Sequential FP64 replay of n proposals on the FP64 replica at `spins`.
void launch_replay(const ExactTables &t, const ExactCons &k, double *spins, int kind, double T, double *sigma_dev,
                   int64_t n, const int64_t *sites, const double *u_phi, const double *u_z, const double *u_acc,
                   uint8_t *accepted, cudaStream_t st);

} // namespace csmc
