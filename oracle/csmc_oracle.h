/*
 * csmc_oracle.h -- CPU FP64 oracle for the ClassicalSpinMC.jl Monte Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * Julia routines (ClassicalSpinMC.jl v1.0.0), used by tests/ as the parity
 * checker and by bench.py as the timed CPU baseline.  The product library
 * (libcsmc.so) never links, loads or calls it.
 *
 * Parity pins: the reference is Julia and cannot run in this build environment,
 * so the oracle is pinned against the reference's own known-answer tests
 * (test/latticetests.jl:17-18,30 and test/mctests.jl:49,57), restated as
 * tests/golden/reference_kats.json.  Cubic and quartic terms have no test in
 * the reference: their parity rests on this restatement alone.
 *
 * Conventions
 *   - site indices are 0-based here; the reference's 1-based indices appear
 *     only in exported tables, where 0 still means "absent" (lattice.jl:179).
 *   - spins are the reference's 3 x N column-major Float64 array, i.e.
 *     interleaved xyz per site (lattice.jl:73, :293-301).
 *   - matrices are row-major m[a*3+b] == M[a,b] (interaction_matrix.jl:2-18);
 *     cubic tensors t[a*9+b*3+c] == C[a,b,c]; quartic t[((a*3+b)*3+c)*3+d].
 *   - all arithmetic keeps the reference's evaluation order and is compiled
 *     with -ffp-contract=off, since Julia does not contract a*b+c into an FMA.
 */
#ifndef CSMC_ORACLE_H
#define CSMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Unit cell + lattice description: the arguments of Lattice(shape, uc, S; bc)
 * together with the term lists of UnitCell (unit_cell.jl:3-18).  Basis indices
 * are 1-based as in the reference API.  Offsets hold `dim` ints per vector:
 * bilinear 1 vector per term, cubic 2 (o2, o3), quartic 3 (o2, o3, o4). */
typedef struct {
    int32_t dim;
    int32_t n_basis;
    int32_t shape[3];
    int32_t periodic;
    double spin_length;
    int32_t n_field;
    const int32_t *field_basis;
    const double *field_vec;
    int32_t n_onsite;
    const int32_t *onsite_basis;
    const double *onsite_mat;
    int32_t n_bilinear;
    const int32_t *bilinear_basis;
    const double *bilinear_mat;
    const int32_t *bilinear_offset;
    int32_t n_cubic;
    const int32_t *cubic_basis;
    const double *cubic_tensor;
    const int32_t *cubic_offset;
    int32_t n_quartic;
    const int32_t *quartic_basis;
    const double *quartic_tensor;
    const int32_t *quartic_offset;
} orc_desc;

typedef struct orc_lattice orc_lattice;

/* Lattice construction (lattice.jl:65-291).  literal_search=1 locates every
 * neighbour by a linear scan of the sorted site list, exactly as the
 * reference's findfirst does (lattice.jl:196,228,273); 0 uses the equivalent
 * index arithmetic.  Returns NULL and fills err on invalid input. */
orc_lattice *orc_lattice_new(const orc_desc *d, int literal_search, char *err, int errlen);
void orc_lattice_free(orc_lattice *lat);
int64_t orc_n_sites(const orc_lattice *lat);
/* N2, N3, N4: per-site tuple lengths == number of unit-cell terms. */
void orc_term_counts(const orc_lattice *lat, int32_t out[3]);
/* Copy out the per-site tables of the Lattice struct (lattice.jl:15-22), with
 * the reference's 1-based neighbour indices (0 = absent).  Any pointer may be
 * NULL.  Shapes: bil_sites N*N2, bil_mats N*N2*9, cub_sites N*N3*2,
 * cub_tens N*N3*27, qua_sites N*N4*3, qua_tens N*N4*81, field N*3, onsite N*9. */
void orc_export_tables(const orc_lattice *lat, int64_t *bil_sites, double *bil_mats,
                       int64_t *cub_sites, double *cub_tens, int64_t *qua_sites,
                       double *qua_tens, double *field, double *onsite);

/* Hamiltonian (hamiltonian.jl). */
void orc_local_field(const orc_lattice *lat, const double *spins, int64_t i, double H[3]);
double orc_site_energy(const orc_lattice *lat, const double *spins, int64_t i);
double orc_total_energy(const orc_lattice *lat, const double *spins);
double orc_magnetization(const orc_lattice *lat, const double *spins);

/* compute_equal_time_correlations (spin_correlations.jl:6-43): for the n_k
 * wavevectors ks (dim x n_k, column-major) and site positions pos (dim x N),
 * S_a(k) = sum_i exp(-i k.r_i) s_i,a and Suv[n*9 + 3a + b] =
 * Re(S_a(k_n) conj(S_b(k_n))) / N (9 x n_k, column-major). */
void orc_structure_factor(const double *spins, int64_t N, const double *pos, int dim, const double *ks,
                          int64_t n_k, double *Suv);

/* Proposals (lattice.jl:306-311, metropolis.jl:84-87) from given uniforms. */
void orc_random_spin_orientation(double S, double u_phi, double u_z, double out[3]);
void orc_gaussian_move(double S, const double s[3], double sigma, double u_phi, double u_z,
                       double out[3]);
/* calculate_energy_diff! core (metropolis.jl:94-110): writes new_spin at site i
 * and returns energy(new) - energy(old). */
double orc_energy_diff(const orc_lattice *lat, double *spins, int64_t i, const double new_spin[3]);

/* Metropolis kinds. */
enum { ORC_UNIFORM = 0, ORC_ADAPTIVE = 1, ORC_FIXED_CONE = 2 };

/* Replay: n proposals with the given sites and uniforms (metropolis.jl:65-153).
 * u_acc[p] is consumed only when dE >= 0, as the reference draws it only
 * then.  For ORC_ADAPTIVE, *sigma is updated once at the end, as after one
 * reference sweep of n proposals.  Returns the accepted count. */
int64_t orc_metropolis_replay(const orc_lattice *lat, double *spins, double T, int kind,
                              double *sigma, int64_t n, const int64_t *site,
                              const double *u_phi, const double *u_z, const double *u_acc,
                              uint8_t *accepted);

/* Constrained Metropolis (metropolis.jl:36-58, 155-179) with the constraint
 * function in the closed form c = g.V + q |V|^2 + p |V| + c0 of
 * V = sum_i w_i s_i (w NULL: all 1), evaluated over the whole lattice at every
 * proposal, as the reference calls mc.constraint(mc.lattice). */
typedef struct {
    const double *w;
    double g[3], q, p, c0;
    double weight;
} orc_constraint;
double orc_constraint_value(const orc_lattice *lat, const double *spins, const orc_constraint *k);
/* Replay of n proposals: cone = 0 uniform proposals (metropolis_constraint!,
 * whose e_diff the reference leaves undefined, read as calculate_energy_diff!
 * with a uniform proposal), cone = 1 cone proposals with *sigma and the
 * adaptive rule of metropolis_constraint_adaptive! at the end (sigma0 when at
 * least half accepted).  *lambda is mc.lambda, updated on every acceptance.
 * u_acc[p] is consumed only when dE - lambda' c >= 0. */
int64_t orc_metropolis_constraint_replay(const orc_lattice *lat, double *spins, double T, int cone,
                                         double *sigma, double sigma0, const orc_constraint *k,
                                         double *lambda, int64_t n, const int64_t *site,
                                         const double *u_phi, const double *u_z, const double *u_acc,
                                         uint8_t *accepted);
/* One constrained sweep of N proposals with the GPU kernel's Philox draws:
 * proposal q takes counter (q, sweep, chain, 5) for the site floor(N w0 / 2^32)
 * and u_acc = u53(w2, w3), and (q, sweep, chain, 6) for u_phi = u53(w0, w1),
 * u_z = u53(w2, w3). */
int64_t orc_metropolis_constraint_sweep(const orc_lattice *lat, double *spins, double T, int cone,
                                        double *sigma, double sigma0, const orc_constraint *k,
                                        double *lambda, uint64_t seed, uint32_t chain, uint32_t sweep);

/* Single-site updates applied in a caller-given order (monte_carlo.jl:126-139
 * and :201-213).  order[] holds 0-based site indices; negative entries are
 * skipped (padding in a device order). */
void orc_overrelax_order(const orc_lattice *lat, double *spins, const int64_t *order, int64_t n);
void orc_deterministic_order(const orc_lattice *lat, double *spins, const int64_t *order,
                             int64_t n);
/* The reference's sequential overrelaxation sweep, sites 1..N in order. */
void orc_overrelax_sweep(const orc_lattice *lat, double *spins);

/* Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
 * "Parallel Random Numbers: As Easy as 1, 2, 3", SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* One Metropolis colour sweep driven by the Philox stream layout of the GPU
 * kernels: order[d] is the reference site at device position d (negative =
 * padding), visited in increasing d.  uniform_bits is 24 (single-precision
 * stream) or 53 (double-precision stream).  Returns the accepted count; for
 * ORC_ADAPTIVE updates *sigma like metropolis_adaptive! (metropolis.jl:113-133). */
int64_t orc_metropolis_colour_sweep(const orc_lattice *lat, double *spins, double T, int kind,
                                    double *sigma, const int64_t *order, int64_t n_order,
                                    uint64_t seed, uint32_t chain, uint32_t sweep,
                                    int uniform_bits);

/* Initial spins from the Philox INIT stream (Lattice initialCondition=:random,
 * lattice.jl:76-79): site i of chain c draws (u_phi, u_z) from counter
 * (i, 0, c, INIT) with 53-bit uniforms. */
void orc_random_spins(const orc_lattice *lat, double *spins, uint64_t seed, uint32_t chain);

/* ---- reference-mode drivers (random sites with replacement) ------------- */

/* xoshiro256++ (Blackman & Vigna) seeded through splitmix64; stands in for
 * Julia's unseeded default task RNG, whose stream cannot be reproduced. */
typedef struct {
    uint64_t s[4];
} orc_rng;
void orc_rng_seed(orc_rng *r, uint64_t seed);
double orc_rng_uniform(orc_rng *r);

/* One reference Metropolis sweep: N proposals at random sites
 * (metropolis.jl:65-153).  Returns the accepted count. */
double orc_metropolis_sweep_ref(const orc_lattice *lat, double *spins, double T, int kind,
                                double *sigma, orc_rng *r);
/* deterministic_updates! (monte_carlo.jl:201-213): t_det-1 random-site updates. */
void orc_deterministic_ref(const orc_lattice *lat, double *spins, int64_t t_det, orc_rng *r);
/* simulated_annealing! (monte_carlo.jl:157-190) over the given temperature
 * sequence (T0, schedule(1), ... down to the last one above the target).
 * Returns the total accepted count. */
double orc_simulated_annealing(const orc_lattice *lat, double *spins, const double *temps,
                               int32_t n_temps, int64_t t_thermalization, int32_t or_rate,
                               int kind, double sigma0, orc_rng *r);

/* parallel_tempering! (monte_carlo.jl:235-398) with the R MPI ranks as R
 * in-process replicas of one lattice.  spins: R arrays of 3N (slot order; a
 * swap exchanges the arrays as MPI.Sendrecv! does).  sweeps between exchange
 * points run on n_threads POSIX threads (one replica per thread at a time).
 * Outputs (any may be NULL): accepted[R], exchanged[R] per slot;
 * probe_E/probe_M[n_probe_cap * R] in probe order.  Returns the number of probes. */
typedef struct {
    int64_t t_thermalization;
    int64_t t_measurement;
    int32_t probe_rate;
    int32_t swap_rate;
    int32_t overrelaxation_rate;
    int32_t kind;
    double sigma0;
    int32_t n_threads;
    uint64_t seed;
} orc_pt_params;
int64_t orc_parallel_tempering(const orc_lattice *lat, double **spins, const double *T,
                               int32_t R, const orc_pt_params *p, double *accepted,
                               double *exchanged, double *probe_E, double *probe_M,
                               int64_t n_probe_cap);

#ifdef __cplusplus
}
#endif
#endif
