/*
 * csmc.h -- C ABI of libcsmc.so, the GB300 (sm_103a) Monte Carlo sweep
 * library for classical spin Hamiltonians with Zeeman, onsite, bilinear,
 * cubic and quartic terms on Bravais lattices with a basis.
 *
 * This is the boundary a host binding (Julia `ccall`, Python `ctypes`, C/C++)
 * calls in place of the sweep routines of ClassicalSpinMC.jl v1.0.0.  Every
 * entry point names the reference routine it replaces (file:line within the
 * ClassicalSpinMC.jl project).  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every function returns CSMC_OK (0) or a CSMC_ERR_* code and never aborts;
 *    csmc_last_error() returns the calling thread's last message.
 *  - Spin arrays on the host use the reference layout: the 3 x N column-major
 *    Float64 array `lattice.spins` (lattice.jl:73), i.e. x,y,z interleaved per
 *    site, sites in the reference's order (basis slowest, last lattice
 *    dimension fastest; lattice.jl:29-33).
 *  - A context holds one or more lattices ("systems"), each with R replicas.
 *    Replica r of a system is temperature slot r: the MPI rank r of the
 *    reference's parallel tempering (monte_carlo.jl:246-259).  Exchanges swap
 *    which configuration sits in which slot; all per-replica inputs and
 *    outputs of this API are indexed by slot, in system order (slot index =
 *    sum of the replica counts of the earlier systems + r).
 *  - Host buffers are borrowed for the duration of the call.  Device memory
 *    is owned by the context.  One host thread per context at a time.
 *  - Basis indices in csmc_lattice_desc are 1-based, as in the reference API.
 */
#ifndef CSMC_H
#define CSMC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSMC_OK 0
#define CSMC_ERR_INVALID 1     /* bad argument or lattice description */
#define CSMC_ERR_OOM 2         /* device or host allocation failed */
#define CSMC_ERR_CUDA 3        /* CUDA runtime error (no device, launch failure, ...) */
#define CSMC_ERR_TIMEOUT 4     /* a bounded device wait gave up */
#define CSMC_ERR_COLOURING 5   /* no valid colouring within CSMC_MAX_COLOURS */
#define CSMC_ERR_UNSUPPORTED 6 /* description valid for the reference, not for these kernels */

#define CSMC_MAX_COLOURS 16

/* precision of a context */
#define CSMC_FP64 0 /* spins, fields and dE in Float64 */
#define CSMC_FP32 1 /* spins, fields and dE in Float32; energies, swap exponent and
                       observable accumulators in Float64 */

/* Metropolis sweep kinds: the FunctionWrapper constructors of metropolis.jl:181-199 */
#define CSMC_METROPOLIS 0           /* Metropolis()          -> metropolis!            :65-82   */
#define CSMC_METROPOLIS_ADAPTIVE 1  /* MetropolisAdaptive()  -> metropolis_adaptive!   :113-133 */
#define CSMC_METROPOLIS_FIXED_CONE 2 /* MetropolisFixedCone() -> metropolis_fixed_cone! :136-153 */
/* the constrained kinds (csmc_constraint): N proposals at random sites per
 * sweep, sequential per replica as in the reference, global path only */
#define CSMC_METROPOLIS_CONSTRAINT 3          /* MetropolisConstraint()         -> metropolis_constraint!          :36-58  */
#define CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE 4 /* MetropolisConstraintAdaptive() -> metropolis_constraint_adaptive! :155-179 */

/* execution path of the multi-sweep drivers */
#define CSMC_PATH_AUTO 0
#define CSMC_PATH_RESIDENT 1 /* persistent kernel, each replica held in shared memory */
#define CSMC_PATH_GLOBAL 2   /* one launch per colour class per sweep, all replicas batched */
#define CSMC_PATH_PER_REPLICA 3 /* like GLOBAL but one replica per launch ("plain" path) */

/* The arguments of `Lattice(shape, uc, S; bc)` (lattice.jl:65-66) with the
 * term lists of the UnitCell (unit_cell.jl:3-18, addZeemanCoupling! :30-32,
 * addOnSite! :37-41, addBilinear! :46-52, addCubic! :57-63, addQuartic! :68-75).
 * Matrices are row-major (m[a*3+b] = M[a,b]); cubic tensors t[(a*3+b)*3+c] =
 * C[a,b,c]; quartic t[((a*3+b)*3+c)*3+d] = R[a,b,c,d].  Offsets hold `dim`
 * ints per vector: bilinear one per term, cubic two (o2, o3), quartic three
 * (o2, o3, o4). */
typedef struct {
    int32_t dim;          /* D = 1, 2 or 3 */
    int32_t n_basis;      /* 0 is treated as one basis site (lattice.jl:68-70) */
    int32_t shape[3];     /* lattice extent per dimension (first `dim` used) */
    int32_t periodic;     /* 1: bc="periodic", 0: bc="open" */
    double spin_length;   /* S */
    int32_t n_field;
    const int32_t *field_basis;
    const double *field_vec;
    int32_t n_onsite;
    const int32_t *onsite_basis;
    const double *onsite_mat;
    int32_t n_bilinear;
    const int32_t *bilinear_basis; /* 2 per term */
    const double *bilinear_mat;    /* 9 per term */
    const int32_t *bilinear_offset;
    int32_t n_cubic;
    const int32_t *cubic_basis;    /* 3 per term */
    const double *cubic_tensor;    /* 27 per term */
    const int32_t *cubic_offset;
    int32_t n_quartic;
    const int32_t *quartic_basis;  /* 4 per term */
    const double *quartic_tensor;  /* 81 per term */
    const int32_t *quartic_offset;
} csmc_lattice_desc;

/* Summary of the flattened interaction tables of one lattice. */
typedef struct {
    int64_t n_sites;        /* N = prod(shape) * n_basis */
    int32_t n_colours;      /* colour classes of the interaction hypergraph */
    int32_t n_bilinear;     /* N2, N3, N4: the reference's per-site tuple lengths */
    int32_t n_cubic;
    int32_t n_quartic;
    int32_t width_bilinear; /* non-self bilinear slots per site in the device tables */
    int32_t width_cubic;
    int32_t width_quartic;
    int32_t n_matrices;     /* distinct 3x3 couplings after deduplication */
    int32_t n_cubic_tensors;
    int32_t n_quartic_tensors;
    int64_t padded_sites;   /* device length of one replica (colour classes padded) */
    int32_t n_isotropic_cubic;   /* distinct cubic tensors of the form kappa eps_abc */
    int32_t n_isotropic_quartic; /* distinct quartic tensors q1 d_ab d_cd + q2 d_ac d_bd + q3 d_ad d_bc */
} csmc_lattice_info;

/* Parameters of a multi-sweep run: the loop of parallel_tempering!
 * (monte_carlo.jl:288-388).  Iterations i = sweep_start .. sweep_start+n_sweeps-1
 * each run, in order: an overrelaxation sweep (if overrelaxation_rate != 0);
 * if i % max(overrelaxation_rate,1) == 0 a Metropolis sweep, the total energy,
 * and if i % swap_rate == 0 a replica exchange between neighbouring slots;
 * then, if i >= t_thermalization and i % probe_rate == 0, a probe recording
 * each slot's energy (from its last Metropolis sweep) and |M|. */
typedef struct {
    int64_t sweep_start;
    int64_t n_sweeps;
    int64_t t_thermalization;
    int32_t overrelaxation_rate;
    int32_t swap_rate;        /* <= 0: no exchanges */
    int32_t probe_rate;       /* <= 0: no probes */
    int32_t kind;             /* CSMC_METROPOLIS* */
    int32_t path;             /* CSMC_PATH_* */
    int32_t resident_block;   /* threads per CTA of the resident kernel: a multiple of 32, capped at the
                                 kernel's largest (896 or 512); 0 = automatic (balanced, or the autotuner's) */
    double *probe_energy;     /* [probe_capacity][n_slots] or NULL */
    double *probe_magnetization; /* [probe_capacity][n_slots] or NULL */
    int64_t probe_capacity;
    double *accepted;         /* [n_slots] accepted Metropolis proposals added, or NULL */
    double *exchanged;        /* [n_slots] accepted exchanges added, or NULL */
    int64_t n_probes_out;     /* set: probes recorded by this call */
} csmc_run_params;

/* ---------------------------------------------------------------- errors */
const char *csmc_last_error(void);
const char *csmc_version(void);

/* ------------------------------------------------ tables (host only, no GPU) */

/* Flatten and colour a lattice; replaces the table build of Lattice()
 * (lattice.jl:65-291) with arithmetic neighbour lookup instead of findfirst. */
int csmc_lattice_plan(const csmc_lattice_desc *desc, csmc_lattice_info *info);

/* Export the per-site tables in the layout of the Lattice struct
 * (lattice.jl:15-22): 1-based neighbour indices, 0 = absent, zero matrices
 * where the site plays no role.  Shapes as csmc_lattice_info's n_sites and
 * N2/N3/N4: bil_sites N*N2, bil_mats N*N2*9, cub_sites N*N3*2, cub_tens
 * N*N3*27, qua_sites N*N4*3, qua_tens N*N4*81, field N*3, onsite N*9.  Any
 * pointer may be NULL. */
int csmc_lattice_tables(const csmc_lattice_desc *desc, int64_t *bil_sites, double *bil_mats,
                        int64_t *cub_sites, double *cub_tens, int64_t *qua_sites,
                        double *qua_tens, double *field, double *onsite);

/* Colour of every site (reference order) and the device order: for device
 * position d < padded_sites, ref_of_device[d] is the 0-based reference site or
 * -1 for padding.  colour_start[c] is the first device position of colour c.
 * Any pointer may be NULL. */
int csmc_lattice_colouring(const csmc_lattice_desc *desc, int32_t *colour_of_site,
                           int64_t *ref_of_device, int64_t *colour_start);

/* ---------------------------------------------------------------- context */

/* Device half of MonteCarlo(T, lattice, params) (monte_carlo.jl:56-118) for
 * n_replicas temperature slots of one lattice.  Spins start at zero; call
 * csmc_random_spins or csmc_set_spins.  seed keys the Philox4x32-10 streams. */
int csmc_create(const csmc_lattice_desc *desc, int32_t precision, int32_t n_replicas,
                uint64_t seed, void **ctx_out);
/* Several lattices in one context, e.g. independent chains of different sizes. */
int csmc_create_batch(const csmc_lattice_desc *descs, int32_t n_lattices,
                      const int32_t *replicas_per_lattice, int32_t precision, uint64_t seed,
                      void **ctx_out);
int csmc_destroy(void *ctx);

int csmc_num_slots(void *ctx, int32_t *n_slots);
int csmc_lattice_info_of(void *ctx, int32_t lattice, csmc_lattice_info *info);

/* lattice.spins of one slot, reference layout (lattice.jl:293-301). */
int csmc_set_spins(void *ctx, int32_t slot, const double *spins);
int csmc_get_spins(void *ctx, int32_t slot, double *spins);
/* All slots, concatenated in slot order.  Pinned (page-locked or registered)
 * host buffers are read or written in place by the layout-conversion kernel
 * across the host link; pageable ones go through one bulk copy to a device
 * staging buffer.  Both return after the host buffer has been read (set) or
 * written (get). */
int csmc_set_spins_all(void *ctx, const double *spins);
int csmc_get_spins_all(void *ctx, double *spins);
/* Uniform random spins of length S from the Philox INIT stream
 * (Lattice initialCondition=:random, lattice.jl:76-79). */
int csmc_random_spins(void *ctx, uint64_t seed);

/* The key of each replica's random streams (Philox counter word 2), one per
 * replica in creation order (replica k starts in slot k and keeps its key
 * when exchanges move it).  Default: k.  A replica given the same key, seed
 * and spins in another context -- alone, or in a different batch -- draws
 * the same numbers and so runs the same chain.  Affects later sweeps and
 * csmc_random_spins.  No counterpart in the reference (its ranks draw from
 * unseeded task-local generators). */
int csmc_set_chain_ids(void *ctx, const uint32_t *ids);
/* mc.T per slot (monte_carlo.jl:72); also resets the slot permutation. */
int csmc_set_temperatures(void *ctx, const double *T);
/* mc.sigma per slot (monte_carlo.jl:79, metropolis.jl:84-87). */
int csmc_set_sigma(void *ctx, const double *sigma);
int csmc_get_sigma(void *ctx, double *sigma);
/* mc.sigma0 (monte_carlo.jl:80) of every slot: the cone width that
 * metropolis_constraint_adaptive! returns to after a sweep accepting at least
 * half of its proposals (metropolis.jl:177).  Default 60. */
int csmc_set_sigma0(void *ctx, double sigma0);

/* The `constraint` and `weight` of MonteCarlo (monte_carlo.jl:57,77-78) in a
 * closed form the device evaluates.  The reference takes any Julia function
 * of the lattice; here it is a function of the order parameter
 *     V = sum_i w_i s_i      (w_i = site_weights[i] in reference site order,
 *                             or 1 for every site when site_weights is NULL):
 *     c(lattice) = g . V + q |V|^2 + p |V| + c0.
 * Linear, quadratic and norm constraints on the uniform or on a staggered
 * magnetisation have this form.  Each constrained proposal evaluates c with
 * the proposed spin in place, sets lambda' = lambda - weight c and accepts
 * when dE - lambda' c < 0 or u < exp(-(dE - lambda' c) / T); an accepted
 * proposal keeps lambda' (metropolis.jl:43-54). */
typedef struct {
    const double *site_weights; /* [n_sites] or NULL */
    double g[3];
    double q, p, c0;
    double weight;
} csmc_constraint;
/* Constraint of every slot of lattice `lattice` (0-based, creation order);
 * NULL restores the reference's default x -> 0.0 with weight 0. */
int csmc_set_constraint(void *ctx, int32_t lattice, const csmc_constraint *constraint);
/* mc.lambda (metropolis.jl:21) of every slot; 0 at creation. */
int csmc_set_lambda(void *ctx, const double *lambda);
int csmc_get_lambda(void *ctx, double *lambda);
/* For each slot, the physical replica whose spins sit there. */
int csmc_get_permutation(void *ctx, int32_t *replica_of_slot);

/* ------------------------------------------------------------ hot path */

/* get_local_field (hamiltonian.jl:3-67) at every site of one slot; H is 3 x N
 * in the reference layout. */
int csmc_local_field(void *ctx, int32_t slot, double *H);
/* calculate_energy_diff! (metropolis.jl:94-110) without mutation: for n
 * proposals (0-based reference sites, new spins 3 per proposal), the energy
 * change of moving that one site, all else fixed. */
int csmc_energy_diff(void *ctx, int32_t slot, int64_t n, const int64_t *sites,
                     const double *new_spins, double *dE);
/* The same energy differences as csmc_energy_diff, with no device allocation.
 * No counterpart in the reference.  csmc_energy_diff allocates and frees its
 * device staging on every call; callers whose memory pool already holds the
 * GPU's memory, or whose proposal loop cannot afford the synchronising
 * cudaFree, use this one: it stages through a 2.5 MiB static device array
 * compiled into the library (held on every GPU that loads it until exit).
 * n may not exceed CSMC_ENERGY_DIFF_STATIC_MAX (CSMC_ERR_INVALID otherwise).
 * The first call on a device looks up the array's address with that device
 * current; make it before any stream capture.  All calls share the array and
 * it keeps the last call's contents (nothing in it needs to start at zero);
 * calls whose GPU work overlaps race on it and must be serialised. */
#define CSMC_ENERGY_DIFF_STATIC_MAX 65536
int csmc_energy_diff_static(void *ctx, int32_t slot, int64_t n, const int64_t *sites,
                            const double *new_spins, double *dE);
/* total_energy (hamiltonian.jl:70-132), one per slot. */
int csmc_total_energy(void *ctx, double *E);
/* get_magnetization (observables.jl:12-18): |sum_i s_i|, one per slot. */
int csmc_magnetization(void *ctx, double *M);

/* alg(mc, T): one Metropolis sweep on every slot at its temperature
 * (metropolis.jl:65-153).  The sweep visits every site once, colour class by
 * colour class; the constrained kinds instead make N proposals at random
 * sites in sequence, one replica per warp, drawing (site, u_acc) from the
 * Philox counter (p, sweep, chain, 5) and (u_phi, u_z) from (p, sweep, chain,
 * 6) for proposal p.  accepted[n_slots] (or NULL) receives the accepted count. */
int csmc_metropolis_sweep(void *ctx, int32_t kind, double *accepted);
/* alg(mc, T) with the temperature the caller passes, as simulated_annealing!
 * calls it with the schedule's T rather than mc.T (monte_carlo.jl:172-182;
 * the FunctionWrapper signature of metropolis.jl:181-199 carries T).  n_T = 1:
 * every slot sweeps at T[0]; n_T = n_slots: slot k sweeps at T[k].  The
 * slots' own temperatures (csmc_set_temperatures) and the slot permutation
 * are left unchanged.  Otherwise as csmc_metropolis_sweep. */
int csmc_metropolis_sweep_at(void *ctx, int32_t kind, const double *T, int32_t n_T, double *accepted);
/* overrelaxation! (monte_carlo.jl:126-139) on every slot. */
int csmc_overrelax_sweep(void *ctx);
/* deterministic_updates! (monte_carlo.jl:201-213) as n_sweeps colour sweeps
 * of s_i <- -S H_i/|H_i| on every slot. */
int csmc_deterministic_sweeps(void *ctx, int64_t n_sweeps);

/* Replay of metropolis!/metropolis_adaptive!/metropolis_fixed_cone!
 * (metropolis.jl:65-153) on one slot, fed with the reference's proposals: n
 * 0-based sites and uniforms.  u_acc[p] is used only where the exponent
 * (dE, or dE - lambda' c for the constrained kinds) is >= 0.  FP64,
 * sequential, the reference's evaluation order without FMA contraction; the
 * constrained kinds evaluate c over the whole lattice at every proposal, as
 * the reference calls its constraint function, and update the slot's lambda.
 * sigma is read (cone kinds) and, for the adaptive kinds, updated. */
int csmc_replay(void *ctx, int32_t slot, int32_t kind, double T, double *sigma, int64_t n,
                const int64_t *sites, const double *u_phi, const double *u_z,
                const double *u_acc, uint8_t *accepted);

/* The sweep loop of parallel_tempering! (monte_carlo.jl:288-388), every slot
 * at its temperature, exchanges on the device (monte_carlo.jl:308-349). */
int csmc_run(void *ctx, csmc_run_params *params);

/* simulated_annealing! (monte_carlo.jl:157-190) on every slot: for each of the
 * n_temps temperatures, sigma reset to sigma0, then t_thermalization-1
 * iterations of [overrelaxation, Metropolis every overrelaxation_rate-th].
 * accepted[n_temps * n_slots] or NULL. */
int csmc_anneal(void *ctx, const double *temps, int32_t n_temps, int64_t t_thermalization,
                int32_t overrelaxation_rate, int32_t kind, double sigma0, int32_t path,
                double *accepted);

/* CTAs per replica of the resident kernel (a thread-block cluster that splits
 * each replica's colour classes): 0 = automatic (the largest of 1, 2, 4 whose
 * clusters all fit on the device with >= 1024 sites per CTA), or force 1, 2
 * or 4.  Sizes above 1 need lattices without cubic/quartic terms and one
 * basis per colour class (CSMC_ERR_UNSUPPORTED otherwise).  A tuning knob of
 * this library; no counterpart in the reference. */
int csmc_set_cluster_size(void *ctx, int32_t ranks);
/* The cluster size in use; 0 while size groups are in use (each group has its own). */
int csmc_cluster_size(void *ctx, int32_t *ranks);

/* Size groups for batches of lattices of very different sizes (a scheduling
 * knob of this library; no counterpart in the reference, which runs one
 * lattice per MPI rank).  On: the lattices are sorted by size and split
 * wherever the size drops below half of the group's largest; each group gets
 * its own resident launch shape -- cluster size as csmc_set_cluster_size(0)
 * picks it for that group alone, and threads per CTA balanced for its largest
 * colour class -- and the groups' launches run side by side on streams of
 * their own, so small replicas run as small CTAs several to an SM while the
 * largest are split over clusters.  Every window is then one launch per group
 * (no persistent multi-window launches).  Off: one launch shape for the whole
 * context (the default; csmc_set_cluster_size also turns size groups off).
 * Chains are the same either way.  csmc_size_groups reports the number of
 * groups in use (0: off). */
int csmc_set_size_groups(void *ctx, int32_t on);
int csmc_size_groups(void *ctx, int32_t *n_groups);

/* compute_equal_time_correlations (spin_correlations.jl:6-43) for every slot
 * of lattice `lattice`: S_a(k) = sum_i exp(-i k.r_i) s_i,a and
 * Suv(k)[3a+b] = Re(S_a(k) conj(S_b(k))) / N.  positions: the reference's
 * site_positions, dim x N column-major (the dim coordinates of a site
 * contiguous, reference site order); ks: dim x n_k column-major; Suv:
 * [replicas of the lattice][n_k][9], the reference's 9 x N_k array per slot
 * in slot order.  Computed in the context's precision (sums of the phases
 * times the spins), the products of the sums in Float64 -- on the tensor
 * cores (csmc_set_tensor_cores) in FP32, the precision of the sums, and
 * returned as Float64.  The tensor-core path keeps its device scratch with
 * the context, grown as needed: the split spins, and partial sums (192 KB per
 * tile of 128 wavevectors x 64 replicas and per CTA its sites are split over,
 * when there are fewer tiles than SMs).  csmc_last_run_stats reports the
 * kernels' device time. */
int csmc_structure_factor(void *ctx, int32_t lattice, int32_t dim, const double *positions, int64_t n_k,
                          const double *ks, double *Suv);

/* Single-precision structure factors (csmc_structure_factor of a CSMC_FP32
 * context) on the tensor cores (on, the default: tcgen05 TF32 matrix
 * multiplies with each operand split into two TF32 halves, FP32 accumulation)
 * or on the CUDA cores (off: FP32 fused multiply-adds).  A choice of this
 * library; no counterpart in the reference.  Double-precision contexts always
 * use the CUDA cores. */
int csmc_set_tensor_cores(void *ctx, int32_t on);

/* Self-test of the bounded device waits (no counterpart in the reference).
 * Runs a kernel whose wait can never complete -- which = 0: an mbarrier phase
 * waiting for 16 bytes no copy delivers; which = 1: a grid barrier expecting
 * one more CTA than the launch has -- and returns what a run returns when a
 * wait gives up: CSMC_ERR_TIMEOUT after the kernel has set the error flag and
 * returned (a 20 ms budget here, one second in the sweep kernels); the flag is cleared and the context stays
 * usable.  Any other code is a failure of the bound. */
int csmc_selftest_timeout(void *ctx, int32_t which);

/* Persistent exchange windows (a tuning knob of this library; no counterpart
 * in the reference).  On (the default): when every replica of the context is
 * resident on the device at once, csmc_run runs up to 128 exchange windows in
 * one cooperative launch of the resident kernel, whose blocks meet at a
 * bounded grid barrier after each window, after which each replica takes the
 * exchange of its own pair (the same decision as its partner's) and writes
 * its own probe record; the replicas stay in shared memory across windows.
 * Off, or if the device refuses the cooperative launch: one launch per window
 * and a separate exchange launch.  Both give the same chain.
 * csmc_persistent reports whether persistent launches are in use. */
int csmc_set_persistent(void *ctx, int32_t on);
int csmc_persistent(void *ctx, int32_t *on);

/* Autotuner of the launch configuration (no counterpart in the reference; the
 * tuning knobs are this library's).  For every cluster size that fits (1, 2
 * or 4 CTAs per replica), two block sizes (the balanced one and the resident
 * kernel's largest), persistent windows on and off (see csmc_set_persistent)
 * size groups when the lattices' sizes differ by more than a factor two, and,
 * when params->path is CSMC_PATH_AUTO, the global colour-sweep path, it
 * times n_windows exchange windows of the
 * schedule in *params on the context's own replicas, restores the replicas and
 * every counter exactly (the chain continues as if no tuning had happened),
 * and keeps the fastest configuration for later CSMC_PATH_AUTO runs (the
 * fastest resident configuration for CSMC_PATH_RESIDENT runs).  entries[capacity]
 * receives the candidates with their device time per window; n_entries the
 * number of candidates (0 when the lattices run on the global path). */
typedef struct {
    int32_t path;          /* CSMC_PATH_RESIDENT or CSMC_PATH_GLOBAL */
    int32_t cluster;       /* CTAs per replica (resident); size groups (csmc_set_size_groups): 0 with
                              each group's own cluster size, -1 with one CTA per replica throughout */
    int32_t block;         /* threads per CTA; size groups: the cap on every group's CTAs (0: none) */
    int32_t persistent;    /* 1: windows and exchanges in one cooperative launch */
    double ms_per_window;  /* device time of one exchange window */
    int32_t chosen;        /* 1 for the configuration kept */
} csmc_tune_entry;
int csmc_autotune(void *ctx, const csmc_run_params *params, int32_t n_windows, csmc_tune_entry *entries,
                  int32_t capacity, int32_t *n_entries);

/* Spin-length renormalisation interval of the single-precision kernels, in
 * sweeps (0 = never).  Default 64. */
int csmc_set_renormalize(void *ctx, int32_t every_sweeps);
/* max over sites and slots of ||s_i| - S| / S. */
int csmc_spin_length_drift(void *ctx, double *drift);

/* Philox4x32-10 (Salmon et al., SC'11), the counter-based generator every
 * random draw of the sweep kernels comes from, evaluated by a device kernel
 * on the current device: out[4q..4q+3] = Philox(ctr[4q..4q+3], key[2q..2q+1])
 * for q < n.  A diagnostic of this library (its published known-answer
 * vectors); no counterpart in the reference, which draws from Julia's
 * default task RNG. */
int csmc_debug_philox(const uint32_t *ctr, const uint32_t *key, int64_t n, uint32_t *out);
/* Device allocations (cudaMalloc calls) the library has made in this process
 * so far, over all contexts: a diagnostic of this library, no counterpart in
 * the reference.  csmc_energy_diff_static leaves it unchanged. */
int csmc_debug_device_allocs(int64_t *count);

/* Device time (CUDA events on the context's stream) of the last csmc_run /
 * csmc_anneal call and the number of kernel launches it issued; of those, the
 * summed time and count of the resident sweep-kernel launches. */
int csmc_last_run_stats(void *ctx, double *device_ms, int64_t *launches, double *sweep_kernel_ms,
                        int64_t *sweep_kernel_launches);

#ifdef __cplusplus
}
#endif
#endif
