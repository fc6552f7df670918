// resident.cuh -- the persistent shared-memory sweep kernel.
//
// Each replica is held in shared memory for a whole window of the
// reference's loop (monte_carlo.jl:295-377: overrelaxation sweeps,
// Metropolis sweeps, the FP64 total energy, probes, spin renormalisation):
// it is staged in with bulk TMA copies (cp.async.bulk, completion on an
// mbarrier, bounded wait), updated colour class by colour class with a
// barrier between classes, and written back once (single precision: bulk
// TMA stores).  A persistent launch (cooperative, every replica resident)
// runs many exchange windows: the replicas stay in shared memory, and between
// windows all CTAs meet at one bounded grid barrier, after which each replica
// takes the exchange of its own pair (monte_carlo.jl:308-349; both replicas of
// a pair reach the same decision) and writes its own probe record.
//
// Shared-memory layout: the replica's spins in the device layout (single
// precision: one float4 per site; double: x | y | z blocks), then, for the
// specialised kernel when it fits, the packed partner words of the CTA's
// sites (one 16-byte word per site, also staged by TMA).
//
// A replica lives either in one CTA (CL = 1; a work list hands replicas out,
// largest first) or in a thread-block cluster of CL CTAs (CL = 2, 4): rank k
// holds part k of every colour class, partners owned by another rank are read
// through distributed shared memory (ld.shared::cluster), and the barrier
// between colour classes is a cluster barrier.  This spreads few replicas
// over more SMs.
//
// The block size is chosen at launch (a multiple of 32, at most NT) so that
// every thread updates the same number of sites between two barriers.
//
// Two physics policies share the driver loop:
//  * ResidentGeneric: per-site pattern, cubic and quartic terms (device.cuh);
//  * ResidentFast: no cubic/quartic terms and one basis per colour class; the
//    couplings of a colour class are loaded once per class into registers
//    (scalar couplings) or staged in shared memory (general 3x3), the onsite
//    matrices are specialised to none / diagonal / general, and the number of
//    bilinear partners per site W (4, 6 or 8) is a compile-time constant.
#pragma once

#include "kernels.cuh"
#include "reduce.cuh"

namespace csmc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// Bulk TMA copy global -> shared, completion counted on the mbarrier.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// Bulk TMA copy shared -> global in the current bulk group.
__device__ __forceinline__ void bulk_s2g(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}
// Close the bulk group and wait until all of its copies have completed.
__device__ __forceinline__ void bulk_commit_and_wait() {
    asm volatile("cp.async.bulk.commit_group;\n\tcp.async.bulk.wait_group 0;" ::: "memory");
}

// Nanoseconds of the global timer: the time bound of every device wait.
__device__ __forceinline__ uint64_t gtimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
constexpr uint64_t WAIT_BUDGET_NS = 1000000000ull; // one second

// Bounded wait on an mbarrier phase: gives up after `budget` nanoseconds and
// reports it through the context's error flag instead of hanging.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *error_flag,
                                                  uint64_t budget = WAIT_BUDGET_NS) {
    if (mbar_try_wait(bar, parity)) return true; // the timer is read only for a phase still open
    const uint64_t t0 = gtimer_ns();
    do {
        if (mbar_try_wait(bar, parity)) return true;
    } while (gtimer_ns() - t0 < budget);
    if (threadIdx.x == 0) atomicExch(error_flag, 1);
    return false;
}

// Barrier across every CTA of a cooperative launch (all CTAs co-resident):
// a monotonic arrival counter, zero at launch; the k-th barrier of the launch
// completes when the counter reaches k * n_blocks.  Bounded: thread 0 gives
// up after `budget` nanoseconds, or as soon as another CTA has reported an
// error, and sets the error flag.  Returns false (block-uniform) on failure.
__device__ __forceinline__ bool grid_barrier(unsigned int *ctr, unsigned int n_blocks, unsigned int &epoch,
                                             int *error_flag, int *s_ok, uint64_t budget = WAIT_BUDGET_NS) {
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch++;
        __threadfence();
        atomicAdd(ctr, 1u);
        const unsigned int target = epoch * n_blocks;
        int ok = 0;
        uint64_t t0 = 0;
        for (int k = 0;; k++) {
            unsigned int v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
            if (v >= target) {
                ok = 1;
                break;
            }
            if (k == 0) t0 = gtimer_ns(); // the timer is read only once the barrier is found open
            else if (gtimer_ns() - t0 >= budget) break;
            if ((k & 63) == 63 && *(volatile int *)error_flag) break;
            __nanosleep(64);
        }
        if (!ok) atomicExch(error_flag, 1);
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// ---- thread-block cluster primitives
// Hardware barrier of every thread of the cluster.  Its wait cannot be
// bounded; it is used only at points that every rank of a cluster reaches the
// same number of times (every decision to leave a loop is made cluster-wide,
// see cluster_all), and the ranks of a cluster are co-scheduled, so it ends.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cluster_ctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_index() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
// shared::cluster address of the same shared variable in CTA `rank`
__device__ __forceinline__ uint32_t map_rank(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
// Loads through the shared::cluster window (this CTA's or another rank's
// shared memory).  Volatile keeps them between the (volatile,
// memory-clobbering) barriers that order them; no memory clobber, since
// within a colour class they read sites no thread writes.
__device__ __forceinline__ double ld_cluster(uint32_t a, double) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a));
    return v;
}
// One site's spin through the cluster window: float4 at a (single
// precision) or x, y, z at a, a + comp, a + 2 comp (double precision).
__device__ __forceinline__ V3<float> cluster_spin(uint32_t a, uint32_t, float) {
    float x, y, z, w;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(x), "=f"(y), "=f"(z), "=f"(w) : "r"(a));
    return {x, y, z};
}
__device__ __forceinline__ V3<double> cluster_spin(uint32_t a, uint32_t comp, double) {
    return {ld_cluster(a, 0.0), ld_cluster(a + comp, 0.0), ld_cluster(a + 2 * comp, 0.0)};
}

__device__ __forceinline__ uint32_t ld_cluster_u32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}
// Cluster-wide AND of a block-uniform flag: every rank publishes its flag in
// `vote` (a shared word of each CTA), all ranks meet, read every rank's word,
// and meet again before the word can be reused.  All ranks return the same
// value, so a loop left on it is left by the whole cluster together: no rank
// exits while a peer can still read its shared memory or arrive on its
// barriers.
template <int CL> __device__ __forceinline__ bool cluster_all(bool ok, uint32_t *vote) {
    if (CL == 1) return ok;
    if (threadIdx.x == 0) *vote = ok ? 1u : 0u;
    cluster_sync_all();
    uint32_t all = 1u;
#pragma unroll
    for (int q = 0; q < CL; q++) all &= ld_cluster_u32(map_rank(smem_u32(vote), (uint32_t)q));
    cluster_sync_all();
    return all != 0u;
}

// Bytes of one site in shared memory per spin component block: 16 (float4
// sites) or 8 (one double of a component block).
template <typename R> constexpr uint32_t site_stride() { return sizeof(R) == 4 ? 16u : 8u; }
// Shared-memory view of `n` local sites starting at `base`.
__device__ __forceinline__ Spins<float> smem_spins(unsigned char *base, int64_t) {
    return {reinterpret_cast<float4 *>(base)};
}
__device__ __forceinline__ Spins<double> smem_spins_d(unsigned char *base, int64_t n) {
    return {reinterpret_cast<double *>(base), n};
}
template <typename R> __device__ __forceinline__ Spins<R> local_spins(unsigned char *base, int64_t n) {
    if constexpr (sizeof(R) == 4) return smem_spins(base, n);
    else return smem_spins_d(base, n);
}
__device__ __forceinline__ const void *spin_base(const Spins<float> &s) { return s.p; }
__device__ __forceinline__ const void *spin_base(const Spins<double> &s) { return s.x; }
// Bytes of the spin part of shared memory for n local sites.
template <typename R> __host__ __device__ constexpr int64_t spin_smem_bytes(int64_t n) {
    return sizeof(R) == 4 ? 16 * n : 24 * n;
}

// Block (CL = 1) or cluster barrier and sums; totals valid in thread 0 of
// every CTA, identical on all ranks (same summation order).
template <int CL> struct Sync {
    double *scratch, *red; // scratch: kSums x 32 doubles; red: kSums doubles (cluster exchange)
    static constexpr int kSums = 5; // the most values summed at once
    int *error_flag;
    // Barrier between colour classes: the block, or every thread of the
    // cluster (hardware cluster barrier, release/acquire at cluster scope, so
    // each rank's shared-memory writes are visible to the others' reads after
    // it).  Every rank runs the same colour loop, so all reach it.
    __device__ __forceinline__ void bar() const {
        if (CL > 1) cluster_sync_all();
        else __syncthreads();
    }
    template <typename T> __device__ double sum(T v) const {
        double t = block_sum_any(v, scratch);
        if (CL == 1) return t;
        if (threadIdx.x == 0) red[0] = t;
        cluster_sync_all();
        double tot = 0.0;
        if (threadIdx.x == 0)
            for (int r = 0; r < CL; r++) tot += ld_cluster(map_rank(smem_u32(red), r), 0.0);
        cluster_sync_all();
        return tot;
    }
    // N totals at once (the energy, the magnetisation and the accepted
    // proposals of a measuring sweep)
    template <int N, typename T> __device__ void sumn(const T (&x)[N], double (&o)[N]) const {
        static_assert(N <= kSums, "scratch holds kSums values");
        block_sumn_any<N>(x, scratch, o);
        if (CL == 1) return;
        if (threadIdx.x == 0)
#pragma unroll
            for (int q = 0; q < N; q++) red[q] = o[q];
        cluster_sync_all();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int q = 0; q < N; q++) o[q] = 0.0;
            for (int r = 0; r < CL; r++) {
                const uint32_t base = map_rank(smem_u32(red), r);
#pragma unroll
                for (int q = 0; q < N; q++) o[q] += ld_cluster(base + 8 * q, 0.0);
            }
        }
        cluster_sync_all();
    }
    template <typename T> __device__ void sum3(T x, T y, T z, double &a, double &b, double &c) const {
        a = block_sum_any(x, scratch);
        b = block_sum_any(y, scratch);
        c = block_sum_any(z, scratch);
        if (CL == 1) return;
        if (threadIdx.x == 0) {
            red[0] = a;
            red[1] = b;
            red[2] = c;
        }
        cluster_sync_all();
        if (threadIdx.x == 0) {
            a = b = c = 0.0;
            for (int r = 0; r < CL; r++) {
                const uint32_t base = map_rank(smem_u32(red), r);
                a += ld_cluster(base, 0.0);
                b += ld_cluster(base + 8, 0.0);
                c += ld_cluster(base + 16, 0.0);
            }
        }
        cluster_sync_all();
    }
};

// Local part of a replica in this CTA and the iteration over its colour class.
template <typename R, int CL> struct ResidentCommon {
    const ResSys<R> &S;
    Spins<R> sp; // this CTA's sites in shared memory (local indices)
    Sync<CL> sy;
    uint32_t key; // the replica's Philox stream key (its chain id)
    int slot, rank;
    R *scoef;

    __device__ __forceinline__ int col_begin(int col) const {
        return CL == 1 ? (int)S.col_start[col] : S.loc_start[rank][col];
    }
    __device__ __forceinline__ int col_size(int col) const {
        return CL == 1 ? (int)S.col_count[col] : S.loc_count[rank][col];
    }
    // device index of local site i of colour class col (the Philox counter)
    __device__ __forceinline__ int device_index(int col, int i) const {
        return CL == 1 ? i : S.src_start[rank][col] + (i - S.loc_start[rank][col]);
    }

    // |sum_i s_i|: each thread adds its sites in R, the block and the cluster
    // add the threads' partials in FP64
    __device__ double magnetization() const { // valid in thread 0
        R ax = R(0), ay = R(0), az = R(0);
        for (int col = 0; col < S.n_colours; col++) { // the sites of this CTA only
            const int st = col_begin(col), n = col_size(col);
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const V3<R> s = sp.get(st + i);
                ax = Fp<R>::add(ax, s.x);
                ay = Fp<R>::add(ay, s.y);
                az = Fp<R>::add(az, s.z);
            }
        }
        double mx, my, mz;
        sy.sum3(ax, ay, az, mx, my, mz);
        return threadIdx.x == 0 ? sqrt(mx * mx + my * my + mz * mz) : 0.0;
    }

    __device__ void renormalize() const {
        for (int col = 0; col < S.n_colours; col++) {
            const int st = col_begin(col), n = col_size(col);
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const V3<R> s = sp.get(st + i);
                const R n2 = dot(s, s);
                if (n2 == R(0)) continue;
                using F = Fp<R>;
                const R f = F::mul(S.S, Math<R>::rsqrt_(n2));
                sp.set(st + i, {F::mul(s.x, f), F::mul(s.y, f), F::mul(s.z, f)});
            }
        }
        sy.bar();
    }
};

// Spins of a replica split over a cluster, as partner_fields sees them:
// entry v = (relative owner << 14) | owner-local index; a partner in this
// CTA's part (top bits clear) is a plain shared-memory load, one in another
// rank's part a load through the shared::cluster window.  With CL = 1 the
// entry is the local index itself.
template <typename R, int CL> struct ClusterView {
    Spins<R> sp;
    uint32_t rb[CL]; // shared::cluster address of local site 0 of rank (rank + q) % CL, by q
    uint32_t comp;   // double precision: bytes between the x, y and z blocks
    __device__ __forceinline__ V3<R> get(int64_t v) const {
        const uint32_t u = (uint32_t)v;
        if (CL == 1 || (u >> 14) == 0u) return sp.get((int64_t)u);
        const uint32_t q = u >> 14, local = u & 0x3FFFu;
        uint32_t b = rb[0];
        if (CL == 2) b = rb[1 % CL];
        if (CL == 4) b = (q & 2u) ? ((q & 1u) ? rb[3 % CL] : rb[2 % CL]) : rb[1 % CL];
        return cluster_spin(b + local * site_stride<R>(), comp, R(0));
    }
};

template <typename R, bool CUB, bool QUA, int CL> struct ResidentGeneric : ResidentCommon<R, CL> {
    static constexpr int kMaxThreads = 512; // 128 registers per thread
    static constexpr int kCoefSmem = 1;
    static constexpr bool kPartnerWords = false;
    static constexpr bool kMeasuringSweep = false; // energy and |M| in separate passes
    using B = ResidentCommon<R, CL>;
    using B::key;
    using B::S;
    using B::sp;
    Tab<uint16_t> tb;      // this rank's tables (local indices; CL = 1: the replica's)
    ClusterView<R, CL> cv; // partner spins
    __device__ ResidentGeneric(const ResSys<R> &s, Spins<R> sp_, Sync<CL> sy_, uint32_t key_, int slot_, int rk,
                               R *coef, const uint4 *, bool)
        : B{s, sp_, sy_, key_, slot_, rk, coef} {
        tb = S.tb;
        cv.sp = sp_;
        cv.comp = (uint32_t)(S.Npl * sizeof(double));
        if (CL > 1) {
            const int64_t n = S.Npl;
            tb.Np = n;
            tb.p2 = S.q2c + (int64_t)rk * tb.W2 * n;
            tb.p3 = S.q3c + (int64_t)rk * tb.W3 * 2 * n;
            tb.p4 = S.q4c + (int64_t)rk * tb.W4 * 3 * n;
            tb.pat = S.patc + (int64_t)rk * n;
            const uint32_t a = smem_u32(spin_base(sp_));
#pragma unroll
            for (int q = 0; q < CL; q++) cv.rb[q] = map_rank(a, (uint32_t)((rk + q) % CL));
        }
    }
    __device__ void prepare() const {}

    template <bool MEASURE = false>
    __device__ unsigned metro_sweep(int kind, R sigma, R invT, double T, uint32_t msweep, R * = nullptr) const {
        unsigned acc = 0;
        for (int col = 0; col < S.n_colours; col++) {
            const int st = this->col_begin(col), n = this->col_size(col);
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int d = st + i;
                const uint32_t dg = (uint32_t)this->device_index(col, d);
                const int b = tb.pat[d];
                V3<R> hb, hc, hq;
                partner_fields<R, uint16_t, CUB, QUA>(tb, S.cf, cv, d, b, hb, hc, hq);
                const V3<R> hext = vsub(vadd(vadd(hb, hc), hq), V3<R>{S.cf.h[3 * b], S.cf.h[3 * b + 1], S.cf.h[3 * b + 2]});
                const V3<R> s = sp.get(d);
                const Draw<R> dr(dg, msweep, this->key, S.k0, S.k1);
                const V3<R> sn = propose<R>(kind, S.S, sigma, s, dr.uphi, dr.uz);
                const R dE = delta_e<R>(S.cf, b, s, sn, hext);
                bool accept = dE < R(0);
                if (!accept) accept = dr.acc(dg, msweep, this->key, S.k0, S.k1) < Math<R>::exp_(boltz_arg(dE, invT, T));
                if (accept) {
                    sp.set(d, sn);
                    acc++;
                }
            }
            this->sy.bar();
        }
        return acc;
    }

    __device__ void or_sweep() const {
        for (int col = 0; col < S.n_colours; col++) {
            const int st = this->col_begin(col), n = this->col_size(col);
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int d = st + i;
                const V3<R> H = local_field<R, uint16_t, CUB, QUA>(tb, S.cf, cv, d, tb.pat[d]);
                if (H.x == R(0) && H.y == R(0) && H.z == R(0)) continue;
                sp.set(d, reflect(sp.get(d), H, false));
            }
            this->sy.bar();
        }
    }

    __device__ double energy() const { // valid in thread 0; per-thread partials in R, their sum in FP64
        R acc = R(0);
        for (int col = 0; col < S.n_colours; col++) {
            const int st = this->col_begin(col), n = this->col_size(col);
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int d = st + i;
                acc = Fp<R>::add(acc, site_energy_share<R, uint16_t, CUB, QUA>(tb, S.cf, cv, d, tb.pat[d]));
            }
        }
        return this->sy.sum(acc);
    }
};

template <typename R, int BIL, int ONS, int W, int CL> struct ResidentFast : ResidentCommon<R, CL> {
    static_assert(W == 4 || W == 6 || W == 8, "partner widths 4, 6 and 8");
    // scalar couplings and at most diagonal onsite terms fit 64 registers per
    // thread (1024 threads); 3x3 couplings or general onsite terms get 128
    static constexpr int kMaxThreads = (BIL == 0 && ONS < 2) ? 896 : 512;
    static constexpr int WMAX = RESIDENT_WMAX;
    // per colour class in shared memory: J[W], A[9], Q[9], E2[9], h[3]; then
    // (3x3 couplings) the matrices [colour][W][9]
    static constexpr int kClassBlock = WMAX + 30;
    static constexpr int kCoefSmem = CSMC_MAX_COLOURS * kClassBlock + (BIL ? CSMC_MAX_COLOURS * WMAX * 9 : 0);
    static constexpr int OFF_A = WMAX, OFF_Q = WMAX + 9, OFF_E2 = WMAX + 18, OFF_H = WMAX + 27;
    static constexpr bool kPartnerWords = true;
    // a Metropolis sweep can also sum the energy and |M| of its final state
    // (two colour classes: every bond joins them)
    static constexpr bool kMeasuringSweep = true;
    using B = ResidentCommon<R, CL>;
    using B::key;
    using B::rank;
    using B::S;
    using B::scoef;
    using B::sp;
    const uint4 *pv; // packed partner words of this CTA's sites, by local index (shared or global memory)
    uint32_t pvs;    // their shared-memory address when staged there, else 0
    uint32_t rb[CL]; // shared::cluster address of local site 0 of rank (rank + q) % CL, by q (CL > 1)
    uint32_t comp;   // double precision: bytes between the x, y and z blocks

    __device__ ResidentFast(const ResSys<R> &s, Spins<R> sp_, Sync<CL> sy_, uint32_t key_, int slot_, int rk,
                            R *coef, const uint4 *pv_, bool pv_shared)
        : B{s, sp_, sy_, key_, slot_, rk, coef}, pv(pv_) {
        pvs = pv_shared ? smem_u32(pv_) : 0u;
        comp = (uint32_t)(S.Npl * sizeof(double));
        if (CL > 1) {
            const uint32_t a = smem_u32(spin_base(sp));
#pragma unroll
            for (int q = 0; q < CL; q++) rb[q] = map_rank(a, (uint32_t)((rk + q) % CL));
        }
    }

    // stage the couplings of every colour class in shared memory (slots
    // beyond the lattice's W2 are zero): the class blocks, and the 3x3
    // matrices at scoef[MAX_COLOURS * kClassBlock + (col*W + t)*9 + e]
    __device__ void prepare() const {
        const int W2 = S.tb.W2;
        for (int k = threadIdx.x; k < S.n_colours * kClassBlock; k += blockDim.x) {
            const int col = k / kClassBlock, e = k - col * kClassBlock, b = S.col_pattern[col];
            R v = R(0);
            if (e < WMAX) v = (BIL == 0 && e < W2) ? S.cf.Js[b * W2 + e] : R(0);
            else if (e < OFF_Q) v = S.cf.A[9 * b + e - OFF_A];
            else if (e < OFF_E2) v = S.cf.Q[9 * b + e - OFF_Q];
            else if (e < OFF_H) v = S.cf.E2[9 * b + e - OFF_E2];
            else v = S.cf.h[3 * b + e - OFF_H];
            scoef[k] = v;
        }
        if (BIL) {
            const int n = S.n_colours * W * 9;
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int col = k / (W * 9), rem = k - col * W * 9, t = rem / 9, e = rem - t * 9;
                const int b = S.col_pattern[col];
                scoef[CSMC_MAX_COLOURS * kClassBlock + k] = t < W2 ? S.cf.mats[9 * S.cf.c2[b * W2 + t] + e] : R(0);
            }
        }
        __syncthreads();
    }

    // per colour class, from shared memory: slot scalars J, the onsite-class
    // matrix m at offset `which` (OFF_A, OFF_Q or OFF_E2) and the field h
    __device__ __forceinline__ void load_coef(int col, int which, R (&J)[W], R (&m)[9], V3<R> &h) const {
        const R *blk = scoef + col * kClassBlock;
#pragma unroll
        for (int t = 0; t < W; t++) J[t] = BIL == 0 ? blk[t] : R(0);
#pragma unroll
        for (int k = 0; k < 9; k++) m[k] = ONS == 0 ? R(0) : blk[which + k];
        h = {blk[OFF_H], blk[OFF_H + 1], blk[OFF_H + 2]};
    }

    __device__ __forceinline__ V3<R> onsite(const R (&m)[9], V3<R> s) const {
        if (ONS == 0) return {R(0), R(0), R(0)};
        if (ONS == 1) return {Fp<R>::mul(m[0], s.x), Fp<R>::mul(m[4], s.y), Fp<R>::mul(m[8], s.z)};
        return matvec(m, s);
    }

    __device__ __forceinline__ void accumulate(V3<R> &hb, int col, int t, const R (&J)[W], V3<R> s) const {
        if (BIL == 0) hb = add_scaled(hb, J[t], s);
        else hb = add_matvec(hb, scoef + CSMC_MAX_COLOURS * kClassBlock + (col * W + t) * 9, s);
    }

    // the spin of cluster partner entry v = (relative owner q << 14) |
    // owner-local index, read through the shared::cluster window
    __device__ __forceinline__ V3<R> partner_cluster(uint32_t v) const {
        const uint32_t q = v >> 14, local = v & 0x3FFFu;
        uint32_t b = rb[0];
        if (CL == 2) b = q ? rb[1 % CL] : rb[0];
        if (CL == 4) b = (q & 2u) ? ((q & 1u) ? rb[3 % CL] : rb[2 % CL]) : ((q & 1u) ? rb[1 % CL] : rb[0]);
        return cluster_spin(b + local * site_stride<R>(), comp, R(0));
    }

    // sum over bilinear slots of J_t s_j at local site i: the partner entries
    // come in one 16-byte word, every partner load is issued before use.  In
    // a cluster, a warp whose sites all have their partners in this CTA reads
    // them with plain shared-memory loads; a warp with any partner in another
    // rank reads all of its partners through the cluster window.
    __device__ __forceinline__ uint4 word(int i) const {
        uint4 w;
        if (pvs) // block-uniform
            asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(w.x), "=r"(w.y), "=r"(w.z), "=r"(w.w)
                         : "r"(pvs + 16u * (uint32_t)i));
        else
            w = pv[i];
        return w;
    }
    // the partner word of the first site of this thread in [st, st + n)
    __device__ __forceinline__ uint4 first_word(int st, int n) const {
        return (int)threadIdx.x < n ? word(st + (int)threadIdx.x) : make_uint4(0u, 0u, 0u, 0u);
    }
    // the partner word of the next site of this thread (loaded one site ahead)
    __device__ __forceinline__ uint4 next_word(int st, int n, int k) const {
        return k + (int)blockDim.x < n ? word(st + k + (int)blockDim.x) : make_uint4(0u, 0u, 0u, 0u);
    }

    __device__ __forceinline__ V3<R> gather(int col, const R (&J)[W], uint4 w, V3<R> init = {R(0), R(0), R(0)}) const {
        const uint32_t v[8] = {w.x & 0xFFFFu, w.x >> 16, w.y & 0xFFFFu, w.y >> 16,
                               w.z & 0xFFFFu, w.z >> 16, w.w & 0xFFFFu, w.w >> 16};
        V3<R> s[W];
        bool local = true;
        if (CL > 1) local = !__any_sync(__activemask(), ((w.x | w.y | w.z | w.w) & 0xC000C000u) != 0u);
        if (local) {
#pragma unroll
            for (int t = 0; t < W; t++) s[t] = sp.get((int)v[t]);
        } else { // per slot: plain loads unless some lane's partner is in another rank
            const unsigned act = __activemask();
#pragma unroll
            for (int t = 0; t < W; t++) {
                const bool far = (v[t] >> 14) != 0u;
                if (__any_sync(act, far)) s[t] = far ? partner_cluster(v[t]) : sp.get((int)v[t]);
                else s[t] = sp.get((int)v[t]);
            }
        }
        V3<R> hb = init;
#pragma unroll
        for (int t = 0; t < W; t++) accumulate(hb, col, t, J, s[t]);
        return hb;
    }

    // the onsite part of the local field added to acc: diagonal terms by one
    // fused multiply-add per component, general matrices by add_matvec
    __device__ __forceinline__ V3<R> add_onsite(V3<R> acc, const R (&m)[9], V3<R> s) const {
        using F = Fp<R>;
        if (ONS == 0) return acc;
        if (ONS == 1) return {F::fma(m[0], s.x, acc.x), F::fma(m[4], s.y, acc.y), F::fma(m[8], s.z, acc.z)};
        return add_matvec(acc, m, s);
    }

    // overrelaxation (monte_carlo.jl:128-137): H = A s + sum_t J_t s_t - h,
    // accumulated from -h; a site without field (|H|^2 = 0) keeps its spin
    __device__ void or_sweep() const {
        using F = Fp<R>;
        for (int col = 0; col < S.n_colours; col++) {
            R J[W], a[9];
            V3<R> h;
            load_coef(col, OFF_A, J, a, h);
            const V3<R> nh = {-h.x, -h.y, -h.z};
            const int st = this->col_begin(col), n = this->col_size(col);
            uint4 wn = first_word(st, n);
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int d = st + k;
                const uint4 w = wn;
                wn = next_word(st, n, k);
                const V3<R> hb = gather(col, J, w, nh);
                const V3<R> s = sp.get(d);
                const V3<R> H = add_onsite(hb, a, s);
                const R den = dot(H, H);
                if (den == R(0)) continue;
                const R proj = Math<R>::div_(F::mul(R(2), dot(s, H)), den);
                sp.set(d, {F::fma(proj, H.x, -s.x), F::fma(proj, H.y, -s.y), F::fma(proj, H.z, -s.z)});
            }
            this->sy.bar();
        }
    }

    // One Metropolis sweep.  MEASURE (lattices of two colour classes): each
    // site's final spin s also adds to this thread's partials meas[0..3] =
    // {energy, M_x, M_y, M_z}: s.(O + P/2).s - s.h for every site, plus s.hb
    // (its whole bilinear field) for the sites of class 1 -- their partners
    // are all of class 0 and already final, and every bond, having one end in
    // each class, is counted once; the sum is total_energy
    // (hamiltonian.jl:70-132) of the state the sweep leaves.
    template <bool MEASURE = false>
    __device__ unsigned metro_sweep(int kind, R sigma, R invT, double T, uint32_t msweep, R *meas = nullptr) const {
        unsigned acc = 0;
        R pe = R(0), pmx = R(0), pmy = R(0), pmz = R(0);
        for (int col = 0; col < S.n_colours; col++) {
            R J[W], q[9], e2[9];
            V3<R> h;
            load_coef(col, OFF_Q, J, q, h);
            if (MEASURE) load_coef(col, OFF_E2, J, e2, h);
            const V3<R> nh = {-h.x, -h.y, -h.z};
            const bool bonds = MEASURE && col == 1;
            const int st = this->col_begin(col), n = this->col_size(col);
            uint4 wn = first_word(st, n);
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int d = st + k;
                const uint4 w = wn;
                wn = next_word(st, n, k);
                const uint32_t dg = (uint32_t)this->device_index(col, d);
                const V3<R> hext = gather(col, J, w, nh); // hb - h, accumulated from -h
                const V3<R> s = sp.get(d);
                const Draw<R> dr(dg, msweep, this->key, S.k0, S.k1);
                const V3<R> sn = propose<R>(kind, S.S, sigma, s, dr.uphi, dr.uz);
                using F = Fp<R>;
                const R dE = F::add(F::sub(dot(sn, onsite(q, sn)), dot(s, onsite(q, s))), dot(vsub(sn, s), hext));
                bool accept = dE < R(0);
                if (!accept) accept = dr.acc(dg, msweep, this->key, S.k0, S.k1) < Math<R>::exp_(boltz_arg(dE, invT, T));
                if (accept) {
                    sp.set(d, sn);
                    acc++;
                }
                if (MEASURE) { // class 1: s.E2.s + s.(hb - h); class 0: s.E2.s - s.h
                    const V3<R> f = accept ? sn : s;
                    const R part = bonds ? F::add(dot(f, onsite(e2, f)), dot(f, hext))
                                         : F::sub(dot(f, onsite(e2, f)), dot(f, h));
                    pe = F::add(pe, part);
                    pmx = F::add(pmx, f.x);
                    pmy = F::add(pmy, f.y);
                    pmz = F::add(pmz, f.z);
                }
            }
            this->sy.bar();
        }
        if (MEASURE) {
            meas[0] = pe;
            meas[1] = pmx;
            meas[2] = pmy;
            meas[3] = pmz;
        }
        return acc;
    }

    __device__ double energy() const { // valid in thread 0; per-thread partials in R, their sum in FP64
        R acc = R(0);
        for (int col = 0; col < S.n_colours; col++) {
            R J[W], m[9];
            V3<R> h;
            load_coef(col, OFF_E2, J, m, h);
            const int st = this->col_begin(col), n = this->col_size(col);
            uint4 wn = first_word(st, n);
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int d = st + k;
                const uint4 w = wn;
                wn = next_word(st, n, k);
                const V3<R> hb = gather(col, J, w);
                const V3<R> s = sp.get(d);
                const R part = Fp<R>::sub(dot(s, onsite(m, s)), dot(s, h));
                acc = Fp<R>::add(acc, Fp<R>::fma(R(0.5), dot(s, hb), part));
            }
        }
        return this->sy.sum(acc);
    }
};

// Probe of iteration q exists?  (q >= t_therm and q % probe_rate == 0)
__device__ __forceinline__ bool is_probe(const RunDesc &rd, int64_t q) {
    return rd.probe_rate > 0 && q >= rd.t_therm && q % rd.probe_rate == 0;
}

// Shared memory of one CTA: the spins of its nl local sites, then (specialised
// kernel, when the lattice's descriptor says so) its nl packed partner words.
template <typename R> __host__ __device__ constexpr int64_t partner_words_offset(int64_t nl) {
    return (spin_smem_bytes<R>(nl) + 15) / 16 * 16;
}

template <typename K, typename R, int NT, int CL>
__global__ void __launch_bounds__(NT, 1)
    k_resident(const ResSys<R> *__restrict__ systems, const int2 *__restrict__ items, int n_items, int *work_ctr,
               ChainState cs, RunDesc rd) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    __shared__ double scratch[Sync<CL>::kSums * 32];
    __shared__ double red[Sync<CL>::kSums];
    __shared__ int s_item;
    __shared__ int s_ok;
    __shared__ uint32_t s_vote;
    __shared__ double s_sigma, s_T;
    __shared__ R s_invT;
    __shared__ int s_slot;
    __shared__ ResSys<R> s_sys;
    __shared__ R s_coef[K::kCoefSmem];
    uint32_t parity = 0;
    const int rank = CL == 1 ? 0 : (int)cluster_ctarank();
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (CL > 1) cluster_sync_all(); // every rank has started before any reads another's shared memory
    const int64_t dosweep = rd.or_rate == 0 ? 1 : rd.or_rate;
    const Sync<CL> sync{scratch, red, cs.error_flag};
    int item = CL == 1 ? 0 : (int)cluster_index();

    for (;; item += (CL == 1 ? 0 : (int)cluster_count())) {
        if (CL == 1) {
            if (threadIdx.x == 0) s_item = atomicAdd(work_ctr, 1);
            __syncthreads();
            item = s_item;
        }
        if (item >= n_items) break;
        const int2 w = items[item];
        { // copy the lattice descriptor into shared memory with all threads
            static_assert(sizeof(ResSys<R>) % 4 == 0, "descriptor copied in 4-byte words");
            const uint32_t *src = reinterpret_cast<const uint32_t *>(systems + w.x);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&s_sys);
            for (int k = threadIdx.x; k < (int)(sizeof(ResSys<R>) / 4); k += blockDim.x) dst[k] = src[k];
        }
        __syncthreads();
        const ResSys<R> &S = s_sys;
        const int r = w.y;
        const int c = S.chain_base + r;
        const int64_t Np = S.tb.Np;
        const int64_t nl = CL == 1 ? Np : S.Npl;
        const Spins<R> g = spins_of(S.spins, Np, r); // the replica in device memory
        const Spins<R> sp = local_spins<R>(smem_raw, nl);
        const bool words = K::kPartnerWords && S.pv_stage;
        const uint4 *gwords = CL == 1 ? S.p2v : S.q2v + (int64_t)rank * S.Npl;
        uint4 *swords = reinterpret_cast<uint4 *>(smem_raw + partner_words_offset<R>(nl));

        // stage this CTA's part of the replica (and its partner words) with bulk TMA copies
        if (threadIdx.x == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            uint32_t total = words ? (uint32_t)(nl * 16) : 0u;
            if (CL == 1) {
                total += (uint32_t)spin_smem_bytes<R>(Np);
            } else {
                for (int col = 0; col < S.n_colours; col++)
                    total += (uint32_t)spin_smem_bytes<R>((S.loc_count[rank][col] + 31) / 32 * 32);
            }
            mbar_expect_tx(&bar, total);
            if (words) bulk_g2s(swords, gwords, (uint32_t)(nl * 16), &bar);
            if (CL == 1) {
                if constexpr (sizeof(R) == 4) {
                    bulk_g2s(sp.p, g.p, (uint32_t)(Np * 16), &bar);
                } else {
                    const uint32_t bytes = (uint32_t)(Np * sizeof(R));
                    bulk_g2s(sp.x, g.x, bytes, &bar);
                    bulk_g2s(sp.x + Np, g.x + Np, bytes, &bar);
                    bulk_g2s(sp.x + 2 * Np, g.x + 2 * Np, bytes, &bar);
                }
            } else {
                for (int col = 0; col < S.n_colours; col++) {
                    const int n = (S.loc_count[rank][col] + 31) / 32 * 32;
                    if (n == 0) continue;
                    const int ls = S.loc_start[rank][col], gs = S.src_start[rank][col];
                    if constexpr (sizeof(R) == 4) {
                        bulk_g2s(sp.p + ls, g.p + gs, (uint32_t)(n * 16), &bar);
                    } else {
                        const uint32_t bytes = (uint32_t)(n * sizeof(R));
                        bulk_g2s(sp.x + ls, g.x + gs, bytes, &bar);
                        bulk_g2s(sp.x + nl + ls, g.x + Np + gs, bytes, &bar);
                        bulk_g2s(sp.x + 2 * nl + ls, g.x + 2 * Np + gs, bytes, &bar);
                    }
                }
            }
        }
        const bool ok = mbar_wait_bounded(&bar, parity, cs.error_flag);
        parity ^= 1;
        const bool local_fail = __syncthreads_or(!ok); // block-uniform
        const bool fail = !cluster_all<CL>(!local_fail, &s_vote); // cluster-uniform: any rank failed
        if (fail) {
            if (local_fail) mbar_wait_bounded(&bar, parity ^ 1, cs.error_flag); // copies still in flight
            __syncthreads();
            if (CL == 1) continue;
            break; // a cluster drops its remaining items together
        }
        if (CL > 1) { // zero this rank's sentinel block, then every rank is staged
            const int sent = S.Npl - 32;
            for (int k = threadIdx.x; k < 32; k += blockDim.x) sp.set(sent + k, {R(0), R(0), R(0)});
            cluster_sync_all();
        }

        const K k(S, sp, sync, __ldg(cs.chain_id + c), 0, rank, s_coef, words ? swords : gwords, words);
        k.prepare();
        const bool writer = threadIdx.x == 0 && rank == 0;
        double E = cs.E_chain[c];
        uint32_t msweep = rd.msweep0;
        // single precision: renormalise |s| = S whenever the context's total
        // sweep count passes a multiple of renorm_every
        uint64_t sweeps = rd.sweeps0;
        const uint64_t every = rd.renorm_every > 0 ? (uint64_t)rd.renorm_every : 0;
        uint64_t next_renorm = every ? (sweeps / every + 1) * every : 0;
        unsigned int epoch = 0;
        int cur_slot = -1; // persistent windows: the slot after the last exchange (-1: read it)

        for (int64_t w0 = rd.it0; w0 < rd.it1;) {
            // the window [w0, w1): the whole launch, or (persistent) up to the
            // next exchange iteration.  The slot of this replica, its
            // temperature and sigma are read per window: the exchange between
            // windows moves replicas between slots (loads bypass L1, other
            // blocks wrote them).
            int64_t w1 = rd.it1;
            if (rd.persistent && rd.swap_enabled) {
                const int64_t q = (w0 + rd.swap_period - 1) / rd.swap_period * rd.swap_period;
                if (q + 1 < w1) w1 = q + 1;
            }
            const int slot = cur_slot >= 0 ? cur_slot : __ldcg(cs.slot_of + c);
            // T, 1/T and sigma of the slot by thread 0, unless the exchange
            // that ended the previous window took them already.  Single
            // precision reads 1/T formed on the host (the same value: FP64
            // division runs at a small fraction of the FP32 rate here).
            if (threadIdx.x == 0 && cur_slot < 0) {
                s_sigma = (rd.reset_sigma && w0 == rd.it0) ? rd.sigma0 : __ldcg(cs.sigma_slot + slot);
                s_T = rd.T_override > 0 ? rd.T_override : __ldcg(cs.T_slot + slot);
                s_invT = (sizeof(R) == 4 && rd.T_override <= 0) ? (R)__ldcg(cs.invT_slot + slot) : (R)(1.0 / s_T);
            }
            __syncthreads();
            const double T = s_T;
            const R invT = s_invT;
            double acc_total = 0.0;
            // accepted proposals of this thread's sites: summed over the block
            // (and cluster) after every Metropolis sweep when the adaptive
            // kind needs the rate, else once at the end of the window
            const bool adaptive = rd.kind == CSMC_METROPOLIS_ADAPTIVE;
            unsigned acc_thread = 0;
            bool acc_summed = false; // the window's accepted proposals already summed (measuring sweep)

            for (int64_t it = w0; it < w1; it++) {
                if (rd.or_rate != 0) {
                    k.or_sweep();
                    sweeps++;
                }
                const bool metro = it % dosweep == 0;
                bool have_M = false; // |M| of this iteration's state summed by its Metropolis sweep
                double M = 0.0;
                if (metro) {
                    // energy needed: exchange point, a probe before the next
                    // Metropolis sweep, or the last Metropolis sweep of the window
                    bool needE = rd.swap_enabled && rd.swap_rate > 0 && it % rd.swap_rate == 0;
                    for (int64_t q = it; q < it + dosweep && q < w1 && !needE; q++) needE = is_probe(rd, q);
                    needE = needE || it + dosweep >= w1;
                    // with two colour classes the sweep itself sums the energy
                    // and |M| of the state it leaves
                    const bool measure = K::kMeasuringSweep && needE && S.n_colours == 2;
                    R meas[4];
                    const unsigned a = measure ? k.template metro_sweep<true>(rd.kind, (R)s_sigma, invT, T, msweep, meas)
                                               : k.template metro_sweep<false>(rd.kind, (R)s_sigma, invT, T, msweep);
                    msweep++;
                    sweeps++;
                    if (adaptive) {
                        const double at = sync.sum(a); // exact: an integer sum per warp
                        if (threadIdx.x == 0) { // metropolis.jl:124-126
                            acc_total += at;
                            const double om = 1 - at / (double)S.n_real;
                            const double f = 0.5 / (om > 0.05 ? om : 0.05);
                            double sg = s_sigma * f;
                            s_sigma = sg < 0.0 ? 0.0 : (sg > 100 ? 100 : sg);
                        }
                        __syncthreads();
                    } else {
                        acc_thread += a;
                    }
                    if (measure) {
                        // the window's last Metropolis sweep also sums the
                        // window's accepted proposals (small integers: exact
                        // in the value type and in FP64)
                        const bool with_acc = !adaptive && it + dosweep >= w1;
                        double o[5];
                        if (with_acc) {
                            const R x[5] = {meas[0], meas[1], meas[2], meas[3], (R)acc_thread};
                            sync.sumn<5>(x, o);
                            acc_summed = true;
                            if (threadIdx.x == 0) acc_total = o[4];
                        } else {
                            const R x[4] = {meas[0], meas[1], meas[2], meas[3]};
                            double o4[4];
                            sync.sumn<4>(x, o4);
                            for (int q = 0; q < 4; q++) o[q] = o4[q];
                        }
                        if (threadIdx.x == 0) { // the totals are thread 0's (FP64 in one lane only)
                            E = o[0];
                            M = sqrt(o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
                        }
                        have_M = true;
                    } else if (needE) {
                        const double e = k.energy();
                        if (threadIdx.x == 0) E = e;
                    }
                }
                // a probe at an exchange iteration (the window's last) is
                // recorded after the exchange, from M_chain
                const bool swap_here = metro && rd.swap_enabled && rd.swap_rate > 0 && it % rd.swap_rate == 0;
                if (is_probe(rd, it)) {
                    if (!have_M) M = k.magnetization();
                    if (writer) {
                        const int64_t kq = (it - rd.probe_first) / rd.probe_rate;
                        if (!swap_here && kq >= 0 && kq < rd.probe_cap) {
                            if (rd.rec_E) rd.rec_E[kq * rd.n_slots + slot] = E;
                            if (rd.rec_M) rd.rec_M[kq * rd.n_slots + slot] = M;
                        }
                        cs.M_chain[c] = M;
                    }
                }
                if (sizeof(R) == 4 && every && sweeps >= next_renorm) {
                    k.renormalize();
                    next_renorm = (sweeps / every + 1) * every;
                }
            }

            if (!adaptive && !acc_summed) {
                const double at = sync.sum(acc_thread);
                if (threadIdx.x == 0) acc_total = at;
            }
            const int64_t last = w1 - 1;
            const bool exchange = rd.persistent && rd.swap_enabled && last % rd.swap_period == 0;
            // the window's energy by slot, for the exchange (buffers alternate
            // by window: a buffer is rewritten only two windows later, after a
            // grid barrier that every reader of it has passed)
            double *const E_slot = cs.E_win + (int64_t)((last / (rd.swap_period > 0 ? rd.swap_period : 1)) & 1) * rd.n_slots;
            if (writer) {
                cs.E_chain[c] = E;
                // one owner adds to a slot's counters per window, windows in
                // order: the additions need no read here (and keep their order)
                atomicAdd(cs.acc_slot + slot, acc_total);
                cs.sigma_slot[slot] = s_sigma;
                if (exchange) E_slot[slot] = E;
            }
            w0 = w1;
            if (!exchange) break;
            // every window's energies written, then each replica takes the
            // exchange of its own pair (the same decision as its partner's)
            // and moves to its new slot: one grid barrier per window, no CTA
            // reads a value another writes before the next barrier.  A barrier
            // that gave up (timeout, or another CTA's error) ends the launch;
            // the ranks of a cluster decide together.
            if (!cluster_all<CL>(grid_barrier(rd.grid_bar, rd.n_blocks, epoch, cs.error_flag, &s_ok), &s_vote)) break;
            if (threadIdx.x == 0) {
                const int2 lat = rd.lattices[w.x];
                // the partner slot's T, 1/T and sigma, loaded beside the decision's operands
                const int ps = exchange_pair_slot(lat.x, lat.y, slot, last, rd.swap_rate);
                double p_sigma = 0.0, p_T = 1.0;
                R p_invT = R(1);
                if (ps >= 0) {
                    p_sigma = __ldcg(cs.sigma_slot + ps);
                    p_T = __ldcg(cs.T_slot + ps);
                    p_invT = sizeof(R) == 4 ? (R)__ldcg(cs.invT_slot + ps) : (R)__ldcg(cs.invT64_slot + ps);
                }
                bool swapped = false;
                const int ns = exchange_partner(cs, E_slot, w.x, lat.x, lat.y, slot, last, rd.swap_rate, rd.k0, rd.k1,
                                                &swapped);
                if (rank == 0) { // the chain's records (each slot has one writer)
                    if (swapped) {
                        atomicAdd(cs.exch_slot + slot, 1.0);
                        cs.slot_of[c] = ns;
                        cs.chain_of[ns] = c;
                    }
                    if (is_probe(rd, last)) { // the probe record of the exchange iteration, by the new slot
                        const int64_t kq = (last - rd.probe_first) / rd.probe_rate;
                        if (kq >= 0 && kq < rd.probe_cap) {
                            if (rd.rec_E) rd.rec_E[kq * rd.n_slots + ns] = E;
                            if (rd.rec_M) rd.rec_M[kq * rd.n_slots + ns] = cs.M_chain[c];
                        }
                    }
                }
                s_slot = ns;
                if (swapped) { // the new slot's T, 1/T and sigma for the next window
                    s_sigma = p_sigma;
                    s_T = p_T;
                    s_invT = p_invT;
                }
            }
            __syncthreads();
            cur_slot = s_slot;
        }
        // every thread's shared-memory accesses are ordered before the bulk
        // copies that follow (the stores below, the next item's staging)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        // write this CTA's part back: bulk TMA stores of the float4 sites
        // (single precision), a store loop over the component blocks (double)
        if constexpr (sizeof(R) == 4) {
            if (threadIdx.x == 0) {
                if (CL == 1) {
                    bulk_s2g(g.p, sp.p, (uint32_t)(Np * 16));
                } else {
                    for (int col = 0; col < S.n_colours; col++) {
                        const int n = S.loc_count[rank][col];
                        if (n > 0) bulk_s2g(g.p + S.src_start[rank][col], sp.p + S.loc_start[rank][col], (uint32_t)(n * 16));
                    }
                }
                bulk_commit_and_wait();
            }
        } else {
            if (CL == 1) {
                for (int64_t i = threadIdx.x; i < 3 * Np; i += blockDim.x) g.x[i] = sp.x[i];
            } else {
                for (int col = 0; col < S.n_colours; col++) {
                    const int n = S.loc_count[rank][col], ls = S.loc_start[rank][col], gs = S.src_start[rank][col];
                    for (int i = threadIdx.x; i < n; i += blockDim.x) {
                        g.x[gs + i] = sp.x[ls + i];
                        g.x[Np + gs + i] = sp.x[nl + ls + i];
                        g.x[2 * Np + gs + i] = sp.x[2 * nl + ls + i];
                    }
                }
            }
        }
        if (CL > 1) cluster_sync_all(); // no rank reads another's shared memory past this point
        __syncthreads();
    }
}

// Kernel entry points of each instantiation family (resident_*.cu).
template <typename R> const void *resident_kernel_generic(bool cub, bool qua, int cl);

template <typename R, bool CUB, bool QUA> const void *resident_generic_for(int cl) {
    constexpr int NT = resident_max_threads(false, 0, 0);
    if (cl == 4) return (const void *)k_resident<ResidentGeneric<R, CUB, QUA, 4>, R, NT, 4>;
    if (cl == 2) return (const void *)k_resident<ResidentGeneric<R, CUB, QUA, 2>, R, NT, 2>;
    return (const void *)k_resident<ResidentGeneric<R, CUB, QUA, 1>, R, NT, 1>;
}
// specialised kernels of width W (defined in resident_fast_<precision>_w<W>.cu)
template <typename R, int W> const void *resident_kernel_fast(int bil, int ons, int cl);

template <typename R, int W, int BIL, int ONS, int CL> const void *resident_fast_kernel() {
    using K = ResidentFast<R, BIL, ONS, W, CL>;
    static_assert(K::kMaxThreads == resident_max_threads(true, BIL, ONS), "launch bound");
    return (const void *)k_resident<K, R, K::kMaxThreads, CL>;
}
template <typename R, int W, int BIL, int ONS> const void *resident_fast_for(int cl) {
    if (cl == 4) return resident_fast_kernel<R, W, BIL, ONS, 4>();
    if (cl == 2) return resident_fast_kernel<R, W, BIL, ONS, 2>();
    return resident_fast_kernel<R, W, BIL, ONS, 1>();
}
// The same scalar-coupling kernels (whose full build is bound to 896 threads
// and so to 72 registers a thread) bound to at most kNarrowThreads threads
// per CTA: up to 85 registers a thread, for launches of that many threads or
// fewer.  Defined for the widths a resident_fast_<precision>_w<W>_narrow.cu
// instantiates; elsewhere (and for other coupling classes) nullptr.
constexpr int kNarrowThreads = 768;
template <typename R, int W> const void *resident_kernel_fast_narrow(int bil, int ons, int cl);
template <typename R, int W, int ONS> const void *resident_fast_narrow_for(int cl) {
    static_assert(resident_max_threads(true, 0, ONS) > kNarrowThreads, "a narrower bound than the full build");
    if (cl == 4) return (const void *)k_resident<ResidentFast<R, 0, ONS, W, 4>, R, kNarrowThreads, 4>;
    if (cl == 2) return (const void *)k_resident<ResidentFast<R, 0, ONS, W, 2>, R, kNarrowThreads, 2>;
    return (const void *)k_resident<ResidentFast<R, 0, ONS, W, 1>, R, kNarrowThreads, 1>;
}

template <typename R, int W> const void *resident_fast_table(int bil, int ons, int cl) {
    if (bil == 0)
        return ons == 0 ? resident_fast_for<R, W, 0, 0>(cl)
                        : ons == 1 ? resident_fast_for<R, W, 0, 1>(cl) : resident_fast_for<R, W, 0, 2>(cl);
    return ons == 0 ? resident_fast_for<R, W, 1, 0>(cl)
                    : ons == 1 ? resident_fast_for<R, W, 1, 1>(cl) : resident_fast_for<R, W, 1, 2>(cl);
}

} // namespace csmc
