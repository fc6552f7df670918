// resident.cuh -- the persistent shared-memory sweep kernel.
//
// Each replica is held in shared memory for a whole window of the
// reference's loop (monte_carlo.jl:295-377: overrelaxation sweeps,
// Metropolis sweeps, the FP64 total energy, probes, spin renormalisation):
// it is staged in with bulk TMA copies (cp.async.bulk, completion on an
// mbarrier, bounded wait), updated colour class by colour class with a
// barrier between classes, and written back once.
//
// A replica lives either in one CTA (CL = 1; a work list hands replicas out,
// largest first) or in a thread-block cluster of CL CTAs (CL = 2, 4): rank k
// holds part k of every colour class, partners owned by another rank are read
// through distributed shared memory (ld.shared::cluster), and the barrier
// between colour classes is a cluster barrier.  This spreads few replicas
// over more SMs.
//
// Two physics policies share the driver loop:
//  * ResidentGeneric: per-site pattern, cubic and quartic terms (device.cuh);
//  * ResidentFast: no cubic/quartic terms and one basis per colour class; the
//    couplings of a colour class are loaded once per class into registers
//    (scalar couplings) or staged in shared memory (general 3x3), and the
//    onsite matrices are specialised to none / diagonal / general.
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

// Bounded wait on an mbarrier phase: gives up after a fixed number of polls
// and reports it through the context's error flag instead of hanging.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *error_flag) {
    for (int k = 0; k < (1 << 22); k++)
        if (mbar_try_wait(bar, parity)) return true;
    if (threadIdx.x == 0) atomicExch(error_flag, 1);
    return false;
}

// ---- thread-block cluster primitives
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
// generic address of the same shared variable in CTA `rank` (plain loads
// through it reach that CTA's shared memory)
template <typename T> __device__ __forceinline__ const T *map_rank_generic(const T *p, uint32_t rank) {
    uint64_t r;
    asm("mapa.u64 %0, %1, %2;" : "=l"(r) : "l"((uint64_t)p), "r"(rank));
    return reinterpret_cast<const T *>(r);
}
// Loads from another CTA's shared memory.  Volatile keeps them between the
// (volatile, memory-clobbering) barriers that order them; no memory clobber,
// since within a colour class they read sites no thread writes.
__device__ __forceinline__ float ld_cluster(uint32_t a, float) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ double ld_cluster(uint32_t a, double) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a));
    return v;
}

// Remote arrive on the mbarrier at shared::cluster address `a` (release at
// cluster scope: this CTA's shared-memory writes become visible to a thread
// that then acquires the barrier phase).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t a) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Block (CL = 1) or cluster barrier and sums; totals valid in thread 0 of
// every CTA, identical on all ranks (same summation order).
template <int NT, int CL> struct Sync {
    double *scratch, *red; // scratch: NT/32 doubles; red: 3 doubles (cluster exchange)
    uint64_t *pbar;        // phase mbarrier of this CTA (CL arrivals per phase)
    uint32_t *pphase;      // its current phase parity (thread 0)
    int *error_flag;
    // Barrier across the cluster between colour classes: every CTA first
    // waits for its own threads (bar.sync), then thread 0 arrives on every
    // rank's phase mbarrier and waits, suspended in try_wait, for the
    // arrivals of all ranks; bounded, reporting a timeout through the
    // error flag.
    __device__ __forceinline__ void bar() const {
        __syncthreads();
        if (CL > 1) {
            if (threadIdx.x == 0) {
                const uint32_t a = smem_u32(pbar);
#pragma unroll
                for (int r = 0; r < CL; r++) mbar_arrive_cluster(map_rank(a, r));
                const uint32_t ph = *pphase;
                bool done = false;
                for (int k = 0; k < (1 << 22) && !done; k++) done = mbar_try_wait_cluster(pbar, ph);
                if (!done) atomicExch(error_flag, 1);
                *pphase = ph ^ 1u;
            }
            __syncthreads();
        }
    }
    __device__ double sum(double v) const {
        double t = block_sum<NT>(v, scratch);
        if (CL == 1) return t;
        if (threadIdx.x == 0) red[0] = t;
        cluster_sync_all();
        double tot = 0.0;
        if (threadIdx.x == 0)
            for (int r = 0; r < CL; r++) tot += ld_cluster(map_rank(smem_u32(red), r), 0.0);
        cluster_sync_all();
        return tot;
    }
    __device__ void sum3(double &a, double &b, double &c) const {
        a = block_sum<NT>(a, scratch);
        b = block_sum<NT>(b, scratch);
        c = block_sum<NT>(c, scratch);
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
template <typename R, int NT, int CL> struct ResidentCommon {
    const ResSys<R> &S;
    R *x, *y, *z; // local shared-memory arrays (stride Npl when CL > 1, else Np)
    Sync<NT, CL> sy;
    int c, slot, rank;
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

    __device__ double magnetization() const { // valid in thread 0
        double mx = 0, my = 0, mz = 0;
        for (int col = 0; col < S.n_colours; col++) { // the sites of this CTA only
            const int st = col_begin(col), n = col_size(col);
            for (int i = threadIdx.x; i < n; i += NT) {
                mx += x[st + i];
                my += y[st + i];
                mz += z[st + i];
            }
        }
        sy.sum3(mx, my, mz);
        return sqrt(mx * mx + my * my + mz * mz);
    }

    __device__ void renormalize() const {
        for (int col = 0; col < S.n_colours; col++) {
            const int st = col_begin(col), n = col_size(col);
            for (int i = threadIdx.x; i < n; i += NT) {
                const int d = st + i;
                const R a = x[d], b = y[d], cc = z[d];
                const R n2 = a * a + b * b + cc * cc;
                if (n2 == R(0)) continue;
                const R f = S.S * Math<R>::rsqrt_(n2);
                x[d] = a * f;
                y[d] = b * f;
                z[d] = cc * f;
            }
        }
        sy.bar();
    }
};

template <typename R, bool CUB, bool QUA, int NT, int CL> struct ResidentGeneric : ResidentCommon<R, NT, CL> {
    static_assert(CL == 1, "the generic resident kernel runs one CTA per replica");
    static constexpr int kCoefSmem = 1;
    using B = ResidentCommon<R, NT, CL>;
    using B::c;
    using B::S;
    using B::x;
    using B::y;
    using B::z;
    __device__ ResidentGeneric(const ResSys<R> &s, R *x_, R *y_, R *z_, Sync<NT, CL> sy_, int c_, int slot_, int rk,
                               R *coef)
        : B{s, x_, y_, z_, sy_, c_, slot_, rk, coef} {}
    __device__ void prepare() const {}

    __device__ unsigned metro_sweep(int kind, R sigma, R invT, double T, uint32_t msweep) const {
        unsigned acc = 0;
        for (int col = 0; col < S.n_colours; col++) {
            const int st = (int)S.col_start[col], n = (int)S.col_count[col];
            for (int i = threadIdx.x; i < n; i += NT) {
                const int d = st + i;
                const int b = S.tb.pat[d];
                V3<R> hb, hc, hq;
                partner_fields<R, uint16_t, CUB, QUA>(S.tb, S.cf, x, y, z, d, b, hb, hc, hq);
                const R *h = S.cf.h + 3 * b;
                const V3<R> hext = {hb.x + hc.x + hq.x - h[0], hb.y + hc.y + hq.y - h[1], hb.z + hc.z + hq.z - h[2]};
                const V3<R> s = {x[d], y[d], z[d]};
                const Draw<R> dr((uint32_t)d, msweep, (uint32_t)c, S.k0, S.k1);
                const V3<R> sn = propose<R>(kind, S.S, sigma, s, dr.uphi, dr.uz);
                const R dE = delta_e<R>(S.cf, b, s, sn, hext);
                bool accept = dE < R(0);
                if (!accept) {
                    const R arg = sizeof(R) == 4 ? -dE * invT : -dE / (R)T;
                    accept = dr.acc((uint32_t)d, msweep, (uint32_t)c, S.k0, S.k1) < Math<R>::exp_(arg);
                }
                if (accept) {
                    x[d] = sn.x;
                    y[d] = sn.y;
                    z[d] = sn.z;
                    acc++;
                }
            }
            __syncthreads();
        }
        return acc;
    }

    __device__ void or_sweep() const {
        for (int col = 0; col < S.n_colours; col++) {
            const int st = (int)S.col_start[col], n = (int)S.col_count[col];
            for (int i = threadIdx.x; i < n; i += NT) {
                const int d = st + i;
                const V3<R> H = local_field<R, uint16_t, CUB, QUA>(S.tb, S.cf, x, y, z, d, S.tb.pat[d]);
                if (H.x == R(0) && H.y == R(0) && H.z == R(0)) continue;
                const V3<R> s = {x[d], y[d], z[d]};
                const R proj = R(2) * dot(s, H) / (H.x * H.x + H.y * H.y + H.z * H.z);
                x[d] = -s.x + proj * H.x;
                y[d] = -s.y + proj * H.y;
                z[d] = -s.z + proj * H.z;
            }
            __syncthreads();
        }
    }

    __device__ double energy() const { // valid in thread 0
        double e = 0.0;
        for (int col = 0; col < S.n_colours; col++) {
            const int st = (int)S.col_start[col], n = (int)S.col_count[col];
            for (int i = threadIdx.x; i < n; i += NT) {
                const int d = st + i;
                e += site_energy_share<R, uint16_t, CUB, QUA>(S.tb, S.cf, x, y, z, d, S.tb.pat[d]);
            }
        }
        return this->sy.sum(e);
    }
};

template <typename R, int BIL, int ONS, int NT, int CL> struct ResidentFast : ResidentCommon<R, NT, CL> {
    static constexpr int WMAX = RESIDENT_WMAX;
    static constexpr int kCoefSmem = BIL ? CSMC_MAX_COLOURS * WMAX * 9 : 1;
    using B = ResidentCommon<R, NT, CL>;
    using B::c;
    using B::rank;
    using B::S;
    using B::scoef;
    using B::x;
    using B::y;
    using B::z;
    const R *xr[CL]; // generic pointer to x in every rank (CL > 1; own rank: x itself)

    __device__ ResidentFast(const ResSys<R> &s, R *x_, R *y_, R *z_, Sync<NT, CL> sy_, int c_, int slot_, int rk,
                            R *coef)
        : B{s, x_, y_, z_, sy_, c_, slot_, rk, coef} {
        if (CL > 1) {
#pragma unroll
            for (int r = 0; r < CL; r++) xr[r] = r == rk ? x_ : map_rank_generic<R>(x_, r);
        }
    }

    // stage the 3x3 couplings of every colour class: scoef[(col*W + t)*9 + e]
    __device__ void prepare() const {
        if (BIL) {
            const int W = S.tb.W2, n = S.n_colours * W * 9;
            for (int k = threadIdx.x; k < n; k += NT) {
                const int col = k / (W * 9), rem = k - col * W * 9, t = rem / 9, e = rem - t * 9;
                const int b = S.col_pattern[col];
                scoef[k] = S.cf.mats[9 * S.cf.c2[b * W + t] + e];
            }
            __syncthreads();
        }
    }

    // per colour class: slot scalars J, an onsite-class matrix m (from A, Q
    // or E2) and the field h
    __device__ __forceinline__ void load_coef(int col, const R *src, R (&J)[WMAX], R (&m)[9], V3<R> &h) const {
        const int b = S.col_pattern[col], W = S.tb.W2;
#pragma unroll
        for (int t = 0; t < WMAX; t++) J[t] = (BIL == 0 && t < W) ? S.cf.Js[b * W + t] : R(0);
#pragma unroll
        for (int k = 0; k < 9; k++) m[k] = ONS == 0 ? R(0) : src[9 * b + k];
        h = {S.cf.h[3 * b], S.cf.h[3 * b + 1], S.cf.h[3 * b + 2]};
    }

    __device__ __forceinline__ V3<R> onsite(const R (&m)[9], V3<R> s) const {
        if (ONS == 0) return {R(0), R(0), R(0)};
        if (ONS == 1) return {m[0] * s.x, m[4] * s.y, m[8] * s.z};
        return matvec(m, s);
    }

    __device__ __forceinline__ const R *rank_x(uint32_t own) const {
        if (CL == 2) return own ? xr[1 % CL] : xr[0];
        if (CL == 4) return own < 2 ? (own ? xr[1 % CL] : xr[0]) : (own == 2 ? xr[2 % CL] : xr[3 % CL]);
        return xr[0];
    }

    __device__ __forceinline__ void accumulate(V3<R> &hb, int col, int t, const R (&J)[WMAX], R sx, R sy_,
                                               R sz) const {
        if (BIL == 0) {
            hb.x += J[t] * sx;
            hb.y += J[t] * sy_;
            hb.z += J[t] * sz;
        } else {
            const R *M = scoef + (col * S.tb.W2 + t) * 9;
            hb.x += M[0] * sx + M[1] * sy_ + M[2] * sz;
            hb.y += M[3] * sx + M[4] * sy_ + M[5] * sz;
            hb.z += M[6] * sx + M[7] * sy_ + M[8] * sz;
        }
    }

    // unpack the 8 16-bit partners of a site from its packed word
    static __device__ __forceinline__ void unpack(const uint4 w, uint32_t (&v)[WMAX]) {
        v[0] = w.x & 0xFFFFu;
        v[1] = w.x >> 16;
        v[2] = w.y & 0xFFFFu;
        v[3] = w.y >> 16;
        v[4] = w.z & 0xFFFFu;
        v[5] = w.z >> 16;
        v[6] = w.w & 0xFFFFu;
        v[7] = w.w >> 16;
    }

    // sum over bilinear slots of J_t s_j at local site i: the partner indices
    // come in one 16-byte load, each partner spin is consumed as soon as it is
    // loaded
    __device__ __forceinline__ V3<R> gather(int col, const R (&J)[WMAX], int i) const {
        V3<R> hb = {R(0), R(0), R(0)};
        const int W = S.tb.W2;
        uint32_t v[WMAX];
        if (CL == 1) {
            unpack(S.p2v[i], v);
#pragma unroll
            for (int t = 0; t < WMAX; t++)
                if (t < W) accumulate(hb, col, t, J, x[v[t]], y[v[t]], z[v[t]]);
        } else {
            const int Npl = S.Npl;
            unpack(S.q2v[(size_t)rank * Npl + i], v);
            // one path for every partner: a generic pointer into the owning
            // CTA's shared memory (this CTA's or, through distributed shared
            // memory, another rank's)
#pragma unroll
            for (int t = 0; t < WMAX; t++)
                if (t < W) {
                    const R *p = rank_x(v[t] >> 14) + (v[t] & 0x3FFFu);
                    accumulate(hb, col, t, J, p[0], p[Npl], p[2 * Npl]);
                }
        }
        return hb;
    }

    __device__ void or_sweep() const {
        for (int col = 0; col < S.n_colours; col++) {
            R J[WMAX], a[9];
            V3<R> h;
            load_coef(col, S.cf.A, J, a, h);
            const int st = this->col_begin(col), n = this->col_size(col);
            for (int k = threadIdx.x; k < n; k += NT) {
                const int d = st + k;
                const V3<R> s = {x[d], y[d], z[d]};
                const V3<R> hb = gather(col, J, d);
                const V3<R> as = onsite(a, s);
                const V3<R> H = {as.x + hb.x - h.x, as.y + hb.y - h.y, as.z + hb.z - h.z};
                if (H.x == R(0) && H.y == R(0) && H.z == R(0)) continue;
                const R proj = Math<R>::div_(R(2) * dot(s, H), H.x * H.x + H.y * H.y + H.z * H.z);
                x[d] = -s.x + proj * H.x;
                y[d] = -s.y + proj * H.y;
                z[d] = -s.z + proj * H.z;
            }
            this->sy.bar();
        }
    }

    __device__ unsigned metro_sweep(int kind, R sigma, R invT, double T, uint32_t msweep) const {
        unsigned acc = 0;
        for (int col = 0; col < S.n_colours; col++) {
            R J[WMAX], q[9];
            V3<R> h;
            load_coef(col, S.cf.Q, J, q, h);
            const int st = this->col_begin(col), n = this->col_size(col);
            for (int k = threadIdx.x; k < n; k += NT) {
                const int d = st + k;
                const uint32_t dg = (uint32_t)this->device_index(col, d);
                const V3<R> s = {x[d], y[d], z[d]};
                const V3<R> hb = gather(col, J, d);
                const V3<R> hext = {hb.x - h.x, hb.y - h.y, hb.z - h.z};
                const Draw<R> dr(dg, msweep, (uint32_t)c, S.k0, S.k1);
                const V3<R> sn = propose<R>(kind, S.S, sigma, s, dr.uphi, dr.uz);
                const V3<R> ds = {sn.x - s.x, sn.y - s.y, sn.z - s.z};
                const R dE = (dot(sn, onsite(q, sn)) - dot(s, onsite(q, s))) + dot(ds, hext);
                bool accept = dE < R(0);
                if (!accept) {
                    const R arg = sizeof(R) == 4 ? -dE * invT : -dE / (R)T;
                    accept = dr.acc(dg, msweep, (uint32_t)c, S.k0, S.k1) < Math<R>::exp_(arg);
                }
                if (accept) {
                    x[d] = sn.x;
                    y[d] = sn.y;
                    z[d] = sn.z;
                    acc++;
                }
            }
            this->sy.bar();
        }
        return acc;
    }

    __device__ double energy() const { // valid in thread 0
        double e = 0.0;
        for (int col = 0; col < S.n_colours; col++) {
            R J[WMAX], m[9];
            V3<R> h;
            load_coef(col, S.cf.E2, J, m, h);
            const int st = this->col_begin(col), n = this->col_size(col);
            for (int k = threadIdx.x; k < n; k += NT) {
                const int d = st + k;
                const V3<R> s = {x[d], y[d], z[d]};
                const V3<R> hb = gather(col, J, d);
                e += (double)(dot(s, onsite(m, s)) - dot(s, h)) + 0.5 * (double)dot(s, hb);
            }
        }
        return this->sy.sum(e);
    }
};

// Probe of iteration q exists?  (q >= t_therm and q % probe_rate == 0)
__device__ __forceinline__ bool is_probe(const RunDesc &rd, int64_t q) {
    return rd.probe_rate > 0 && q >= rd.t_therm && q % rd.probe_rate == 0;
}

template <typename K, typename R, int NT, int CL>
__global__ void __launch_bounds__(NT, 1)
    k_resident(const ResSys<R> *__restrict__ systems, const int2 *__restrict__ items, int n_items, int *work_ctr,
               ChainState cs, RunDesc rd) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    __shared__ double scratch[32];
    __shared__ double red[4];
    __shared__ int s_item;
    __shared__ double s_sigma;
    __shared__ ResSys<R> s_sys;
    __shared__ R s_coef[K::kCoefSmem];
    __shared__ uint64_t pbar;
    __shared__ uint32_t pphase;
    uint32_t parity = 0;
    const int rank = CL == 1 ? 0 : (int)cluster_ctarank();
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init(&pbar, CL);
        pphase = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (CL > 1) cluster_sync_all(); // every rank's phase barrier exists before any remote arrive
    const int64_t dosweep = rd.or_rate == 0 ? 1 : rd.or_rate;
    const Sync<NT, CL> sync{scratch, red, &pbar, &pphase, cs.error_flag};
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
            for (int k = threadIdx.x; k < (int)(sizeof(ResSys<R>) / 4); k += NT) dst[k] = src[k];
        }
        __syncthreads();
        const ResSys<R> &S = s_sys;
        const int r = w.y;
        const int c = S.chain_base + r;
        const int64_t Np = S.tb.Np;
        const int64_t nl = CL == 1 ? Np : S.Npl;
        R *gx = S.spins + (int64_t)r * 3 * Np;
        R *x = reinterpret_cast<R *>(smem_raw), *y = x + nl, *z = y + nl;

        // stage this CTA's part of the replica with bulk TMA copies
        if (threadIdx.x == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            if (CL == 1) {
                const uint32_t bytes = (uint32_t)(Np * sizeof(R));
                mbar_expect_tx(&bar, 3 * bytes);
                bulk_g2s(x, gx, bytes, &bar);
                bulk_g2s(y, gx + Np, bytes, &bar);
                bulk_g2s(z, gx + 2 * Np, bytes, &bar);
            } else {
                uint32_t total = 0;
                for (int col = 0; col < S.n_colours; col++)
                    total += 3u * (uint32_t)(((S.loc_count[rank][col] + 31) / 32 * 32) * sizeof(R));
                mbar_expect_tx(&bar, total);
                for (int col = 0; col < S.n_colours; col++) {
                    const int n = (S.loc_count[rank][col] + 31) / 32 * 32;
                    if (n == 0) continue;
                    const uint32_t bytes = (uint32_t)(n * sizeof(R));
                    const int ls = S.loc_start[rank][col], gs = S.src_start[rank][col];
                    bulk_g2s(x + ls, gx + gs, bytes, &bar);
                    bulk_g2s(y + ls, gx + Np + gs, bytes, &bar);
                    bulk_g2s(z + ls, gx + 2 * Np + gs, bytes, &bar);
                }
            }
        }
        const bool ok = mbar_wait_bounded(&bar, parity, cs.error_flag);
        parity ^= 1;
        const bool local_fail = __syncthreads_or(!ok); // block-uniform
        bool fail = local_fail;
        if (CL > 1) { // cluster-uniform: any rank failed
            if (threadIdx.x == 0) red[3] = local_fail ? 1.0 : 0.0;
            cluster_sync_all();
            double n_fail = 0.0;
            for (int q = 0; q < CL; q++) n_fail += ld_cluster(map_rank(smem_u32(&red[3]), q), 0.0);
            cluster_sync_all();
            fail = n_fail > 0.0;
        }
        if (fail) {
            if (local_fail) mbar_wait_bounded(&bar, parity ^ 1, cs.error_flag); // copies still in flight
            __syncthreads();
            if (CL == 1) continue;
            break; // a cluster drops its remaining items together
        }
        if (CL > 1) { // zero this rank's sentinel block, then every rank is staged
            const int sent = S.Npl - 32;
            for (int k = threadIdx.x; k < 32; k += NT) x[sent + k] = y[sent + k] = z[sent + k] = R(0);
            cluster_sync_all();
        }

        const int slot = cs.slot_of[c];
        const double T = rd.T_override > 0 ? rd.T_override : cs.T_slot[slot];
        if (threadIdx.x == 0) s_sigma = rd.reset_sigma ? rd.sigma0 : cs.sigma_slot[slot];
        __syncthreads();
        const K k(S, x, y, z, sync, c, slot, rank, s_coef);
        k.prepare();
        const R invT = (R)(1.0 / T);
        const bool writer = threadIdx.x == 0 && rank == 0;
        double E = cs.E_chain[c];
        double acc_total = 0.0;
        uint32_t msweep = rd.msweep0;
        // single precision: renormalise |s| = S whenever the context's total
        // sweep count passes a multiple of renorm_every
        uint64_t sweeps = rd.sweeps0;
        const uint64_t every = rd.renorm_every > 0 ? (uint64_t)rd.renorm_every : 0;
        uint64_t next_renorm = every ? (sweeps / every + 1) * every : 0;

        if (rd.pending_probe) { // probe of the exchange iteration it0-1
            const int64_t q = rd.it0 - 1;
            const double M = k.magnetization();
            if (writer) {
                const int64_t kq = (q - rd.probe_first) / rd.probe_rate;
                if (kq >= 0 && kq < rd.probe_cap) {
                    if (rd.rec_E) rd.rec_E[kq * rd.n_slots + slot] = E;
                    if (rd.rec_M) rd.rec_M[kq * rd.n_slots + slot] = M;
                }
                cs.M_chain[c] = M;
            }
        }

        for (int64_t it = rd.it0; it < rd.it1; it++) {
            if (rd.or_rate != 0) {
                k.or_sweep();
                sweeps++;
            }
            const bool metro = it % dosweep == 0;
            if (metro) {
                const unsigned a = k.metro_sweep(rd.kind, (R)s_sigma, invT, T, msweep);
                msweep++;
                sweeps++;
                const double at = sync.sum((double)a);
                if (threadIdx.x == 0) {
                    acc_total += at;
                    if (rd.kind == CSMC_METROPOLIS_ADAPTIVE) { // metropolis.jl:124-126
                        const double om = 1 - at / (double)S.n_real;
                        const double f = 0.5 / (om > 0.05 ? om : 0.05);
                        double sg = s_sigma * f;
                        s_sigma = sg < 0.0 ? 0.0 : (sg > 100 ? 100 : sg);
                    }
                }
                __syncthreads();
                // energy needed: exchange point, a probe before the next
                // Metropolis sweep, or the last Metropolis sweep of the window
                bool needE = rd.swap_enabled && rd.swap_rate > 0 && it % rd.swap_rate == 0;
                for (int64_t q = it; q < it + dosweep && q < rd.it1 && !needE; q++) needE = is_probe(rd, q);
                needE = needE || it + dosweep >= rd.it1;
                if (needE) {
                    const double e = k.energy();
                    if (threadIdx.x == 0) E = e;
                }
            }
            const bool swap_here = metro && rd.swap_enabled && rd.swap_rate > 0 && it % rd.swap_rate == 0;
            if (is_probe(rd, it) && !swap_here) {
                const double M = k.magnetization();
                if (writer) {
                    const int64_t kq = (it - rd.probe_first) / rd.probe_rate;
                    if (kq >= 0 && kq < rd.probe_cap) {
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

        if (writer) {
            cs.E_chain[c] = E;
            cs.acc_slot[slot] += acc_total;
            cs.sigma_slot[slot] = s_sigma;
        }
        __syncthreads();
        // write this CTA's part back (x, y, z are contiguous in both memories)
        if (CL == 1) {
            for (int64_t i = threadIdx.x; i < 3 * Np; i += NT) gx[i] = x[i];
        } else {
            for (int col = 0; col < S.n_colours; col++) {
                const int n = S.loc_count[rank][col], ls = S.loc_start[rank][col], gs = S.src_start[rank][col];
                for (int i = threadIdx.x; i < n; i += NT) {
                    gx[gs + i] = x[ls + i];
                    gx[Np + gs + i] = y[ls + i];
                    gx[2 * Np + gs + i] = z[ls + i];
                }
            }
            cluster_sync_all(); // no rank reads another's shared memory past this point
        }
        __syncthreads();
    }
}

// Kernel entry points of each instantiation family (resident_*.cu).
template <typename R> const void *resident_kernel_generic(int block, bool cub, bool qua);

} // namespace csmc
