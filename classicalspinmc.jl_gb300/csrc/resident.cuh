// resident.cuh -- the persistent shared-memory sweep kernel.
//
// One CTA per replica (a work list hands replicas out, largest first): the
// replica's spins are staged into shared memory with three bulk TMA copies
// (cp.async.bulk, completion on an mbarrier, bounded wait), a whole window of
// the reference's loop (monte_carlo.jl:295-377: overrelaxation sweeps,
// Metropolis sweeps, the FP64 total energy, probes, spin renormalisation) runs
// there with __syncthreads between colour classes, and the replica is written
// back once.  The partner tables (16-bit) and couplings are read from L2/L1.
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

// Magnetisation and renormalisation, common to both policies.
template <typename R, int NT> struct ResidentCommon {
    const ResSys<R> &S;
    R *x, *y, *z;
    double *scratch;
    int c, slot;
    R *scoef;

    __device__ double magnetization() const { // valid in thread 0
        double mx = 0, my = 0, mz = 0;
        const int Np = (int)S.tb.Np;
        for (int d = threadIdx.x; d < Np; d += NT) { // padding holds zeros
            mx += x[d];
            my += y[d];
            mz += z[d];
        }
        mx = block_sum<NT>(mx, scratch);
        my = block_sum<NT>(my, scratch);
        mz = block_sum<NT>(mz, scratch);
        return sqrt(mx * mx + my * my + mz * mz);
    }

    __device__ void renormalize() const {
        for (int col = 0; col < S.n_colours; col++) {
            const int st = (int)S.col_start[col], n = (int)S.col_count[col];
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
        __syncthreads();
    }
};

template <typename R, bool CUB, bool QUA, int NT> struct ResidentGeneric : ResidentCommon<R, NT> {
    static constexpr int kCoefSmem = 1;
    using B = ResidentCommon<R, NT>;
    using B::c;
    using B::S;
    using B::x;
    using B::y;
    using B::z;
    __device__ ResidentGeneric(const ResSys<R> &s, R *x_, R *y_, R *z_, double *sc, int c_, int slot_, R *coef)
        : B{s, x_, y_, z_, sc, c_, slot_, coef} {}
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
        return block_sum<NT>(e, this->scratch);
    }
};

template <typename R, int BIL, int ONS, int NT> struct ResidentFast : ResidentCommon<R, NT> {
    static constexpr int WMAX = RESIDENT_WMAX;
    static constexpr int kCoefSmem = BIL ? CSMC_MAX_COLOURS * WMAX * 9 : 1;
    using B = ResidentCommon<R, NT>;
    using B::c;
    using B::S;
    using B::scoef;
    using B::x;
    using B::y;
    using B::z;
    __device__ ResidentFast(const ResSys<R> &s, R *x_, R *y_, R *z_, double *sc, int c_, int slot_, R *coef)
        : B{s, x_, y_, z_, sc, c_, slot_, coef} {}

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

    // sum over bilinear slots of J_t s_j
    __device__ __forceinline__ V3<R> gather(int col, const R (&J)[WMAX], int d) const {
        V3<R> hb = {R(0), R(0), R(0)};
        const int W = S.tb.W2, Np = (int)S.tb.Np;
        const uint16_t *p2 = S.tb.p2;
        int j[WMAX];
#pragma unroll
        for (int t = 0; t < WMAX; t++) j[t] = t < W ? p2[t * Np + d] : 0;
#pragma unroll
        for (int t = 0; t < WMAX; t++) {
            if (t < W) {
                const R sx = x[j[t]], sy = y[j[t]], sz = z[j[t]];
                if (BIL == 0) {
                    hb.x += J[t] * sx;
                    hb.y += J[t] * sy;
                    hb.z += J[t] * sz;
                } else {
                    const R *M = scoef + (col * W + t) * 9;
                    hb.x += M[0] * sx + M[1] * sy + M[2] * sz;
                    hb.y += M[3] * sx + M[4] * sy + M[5] * sz;
                    hb.z += M[6] * sx + M[7] * sy + M[8] * sz;
                }
            }
        }
        return hb;
    }

    __device__ void or_sweep() const {
        for (int col = 0; col < S.n_colours; col++) {
            R J[WMAX], a[9];
            V3<R> h;
            load_coef(col, S.cf.A, J, a, h);
            const int st = (int)S.col_start[col], n = (int)S.col_count[col];
            for (int i = threadIdx.x; i < n; i += NT) {
                const int d = st + i;
                const V3<R> s = {x[d], y[d], z[d]};
                const V3<R> hb = gather(col, J, d);
                const V3<R> as = onsite(a, s);
                const V3<R> H = {as.x + hb.x - h.x, as.y + hb.y - h.y, as.z + hb.z - h.z};
                if (H.x == R(0) && H.y == R(0) && H.z == R(0)) continue;
                const R proj = R(2) * dot(s, H) / (H.x * H.x + H.y * H.y + H.z * H.z);
                x[d] = -s.x + proj * H.x;
                y[d] = -s.y + proj * H.y;
                z[d] = -s.z + proj * H.z;
            }
            __syncthreads();
        }
    }

    __device__ unsigned metro_sweep(int kind, R sigma, R invT, double T, uint32_t msweep) const {
        unsigned acc = 0;
        for (int col = 0; col < S.n_colours; col++) {
            R J[WMAX], q[9];
            V3<R> h;
            load_coef(col, S.cf.Q, J, q, h);
            const int st = (int)S.col_start[col], n = (int)S.col_count[col];
            for (int i = threadIdx.x; i < n; i += NT) {
                const int d = st + i;
                const V3<R> s = {x[d], y[d], z[d]};
                const V3<R> hb = gather(col, J, d);
                const V3<R> hext = {hb.x - h.x, hb.y - h.y, hb.z - h.z};
                const Draw<R> dr((uint32_t)d, msweep, (uint32_t)c, S.k0, S.k1);
                const V3<R> sn = propose<R>(kind, S.S, sigma, s, dr.uphi, dr.uz);
                const V3<R> ds = {sn.x - s.x, sn.y - s.y, sn.z - s.z};
                const R dE = (dot(sn, onsite(q, sn)) - dot(s, onsite(q, s))) + dot(ds, hext);
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

    __device__ double energy() const { // valid in thread 0
        double e = 0.0;
        for (int col = 0; col < S.n_colours; col++) {
            R J[WMAX], m[9];
            V3<R> h;
            load_coef(col, S.cf.E2, J, m, h);
            const int st = (int)S.col_start[col], n = (int)S.col_count[col];
            for (int i = threadIdx.x; i < n; i += NT) {
                const int d = st + i;
                const V3<R> s = {x[d], y[d], z[d]};
                const V3<R> hb = gather(col, J, d);
                e += (double)(dot(s, onsite(m, s)) - dot(s, h)) + 0.5 * (double)dot(s, hb);
            }
        }
        return block_sum<NT>(e, this->scratch);
    }
};

// Probe of iteration q exists?  (q >= t_therm and q % probe_rate == 0)
__device__ __forceinline__ bool is_probe(const RunDesc &rd, int64_t q) {
    return rd.probe_rate > 0 && q >= rd.t_therm && q % rd.probe_rate == 0;
}

template <typename K, typename R, int NT>
__global__ void __launch_bounds__(NT, 1)
    k_resident(const ResSys<R> *__restrict__ systems, const int2 *__restrict__ items, int n_items, int *work_ctr,
               ChainState cs, RunDesc rd) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    __shared__ double scratch[32];
    __shared__ int s_item;
    __shared__ double s_sigma;
    __shared__ ResSys<R> s_sys;
    __shared__ R s_coef[K::kCoefSmem];
    uint32_t parity = 0;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int64_t dosweep = rd.or_rate == 0 ? 1 : rd.or_rate;

    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(work_ctr, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= n_items) break;
        const int2 w = items[item];
        if (threadIdx.x == 0) s_sys = systems[w.x];
        __syncthreads();
        const ResSys<R> &S = s_sys;
        const int r = w.y;
        const int c = S.chain_base + r;
        const int64_t Np = S.tb.Np;
        R *gx = S.spins + (int64_t)r * 3 * Np;
        R *x = reinterpret_cast<R *>(smem_raw), *y = x + Np, *z = y + Np;

        // stage the replica: three bulk TMA copies of Np elements
        if (threadIdx.x == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const uint32_t bytes = (uint32_t)(Np * sizeof(R));
            mbar_expect_tx(&bar, 3 * bytes);
            bulk_g2s(x, gx, bytes, &bar);
            bulk_g2s(y, gx + Np, bytes, &bar);
            bulk_g2s(z, gx + 2 * Np, bytes, &bar);
        }
        const bool ok = mbar_wait_bounded(&bar, parity, cs.error_flag);
        parity ^= 1;
        if (__syncthreads_or(!ok)) { // block-uniform: wait once more for the copies in flight, drop the item
            mbar_wait_bounded(&bar, parity ^ 1, cs.error_flag);
            __syncthreads();
            continue;
        }

        const int slot = cs.slot_of[c];
        const double T = rd.T_override > 0 ? rd.T_override : cs.T_slot[slot];
        if (threadIdx.x == 0) s_sigma = rd.reset_sigma ? rd.sigma0 : cs.sigma_slot[slot];
        __syncthreads();
        const K k(S, x, y, z, scratch, c, slot, s_coef);
        k.prepare();
        const R invT = (R)(1.0 / T);
        double E = cs.E_chain[c];
        double acc_total = 0.0;
        uint32_t msweep = rd.msweep0;
        int sweeps_since_renorm = 0;

        if (rd.pending_probe) { // probe of the exchange iteration it0-1
            const int64_t q = rd.it0 - 1;
            const double M = k.magnetization();
            if (threadIdx.x == 0) {
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
                sweeps_since_renorm++;
            }
            const bool metro = it % dosweep == 0;
            if (metro) {
                const unsigned a = k.metro_sweep(rd.kind, (R)s_sigma, invT, T, msweep);
                msweep++;
                sweeps_since_renorm++;
                const double at = block_sum<NT>((double)a, scratch);
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
                if (threadIdx.x == 0) {
                    const int64_t kq = (it - rd.probe_first) / rd.probe_rate;
                    if (kq >= 0 && kq < rd.probe_cap) {
                        if (rd.rec_E) rd.rec_E[kq * rd.n_slots + slot] = E;
                        if (rd.rec_M) rd.rec_M[kq * rd.n_slots + slot] = M;
                    }
                    cs.M_chain[c] = M;
                }
            }
            if (sizeof(R) == 4 && rd.renorm_every > 0 && sweeps_since_renorm >= rd.renorm_every) {
                k.renormalize();
                sweeps_since_renorm = 0;
            }
        }
        if (sizeof(R) == 4 && rd.renorm_every > 0 && sweeps_since_renorm > 0) k.renormalize();

        if (threadIdx.x == 0) {
            cs.E_chain[c] = E;
            cs.acc_slot[slot] += acc_total;
            cs.sigma_slot[slot] = s_sigma;
        }
        __syncthreads();
        // write the replica back (x, y, z are contiguous in both memories)
        for (int64_t i = threadIdx.x; i < 3 * Np; i += NT) gx[i] = x[i];
        __syncthreads();
    }
}

// Kernel entry points of each instantiation family (resident_*.cu).
template <typename R> const void *resident_kernel_generic(int block, bool cub, bool qua);
template <typename R> const void *resident_kernel_fast(int block, int bil, int ons);

} // namespace csmc
