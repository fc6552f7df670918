// kernels.cu -- sm_103a colour-sweep kernels of the global path: one launch
// per colour class, all replicas of a lattice in the grid's y dimension (or
// one replica per launch for the plain path), spins in HBM/L2, 32-bit partner
// tables; plus the energy and magnetisation reductions, the replica exchange
// and the layout conversions.  The persistent shared-memory kernel is in
// resident.cuh.
//
// The physics per site restates hamiltonian.jl, metropolis.jl and
// monte_carlo.jl (see device.cuh).  Colour classes make every update within
// a class independent, so each class is one parallel step.
#include <cstdlib>

#include "kernels.cuh"
#include "launch.hpp"
#include "reduce.cuh"

namespace csmc {

constexpr int GB = 256; // block size of the global-path kernels

// ------------------------------------------------------------ global path

template <typename R> __device__ __forceinline__ Spins<R> replica(const SysArgs<R> &a, int r) {
    return spins_of(a.spins, a.tb.Np, r);
}

// One Metropolis colour step: every site of the class proposes once
// (metropolis.jl:65-82, with site order given by the colouring).
// The colour-sweep kernels are launched as programmatic dependents of the
// kernel before them (launch_dep): the launch overlaps the end of that kernel,
// and this wait -- a no-op for an ordinary launch -- holds every thread until
// that kernel has completed and its writes are visible.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename R, bool CUB, bool QUA>
__global__ void __launch_bounds__(GB) k_metro_colour(SysArgs<R> a, ChainState cs, int start, int count, int chain_lo,
                                                     int kind, uint32_t msweep, double T_override,
                                                     float invT_override) {
    pdl_wait();
    const int r = chain_lo + blockIdx.y;
    const int c = a.chain_base + r;
    const Spins<R> p = replica(a, r);
    // 1/T and sigma of the block's replica.  Single precision reads 1/T
    // formed on the host (FP64 arithmetic -- even one division or comparison
    // per block -- runs at a small fraction of the FP32 rate on this device);
    // double precision divides by T itself.
    __shared__ R s_invT, s_sigma;
    __shared__ double s_T;
    __shared__ uint32_t s_key;
    if (threadIdx.x == 0) {
        const int slot = cs.slot_of[c];
        s_key = cs.chain_id[c];
        if constexpr (sizeof(R) == 4) {
            s_invT = invT_override > 0.f ? invT_override : cs.invT_slot[slot];
        } else {
            s_T = T_override > 0 ? T_override : cs.T_slot[slot];
            s_invT = (R)(1.0 / s_T);
        }
        s_sigma = (R)cs.sigma_slot[slot];
    }
    __syncthreads();
    const R invT = s_invT, sigma = s_sigma;
    const uint32_t key = s_key; // the replica's Philox stream key
    const double T = sizeof(R) == 4 ? 0.0 : s_T; // used by the double-precision acceptance only
    unsigned acc = 0;
    if constexpr (!CUB && !QUA) { // two sites per thread, their gathers in flight together
        const int i0 = (int)blockIdx.x * (2 * GB) + (int)threadIdx.x, i1 = i0 + GB;
        if (i0 < count) {
            const bool two = i1 < count;
            const int dd[2] = {start + i0, start + (two ? i1 : i0)};
            const int bb[2] = {a.tb.pat[dd[0]], a.tb.pat[dd[1]]};
            V3<R> hb[2];
            bilinear_fields2(a.tb, a.cf, p, dd[0], dd[1], bb[0], bb[1], hb[0], hb[1]);
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (q == 1 && !two) break;
                const int d = dd[q], b = bb[q];
                // no cubic or quartic fields to add (hb + 0 + 0 is hb)
                const V3<R> hext = vsub(hb[q], V3<R>{a.cf.h[3 * b], a.cf.h[3 * b + 1], a.cf.h[3 * b + 2]});
                const V3<R> s = p.get(d);
                const Draw<R> dr((uint32_t)d, msweep, key, a.k0, a.k1);
                const V3<R> sn = propose<R>(kind, a.S, sigma, s, dr.uphi, dr.uz);
                const R dE = delta_e<R>(a.cf, b, s, sn, hext);
                bool accept = dE < R(0);
                if (!accept)
                    accept = dr.acc((uint32_t)d, msweep, key, a.k0, a.k1) < Math<R>::exp_(boltz_arg(dE, invT, T));
                if (accept) {
                    p.set(d, sn);
                    acc++;
                }
            }
        }
    } else {
    const int i = (int)blockIdx.x * GB + (int)threadIdx.x;
    if (i < count) {
        const int d = start + i;
        const int b = a.tb.pat[d];
        V3<R> hb, hc, hq;
        partner_fields<R, uint32_t, CUB, QUA>(a.tb, a.cf, p, d, b, hb, hc, hq);
        const V3<R> hext = vsub(vadd(vadd(hb, hc), hq), V3<R>{a.cf.h[3 * b], a.cf.h[3 * b + 1], a.cf.h[3 * b + 2]});
        const V3<R> s = p.get(d);
        const Draw<R> dr((uint32_t)d, msweep, key, a.k0, a.k1);
        const V3<R> sn = propose<R>(kind, a.S, sigma, s, dr.uphi, dr.uz);
        const R dE = delta_e<R>(a.cf, b, s, sn, hext);
        bool accept = dE < R(0);
        if (!accept) accept = dr.acc((uint32_t)d, msweep, key, a.k0, a.k1) < Math<R>::exp_(boltz_arg(dE, invT, T));
        if (accept) {
            p.set(d, sn);
            acc = 1;
        }
    }
    }
    acc = warp_sum_u(acc);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&cs.sweep_acc[c], (unsigned long long)acc);
}

// metropolis_constraint! / metropolis_constraint_adaptive! (metropolis.jl:36-58,
// 155-179) on every replica of a lattice, one warp per replica: the warp sums
// the order parameter V of the constraint, then lane 0 makes the sweep's N
// proposals in sequence -- random site, uniform (kind 3) or cone (kind 4)
// proposal, dE, the constraint c on V with the proposed spin in place
// (V updated by the site's weighted change), lambda' = lambda - weight c,
// acceptance of dE - lambda' c -- since every proposal depends on lambda and V
// as left by the one before.  Proposal q draws (site, u_acc) from Philox
// counter (q, msweep, chain, CONS_A) and (u_phi, u_z) from (q, msweep, chain,
// CONS_B); the site is floor(N x / 2^32) of the first word.  The uniforms
// are 53-bit in double precision; a single-precision context takes 24-bit
// uniforms (the top bits of the first word of each pair) and evaluates the
// constraint, lambda' and the acceptance in single precision -- on this
// device FP64 runs at a small fraction of the FP32 rate and the sequential
// proposals would wait on it -- with V summed in FP64 at the start of the
// sweep and lambda kept in FP64 between sweeps.
// V = sum_d w[d] s_d of a replica, summed by the calling warp in FP64 (every
// lane gets it)
template <typename R>
__device__ __forceinline__ void constraint_v_sum(const SysArgs<R> &a, const Spins<R> &p, const ConsArgs &k, double &vx,
                                                 double &vy, double &vz) {
    vx = vy = vz = 0.0;
    for (int64_t d = threadIdx.x; d < a.tb.Np; d += 32) {
        const V3<R> s = p.get(d);
        const double w = k.w ? k.w[d] : 1.0;
        vx += w * (double)s.x;
        vy += w * (double)s.y;
        vz += w * (double)s.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vx += __shfl_xor_sync(0xffffffffu, vx, o);
        vy += __shfl_xor_sync(0xffffffffu, vy, o);
        vz += __shfl_xor_sync(0xffffffffu, vz, o);
    }
}
// w_d (s' - s): the change of V when site d moves from s to s'
template <typename R> __device__ __forceinline__ V3<R> constraint_step(const ConsArgs &k, int64_t d, V3<R> s, V3<R> sn) {
    using F = Fp<R>;
    const R w = k.w ? (R)k.w[d] : R(1);
    return {F::mul(w, F::sub(sn.x, s.x)), F::mul(w, F::sub(sn.y, s.y)), F::mul(w, F::sub(sn.z, s.z))};
}

template <typename R, bool CUB, bool QUA>
__global__ void __launch_bounds__(32) k_metro_constraint(SysArgs<R> a, ChainState cs, ConsArgs k, int kind,
                                                        uint32_t msweep, double T_override) {
    const int r = blockIdx.x;
    const int c = a.chain_base + r;
    const uint32_t key = cs.chain_id[c];
    const Spins<R> p = replica(a, r);
    double vx, vy, vz;
    constraint_v_sum(a, p, k, vx, vy, vz);
    if (threadIdx.x != 0) return;
    const int slot = cs.slot_of[c];
    const double T = T_override > 0 ? T_override : cs.T_slot[slot];
    const R sigma = (R)cs.sigma_slot[slot];
    const int pk = kind == CSMC_METROPOLIS_CONSTRAINT ? CSMC_METROPOLIS : CSMC_METROPOLIS_ADAPTIVE;
    R lambda = (R)k.lambda_slot[slot];
    R ux = (R)vx, uy = (R)vy, uz = (R)vz; // V in R from here on
    const R invT = (R)(1.0 / T);
    auto uniform = [](uint32_t a, uint32_t b) -> R {
        if (sizeof(R) == 4) return (R)u24(a);
        return (R)u53(a, b);
    };
    unsigned long long acc = 0;
    const uint64_t n = (uint64_t)a.n_real;
    // the draws of proposal q + 1 are computed while proposal q waits for its
    // spins (they depend on nothing the proposal changes)
    U4 A = philox4x32_10(0u, msweep, key, PURPOSE_CONS_A, a.k0, a.k1);
    U4 B = philox4x32_10(0u, msweep, key, PURPOSE_CONS_B, a.k0, a.k1);
    for (uint64_t q = 0; q < n; q++) {
        const U4 An = philox4x32_10((uint32_t)(q + 1), msweep, key, PURPOSE_CONS_A, a.k0, a.k1);
        const U4 Bn = philox4x32_10((uint32_t)(q + 1), msweep, key, PURPOSE_CONS_B, a.k0, a.k1);
        const int64_t i = (int64_t)(((uint64_t)A.x * n) >> 32);
        const int64_t d = a.ref2dev[i];
        const int b = a.tb.pat[d];
        V3<R> hb, hc, hq;
        partner_fields<R, uint32_t, CUB, QUA>(a.tb, a.cf, p, d, b, hb, hc, hq);
        const V3<R> hext = vsub(vadd(vadd(hb, hc), hq), V3<R>{a.cf.h[3 * b], a.cf.h[3 * b + 1], a.cf.h[3 * b + 2]});
        const V3<R> s = p.get(d);
        const V3<R> sn = propose<R>(pk, a.S, sigma, s, uniform(B.x, B.y), uniform(B.z, B.w));
        const R dE = delta_e<R>(a.cf, b, s, sn, hext);
        const V3<R> dv = constraint_step(k, d, s, sn);
        const R nx = Fp<R>::add(ux, dv.x), ny = Fp<R>::add(uy, dv.y), nz = Fp<R>::add(uz, dv.z);
        const R cv = constraint_value<R>(k, nx, ny, nz);
        const R nl = Fp<R>::sub(lambda, Fp<R>::mul((R)k.weight, cv));
        const R x = Fp<R>::sub(dE, Fp<R>::mul(nl, cv));
        const bool accept = x < R(0) ? true : uniform(A.z, A.w) < Math<R>::exp_(boltz_arg(x, invT, T));
        if (accept) {
            p.set(d, sn);
            ux = nx;
            uy = ny;
            uz = nz;
            lambda = nl;
            acc++;
        }
        A = An;
        B = Bn;
    }
    k.lambda_slot[slot] = (double)lambda;
    cs.sweep_acc[c] += acc;
}

// The same sweep for lattices with bilinear terms only and at most CONS_NB
// partners per site, 32 proposals at a time: lane j takes proposal q0 + j and
// evaluates it against the state at the start of the batch (its draws, site,
// proposed spin, dE, the change of V); the warp then decides the proposals
// in order, in lockstep, exactly as the sequential kernel would (lambda and V
// carried from one decision to the next), up to the first proposal whose
// site or partners an accepted earlier proposal of the batch has changed;
// that one and the rest are drawn again (same counters) in the next batch.
// Every decision and every value equals the sequential kernel's.
constexpr int CONS_NB = 15;
template <typename R>
__global__ void __launch_bounds__(32) k_metro_constraint_batch(SysArgs<R> a, ChainState cs, ConsArgs k, int kind,
                                                              uint32_t msweep, double T_override) {
    using F = Fp<R>;
    constexpr unsigned FULL = 0xffffffffu;
    const int r = blockIdx.x, lane = threadIdx.x;
    const int c = a.chain_base + r;
    const uint32_t key = cs.chain_id[c];
    const Spins<R> p = replica(a, r);
    double vx, vy, vz;
    constraint_v_sum(a, p, k, vx, vy, vz);
    const int slot = cs.slot_of[c];
    const double T = T_override > 0 ? T_override : cs.T_slot[slot];
    const R sigma = (R)cs.sigma_slot[slot];
    const int pk = kind == CSMC_METROPOLIS_CONSTRAINT ? CSMC_METROPOLIS : CSMC_METROPOLIS_ADAPTIVE;
    R lambda = (R)k.lambda_slot[slot];
    R ux = (R)vx, uy = (R)vy, uz = (R)vz;
    const R invT = (R)(1.0 / T);
    auto uniform = [](uint32_t x, uint32_t y) -> R {
        if (sizeof(R) == 4) return (R)u24(x);
        return (R)u53(x, y);
    };
    const uint64_t n = (uint64_t)a.n_real;
    const int64_t Np = a.tb.Np;
    const int W2 = a.tb.W2;
    unsigned long long acc = 0;
    uint64_t q0 = 0;
    // What does not depend on the spins -- the draws, the site, its pattern
    // and partner indices -- is fetched for the next batch of 32 while the
    // warp decides the current one; it is used when the current batch is
    // not cut short (else fetched again).
    uint64_t pf_q0 = UINT64_MAX;
    U4 pA = {0u, 0u, 0u, 0u}, pB = {0u, 0u, 0u, 0u};
    int64_t pd = -1, pnb[CONS_NB];
    int pbs = 0;
    auto fetch = [&](uint64_t qq, U4 &A, U4 &B, int64_t &dd, int &bb, int64_t *nn) {
        A = philox4x32_10((uint32_t)qq, msweep, key, PURPOSE_CONS_A, a.k0, a.k1);
        B = philox4x32_10((uint32_t)qq, msweep, key, PURPOSE_CONS_B, a.k0, a.k1);
        dd = a.ref2dev[(int64_t)(((uint64_t)A.x * n) >> 32)];
        bb = a.tb.pat[dd];
#pragma unroll
        for (int t = 0; t < CONS_NB; t++) nn[t] = t < W2 ? (int64_t)a.tb.p2[t * Np + dd] : -1;
    };
    while (q0 < n) {
        const uint64_t q = q0 + (uint64_t)lane;
        const bool live = q < n;
        int64_t d = -1;
        int64_t nb[CONS_NB];
#pragma unroll
        for (int t = 0; t < CONS_NB; t++) nb[t] = -1;
        V3<R> sn = {R(0), R(0), R(0)}, dv = {R(0), R(0), R(0)};
        R dE = R(0), u = R(0);
        if (live) {
            U4 A, B;
            int b;
            if (pf_q0 == q0) {
                A = pA;
                B = pB;
                d = pd;
                b = pbs;
#pragma unroll
                for (int t = 0; t < CONS_NB; t++) nb[t] = pnb[t];
            } else {
                fetch(q, A, B, d, b, nb);
            }
            V3<R> hb, hc, hq;
            partner_fields<R, uint32_t, false, false>(a.tb, a.cf, p, d, b, hb, hc, hq);
            const V3<R> hext = vsub(vadd(vadd(hb, hc), hq), V3<R>{a.cf.h[3 * b], a.cf.h[3 * b + 1], a.cf.h[3 * b + 2]});
            const V3<R> s = p.get(d);
            sn = propose<R>(pk, a.S, sigma, s, uniform(B.x, B.y), uniform(B.z, B.w));
            dE = delta_e<R>(a.cf, b, s, sn, hext);
            dv = constraint_step(k, d, s, sn);
            u = uniform(A.z, A.w);
        }
        pf_q0 = q0 + 32;
        if (pf_q0 + (uint64_t)lane < n) fetch(pf_q0 + (uint64_t)lane, pA, pB, pd, pbs, pnb);
        // Decisions in order, one accepted proposal per round: every lane of
        // [start, stop) decides against the current state (V, lambda), which
        // is the state the sequential order gives it up to the first lane
        // that accepts; that lane's V and lambda become the state, the lanes
        // after it decide again in the next round, and the first later lane
        // that shares a site with it bounds the batch.  The arithmetic of
        // every decision is the sequential kernel's.
        const int nvalid = n - q0 < 32 ? (int)(n - q0) : 32;
        unsigned taken = 0;
        int stop = nvalid, start = 0;
        while (start < stop) {
            const R nx = F::add(ux, dv.x), ny = F::add(uy, dv.y), nz = F::add(uz, dv.z);
            const R cv = constraint_value<R>(k, nx, ny, nz);
            const R nl = F::sub(lambda, F::mul((R)k.weight, cv));
            const R x = F::sub(dE, F::mul(nl, cv));
            const bool in = lane >= start && lane < stop;
            const bool accept = in && (x < R(0) ? true : u < Math<R>::exp_(boltz_arg(x, invT, T)));
            const unsigned ball = __ballot_sync(FULL, accept);
            if (ball == 0u) break;
            const int j = __ffs((int)ball) - 1;
            taken |= 1u << j;
            ux = __shfl_sync(FULL, nx, j);
            uy = __shfl_sync(FULL, ny, j);
            uz = __shfl_sync(FULL, nz, j);
            lambda = __shfl_sync(FULL, nl, j);
            // the later lanes whose site is the accepted site or a partner of theirs
            const int64_t dj = __shfl_sync(FULL, d, j);
            bool hit = dj == d;
#pragma unroll
            for (int t = 0; t < CONS_NB; t++) hit = hit || nb[t] == dj;
            const unsigned conf = __ballot_sync(FULL, lane > j && lane < stop && hit);
            if (conf != 0u) stop = __ffs((int)conf) - 1;
            start = j + 1;
        }
        if (live && lane < stop && ((taken >> lane) & 1u)) p.set(d, sn);
        acc += (unsigned long long)__popc(taken);
        q0 += (uint64_t)stop;
        __syncwarp();
    }
    if (lane == 0) {
        k.lambda_slot[slot] = (double)lambda;
        cs.sweep_acc[c] += acc;
    }
}

// overrelaxation! body (monte_carlo.jl:128-137) on one colour class.
template <typename R, bool CUB, bool QUA>
__global__ void __launch_bounds__(GB) k_or_colour(SysArgs<R> a, int start, int count, int chain_lo) {
    pdl_wait();
    const int r = chain_lo + blockIdx.y;
    const Spins<R> p = replica(a, r);
    const int i = (int)blockIdx.x * GB + (int)threadIdx.x;
    if (i >= count) return;
    const int d = start + i;
    const int b = a.tb.pat[d];
    const V3<R> H = local_field<R, uint32_t, CUB, QUA>(a.tb, a.cf, p, d, b);
    if (H.x == R(0) && H.y == R(0) && H.z == R(0)) return;
    p.set(d, reflect(p.get(d), H, false));
}

// deterministic_updates! body (monte_carlo.jl:205-210) on one colour class.
template <typename R, bool CUB, bool QUA>
__global__ void __launch_bounds__(GB) k_det_colour(SysArgs<R> a, int start, int count, int chain_lo) {
    pdl_wait();
    const int r = chain_lo + blockIdx.y;
    const Spins<R> p = replica(a, r);
    const int i = (int)blockIdx.x * GB + (int)threadIdx.x;
    if (i >= count) return;
    const int d = start + i;
    const int b = a.tb.pat[d];
    const V3<R> H = local_field<R, uint32_t, CUB, QUA>(a.tb, a.cf, p, d, b);
    if (H.x == R(0) && H.y == R(0) && H.z == R(0)) return;
    const R n = Math<R>::sqrt_(H.x * H.x + H.y * H.y + H.z * H.z);
    p.set(d, {-H.x / n * a.S, -H.y / n * a.S, -H.z / n * a.S});
}

// The reductions give each thread RK sites (stride GB) of a block's RB = GB x
// RK: the thread and then its warp sum them in R, the block sums the warps'
// partials in FP64.
constexpr int RK = 8, RB = GB * RK;

// Per-block partial sums of total_energy (hamiltonian.jl:70-132).
template <typename R, bool CUB, bool QUA>
__global__ void __launch_bounds__(GB) k_energy_part(SysArgs<R> a, int chain_lo, double *part) {
    pdl_wait();
    __shared__ double scratch[GB / 32];
    const int r = chain_lo + blockIdx.y;
    const Spins<R> p = replica(a, r);
    R acc = R(0);
#pragma unroll 1
    for (int k = 0; k < RK; k++) {
        const int d = (int)blockIdx.x * RB + k * GB + (int)threadIdx.x;
        if (d < a.tb.Np && a.dev2ref[d] >= 0)
            acc = Fp<R>::add(acc, site_energy_share<R, uint32_t, CUB, QUA>(a.tb, a.cf, p, d, a.tb.pat[d]));
    }
    const double e = block_sum<GB>(acc, scratch);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = e;
}

// Per-block partial sums of sum_i s_i (observables.jl:12-18).
template <typename R> __global__ void __launch_bounds__(GB) k_magnet_part(SysArgs<R> a, int chain_lo, double *part) {
    pdl_wait();
    __shared__ double scratch[GB / 32];
    const int r = chain_lo + blockIdx.y;
    const Spins<R> p = replica(a, r);
    R ax = R(0), ay = R(0), az = R(0);
#pragma unroll 2
    for (int k = 0; k < RK; k++) {
        const int d = (int)blockIdx.x * RB + k * GB + (int)threadIdx.x;
        if (d < a.tb.Np) { // padding holds zero spins
            const V3<R> s = p.get(d);
            ax = Fp<R>::add(ax, s.x);
            ay = Fp<R>::add(ay, s.y);
            az = Fp<R>::add(az, s.z);
        }
    }
    const double mx = block_sum<GB>(ax, scratch), my = block_sum<GB>(ay, scratch), mz = block_sum<GB>(az, scratch);
    if (threadIdx.x == 0) {
        int64_t o = ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * 3;
        part[o] = mx;
        part[o + 1] = my;
        part[o + 2] = mz;
    }
}

// Deterministic fixed-order sum of per-block partials, one block per replica.
// width = values per block entry (1: energy, 3: magnetisation -> norm).
__global__ void k_reduce_rows(const double *part, int64_t nblk, int width, double *out_chain, int chain_base,
                              int chain_lo) {
    pdl_wait();
    __shared__ double scratch[GB / 32];
    const int row = blockIdx.x;
    double v[3] = {0, 0, 0};
    for (int64_t k = threadIdx.x; k < nblk; k += GB)
        for (int q = 0; q < width; q++) v[q] += part[((int64_t)row * nblk + k) * width + q];
    double t[3];
    for (int q = 0; q < width; q++) t[q] = block_sum<GB>(v[q], scratch);
    if (threadIdx.x == 0) {
        double res = width == 1 ? t[0] : sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        out_chain[chain_base + chain_lo + row] = res;
    }
}

// After one Metropolis sweep of replicas [chain_base+lo, +n): move the sweep's
// accepted count into the slot counters and adapt sigma like
// metropolis_adaptive! (metropolis.jl:124-126) or
// metropolis_constraint_adaptive! (:175-177).
__global__ void k_after_metro(ChainState cs, int chain_first, int n, int kind, double n_sites, double sigma0,
                              double *last_acc) {
    pdl_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int c = chain_first + k;
    const int slot = cs.slot_of[c];
    const double a = (double)cs.sweep_acc[c];
    cs.sweep_acc[c] = 0ull;
    cs.acc_slot[slot] += a;
    if (last_acc) last_acc[slot] = a;
    if (kind == CSMC_METROPOLIS_ADAPTIVE) {
        const double rate = a / n_sites;
        const double om = 1 - rate;
        const double f = 0.5 / (om > 0.05 ? om : 0.05);
        double s = cs.sigma_slot[slot] * f;
        s = s < 0.0 ? 0.0 : (s > 100 ? 100 : s);
        cs.sigma_slot[slot] = s;
    } else if (kind == CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE) { // metropolis.jl:175-177
        const double rate = a / n_sites;
        const double f = 0.5 / (1 - rate);
        cs.sigma_slot[slot] = rate < 0.5 ? cs.sigma_slot[slot] * f : sigma0;
    }
}

// Replica exchange of every lattice of the context followed by the probe
// record of the same iteration (monte_carlo.jl:308-349 then :368-370): one
// block per lattice; the pairs of a lattice are decided in parallel (they
// are disjoint), then, after the block barrier, every slot records the energy
// and |M| of the replica that now sits in it.  kq < 0: no record.
__global__ void k_exchange(ChainState cs, const int2 *lattices, int64_t it, int swap_rate, uint32_t k0, uint32_t k1,
                           int do_swap, double *rec_E, double *rec_M, int64_t kq, int n_slots) {
    pdl_wait();
    const int sys = blockIdx.x;
    const int slot_base = lattices[sys].x, n_rep = lattices[sys].y;
    if (do_swap) exchange_slots(cs, sys, slot_base, n_rep, it, swap_rate, k0, k1);
    if (kq < 0) return;
    __syncthreads();
    record_slots(cs, slot_base, n_rep, rec_E, rec_M, kq, n_slots);
}

// Reference layout (interleaved FP64, reference order) <-> device order.
// One thread per element e = 3 i + k (site i, component k) of a slot's 3 x N
// array, so the FP64 buffer is read (scatter) or written (gather) once and
// contiguously across a warp; `buf` may be device memory or pinned host
// memory mapped into the device's address space.  The slot's replica is
// looked up on the device (chain_of), so a batch of slots is one launch
// whatever the exchange permutation.
template <typename R>
__global__ void k_scatter(SysArgs<R> a, const int32_t *chain_of, int slot_first, const double *src) {
    const int64_t e = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (e >= 3 * a.n_real) return;
    const int r = chain_of[slot_first + blockIdx.y] - a.chain_base;
    const int64_t i = e / 3;
    replica(a, r).set1(a.ref2dev[i], (int)(e - 3 * i), (R)src[(int64_t)blockIdx.y * 3 * a.n_real + e]);
}

template <typename R>
__global__ void k_gather(SysArgs<R> a, const int32_t *chain_of, int slot_first, double *dst) {
    const int64_t e = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (e >= 3 * a.n_real) return;
    const int r = chain_of[slot_first + blockIdx.y] - a.chain_base;
    const int64_t i = e / 3;
    dst[(int64_t)blockIdx.y * 3 * a.n_real + e] = (double)replica(a, r).get1(a.ref2dev[i], (int)(e - 3 * i));
}

// The same, two consecutive values per thread: 16-byte accesses of the FP64
// buffer, which cross the host link faster when it is pinned host memory
// read or written in place.  For blocks of 3 N values that start on 16-byte
// boundaries (N even, buffer 16-byte aligned).
template <typename R>
__global__ void k_scatter2(SysArgs<R> a, const int32_t *chain_of, int slot_first, const double *src) {
    const int64_t n = 3 * a.n_real, e = 2 * ((int64_t)blockIdx.x * GB + threadIdx.x);
    if (e >= n) return;
    const int r = chain_of[slot_first + blockIdx.y] - a.chain_base;
    const double2 v = *reinterpret_cast<const double2 *>(src + (int64_t)blockIdx.y * n + e);
    const Spins<R> p = replica(a, r);
    int64_t i = e / 3;
    int comp = (int)(e - 3 * i);
    p.set1(a.ref2dev[i], comp, (R)v.x);
    if (++comp == 3) {
        comp = 0;
        i++;
    }
    p.set1(a.ref2dev[i], comp, (R)v.y);
}

template <typename R>
__global__ void k_gather2(SysArgs<R> a, const int32_t *chain_of, int slot_first, double *dst) {
    const int64_t n = 3 * a.n_real, e = 2 * ((int64_t)blockIdx.x * GB + threadIdx.x);
    if (e >= n) return;
    const int r = chain_of[slot_first + blockIdx.y] - a.chain_base;
    const Spins<R> p = replica(a, r);
    int64_t i = e / 3;
    int comp = (int)(e - 3 * i);
    double2 v;
    v.x = (double)p.get1(a.ref2dev[i], comp);
    if (++comp == 3) {
        comp = 0;
        i++;
    }
    v.y = (double)p.get1(a.ref2dev[i], comp);
    *reinterpret_cast<double2 *>(dst + (int64_t)blockIdx.y * n + e) = v;
}

// Uniform spins from the INIT stream, counter (reference site, 0, chain, INIT).
template <typename R>
__global__ void k_random_spins(SysArgs<R> a, const uint32_t *chain_id, uint32_t k0, uint32_t k1) {
    const int r = blockIdx.y;
    const Spins<R> p = replica(a, r);
    const int64_t d = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (d >= a.tb.Np) return;
    const int64_t i = a.dev2ref[d];
    if (i < 0) return;
    const U4 w = philox4x32_10((uint32_t)i, 0u, chain_id[a.chain_base + r], PURPOSE_INIT, k0, k1);
    const double uphi = u53(w.x, w.y), uz = u53(w.z, w.w);
    double sp, cp;
    sincospi(2.0 * uphi, &sp, &cp);
    const double z = 2.0 * uz - 1.0;
    const double rr = sqrt(fmax(1.0 - z * z, 0.0));
    const double S = (double)a.S;
    p.set(d, {(R)(S * (rr * cp)), (R)(S * (rr * sp)), (R)(S * z)});
}

template <typename R, bool CUB, bool QUA> __global__ void k_local_field(SysArgs<R> a, int r, double *out) {
    const Spins<R> p = replica(a, r);
    const int64_t d = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (d >= a.tb.Np) return;
    const int64_t i = a.dev2ref[d];
    if (i < 0) return;
    const V3<R> H = local_field<R, uint32_t, CUB, QUA>(a.tb, a.cf, p, d, a.tb.pat[d]);
    out[3 * i] = (double)H.x;
    out[3 * i + 1] = (double)H.y;
    out[3 * i + 2] = (double)H.z;
}

// The replica in `slot` is looked up on the device (chain_of), so the call
// needs no device-to-host read before the launch.
template <typename R, bool CUB, bool QUA>
__global__ void k_energy_diff(SysArgs<R> a, const int32_t *chain_of, int slot, int64_t n, const int64_t *sites,
                              const double *ns, double *dE) {
    const Spins<R> p = replica(a, chain_of[slot] - a.chain_base);
    const int64_t q = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (q >= n) return;
    const int64_t d = a.ref2dev[sites[q]];
    const int b = a.tb.pat[d];
    V3<R> hb, hc, hq;
    partner_fields<R, uint32_t, CUB, QUA>(a.tb, a.cf, p, d, b, hb, hc, hq);
    const V3<R> hext = vsub(vadd(vadd(hb, hc), hq), V3<R>{a.cf.h[3 * b], a.cf.h[3 * b + 1], a.cf.h[3 * b + 2]});
    const V3<R> s = p.get(d);
    const V3<R> sn = {(R)ns[3 * q], (R)ns[3 * q + 1], (R)ns[3 * q + 2]};
    dE[q] = (double)delta_e<R>(a.cf, b, s, sn, hext);
}

template <typename R> __global__ void k_renorm(SysArgs<R> a, int chain_lo) {
    const int r = chain_lo + blockIdx.y;
    const Spins<R> p = replica(a, r);
    const int64_t d = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (d >= a.tb.Np || a.dev2ref[d] < 0) return;
    const V3<R> s = p.get(d);
    const R n2 = s.x * s.x + s.y * s.y + s.z * s.z;
    if (n2 == R(0)) return;
    const R f = a.S * Math<R>::rsqrt_(n2);
    p.set(d, {s.x * f, s.y * f, s.z * f});
}

template <typename R> __global__ void k_drift(SysArgs<R> a, unsigned int *bits) {
    const int r = blockIdx.y;
    const Spins<R> p = replica(a, r);
    const int64_t d = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (d >= a.tb.Np || a.dev2ref[d] < 0) return;
    const V3<R> s = p.get(d);
    const double x = s.x, y = s.y, z = s.z;
    const double S = (double)a.S;
    const float e = (float)(fabs(sqrt(x * x + y * y + z * z) - S) / (S != 0 ? S : 1.0));
    atomicMax(bits, __float_as_uint(e));
}

// Philox4x32-10 blocks of n (counter, key) pairs: the generator the sweep
// kernels draw from, exposed for its published known-answer vectors.
__global__ void k_philox(const uint32_t *ctr, const uint32_t *key, int64_t n, uint32_t *out) {
    const int64_t q = (int64_t)blockIdx.x * GB + threadIdx.x;
    if (q >= n) return;
    const U4 w = philox4x32_10(ctr[4 * q], ctr[4 * q + 1], ctr[4 * q + 2], ctr[4 * q + 3], key[2 * q], key[2 * q + 1]);
    out[4 * q] = w.x;
    out[4 * q + 1] = w.y;
    out[4 * q + 2] = w.z;
    out[4 * q + 3] = w.w;
}

void launch_philox(const uint32_t *ctr, const uint32_t *key, int64_t n, uint32_t *out, cudaStream_t st) {
    if (n <= 0) return;
    k_philox<<<(unsigned)((n + GB - 1) / GB), GB, 0, st>>>(ctr, key, n, out);
}

// ------------------------------------------------------------ launchers

template <typename R> static dim3 grid_for(int64_t n, int chains) {
    return dim3((unsigned)((n + GB - 1) / GB), (unsigned)chains);
}

#define DISPATCH_CQ(a, KERNEL, ...)                                                                                    \
    do {                                                                                                               \
        if ((a).cub && (a).qua) KERNEL<R, true, true> __VA_ARGS__;                                                     \
        else if ((a).cub) KERNEL<R, true, false> __VA_ARGS__;                                                          \
        else if ((a).qua) KERNEL<R, false, true> __VA_ARGS__;                                                          \
        else KERNEL<R, false, false> __VA_ARGS__;                                                                      \
    } while (0)

// Programmatic stream serialization is left off in a process with a tool
// injected (CUDA_INJECTION64_PATH: kernel profilers), which serialise and
// intercept every launch; the kernels then run as ordinary launches, with the
// same results (their griddepcontrol.wait does nothing).
static bool pdl_allowed() {
    static const bool ok = std::getenv("CUDA_INJECTION64_PATH") == nullptr;
    return ok;
}

// A launch with programmatic stream serialization (see pdl_wait).
template <typename... KArgs, typename... Args>
static void launch_dep_b(void (*kern)(KArgs...), dim3 g, int block, cudaStream_t st, Args... args) {
    if (!pdl_allowed()) {
        kern<<<g, block, 0, st>>>(static_cast<KArgs>(args)...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...) != cudaSuccess) {
        (void)cudaGetLastError();
        kern<<<g, block, 0, st>>>(static_cast<KArgs>(args)...); // an ordinary launch reports its own error
    }
}

template <typename... KArgs, typename... Args>
static void launch_dep(void (*kern)(KArgs...), dim3 g, cudaStream_t st, Args... args) {
    launch_dep_b(kern, g, GB, st, args...);
}

#define PICK_CQ(a, KERNEL)                                                                                             \
    ((a).cub && (a).qua ? KERNEL<R, true, true>                                                                       \
                        : (a).cub ? KERNEL<R, true, false> : (a).qua ? KERNEL<R, false, true> : KERNEL<R, false, false>)

// (the host admits lattices of fewer than 2^31 / W device sites, so colour
// class starts and counts fit 32 bits)

// Threads of a Metropolis colour-sweep launch over `count` sites: lattices
// without cubic and quartic terms take two sites per thread (k_metro_colour:
// 151 vs 206 us per launch on SC L=64 x 64; the overrelaxation kernel, with
// less arithmetic per gather, was slower that way, 125 vs 98 us).
template <typename R> static int64_t sweep_threads(const SysArgs<R> &a, int64_t count) {
    return (a.cub || a.qua) ? count : (count + 1) / 2;
}
template <typename R>
void launch_metro_colour(const SysArgs<R> &a, const ChainState &cs, int64_t start, int64_t count, int chain_lo,
                         int n_chains, int kind, uint32_t msweep, double T_override, cudaStream_t st) {
    if (count <= 0 || n_chains <= 0) return;
    const float invT_override = T_override > 0 ? (float)(1.0 / T_override) : 0.f;
    launch_dep(PICK_CQ(a, k_metro_colour), grid_for<R>(sweep_threads(a, count), n_chains), st, a, cs, (int)start,
               (int)count, chain_lo, kind, msweep, T_override, invT_override);
}

template <typename R>
void launch_or_colour(const SysArgs<R> &a, int64_t start, int64_t count, int chain_lo, int n_chains,
                      cudaStream_t st) {
    if (count <= 0 || n_chains <= 0) return;
    launch_dep(PICK_CQ(a, k_or_colour), grid_for<R>(count, n_chains), st, a, (int)start, (int)count, chain_lo);
}

template <typename R>
void launch_det_colour(const SysArgs<R> &a, int64_t start, int64_t count, int chain_lo, int n_chains,
                       cudaStream_t st) {
    if (count <= 0 || n_chains <= 0) return;
    launch_dep(PICK_CQ(a, k_det_colour), grid_for<R>(count, n_chains), st, a, (int)start, (int)count, chain_lo);
}

int64_t partial_blocks(int64_t Np) { return (Np + RB - 1) / RB; }

template <typename R>
void launch_energy(const SysArgs<R> &a, const ChainState &cs, int chain_lo, int n_chains, double *part,
                   cudaStream_t st) {
    if (n_chains <= 0) return;
    const dim3 g((unsigned)partial_blocks(a.tb.Np), (unsigned)n_chains);
    launch_dep(PICK_CQ(a, k_energy_part), g, st, a, chain_lo, part);
    launch_dep(k_reduce_rows, dim3(n_chains), st, (const double *)part, (int64_t)g.x, 1, cs.E_chain, a.chain_base,
               chain_lo);
}

template <typename R>
void launch_magnet(const SysArgs<R> &a, const ChainState &cs, int chain_lo, int n_chains, double *part,
                   cudaStream_t st) {
    if (n_chains <= 0) return;
    const dim3 g((unsigned)partial_blocks(a.tb.Np), (unsigned)n_chains);
    launch_dep(k_magnet_part<R>, g, st, a, chain_lo, part);
    launch_dep(k_reduce_rows, dim3(n_chains), st, (const double *)part, (int64_t)g.x, 3, cs.M_chain, a.chain_base,
               chain_lo);
}

void launch_after_metro(const ChainState &cs, int chain_first, int n, int kind, int64_t n_sites, double sigma0,
                        double *last_acc, cudaStream_t st) {
    if (n <= 0) return;
    launch_dep_b(k_after_metro, dim3((n + 127) / 128), 128, st, cs, chain_first, n, kind, (double)n_sites, sigma0,
                 last_acc);
}

template <typename R>
void launch_metro_constraint(const SysArgs<R> &a, const ChainState &cs, const ConsArgs &k, int kind, uint32_t msweep,
                             double T_override, cudaStream_t st) {
    if (a.n_rep <= 0 || a.n_real <= 0) return;
    if (!a.cub && !a.qua && a.tb.W2 <= CONS_NB)
        k_metro_constraint_batch<R><<<a.n_rep, 32, 0, st>>>(a, cs, k, kind, msweep, T_override);
    else
        DISPATCH_CQ(a, k_metro_constraint, <<<a.n_rep, 32, 0, st>>>(a, cs, k, kind, msweep, T_override));
}

void launch_exchange(const ChainState &cs, const int2 *lattices, int n_lattices, int64_t it, int swap_rate, uint32_t k0,
                     uint32_t k1, bool do_swap, double *rec_E, double *rec_M, int64_t kq, int n_slots, cudaStream_t st) {
    launch_dep_b(k_exchange, dim3(n_lattices), 256, st, cs, lattices, it, swap_rate, k0, k1, do_swap ? 1 : 0, rec_E,
                 rec_M, kq, n_slots);
}

template <typename R>
void launch_scatter(const SysArgs<R> &a, const int32_t *chain_of, int slot_first, int n_slots, const double *src,
                    cudaStream_t st) {
    if (a.n_real % 2 == 0 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0)
        k_scatter2<R><<<grid_for<R>(3 * a.n_real / 2, n_slots), GB, 0, st>>>(a, chain_of, slot_first, src);
    else
        k_scatter<R><<<grid_for<R>(3 * a.n_real, n_slots), GB, 0, st>>>(a, chain_of, slot_first, src);
}
template <typename R>
void launch_gather(const SysArgs<R> &a, const int32_t *chain_of, int slot_first, int n_slots, double *dst,
                   cudaStream_t st) {
    if (a.n_real % 2 == 0 && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0)
        k_gather2<R><<<grid_for<R>(3 * a.n_real / 2, n_slots), GB, 0, st>>>(a, chain_of, slot_first, dst);
    else
        k_gather<R><<<grid_for<R>(3 * a.n_real, n_slots), GB, 0, st>>>(a, chain_of, slot_first, dst);
}
template <typename R>
void launch_random_spins(const SysArgs<R> &a, const uint32_t *chain_id, uint32_t k0, uint32_t k1, cudaStream_t st) {
    k_random_spins<R><<<grid_for<R>(a.tb.Np, a.n_rep), GB, 0, st>>>(a, chain_id, k0, k1);
}
template <typename R> void launch_local_field(const SysArgs<R> &a, int r, double *out, cudaStream_t st) {
    dim3 g = grid_for<R>(a.tb.Np, 1);
    DISPATCH_CQ(a, k_local_field, <<<g, GB, 0, st>>>(a, r, out));
}
template <typename R>
void launch_energy_diff(const SysArgs<R> &a, const int32_t *chain_of, int slot, int64_t n, const int64_t *sites,
                        const double *ns, double *dE, cudaStream_t st) {
    if (n <= 0) return;
    dim3 g = grid_for<R>(n, 1);
    DISPATCH_CQ(a, k_energy_diff, <<<g, GB, 0, st>>>(a, chain_of, slot, n, sites, ns, dE));
}
template <typename R> void launch_renorm(const SysArgs<R> &a, int chain_lo, int n_chains, cudaStream_t st) {
    k_renorm<R><<<grid_for<R>(a.tb.Np, n_chains), GB, 0, st>>>(a, chain_lo);
}
template <typename R> void launch_drift(const SysArgs<R> &a, unsigned int *bits, cudaStream_t st) {
    k_drift<R><<<grid_for<R>(a.tb.Np, a.n_rep), GB, 0, st>>>(a, bits);
}

#define INSTANTIATE(R)                                                                                                 \
    template void launch_metro_colour<R>(const SysArgs<R> &, const ChainState &, int64_t, int64_t, int, int, int,     \
                                         uint32_t, double, cudaStream_t);                                              \
    template void launch_metro_constraint<R>(const SysArgs<R> &, const ChainState &, const ConsArgs &, int, uint32_t, \
                                             double, cudaStream_t);                                                    \
    template void launch_or_colour<R>(const SysArgs<R> &, int64_t, int64_t, int, int, cudaStream_t);                  \
    template void launch_det_colour<R>(const SysArgs<R> &, int64_t, int64_t, int, int, cudaStream_t);                 \
    template void launch_energy<R>(const SysArgs<R> &, const ChainState &, int, int, double *, cudaStream_t);         \
    template void launch_magnet<R>(const SysArgs<R> &, const ChainState &, int, int, double *, cudaStream_t);         \
    template void launch_scatter<R>(const SysArgs<R> &, const int32_t *, int, int, const double *, cudaStream_t);     \
    template void launch_gather<R>(const SysArgs<R> &, const int32_t *, int, int, double *, cudaStream_t);            \
    template void launch_random_spins<R>(const SysArgs<R> &, const uint32_t *, uint32_t, uint32_t, cudaStream_t);     \
    template void launch_local_field<R>(const SysArgs<R> &, int, double *, cudaStream_t);                             \
    template void launch_energy_diff<R>(const SysArgs<R> &, const int32_t *, int, int64_t, const int64_t *,          \
                                        const double *, double *, cudaStream_t);                                       \
    template void launch_renorm<R>(const SysArgs<R> &, int, int, cudaStream_t);                                       \
    template void launch_drift<R>(const SysArgs<R> &, unsigned int *, cudaStream_t);

INSTANTIATE(float)
INSTANTIATE(double)

} // namespace csmc
