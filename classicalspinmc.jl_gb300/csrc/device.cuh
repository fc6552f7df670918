// device.cuh -- device-side data views and per-site physics shared by the
// colour-sweep kernels (kernels.cu) and the replay kernel (exact.cu).
#pragma once

#include <type_traits>

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/csmc.h"

namespace csmc {

// Philox stream purposes (counter word 3); the oracle uses the same values.
enum : uint32_t {
    PURPOSE_METRO_A = 1,
    PURPOSE_METRO_B = 2,
    PURPOSE_SWAP = 3,
    PURPOSE_INIT = 4,
    PURPOSE_CONS_A = 5, // constrained Metropolis: site and acceptance uniform
    PURPOSE_CONS_B = 6  // constrained Metropolis: proposal uniforms
};

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of the
// multiply-xor S-box with Weyl key schedule.
struct U4 {
    uint32_t x, y, z, w;
};
__host__ __device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                     uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        // each 32 x 32 -> 64-bit product as one wide multiply (both halves)
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

__host__ __device__ __forceinline__ float u24(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }
__host__ __device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)m * (1.0 / 9007199254740992.0);
}

// One lattice ("system") as the kernels see it.  Idx is the partner index
// type: uint32 for the global path, uint16 for shared-memory residents.
template <typename Idx> struct Tab {
    const Idx *p2, *p3, *p4; // [W][k][Np]
    const uint8_t *pat;      // basis (pattern) of each device site
    int64_t Np;
    int W2, W3, W4;
};

// Coupling coefficients in the arithmetic type R; pattern b = basis, nb =
// padding.  Pointers may point to global or shared memory.
template <typename R> struct Coef {
    const R *mats, *cubs, *quas; // deduplicated tensors, id 0 = zeros
    const R *O, *P, *h;          // per pattern: onsite (9), folded self loops (9), field (3)
    const int32_t *c2, *c3, *c4; // per pattern x slot: coefficient ids
    // per pattern, for the specialised resident kernel: 2O+P (local field),
    // O+P (dE), O+P/2 (energy share), and the scalar of each bilinear slot
    // when every coupling is a multiple of the identity
    const R *A, *Q, *E2, *Js;
    // 1: every bilinear coupling of the lattice is c I, and Js[b * W2 + t]
    // holds its c (the same value as miso's) -- one table read per partner
    // instead of the coupling id and its isotropy record
    int32_t iso2;
    // 1: every pattern's onsite matrix O and self-loop matrix P is diagonal;
    // the onsite products then read and multiply the diagonals alone (the
    // zero off-diagonal terms of the full products add nothing)
    int32_t ons_diag;
    // per tensor id: isotropic bilinear {flag, J}, cubic {flag, kappa},
    // quartic {flag, q1, q2, q3}
    const R *miso, *ciso, *qiso;
};

template <typename R> struct V3 {
    R x, y, z;
};

// Arithmetic with explicit rounding: every product, sum and fused
// multiply-add below is spelled out, so the compiler cannot contract or
// re-associate differently in different kernels.  The resident kernel's
// instantiations (one CTA or a cluster per replica) and the colour-sweep
// kernels therefore compute bit-identical values for the same site.
template <typename R> struct Fp;
template <> struct Fp<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <> struct Fp<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};
// acc + M s, one fused multiply-add per term in the order M[0] s.x, M[1] s.y,
// M[2] s.z (a matrix c*I gives exactly acc + c s)
template <typename R> __device__ __forceinline__ V3<R> add_matvec(V3<R> acc, const R *M, V3<R> s) {
    using F = Fp<R>;
    return {F::fma(M[2], s.z, F::fma(M[1], s.y, F::fma(M[0], s.x, acc.x))),
            F::fma(M[5], s.z, F::fma(M[4], s.y, F::fma(M[3], s.x, acc.y))),
            F::fma(M[8], s.z, F::fma(M[7], s.y, F::fma(M[6], s.x, acc.z)))};
}
template <typename R> __device__ __forceinline__ V3<R> add_scaled(V3<R> acc, R c, V3<R> s) {
    using F = Fp<R>;
    return {F::fma(c, s.x, acc.x), F::fma(c, s.y, acc.y), F::fma(c, s.z, acc.z)};
}
template <typename R> __device__ __forceinline__ V3<R> vadd(V3<R> a, V3<R> b) {
    return {Fp<R>::add(a.x, b.x), Fp<R>::add(a.y, b.y), Fp<R>::add(a.z, b.z)};
}
template <typename R> __device__ __forceinline__ V3<R> vsub(V3<R> a, V3<R> b) {
    return {Fp<R>::sub(a.x, b.x), Fp<R>::sub(a.y, b.y), Fp<R>::sub(a.z, b.z)};
}

// The spins of one replica in device memory.  Single precision: one float4
// (x, y, z, 0) per device site, so a site is a single 16-byte load and a
// replica one contiguous block of 16 * Np bytes.  Double precision: three
// blocks x[Np] | y[Np] | z[Np].  get/set take the device site index.
template <typename R> struct Spins;
template <> struct Spins<float> {
    float4 *p;
    static constexpr int kWords = 4; // floats per site
    __device__ __forceinline__ V3<float> get(int64_t j) const {
        const float4 v = p[j];
        return {v.x, v.y, v.z};
    }
    __device__ __forceinline__ void set(int64_t j, V3<float> s) const { p[j] = make_float4(s.x, s.y, s.z, 0.f); }
    // component k (0, 1, 2) of site j
    __device__ __forceinline__ float get1(int64_t j, int k) const { return reinterpret_cast<const float *>(p)[4 * j + k]; }
    __device__ __forceinline__ void set1(int64_t j, int k, float v) const { reinterpret_cast<float *>(p)[4 * j + k] = v; }
};
template <> struct Spins<double> {
    double *x;
    int64_t n;
    static constexpr int kWords = 3; // doubles per site
    __device__ __forceinline__ V3<double> get(int64_t j) const { return {x[j], x[n + j], x[2 * n + j]}; }
    __device__ __forceinline__ void set(int64_t j, V3<double> s) const {
        x[j] = s.x;
        x[n + j] = s.y;
        x[2 * n + j] = s.z;
    }
    __device__ __forceinline__ double get1(int64_t j, int k) const { return x[k * n + j]; }
    __device__ __forceinline__ void set1(int64_t j, int k, double v) const { x[k * n + j] = v; }
};
// Replica r of a spin array of Np device sites per replica.
__host__ __device__ __forceinline__ Spins<float> spins_of(float *base, int64_t Np, int64_t r) {
    return {reinterpret_cast<float4 *>(base) + r * Np};
}
__host__ __device__ __forceinline__ Spins<double> spins_of(double *base, int64_t Np, int64_t r) {
    return {base + r * 3 * Np, Np};
}

// Fields on site d from its partners, split by term order, without onsite,
// self loops or the Zeeman field:
//   hb = sum_n J_n s_j (bilinear), hc_a = sum C[a,b,c] s_j,b s_k,c,
//   hq_a = sum R[a,b,c,d] s_j,b s_k,c s_l,d  (hamiltonian.jl:24-65).
// SV is a spin view with get(j) (Spins<R> or a shared-memory view).
template <typename R, typename Idx, bool CUB, bool QUA, class SV>
__device__ __forceinline__ void partner_fields(const Tab<Idx> &tb, const Coef<R> &cf, const SV &sv, int64_t d, int b,
                                               V3<R> &hb, V3<R> &hc, V3<R> &hq) {
    using F = Fp<R>;
    hb = {R(0), R(0), R(0)};
    hc = {R(0), R(0), R(0)};
    hq = {R(0), R(0), R(0)};
    // 32-bit table offsets: the host admits lattices with W * Np < 2^31
    const int Np = (int)tb.Np, di = (int)d;
    // one term of each kind, its partner spins given
    auto bil = [&](int t, V3<R> sj) {
        if (cf.iso2) { // block-uniform
            hb = add_scaled(hb, cf.Js[b * tb.W2 + t], sj);
            return;
        }
        const int id = cf.c2[b * tb.W2 + t];
        if (cf.miso[2 * id] != R(0)) hb = add_scaled(hb, cf.miso[2 * id + 1], sj); // J I
        else hb = add_matvec(hb, cf.mats + 9 * id, sj);
    };
    auto cub = [&](int t, V3<R> sj, V3<R> sk) {
        const int id = cf.c3[b * tb.W3 + t];
        if (cf.ciso[2 * id] != R(0)) { // kappa eps_abc: kappa (s_j x s_k)
            const R kap = cf.ciso[2 * id + 1];
            const V3<R> x = {F::fma(sj.y, sk.z, -F::mul(sj.z, sk.y)), F::fma(sj.z, sk.x, -F::mul(sj.x, sk.z)),
                             F::fma(sj.x, sk.y, -F::mul(sj.y, sk.x))};
            hc = add_scaled(hc, kap, x);
            return;
        }
        const R *C = cf.cubs + 27 * id;
        const R a0 = sj.x, a1 = sj.y, a2 = sj.z, b0 = sk.x, b1 = sk.y, b2 = sk.z;
        const R o[9] = {F::mul(a0, b0), F::mul(a0, b1), F::mul(a0, b2), F::mul(a1, b0), F::mul(a1, b1),
                        F::mul(a1, b2), F::mul(a2, b0), F::mul(a2, b1), F::mul(a2, b2)};
        R sx = 0, sy = 0, sz = 0;
#pragma unroll
        for (int q = 0; q < 9; q++) {
            sx = F::fma(C[q], o[q], sx);
            sy = F::fma(C[9 + q], o[q], sy);
            sz = F::fma(C[18 + q], o[q], sz);
        }
        hc = vadd(hc, V3<R>{sx, sy, sz});
    };
    auto qua = [&](int t, V3<R> sj, V3<R> sk, V3<R> sl) {
        const int id = cf.c4[b * tb.W4 + t];
        if (cf.qiso[4 * id] != R(0)) { // q1 s_j (s_k.s_l) + q2 s_k (s_j.s_l) + q3 s_l (s_j.s_k)
            const R w1 = F::mul(cf.qiso[4 * id + 1], dot(sk, sl)), w2 = F::mul(cf.qiso[4 * id + 2], dot(sj, sl)),
                    w3 = F::mul(cf.qiso[4 * id + 3], dot(sj, sk));
            hq = add_scaled(add_scaled(add_scaled(hq, w1, sj), w2, sk), w3, sl);
            return;
        }
        const R *Q = cf.quas + 81 * id;
        const R a[3] = {sj.x, sj.y, sj.z}, bb[3] = {sk.x, sk.y, sk.z}, c[3] = {sl.x, sl.y, sl.z};
        R sx = 0, sy = 0, sz = 0;
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                const R ab = F::mul(a[p], bb[q]);
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    const R o = F::mul(ab, c[r]);
                    const int idx = (p * 3 + q) * 3 + r;
                    sx = F::fma(Q[idx], o, sx);
                    sy = F::fma(Q[27 + idx], o, sy);
                    sz = F::fma(Q[54 + idx], o, sz);
                }
            }
        hq = vadd(hq, V3<R>{sx, sy, sz});
    };
    // Spins in global memory: terms in groups (bilinear threes, cubic and
    // quartic pairs), the group's partner indices and then its partner spins
    // loaded before any is used (several gathers in flight per dependent
    // step instead of one); same arithmetic order.
    constexpr bool kPairs = std::is_same<SV, Spins<R>>::value;
    int t = 0;
    if (kPairs) { // bilinear terms in threes
        constexpr int G = 3;
        for (; t + G <= tb.W2; t += G) {
            int j[G];
            V3<R> sj[G];
#pragma unroll
            for (int u = 0; u < G; u++) j[u] = (int)tb.p2[(t + u) * Np + di];
#pragma unroll
            for (int u = 0; u < G; u++) sj[u] = sv.get(j[u]);
#pragma unroll
            for (int u = 0; u < G; u++) bil(t + u, sj[u]);
        }
    }
    for (; t < tb.W2; t++) bil(t, sv.get(tb.p2[t * Np + di]));
    if (CUB) {
        t = 0;
        if (kPairs)
            for (; t + 2 <= tb.W3; t += 2) {
                const int j0 = (int)tb.p3[(2 * t) * Np + di], k0 = (int)tb.p3[(2 * t + 1) * Np + di];
                const int j1 = (int)tb.p3[(2 * t + 2) * Np + di], k1 = (int)tb.p3[(2 * t + 3) * Np + di];
                const V3<R> sj0 = sv.get(j0), sk0 = sv.get(k0), sj1 = sv.get(j1), sk1 = sv.get(k1);
                cub(t, sj0, sk0);
                cub(t + 1, sj1, sk1);
            }
        for (; t < tb.W3; t++) cub(t, sv.get(tb.p3[(2 * t) * Np + di]), sv.get(tb.p3[(2 * t + 1) * Np + di]));
    }
    if (QUA) {
        t = 0;
        if (kPairs)
            for (; t + 2 <= tb.W4; t += 2) {
                const int j0 = (int)tb.p4[(3 * t) * Np + di], k0 = (int)tb.p4[(3 * t + 1) * Np + di],
                              l0 = (int)tb.p4[(3 * t + 2) * Np + di];
                const int j1 = (int)tb.p4[(3 * t + 3) * Np + di], k1 = (int)tb.p4[(3 * t + 4) * Np + di],
                              l1 = (int)tb.p4[(3 * t + 5) * Np + di];
                const V3<R> sj0 = sv.get(j0), sk0 = sv.get(k0), sl0 = sv.get(l0);
                const V3<R> sj1 = sv.get(j1), sk1 = sv.get(k1), sl1 = sv.get(l1);
                qua(t, sj0, sk0, sl0);
                qua(t + 1, sj1, sk1, sl1);
            }
        for (; t < tb.W4; t++)
            qua(t, sv.get(tb.p4[(3 * t) * Np + di]), sv.get(tb.p4[(3 * t + 1) * Np + di]),
                sv.get(tb.p4[(3 * t + 2) * Np + di]));
    }
}

// The bilinear fields hb of two sites d0, d1 of a lattice without cubic and
// quartic terms, spins in global memory: per group of three slots, both
// sites' partner indices, then both sites' partner spins are loaded before
// any is used, so twice as many gathers are in flight per dependent step.
// Each site's sum is formed in partner_fields' order (bit for bit the same).
template <typename R, class SV>
__device__ __forceinline__ void bilinear_fields2(const Tab<uint32_t> &tb, const Coef<R> &cf, const SV &sv, int d0,
                                                 int d1, int b0, int b1, V3<R> &hb0, V3<R> &hb1) {
    hb0 = {R(0), R(0), R(0)};
    hb1 = {R(0), R(0), R(0)};
    const int Np = (int)tb.Np;
    auto bil = [&](int b, int t, V3<R> sj, V3<R> &hb) {
        if (cf.iso2) { // block-uniform
            hb = add_scaled(hb, cf.Js[b * tb.W2 + t], sj);
            return;
        }
        const int id = cf.c2[b * tb.W2 + t];
        if (cf.miso[2 * id] != R(0)) hb = add_scaled(hb, cf.miso[2 * id + 1], sj); // J I
        else hb = add_matvec(hb, cf.mats + 9 * id, sj);
    };
    constexpr int G = 3;
    int t = 0;
    for (; t + G <= tb.W2; t += G) {
        int j0[G], j1[G];
        V3<R> s0[G], s1[G];
#pragma unroll
        for (int u = 0; u < G; u++) {
            j0[u] = (int)tb.p2[(t + u) * Np + d0];
            j1[u] = (int)tb.p2[(t + u) * Np + d1];
        }
#pragma unroll
        for (int u = 0; u < G; u++) {
            s0[u] = sv.get(j0[u]);
            s1[u] = sv.get(j1[u]);
        }
#pragma unroll
        for (int u = 0; u < G; u++) bil(b0, t + u, s0[u], hb0);
#pragma unroll
        for (int u = 0; u < G; u++) bil(b1, t + u, s1[u], hb1);
    }
    for (; t < tb.W2; t++) {
        const V3<R> s0r = sv.get(tb.p2[t * Np + d0]), s1r = sv.get(tb.p2[t * Np + d1]);
        bil(b0, t, s0r, hb0);
        bil(b1, t, s1r, hb1);
    }
}

template <typename R> __device__ __forceinline__ V3<R> matvec(const R *M, V3<R> s) {
    using F = Fp<R>;
    return {F::fma(M[2], s.z, F::fma(M[1], s.y, F::mul(M[0], s.x))),
            F::fma(M[5], s.z, F::fma(M[4], s.y, F::mul(M[3], s.x))),
            F::fma(M[8], s.z, F::fma(M[7], s.y, F::mul(M[6], s.x)))};
}
// matvec of a diagonal matrix: M[0] s.x, M[4] s.y, M[8] s.z -- the values
// matvec gives when the off-diagonal entries are zero
template <typename R> __device__ __forceinline__ V3<R> diagvec(const R *M, V3<R> s) {
    using F = Fp<R>;
    return {F::mul(M[0], s.x), F::mul(M[4], s.y), F::mul(M[8], s.z)};
}
template <typename R> __device__ __forceinline__ R dot(V3<R> a, V3<R> b) {
    using F = Fp<R>;
    return F::fma(a.z, b.z, F::fma(a.y, b.y, F::mul(a.x, b.x)));
}

// get_local_field (hamiltonian.jl:3-67) of site spin s of pattern b from its
// partners' fields: 2 O s + (self loops) + hb + hc + hq - h.
// CUB / QUA false: hc / hq are zero and not added (x + 0 is x).
template <typename R, bool CUB = true, bool QUA = true>
__device__ __forceinline__ V3<R> field_of(const Coef<R> &cf, int b, V3<R> s, V3<R> hb, V3<R> hc, V3<R> hq) {
    const V3<R> os = cf.ons_diag ? diagvec(cf.O + 9 * b, s) : matvec(cf.O + 9 * b, s),
                ps = cf.ons_diag ? diagvec(cf.P + 9 * b, s) : matvec(cf.P + 9 * b, s);
    const V3<R> h = {cf.h[3 * b], cf.h[3 * b + 1], cf.h[3 * b + 2]};
    const V3<R> two_os = {Fp<R>::mul(R(2), os.x), Fp<R>::mul(R(2), os.y), Fp<R>::mul(R(2), os.z)};
    V3<R> f = vadd(vadd(two_os, ps), hb);
    if (CUB) f = vadd(f, hc);
    if (QUA) f = vadd(f, hq);
    return vsub(f, h);
}

// get_local_field (hamiltonian.jl:3-67) at device site d.
template <typename R, typename Idx, bool CUB, bool QUA, class SV>
__device__ __forceinline__ V3<R> local_field(const Tab<Idx> &tb, const Coef<R> &cf, const SV &sv, int64_t d, int b) {
    V3<R> hb, hc, hq;
    partner_fields<R, Idx, CUB, QUA>(tb, cf, sv, d, b, hb, hc, hq);
    return field_of<R, CUB, QUA>(cf, b, sv.get(d), hb, hc, hq);
}

// Energy of moving site d from s to sn with all other spins fixed:
// e(s) = s.(O+P).s + s.(hb + hc + hq - h)  (hamiltonian.jl:139-196), so
// dE = sn.Q.sn - s.Q.s + (sn - s).hext.
template <typename R>
__device__ __forceinline__ R delta_e(const Coef<R> &cf, int b, V3<R> s, V3<R> sn, V3<R> hext) {
    using F = Fp<R>;
    const R *O = cf.O + 9 * b, *P = cf.P + 9 * b;
    R q[9];
    if (cf.ons_diag) { // block-uniform
#pragma unroll
        for (int k = 0; k < 9; k += 4) q[k] = F::add(O[k], P[k]);
        const R en = dot(sn, diagvec(q, sn)), eo = dot(s, diagvec(q, s));
        return F::add(F::sub(en, eo), dot(vsub(sn, s), hext));
    }
#pragma unroll
    for (int k = 0; k < 9; k++) q[k] = F::add(O[k], P[k]);
    const R en = dot(sn, matvec(q, sn)), eo = dot(s, matvec(q, s));
    return F::add(F::sub(en, eo), dot(vsub(sn, s), hext));
}

// Contribution of site d to total_energy (hamiltonian.jl:70-132):
// -s.h + s.O.s + (s.hb + s.P.s)/2 + s.hc/3 + s.hq/4, in the arithmetic type R.
// Callers add a few sites' shares in R per thread and sum those partials in
// FP64 (on this device FP64 runs at a small fraction of the FP32 rate, and a
// per-site FP64 sum made the energy kernels FP64-bound).
template <typename R, typename Idx, bool CUB, bool QUA, class SV>
__device__ __forceinline__ R site_energy_share(const Tab<Idx> &tb, const Coef<R> &cf, const SV &sv, int64_t d, int b) {
    using F = Fp<R>;
    V3<R> hb, hc, hq;
    partner_fields<R, Idx, CUB, QUA>(tb, cf, sv, d, b, hb, hc, hq);
    const V3<R> s = sv.get(d);
    const V3<R> h = {cf.h[3 * b], cf.h[3 * b + 1], cf.h[3 * b + 2]};
    const R eo = dot(s, matvec(cf.O + 9 * b, s));
    const R ep = dot(s, matvec(cf.P + 9 * b, s));
    const R ez = dot(s, h);
    R e = F::add(F::sub(eo, ez), F::mul(R(0.5), F::add(dot(s, hb), ep)));
    if (CUB) e = F::add(e, F::div(dot(s, hc), R(3)));
    if (QUA) e = F::fma(R(0.25), dot(s, hq), e);
    return e;
}

template <typename R> struct Math;
template <> struct Math<float> {
    // sin and cos of 2*pi*u for u in [0,1): the hardware approximation on the
    // angle shifted into [-pi, pi) (absolute error below 2^-21), then
    // sin(a + pi) = -sin(a), cos(a + pi) = -cos(a)
    static __device__ __forceinline__ void sincospi2(float u, float *s, float *c) {
        float sa, ca;
        __sincosf(6.28318530718f * (u - 0.5f), &sa, &ca);
        *s = -sa;
        *c = -ca;
    }
    static __device__ __forceinline__ float sqrt_(float v) { return sqrtf(v); }
    static __device__ __forceinline__ float rsqrt_(float v) { return rsqrtf(v); }
    static __device__ __forceinline__ float exp_(float v) { return __expf(v); }
    // a / b within 2 ulp for 2^-126 <= |b| <= 2^126 (the squared local field)
    static __device__ __forceinline__ float div_(float a, float b) { return __fdividef(a, b); }
};
template <> struct Math<double> {
    static __device__ __forceinline__ void sincospi2(double u, double *s, double *c) { sincospi(2.0 * u, s, c); }
    static __device__ __forceinline__ double sqrt_(double v) { return sqrt(v); }
    static __device__ __forceinline__ double rsqrt_(double v) { return rsqrt(v); }
    static __device__ __forceinline__ double exp_(double v) { return exp(v); }
    static __device__ __forceinline__ double div_(double a, double b) { return a / b; }
};

// Overrelaxation (monte_carlo.jl:135-137): s <- -s + 2 (s.H)/|H|^2 H, with
// explicit rounding; `fast` uses the single-precision fast division.
template <typename R> __device__ __forceinline__ V3<R> reflect(V3<R> s, V3<R> H, bool fast) {
    using F = Fp<R>;
    const R num = F::mul(R(2), dot(s, H)), den = dot(H, H);
    const R proj = fast ? Math<R>::div_(num, den) : num / den;
    return {F::fma(proj, H.x, -s.x), F::fma(proj, H.y, -s.y), F::fma(proj, H.z, -s.z)};
}
// The exponent -dE/T of the acceptance test (metropolis.jl:73): by the
// reciprocal temperature in single precision, by division in double.
template <typename R> __device__ __forceinline__ R boltz_arg(R dE, R invT, double T) {
    if (sizeof(R) == 4) return Fp<R>::mul(-dE, invT);
    return -dE / (R)T;
}

// Uniforms of one Metropolis proposal from the Philox stream keyed by the
// context seed; counter = (device site, Metropolis sweep, replica, purpose).
template <typename R> struct Draw;
template <> struct Draw<float> {
    float uphi, uz, uacc;
    __device__ __forceinline__ Draw(uint32_t d, uint32_t sweep, uint32_t chain, uint32_t k0, uint32_t k1) {
        U4 w = philox4x32_10(d, sweep, chain, PURPOSE_METRO_A, k0, k1);
        uphi = u24(w.x);
        uz = u24(w.y);
        uacc = u24(w.z);
    }
    __device__ __forceinline__ float acc(uint32_t, uint32_t, uint32_t, uint32_t, uint32_t) const { return uacc; }
};
template <> struct Draw<double> {
    double uphi, uz;
    __device__ __forceinline__ Draw(uint32_t d, uint32_t sweep, uint32_t chain, uint32_t k0, uint32_t k1) {
        U4 w = philox4x32_10(d, sweep, chain, PURPOSE_METRO_A, k0, k1);
        uphi = u53(w.x, w.y);
        uz = u53(w.z, w.w);
    }
    __device__ __forceinline__ double acc(uint32_t d, uint32_t sweep, uint32_t chain, uint32_t k0, uint32_t k1) const {
        U4 w = philox4x32_10(d, sweep, chain, PURPOSE_METRO_B, k0, k1);
        return u53(w.x, w.y);
    }
};

// random_spin_orientation (lattice.jl:306-311) and gaussian_move
// (metropolis.jl:84-87) for uniforms (uphi, uz).
template <typename R>
__device__ __forceinline__ V3<R> propose(int kind, R S, R sigma, V3<R> s, R uphi, R uz) {
    using F = Fp<R>;
    R sp, cp;
    Math<R>::sincospi2(uphi, &sp, &cp);
    const R zz = F::sub(F::mul(R(2), uz), R(1));
    const R r2 = F::sub(R(1), F::mul(zz, zz));
    const R r = Math<R>::sqrt_(r2 > R(0) ? r2 : R(0));
    const V3<R> u = {F::mul(S, F::mul(r, cp)), F::mul(S, F::mul(r, sp)), F::mul(S, zz)};
    if (kind == CSMC_METROPOLIS) return u;
    const V3<R> v = vadd(s, V3<R>{F::mul(sigma, u.x), F::mul(sigma, u.y), F::mul(sigma, u.z)});
    const R inv = F::mul(S, Math<R>::rsqrt_(dot(v, v)));
    return {F::mul(v.x, inv), F::mul(v.y, inv), F::mul(v.z, inv)};
}

} // namespace csmc
