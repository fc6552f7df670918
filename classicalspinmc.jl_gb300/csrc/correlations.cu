// correlations.cu -- equal-time spin correlations in momentum space,
// compute_equal_time_correlations (spin_correlations.jl:6-43), for every
// replica of a lattice at once:
//
//   S_a(k) = sum_i exp(-i k.r_i) s_i,a,   Suv[3a+b](k) = Re(S_a(k) conj(S_b(k))) / N.
//
// A contraction of the phase matrix [n_k x N] with the spins [N x 3R]; the
// phases are generated on the fly, never stored.  One CTA computes a tile of
// KT wavevectors x RG replicas: per chunk of CH sites it stages the phases
// (KT x CH sincos) and the replicas' spins in shared memory, then every
// thread accumulates KK wavevectors x 3 components of one replica over the
// chunk (register tile: 1 + 2 KK shared loads for 6 KK fused multiply-adds
// per site).  Summation is sequential over sites in device order per thread.
#include "launch.hpp"

namespace csmc {

namespace {
constexpr int SF_THREADS = 256;
constexpr int SF_RG = 16;                               // replicas per CTA
constexpr int SF_KK = 4;                                // wavevectors per thread
constexpr int SF_KT = SF_KK * (SF_THREADS / SF_RG);     // 64 wavevectors per CTA
// sites per chunk: 24 KB of shared memory per CTA in either precision
template <typename R> constexpr int sf_chunk() { return sizeof(R) == 4 ? 32 : 16; }

template <typename R> struct Vec4;
template <> struct Vec4<float> {
    using T = float4;
};
template <> struct Vec4<double> {
    using T = double4;
};

// Single precision: t reduced to [-pi, pi] by Cody-Waite reduction with 2 pi
// split in two floats (W. J. Cody and W. Waite, Software Manual for the
// Elementary Functions, 1980), then the hardware sine and cosine (absolute
// error about 2^-21 on that interval).  t itself carries the rounding of the
// single-precision dot product k.r, about 2^-24 |t|.
__device__ __forceinline__ void sincos_(float t, float *s, float *c) {
    const float n = rintf(t * 0.159154943091895336f);    // t / (2 pi), nearest integer
    float r = __fmaf_rn(-n, 6.28318548202514648f, t);      // 2 pi rounded to float
    r = __fmaf_rn(-n, -1.74845553146951305e-7f, r);        // 2 pi - that float
    __sincosf(r, s, c);
}
__device__ __forceinline__ void sincos_(double t, double *s, double *c) { sincos(t, s, c); }
} // namespace

// pos: device order, 3 per site (padding sites: any position, zero spin);
// ks: 3 per wavevector (unused dimensions zero); out[r][n][9] per replica r
// of the lattice (chain index), written in the slot order of `slot_of`.
template <typename R>
__global__ void __launch_bounds__(SF_THREADS)
    k_structure_factor(const R *__restrict__ spins, int64_t Np, int n_rep, const R *__restrict__ pos,
                       const R *__restrict__ ks, int64_t n_k, int64_t n_real, const int32_t *slot_of,
                       int chain_base, int slot_base, double *__restrict__ out) {
    using V4 = typename Vec4<R>::T;
    constexpr int SF_CH = sf_chunk<R>();
    // phases stored [site][wavevector]: a thread's SF_KK wavevectors of one
    // site are one vector load
    __shared__ __align__(16) R s_cos[SF_CH][SF_KT];
    __shared__ __align__(16) R s_sin[SF_CH][SF_KT];
    __shared__ V4 s_spin[SF_CH][SF_RG];
    const int rl = threadIdx.x % SF_RG, kg = threadIdx.x / SF_RG;
    const int64_t k0 = (int64_t)blockIdx.x * SF_KT;
    const int r0 = blockIdx.y * SF_RG;
    R re[SF_KK][3], im[SF_KK][3];
#pragma unroll
    for (int q = 0; q < SF_KK; q++)
#pragma unroll
        for (int a = 0; a < 3; a++) re[q][a] = im[q][a] = R(0);

    for (int64_t c0 = 0; c0 < Np; c0 += SF_CH) {
        __syncthreads(); // the previous chunk is consumed
        for (int e = threadIdx.x; e < SF_KT * SF_CH; e += SF_THREADS) {
            const int ii = e / SF_KT, kk = e - ii * SF_KT;
            const int64_t k = k0 + kk, i = c0 + ii;
            R c = R(0), s = R(0);
            if (k < n_k && i < Np) {
                // t = k.r summed over the dimensions in order; exp(-i t) = cos t - i sin t
                const R t = Fp<R>::fma(ks[3 * k + 2], pos[3 * i + 2],
                                       Fp<R>::fma(ks[3 * k + 1], pos[3 * i + 1], Fp<R>::mul(ks[3 * k], pos[3 * i])));
                sincos_(t, &s, &c);
            }
            s_cos[ii][kk] = c;
            s_sin[ii][kk] = -s;
        }
        for (int e = threadIdx.x; e < SF_CH * SF_RG; e += SF_THREADS) {
            const int ii = e / SF_RG, rr = e - ii * SF_RG;
            const int64_t i = c0 + ii;
            const int r = r0 + rr;
            V4 v;
            v.x = v.y = v.z = v.w = R(0);
            if (i < Np && r < n_rep) {
                const V3<R> sp = spins_of(const_cast<R *>(spins), Np, r).get(i);
                v.x = sp.x;
                v.y = sp.y;
                v.z = sp.z;
            }
            s_spin[ii][rr] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int ii = 0; ii < SF_CH; ii++) {
            const V4 v = s_spin[ii][rl];
            R cq[SF_KK], sq[SF_KK];
            if constexpr (sizeof(R) == 4 && SF_KK % 4 == 0) {
#pragma unroll
                for (int q = 0; q < SF_KK; q += 4) {
                    const float4 c4 = *reinterpret_cast<const float4 *>(&s_cos[ii][kg * SF_KK + q]);
                    const float4 s4 = *reinterpret_cast<const float4 *>(&s_sin[ii][kg * SF_KK + q]);
                    cq[q] = c4.x, cq[q + 1] = c4.y, cq[q + 2] = c4.z, cq[q + 3] = c4.w;
                    sq[q] = s4.x, sq[q + 1] = s4.y, sq[q + 2] = s4.z, sq[q + 3] = s4.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < SF_KK; q++) cq[q] = s_cos[ii][kg * SF_KK + q], sq[q] = s_sin[ii][kg * SF_KK + q];
            }
#pragma unroll
            for (int q = 0; q < SF_KK; q++) {
                const R c = cq[q], s = sq[q];
                re[q][0] = Fp<R>::fma(c, v.x, re[q][0]);
                re[q][1] = Fp<R>::fma(c, v.y, re[q][1]);
                re[q][2] = Fp<R>::fma(c, v.z, re[q][2]);
                im[q][0] = Fp<R>::fma(s, v.x, im[q][0]);
                im[q][1] = Fp<R>::fma(s, v.y, im[q][1]);
                im[q][2] = Fp<R>::fma(s, v.z, im[q][2]);
            }
        }
    }
    const int r = r0 + rl;
    if (r >= n_rep) return;
    const int slot = slot_of[chain_base + r] - slot_base;
    const double inv_n = 1.0 / (double)n_real;
#pragma unroll
    for (int q = 0; q < SF_KK; q++) {
        const int64_t k = k0 + kg * SF_KK + q;
        if (k >= n_k) continue;
        double *o = out + ((int64_t)slot * n_k + k) * 9;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) // Re((re_a + i im_a)(re_b - i im_b))
                o[3 * a + b] = ((double)re[q][a] * (double)re[q][b] + (double)im[q][a] * (double)im[q][b]) * inv_n;
    }
}

template <typename R>
void launch_structure_factor(const SysArgs<R> &a, const R *pos, const R *ks, int64_t n_k, const int32_t *slot_of,
                             int slot_base, double *out, cudaStream_t st) {
    if (n_k <= 0) return;
    const dim3 grid((unsigned)((n_k + SF_KT - 1) / SF_KT), (unsigned)((a.n_rep + SF_RG - 1) / SF_RG));
    k_structure_factor<R><<<grid, SF_THREADS, 0, st>>>(a.spins, a.tb.Np, a.n_rep, pos, ks, n_k, a.n_real,
                                                       slot_of, a.chain_base, slot_base, out);
}

template void launch_structure_factor<float>(const SysArgs<float> &, const float *, const float *, int64_t,
                                             const int32_t *, int, double *, cudaStream_t);
template void launch_structure_factor<double>(const SysArgs<double> &, const double *, const double *, int64_t,
                                              const int32_t *, int, double *, cudaStream_t);

} // namespace csmc
