// exact.cu -- sequential FP64 replay of Metropolis proposals with the
// reference's arithmetic: energy(lattice, point) (hamiltonian.jl:139-196)
// evaluated term by term in the reference's order and association, over the
// reference-layout per-site tables, and calculate_energy_diff! /
// metropolis!'s accept rule (metropolis.jl:65-110), or the constrained rule
// of metropolis_constraint(_adaptive)! (:36-58, :155-179).  This translation unit is
// compiled with -fmad=false so that no a*b+c is contracted into an FMA, as
// Julia does not contract.  The cubic/quartic contractions follow Einsum.jl
// 0.4.1's loop expansion: a fresh accumulator, first summed index innermost.
#include "launch.hpp"

namespace csmc {

struct SpinView {
    const int64_t *ref2dev;
    int64_t Np;
    double *sp;
    __device__ __forceinline__ double get(int64_t i, int k) const { return sp[k * Np + ref2dev[i]]; }
    __device__ __forceinline__ void set(int64_t i, double a, double b, double c) const {
        const int64_t d = ref2dev[i];
        sp[d] = a;
        sp[Np + d] = b;
        sp[2 * Np + d] = c;
    }
};

__device__ double site_energy_ref(const ExactTables &t, const SpinView &v, int64_t i) {
    const double *o = t.onsite + i * 9;
    const double s[3] = {v.get(i, 0), v.get(i, 1), v.get(i, 2)};
    double E = 0.0;
    E += s[0] * (o[0] * s[0] + o[1] * s[1] + o[2] * s[2]) + s[1] * (o[3] * s[0] + o[4] * s[1] + o[5] * s[2]) +
         s[2] * (o[6] * s[0] + o[7] * s[1] + o[8] * s[2]);
    for (int n = 0; n < t.N2; n++) {
        const int64_t j = t.bs[i * t.N2 + n];
        if (j < 0) continue;
        const double *J = t.bm + (i * t.N2 + n) * 9;
        const double q[3] = {v.get(j, 0), v.get(j, 1), v.get(j, 2)};
        E += s[0] * (J[0] * q[0] + J[1] * q[1] + J[2] * q[2]) + s[1] * (J[3] * q[0] + J[4] * q[1] + J[5] * q[2]) +
             s[2] * (J[6] * q[0] + J[7] * q[1] + J[8] * q[2]);
    }
    for (int n = 0; n < t.N3; n++) {
        const int64_t *jk = t.cs + (i * t.N3 + n) * 2;
        if (jk[0] < 0) continue;
        const double *C = t.ct + (i * t.N3 + n) * 27;
        const double sj[3] = {v.get(jk[0], 0), v.get(jk[0], 1), v.get(jk[0], 2)};
        const double sk[3] = {v.get(jk[1], 0), v.get(jk[1], 1), v.get(jk[1], 2)};
        double acc = 0.0;
        for (int c = 0; c < 3; c++)
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) acc += C[(a * 3 + b) * 3 + c] * s[a] * sj[b] * sk[c];
        E += acc;
    }
    for (int n = 0; n < t.N4; n++) {
        const int64_t *jkl = t.qs + (i * t.N4 + n) * 3;
        if (jkl[0] < 0) continue;
        const double *Q = t.qt + (i * t.N4 + n) * 81;
        const double sj[3] = {v.get(jkl[0], 0), v.get(jkl[0], 1), v.get(jkl[0], 2)};
        const double sk[3] = {v.get(jkl[1], 0), v.get(jkl[1], 1), v.get(jkl[1], 2)};
        const double sl[3] = {v.get(jkl[2], 0), v.get(jkl[2], 1), v.get(jkl[2], 2)};
        double acc = 0.0;
        for (int e = 0; e < 3; e++)
            for (int c = 0; c < 3; c++)
                for (int b = 0; b < 3; b++)
                    for (int a = 0; a < 3; a++)
                        acc += Q[((a * 3 + b) * 3 + c) * 3 + e] * s[a] * sj[b] * sk[c] * sl[e];
        E += acc;
    }
    const double *h = t.field + i * 3;
    return E - (s[0] * h[0] + s[1] * h[1] + s[2] * h[2]);
}

// The constraint function evaluated on the whole lattice, as the reference
// calls mc.constraint(mc.lattice) (metropolis.jl:45,164): V summed over
// sites 1..N in order, then c = g.V + q |V|^2 + p |V| + c0.
__device__ double constraint_full(const ExactTables &t, const SpinView &v, const ExactCons &k) {
    double V0 = 0.0, V1 = 0.0, V2 = 0.0;
    for (int64_t i = 0; i < t.N; i++) {
        const double w = k.w ? k.w[i] : 1.0;
        V0 = V0 + w * v.get(i, 0);
        V1 = V1 + w * v.get(i, 1);
        V2 = V2 + w * v.get(i, 2);
    }
    const double vv = V0 * V0 + V1 * V1 + V2 * V2;
    return k.g[0] * V0 + k.g[1] * V1 + k.g[2] * V2 + k.q * vv + k.p * sqrt(vv) + k.c0;
}

__global__ void k_replay(ExactTables t, ExactCons k, double *spins, int kind, double T, double *sigma_dev, int64_t n,
                         const int64_t *sites, const double *u_phi, const double *u_z, const double *u_acc,
                         uint8_t *accepted) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const SpinView v{t.ref2dev, t.Np, spins};
    const double S = t.S;
    const double sigma = sigma_dev ? *sigma_dev : 60.0;
    const double two_pi = 6.283185307179586; // 2.0 * pi in Float64
    const bool constrained = kind >= CSMC_METROPOLIS_CONSTRAINT;
    const bool uniform = kind == CSMC_METROPOLIS || kind == CSMC_METROPOLIS_CONSTRAINT;
    double lambda = constrained && k.lambda ? *k.lambda : 0.0;
    double acc = 0.0;
    for (int64_t p = 0; p < n; p++) {
        const int64_t i = sites[p];
        const double old[3] = {v.get(i, 0), v.get(i, 1), v.get(i, 2)};
        // random_spin_orientation (lattice.jl:306-311)
        const double phi = two_pi * u_phi[p];
        const double z = 2.0 * u_z[p] - 1.0;
        const double r = sqrt(1.0 - z * z);
        double ns[3] = {S * (r * cos(phi)), S * (r * sin(phi)), S * z};
        if (!uniform) { // gaussian_move (metropolis.jl:84-87)
            const double a = old[0] + sigma * ns[0], b = old[1] + sigma * ns[1], c = old[2] + sigma * ns[2];
            const double nn = sqrt(a * a + b * b + c * c);
            ns[0] = a / nn * S;
            ns[1] = b / nn * S;
            ns[2] = c / nn * S;
        }
        const double E_old = site_energy_ref(t, v, i);
        v.set(i, ns[0], ns[1], ns[2]);
        const double E_new = site_energy_ref(t, v, i);
        const double dE = E_new - E_old;
        bool accept;
        if (!constrained) {
            accept = (dE < 0) ? true : (u_acc[p] < exp(-(dE) / T));
        } else { // metropolis.jl:45-48, 164-167
            const double c = constraint_full(t, v, k);
            const double new_lambda = lambda - k.weight * c;
            const double x = dE - (new_lambda * c);
            accept = x < 0 ? true : u_acc[p] < exp(-(x) / T);
            if (accept) lambda = new_lambda;
        }
        if (!accept) v.set(i, old[0], old[1], old[2]);
        else acc += 1;
        accepted[p] = accept ? 1 : 0;
    }
    if (constrained && k.lambda) *k.lambda = lambda;
    if (kind == CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE && sigma_dev) { // metropolis.jl:175-177
        const double a = acc / (double)n;
        const double f = 0.5 / (1 - a);
        *sigma_dev = a < 0.5 ? sigma * f : k.sigma0;
    }
    if (kind == CSMC_METROPOLIS_ADAPTIVE && sigma_dev) { // metropolis.jl:124-126
        const double a = acc / (double)n;
        const double om = 1 - a;
        const double f = 0.5 / (om > 0.05 ? om : 0.05);
        double s = sigma * f;
        *sigma_dev = s < 0.0 ? 0.0 : (s > 100 ? 100 : s);
    }
}

void launch_replay(const ExactTables &t, const ExactCons &k, double *spins, int kind, double T, double *sigma_dev,
                   int64_t n, const int64_t *sites, const double *u_phi, const double *u_z, const double *u_acc,
                   uint8_t *accepted, cudaStream_t st) {
    k_replay<<<1, 32, 0, st>>>(t, k, spins, kind, T, sigma_dev, n, sites, u_phi, u_z, u_acc, accepted);
}

} // namespace csmc
