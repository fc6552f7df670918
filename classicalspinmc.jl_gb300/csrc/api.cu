// api.cu -- the C ABI of libcsmc.so (include/csmc.h): contexts, host<->device
// layout conversion, and the multi-sweep drivers that schedule the kernels of
// kernels.cu in the cadence of simulated_annealing! / parallel_tempering!
// (monte_carlo.jl:157-190, :288-388).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "launch.hpp"
#include "plan.hpp"

namespace csmc {

static thread_local std::string g_err;

// A failed runtime call throws; the runtime's last-error slot is read (and so
// cleared) first, so that a recoverable failure such as an allocation that
// does not fit is not reported again by a later, unrelated check.
#define CK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) {                                                                                       \
            (void)cudaGetLastError();                                                                                  \
            throw Error(e_ == cudaErrorMemoryAllocation ? CSMC_ERR_OOM : CSMC_ERR_CUDA,                                \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                                           \
        }                                                                                                              \
    } while (0)

static void require(bool ok, int code, const std::string &msg) {
    if (!ok) throw Error(code, msg);
}

// Device allocations made by the library since the process started
// (csmc_debug_device_allocs).
static std::atomic<int64_t> g_device_allocs{0};

template <typename T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    void alloc(size_t count) {
        if (p) cudaFree(p);
        p = nullptr;
        n = count;
        if (count) {
            g_device_allocs++;
            CK(cudaMalloc(&p, count * sizeof(T)));
        }
    }
    void upload(const T *src, size_t count) {
        alloc(count);
        if (count) CK(cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice));
    }
    template <class V> void upload(const V &v) { upload(v.data(), v.size()); }
    // at least `count` elements, reallocating only to grow (contents not kept)
    void reserve(size_t count) {
        if (count > n) alloc(count);
    }
    void zero(cudaStream_t st) {
        if (n) CK(cudaMemsetAsync(p, 0, n * sizeof(T), st));
    }
};

struct System {
    Plan plan;
    int R = 0, base = 0; // replicas, first chain/slot
    bool cub = false, qua = false;
    DevBuf<uint32_t> p2, p3, p4;
    DevBuf<uint16_t> q2, q3, q4;
    DevBuf<uint8_t> pat;
    DevBuf<int32_t> dev2ref, c2, c3, c4;
    DevBuf<int64_t> ref2dev;
    DevBuf<float> fmats, fcubs, fquas, fO, fP, fh, fspins, fA, fQ, fE2, fJs, fmiso, fciso, fqiso;
    DevBuf<double> dmats, dcubs, dquas, dO, dP, dh, dspins, dA, dQ, dE2, dJs, dmiso, dciso, dqiso;
    SysArgs<float> fa{};
    SysArgs<double> da{};
    bool resident_ok = false;
    // specialised resident kernel: eligible, bilinear and onsite classes, and
    // the single basis of each colour class
    bool fast_ok = false;
    int bil_class = 1, ons_class = 2;
    bool pv_stage = false; // partner words staged in shared memory beside the spins
    std::vector<int32_t> col_pattern;
    // split over a thread-block cluster (context-wide cluster size > 1)
    ClusterLayout cl_layout;
    // bilinear partners packed 8 x 16 bit per site (specialised kernel)
    DevBuf<uint4> p2v, q2v;
    // per-rank partner tables and local patterns (generic kernel on a cluster)
    DevBuf<uint16_t> q2c, q3c, q4c;
    DevBuf<uint8_t> patc;
    size_t resident_smem = 0;
    // reference-layout tables for the replay kernel (built on first use)
    DevBuf<int64_t> xbs, xcs, xqs;
    DevBuf<double> xbm, xct, xqt, xfield, xonsite;
    bool exact_ready = false;
    // constraint of the constrained Metropolis kinds (csmc_set_constraint):
    // weights by device position (cw) and by reference site (cw_ref), both
    // empty for unit weights
    ConsArgs cons{};
    DevBuf<double> cw, cw_ref;
};

// Lattices that share one resident launch: its CTAs per replica (cluster
// size), threads per CTA, shared-memory size and work list.  A context is one
// group, or -- size groups, for batches of lattices of very different sizes --
// one group per band of replica sizes, whose launches run side by side on
// streams of their own (small replicas in small CTAs, several per SM; the
// largest split over clusters).
struct Group {
    std::vector<int> sys; // lattices (indices into Ctx::sys)
    int cl = 1;           // CTAs per replica
    int n_items = 0;      // replicas of the group
    DevBuf<int2> items;   // {lattice, replica}, largest replicas first
    DevBuf<int> work_ctr;
    cudaStream_t st = nullptr; // own stream (size groups only)
    cudaEvent_t done = nullptr;
    Group() = default;
    Group(const Group &) = delete;
    Group &operator=(const Group &) = delete;
    ~Group() {
        if (done) cudaEventDestroy(done);
        if (st) cudaStreamDestroy(st);
    }
};

struct Ctx {
    int precision = CSMC_FP64;
    uint64_t seed = 0;
    uint32_t k0 = 0, k1 = 0;
    int device = 0, n_sms = 0, max_smem = 0;
    std::vector<std::unique_ptr<System>> sys;
    int n_chains = 0;
    cudaStream_t st = nullptr;
    DevBuf<int32_t> slot_of, chain_of;
    DevBuf<double> T_slot, sigma_slot, acc_slot, exch_slot, E_chain, M_chain, last_acc;
    DevBuf<double> E_win; // persistent windows: energies by slot, two alternating buffers
    DevBuf<double> T_stash; // mc.T of every slot during a csmc_metropolis_sweep_at call
    DevBuf<float> invT_slot, invT_stash; // (float)(1 / T) per slot (single-precision sweeps)
    DevBuf<double> invT64_slot;          // 1 / T per slot (the persistent exchange's exponent)
    DevBuf<uint32_t> chain_id;           // per chain: the key of its Philox streams
    DevBuf<unsigned long long> sweep_acc;
    DevBuf<unsigned int> drift_bits;
    DevBuf<int> error_flag;
    DevBuf<unsigned int> grid_bar; // arrival counter of the persistent kernel's grid barrier
    bool persistent_ok = true;     // cleared if a cooperative launch is refused
    bool persistent_on = true;     // csmc_set_persistent
    DevBuf<double> part, stage, rec_E, rec_M;
    DevBuf<ResSys<float>> fres;
    DevBuf<ResSys<double>> dres;
    DevBuf<int2> lattices; // per lattice {first slot, replicas} (exchange kernel)
    int n_items = 0;       // replicas of every lattice
    std::vector<std::unique_ptr<Group>> groups; // one, or the size groups
    bool size_groups = false;                   // csmc_set_size_groups / the autotuner's choice
    bool sf_tensor = true; // single-precision structure factors on the tensor cores (csmc_set_tensor_cores)
    DevBuf<float> sf_packed, sf_partial; // their scratch (split spins, partial sums), kept and grown
    int group_block_cap = 0; // size groups: at most this many threads per CTA (0: none), so CTAs of
                             // several groups share an SM (the autotuner's choice)
    cudaEvent_t fork = nullptr;                 // size groups start after the work queued before them
    int cl = 1;         // CTAs per replica of the resident kernel (one group; 0 with size groups)
    int block_pref = 0; // threads per CTA chosen by csmc_autotune (0: automatic)
    bool global_pref = false; // csmc_autotune found the global path faster for CSMC_PATH_AUTO runs
    DevBuf<double> lambda_slot; // mc.lambda per slot (constrained kinds)
    double sigma0 = 60.0;       // mc.sigma0 (constrained adaptive kind)
    uint32_t msweep = 0;   // Metropolis sweeps so far (the Philox counter)
    uint64_t nsweeps = 0;  // sweeps of every kind so far (renormalisation cadence)
    int renorm_every = 64;
    double last_ms = 0.0;
    int64_t last_launches = 0;
    // CUDA events bracketing each resident-kernel launch of the current run
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> kev;
    size_t kev_used = 0;
    double last_kernel_ms = 0.0;
    int64_t last_kernel_launches = 0;
    ChainState cs{};
    // pinned host staging for the results of a run (error flag, probe
    // records, counters): copied back together, read after one synchronisation
    int *h_flag = nullptr;
    double *h_box = nullptr;
    size_t h_box_n = 0;
    cudaEvent_t run_e0 = nullptr, run_e1 = nullptr;

    ~Ctx() {
        for (auto &e : kev) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
        groups.clear(); // their streams before the context's
        if (fork) cudaEventDestroy(fork);
        if (run_e0) cudaEventDestroy(run_e0);
        if (run_e1) cudaEventDestroy(run_e1);
        if (h_flag) cudaFreeHost(h_flag);
        if (h_box) cudaFreeHost(h_box);
        if (st) cudaStreamDestroy(st);
    }
    double *host_box(size_t n) {
        if (n > h_box_n) {
            if (h_box) cudaFreeHost(h_box);
            h_box = nullptr;
            h_box_n = 0;
            CK(cudaHostAlloc((void **)&h_box, n * sizeof(double), cudaHostAllocDefault));
            h_box_n = n;
        }
        return h_box;
    }
    std::pair<cudaEvent_t, cudaEvent_t> next_kernel_events() {
        if (kev_used == kev.size()) {
            std::pair<cudaEvent_t, cudaEvent_t> e;
            CK(cudaEventCreate(&e.first));
            CK(cudaEventCreate(&e.second));
            kev.push_back(e);
        }
        return kev[kev_used++];
    }
    void reset_kernel_time() {
        kev_used = 0;
        last_kernel_ms = 0.0;
        last_kernel_launches = 0;
    }
    // after the stream has been synchronised: add the time of the bracketed launches
    void collect_kernel_time() {
        for (size_t k = 0; k < kev_used; k++) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, kev[k].first, kev[k].second));
            last_kernel_ms += ms;
        }
        last_kernel_launches += (int64_t)kev_used;
        kev_used = 0;
    }
    int sys_of_slot(int slot) const {
        for (size_t k = 0; k < sys.size(); k++)
            if (slot >= sys[k]->base && slot < sys[k]->base + sys[k]->R) return (int)k;
        throw Error(CSMC_ERR_INVALID, "slot " + std::to_string(slot) + " out of range");
    }
};

template <typename V> static std::vector<float> to_f(const V &v) { return std::vector<float>(v.begin(), v.end()); }

// Pack a slot-major partner table [W][n] (16-bit values) into one 16-byte
// word per site, slots >= W filled with pad(i).
template <typename T, class Pad>
static std::vector<uint4> pack8(const std::vector<T> &tab, int W, int64_t n, Pad pad) {
    std::vector<uint4> out((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        uint32_t v[8];
        for (int t = 0; t < 8; t++) v[t] = (t < W ? (uint32_t)tab[(size_t)t * n + i] : pad(i)) & 0xFFFFu;
        out[i] = make_uint4(v[0] | v[1] << 16, v[2] | v[3] << 16, v[4] | v[5] << 16, v[6] | v[7] << 16);
    }
    return out;
}

static void upload_system(Ctx &C, System &S) {
    const Plan &P = S.plan;
    const int nb = P.desc.nb;
    S.p2.upload(P.p2);
    S.p3.upload(P.p3);
    S.p4.upload(P.p4);
    S.pat.upload(P.pat);
    std::vector<int32_t> d2r(P.dev2ref.begin(), P.dev2ref.end());
    S.dev2ref.upload(d2r);
    S.ref2dev.upload(P.ref2dev);
    S.c2.upload(P.c2);
    S.c3.upload(P.c3);
    S.c4.upload(P.c4);
    // per-pattern onsite, folded self loops and field; pattern nb is padding
    std::vector<double> O((nb + 1) * 9, 0.0), Pm((nb + 1) * 9, 0.0), h((nb + 1) * 3, 0.0);
    for (int b = 0; b < nb; b++) {
        for (int k = 0; k < 9; k++) {
            O[b * 9 + k] = P.onsite_b[b][k];
            Pm[b * 9 + k] = P.self_b[b][k];
        }
        for (int k = 0; k < 3; k++) h[b * 3 + k] = P.field_b[b][k];
    }
    S.cub = P.W3 > 0;
    S.qua = P.W4 > 0;
    int ons_diag = 1;
    for (int b = 0; b < nb; b++)
        for (int k = 0; k < 9; k++)
            if (k % 4 != 0 && (O[b * 9 + k] != 0.0 || Pm[b * 9 + k] != 0.0)) ons_diag = 0;
    // per pattern: 2O+P (local field), O+P (dE), O+P/2 (energy share)
    std::vector<double> A((nb + 1) * 9, 0.0), Qm((nb + 1) * 9, 0.0), E2((nb + 1) * 9, 0.0);
    for (int k = 0; k < (nb + 1) * 9; k++) {
        A[k] = 2 * O[k] + Pm[k];
        Qm[k] = O[k] + Pm[k];
        E2[k] = O[k] + 0.5 * Pm[k];
    }
    S.ons_class = 0;
    for (int b = 0; b <= nb; b++)
        for (int k = 0; k < 9; k++) {
            const bool diag = k == 0 || k == 4 || k == 8;
            if (A[b * 9 + k] != 0.0 || Qm[b * 9 + k] != 0.0) S.ons_class = std::max(S.ons_class, diag ? 1 : 2);
        }
    // scalar couplings: every bilinear slot matrix is c * I
    const int W2 = std::max(P.W2, 1);
    std::vector<double> Js((size_t)(nb + 1) * W2, 0.0);
    S.bil_class = 0;
    for (int b = 0; b < nb; b++)
        for (int t = 0; t < P.W2; t++) {
            const double *M = &P.mats[9 * (size_t)P.c2[(size_t)b * P.W2 + t]];
            const bool scalar = M[1] == 0 && M[2] == 0 && M[3] == 0 && M[5] == 0 && M[6] == 0 && M[7] == 0 &&
                                M[0] == M[4] && M[4] == M[8];
            if (!scalar) S.bil_class = 1;
            Js[(size_t)b * W2 + t] = M[0];
        }
    S.col_pattern.assign(P.n_colours, -1);
    bool uniform = true;
    for (int col = 0; col < P.n_colours; col++) {
        int pb = -1;
        for (int64_t d = P.col_start[col]; d < P.col_start[col] + P.col_count[col]; d++) {
            if (pb < 0) pb = P.pat[d];
            if (P.pat[d] != pb) uniform = false;
        }
        S.col_pattern[col] = pb < 0 ? nb : pb;
    }
    S.fast_ok = uniform && !S.cub && !S.qua && P.W2 <= RESIDENT_WMAX;
    if (S.fast_ok && P.Np <= 65536) S.p2v.upload(pack8(P.p2, P.W2, P.Np, [&](int64_t) { return (uint32_t)P.sentinel; }));
    const int64_t Np = P.Np;
    if (P.Np <= 65536) {
        std::vector<uint16_t> a(P.p2.begin(), P.p2.end()), b(P.p3.begin(), P.p3.end()), c(P.p4.begin(), P.p4.end());
        S.q2.upload(a);
        S.q3.upload(b);
        S.q4.upload(c);
    }
    auto fill_args = [&](auto &a, auto *spins, auto *mats, auto *cubs, auto *quas, auto *Oo, auto *Pp, auto *hh) {
        a.tb.p2 = S.p2.p;
        a.tb.p3 = S.p3.p;
        a.tb.p4 = S.p4.p;
        a.tb.pat = S.pat.p;
        a.tb.Np = Np;
        a.tb.W2 = P.W2;
        a.tb.W3 = P.W3;
        a.tb.W4 = P.W4;
        a.cf.mats = mats;
        a.cf.cubs = cubs;
        a.cf.quas = quas;
        a.cf.O = Oo;
        a.cf.P = Pp;
        a.cf.h = hh;
        a.cf.c2 = S.c2.p;
        a.cf.c3 = S.c3.p;
        a.cf.c4 = S.c4.p;
        a.spins = spins;
        a.dev2ref = S.dev2ref.p;
        a.ref2dev = S.ref2dev.p;
        a.chain_base = S.base;
        a.n_rep = S.R;
        a.n_real = P.N;
        a.k0 = C.k0;
        a.k1 = C.k1;
        a.cub = S.cub;
        a.qua = S.qua;
    };
    if (C.precision == CSMC_FP32) {
        const size_t nsp = (size_t)S.R * 4 * Np; // one float4 per site
        S.fmats.upload(to_f(P.mats));
        S.fcubs.upload(to_f(P.cubs));
        S.fquas.upload(to_f(P.quas));
        S.fmiso.upload(to_f(P.mat_iso));
        S.fciso.upload(to_f(P.cub_iso));
        S.fqiso.upload(to_f(P.qua_iso));
        S.fO.upload(to_f(O));
        S.fP.upload(to_f(Pm));
        S.fh.upload(to_f(h));
        S.fspins.alloc(nsp);
        CK(cudaMemset(S.fspins.p, 0, nsp * sizeof(float)));
        fill_args(S.fa, S.fspins.p, S.fmats.p, S.fcubs.p, S.fquas.p, S.fO.p, S.fP.p, S.fh.p);
        S.fa.cf.miso = S.fmiso.p;
        S.fa.cf.ciso = S.fciso.p;
        S.fa.cf.qiso = S.fqiso.p;
        S.fA.upload(to_f(A));
        S.fQ.upload(to_f(Qm));
        S.fE2.upload(to_f(E2));
        S.fJs.upload(to_f(Js));
        S.fa.cf.A = S.fA.p;
        S.fa.cf.Q = S.fQ.p;
        S.fa.cf.E2 = S.fE2.p;
        S.fa.cf.Js = S.fJs.p;
        S.fa.cf.iso2 = S.bil_class == 0 ? 1 : 0;
        S.fa.cf.ons_diag = ons_diag;
        S.fa.S = (float)P.desc.S;
    } else {
        const size_t nsp = (size_t)S.R * 3 * Np; // x | y | z blocks
        S.dmats.upload(P.mats);
        S.dcubs.upload(P.cubs);
        S.dquas.upload(P.quas);
        S.dmiso.upload(P.mat_iso);
        S.dciso.upload(P.cub_iso);
        S.dqiso.upload(P.qua_iso);
        S.dO.upload(O);
        S.dP.upload(Pm);
        S.dh.upload(h);
        S.dspins.alloc(nsp);
        CK(cudaMemset(S.dspins.p, 0, nsp * sizeof(double)));
        fill_args(S.da, S.dspins.p, S.dmats.p, S.dcubs.p, S.dquas.p, S.dO.p, S.dP.p, S.dh.p);
        S.da.cf.miso = S.dmiso.p;
        S.da.cf.ciso = S.dciso.p;
        S.da.cf.qiso = S.dqiso.p;
        S.dA.upload(A);
        S.dQ.upload(Qm);
        S.dE2.upload(E2);
        S.dJs.upload(Js);
        S.da.cf.A = S.dA.p;
        S.da.cf.Q = S.dQ.p;
        S.da.cf.E2 = S.dE2.p;
        S.da.cf.Js = S.dJs.p;
        S.da.cf.iso2 = S.bil_class == 0 ? 1 : 0;
        S.da.cf.ons_diag = ons_diag;
        S.da.S = P.desc.S;
    }
}

template <typename R> static ResSys<R> make_res(const System &S, const SysArgs<R> &a) {
    ResSys<R> r{};
    r.tb.p2 = S.q2.p;
    r.tb.p3 = S.q3.p;
    r.tb.p4 = S.q4.p;
    r.tb.pat = S.pat.p;
    r.tb.Np = a.tb.Np;
    r.tb.W2 = a.tb.W2;
    r.tb.W3 = a.tb.W3;
    r.tb.W4 = a.tb.W4;
    r.cf = a.cf;
    r.spins = a.spins;
    r.chain_base = a.chain_base;
    r.n_rep = a.n_rep;
    r.n_colours = S.plan.n_colours;
    r.nb = S.plan.desc.nb;
    for (int c = 0; c <= S.plan.n_colours; c++) r.col_start[c] = S.plan.col_start[c];
    for (int c = 0; c < S.plan.n_colours; c++) r.col_count[c] = S.plan.col_count[c];
    for (int c = 0; c < S.plan.n_colours; c++) r.col_pattern[c] = S.col_pattern[c];
    r.n_real = S.plan.N;
    r.S = a.S;
    r.k0 = a.k0;
    r.k1 = a.k1;
    const ClusterLayout &L = S.cl_layout;
    r.cl = L.ranks;
    r.Npl = (int32_t)L.Npl;
    r.p2v = S.p2v.p;
    r.q2v = S.q2v.p;
    r.pv_stage = S.pv_stage ? 1 : 0;
    r.q2c = S.q2c.p;
    r.q3c = S.q3c.p;
    r.q4c = S.q4c.p;
    r.patc = S.patc.p;
    if (L.ranks > 1)
        for (int k = 0; k < L.ranks; k++)
            for (int c = 0; c < S.plan.n_colours; c++) {
                r.loc_start[k][c] = (int32_t)L.loc_start[k * S.plan.n_colours + c];
                r.loc_count[k][c] = (int32_t)L.loc_count[k * S.plan.n_colours + c];
                r.src_start[k][c] = (int32_t)L.src_start[k * S.plan.n_colours + c];
            }
    return r;
}

// Bytes of shared memory for the spins of n sites (float4 or three doubles per site).
static int64_t spin_bytes(const Ctx &C, int64_t n) { return C.precision == CSMC_FP32 ? 16 * n : 24 * n; }
// Dynamic shared memory a resident CTA may use: the opt-in maximum less a
// reserve for the kernel's static shared memory (at most about 6 KB).
static int64_t dynamic_smem_limit(const Ctx &C) { return (int64_t)C.max_smem - 8 * 1024; }

// Does a cluster size of c CTAs per replica fit the lattices `idx` (n_items
// replicas)?  Parts of at most 16383 sites (14-bit owner-local indices) that
// fit shared memory; `prefer`: also at least 1024 sites per rank and all
// clusters of the group on the device at once.
static bool cluster_fits(const Ctx &C, const std::vector<int> &idx, int n_items, int c, bool prefer) {
    const int64_t limit = dynamic_smem_limit(C);
    if (c == 1) {
        for (int k : idx)
            if (C.sys[k]->plan.Np > 65536 || spin_bytes(C, C.sys[k]->plan.Np) > limit) return false;
        return true;
    }
    for (int k : idx) {
        const Plan &P = C.sys[k]->plan;
        const int64_t per_rank = (P.Np + c - 1) / c + 32 * (P.n_colours + 1);
        if (per_rank > 16384 || spin_bytes(C, per_rank) > limit) return false;
        if (prefer && P.N / c < 1024) return false;
    }
    return !prefer || (int64_t)n_items * c <= C.n_sms;
}

// Cluster size of a group: the largest of 2 and 4 whose clusters all fit on
// the device at once with at least 1024 sites per rank, else 1; a larger size
// when a replica fits shared memory only split.  `requested` = 0 picks
// automatically; 1, 2 or 4 forces that size (if the parts fit shared memory).
static int pick_cluster(const Ctx &C, const std::vector<int> &idx, int n_items, int requested) {
    if (requested > 0) {
        require(requested == 1 || requested == 2 || requested == 4, CSMC_ERR_INVALID, "cluster size must be 1, 2 or 4");
        require(requested == 1 || cluster_fits(C, idx, n_items, requested, false), CSMC_ERR_UNSUPPORTED,
                "this cluster size needs parts of at most 16383 sites that fit shared memory");
        return requested;
    }
    int pick = 0;
    for (int c : {1, 2, 4})
        if (cluster_fits(C, idx, n_items, c, true)) pick = c;
    if (!pick) // no preferred size: the smallest one that fits
        for (int c : {1, 2, 4})
            if (cluster_fits(C, idx, n_items, c, false)) {
                pick = c;
                break;
            }
    return pick ? pick : 1;
}

// Lay a lattice out for clusters of `cl` CTAs per replica (cl = 1: one CTA).
static void layout_for_cluster(Ctx &C, System &S, int cl) {
    const int64_t limit = dynamic_smem_limit(C);
    if (cl > 1) {
        S.cl_layout = make_cluster_layout(S.plan, cl);
        S.q2c.upload(S.cl_layout.q2);
        S.q3c.upload(S.cl_layout.q3);
        S.q4c.upload(S.cl_layout.q4);
        S.patc.upload(S.cl_layout.pat);
        if (S.fast_ok) {
            const ClusterLayout &L = S.cl_layout;
            const int W = std::max(S.plan.W2, 1);
            std::vector<uint4> all;
            for (int k = 0; k < L.ranks; k++) {
                std::vector<uint16_t> part(L.q2.begin() + (size_t)k * W * L.Npl,
                                           L.q2.begin() + (size_t)(k + 1) * W * L.Npl);
                const uint32_t sent = (uint32_t)(L.Npl - 32);
                std::vector<uint4> pk = pack8(part, S.plan.W2, L.Npl, [&](int64_t) { return sent; });
                all.insert(all.end(), pk.begin(), pk.end());
            }
            S.q2v.upload(all);
        }
        S.resident_smem = (size_t)spin_bytes(C, S.cl_layout.Npl);
        S.resident_ok = (int64_t)S.resident_smem <= limit && S.plan.n_colours <= CSMC_MAX_COLOURS;
    } else {
        S.cl_layout = ClusterLayout();
        S.resident_smem = (size_t)spin_bytes(C, S.plan.Np);
        S.resident_ok =
            S.plan.Np <= 65536 && (int64_t)S.resident_smem <= limit && S.plan.n_colours <= CSMC_MAX_COLOURS;
    }
}

static int group_items(const Ctx &C, const std::vector<int> &idx) {
    int n = 0;
    for (int k : idx) n += C.sys[k]->R;
    return n;
}

// One group of every lattice with the cluster size `requested` (0: automatic).
static void choose_cluster(Ctx &C, int requested) {
    std::vector<int> all(C.sys.size());
    std::iota(all.begin(), all.end(), 0);
    const int cl = pick_cluster(C, all, C.n_items, requested);
    for (auto &S : C.sys) layout_for_cluster(C, *S, cl);
    C.groups.clear();
    C.groups.push_back(std::make_unique<Group>());
    C.groups[0]->sys = all;
    C.groups[0]->cl = cl;
    C.groups[0]->n_items = C.n_items;
    C.cl = cl;
    C.size_groups = false;
}

// Size groups: lattices sorted by size, a new group wherever the padded size
// drops below half of the group's largest; each group picks its own cluster
// size (or, clusters = false, one CTA per replica).  Fewer than two groups:
// one group (choose_cluster).  Returns whether size groups are in use.
static bool make_size_groups(Ctx &C, bool clusters = true) {
    std::vector<int> order(C.sys.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return C.sys[a]->plan.Np > C.sys[b]->plan.Np; });
    std::vector<std::vector<int>> bands;
    for (int k : order) {
        if (bands.empty() || 2 * C.sys[k]->plan.Np < C.sys[bands.back()[0]]->plan.Np) bands.emplace_back();
        bands.back().push_back(k);
    }
    if (bands.size() < 2) {
        choose_cluster(C, 0);
        return false;
    }
    C.groups.clear();
    for (auto &band : bands) {
        auto G = std::make_unique<Group>();
        G->sys = band;
        G->n_items = group_items(C, band);
        G->cl = clusters ? pick_cluster(C, band, G->n_items, 0) : 1;
        for (int k : band) layout_for_cluster(C, *C.sys[k], G->cl);
        CK(cudaStreamCreateWithFlags(&G->st, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&G->done, cudaEventDisableTiming));
        G->work_ctr.alloc(1);
        C.groups.push_back(std::move(G));
    }
    if (!C.fork) CK(cudaEventCreateWithFlags(&C.fork, cudaEventDisableTiming));
    C.cl = 0;
    C.size_groups = true;
    return true;
}

static ResidentSel resident_selection(const Ctx &C, const Group &G);

// Resident descriptors of every lattice and the work list of each group
// (largest replicas first).  The specialised kernel also stages each CTA's
// packed partner words in shared memory when they fit beside the spins of
// every lattice of the group.
static void upload_resident(Ctx &C) {
    for (auto &Gp : C.groups) {
        Group &G = *Gp;
        const ResidentSel sel = resident_selection(C, G);
        const int stat = !sel.fast ? -1
                         : C.precision == CSMC_FP32 ? resident_static_smem<float>(sel)
                                                    : resident_static_smem<double>(sel);
        bool stage = sel.fast && stat >= 0;
        for (int k : G.sys) {
            const System &S = *C.sys[k];
            const int64_t nl = G.cl > 1 ? S.cl_layout.Npl : S.plan.Np;
            const int64_t spins = (spin_bytes(C, nl) + 15) / 16 * 16;
            stage = stage && spins + 16 * nl + stat <= (int64_t)C.max_smem;
        }
        std::vector<int2> items;
        for (int k : G.sys) {
            System &S = *C.sys[k];
            const int64_t nl = G.cl > 1 ? S.cl_layout.Npl : S.plan.Np;
            S.pv_stage = stage;
            S.resident_smem = (size_t)(stage ? (spin_bytes(C, nl) + 15) / 16 * 16 + 16 * nl : spin_bytes(C, nl));
            for (int r = 0; r < S.R; r++) items.push_back(make_int2(k, r));
        }
        std::stable_sort(items.begin(), items.end(),
                         [&](int2 a, int2 b) { return C.sys[a.x]->plan.Np > C.sys[b.x]->plan.Np; });
        G.items.upload(items);
        G.n_items = (int)items.size();
        if (!G.work_ctr.n) G.work_ctr.alloc(1);
    }
    std::vector<ResSys<float>> fr;
    std::vector<ResSys<double>> dr;
    for (auto &Sp : C.sys) {
        if (C.precision == CSMC_FP32) fr.push_back(make_res(*Sp, Sp->fa));
        else dr.push_back(make_res(*Sp, Sp->da));
    }
    if (C.precision == CSMC_FP32) C.fres.upload(fr);
    else C.dres.upload(dr);
}

// (float)(1 / T[k]): the reciprocal temperatures the single-precision sweeps
// multiply by, rounded once from the FP64 quotient
static std::vector<float> reciprocals(const double *T, int n) {
    std::vector<float> v((size_t)n);
    for (int k = 0; k < n; k++) v[k] = (float)(1.0 / T[k]);
    return v;
}

static Ctx *create(const csmc_lattice_desc *descs, int n, const int32_t *reps, int precision, uint64_t seed) {
    require(n >= 1, CSMC_ERR_INVALID, "need at least one lattice");
    require(precision == CSMC_FP32 || precision == CSMC_FP64, CSMC_ERR_INVALID, "precision must be CSMC_FP32 or CSMC_FP64");
    std::unique_ptr<Ctx> C(new Ctx());
    C->precision = precision;
    C->seed = seed;
    C->k0 = (uint32_t)seed;
    C->k1 = (uint32_t)(seed >> 32);
    int chains = 0;
    for (int k = 0; k < n; k++) { // host-side validation and flattening first
        require(reps[k] >= 1, CSMC_ERR_INVALID, "replica count must be >= 1");
        auto S = std::make_unique<System>();
        S->plan = make_plan(&descs[k]);
        const Plan &P = S->plan;
        // the sweep kernels index the [slot][site] partner tables in 32 bits
        require((int64_t)std::max({P.W2, 2 * P.W3, 3 * P.W4, 1}) * P.Np < ((int64_t)1 << 31), CSMC_ERR_UNSUPPORTED,
                "lattice too large: partner slots x padded sites must stay below 2^31");
        S->R = reps[k];
        S->base = chains;
        chains += reps[k];
        C->sys.push_back(std::move(S));
    }
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    require(ndev > 0, CSMC_ERR_CUDA, "no CUDA device");
    CK(cudaGetDevice(&C->device));
    CK(cudaDeviceGetAttribute(&C->n_sms, cudaDevAttrMultiProcessorCount, C->device));
    CK(cudaDeviceGetAttribute(&C->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, C->device));
    CK(cudaStreamCreateWithFlags(&C->st, cudaStreamNonBlocking));
    C->n_chains = chains;
    // With a tool injected into the process (CUDA_INJECTION64_PATH: kernel
    // profilers), multi-window cooperative launches are not issued: such tools
    // serialise and intercept every launch, and a cooperative cluster launch
    // under one failed to start.  Exchange windows then run one launch each.
    if (std::getenv("CUDA_INJECTION64_PATH")) C->persistent_ok = false;
    for (auto &S : C->sys) upload_system(*C, *S);

    const int nc = chains;
    std::vector<int32_t> ident(nc);
    std::iota(ident.begin(), ident.end(), 0);
    C->slot_of.upload(ident);
    C->chain_of.upload(ident);
    std::vector<double> ones(nc, 1.0), sig(nc, 60.0), zeros(nc, 0.0);
    C->T_slot.upload(ones);
    C->T_stash.upload(ones);
    std::vector<float> fones(nc, 1.0f);
    C->invT_slot.upload(fones);
    C->invT_stash.upload(fones);
    C->invT64_slot.upload(ones);
    C->sigma_slot.upload(sig);
    C->acc_slot.upload(zeros);
    C->exch_slot.upload(zeros);
    C->E_chain.upload(zeros);
    C->M_chain.upload(zeros);
    C->E_win.alloc(2 * (size_t)nc);
    C->last_acc.upload(zeros);
    C->lambda_slot.upload(zeros);
    for (auto &S : C->sys) S->cons.lambda_slot = C->lambda_slot.p;
    std::vector<unsigned long long> z64(nc, 0ull);
    C->sweep_acc.upload(z64);
    unsigned int zb = 0;
    C->drift_bits.upload(&zb, 1);
    int zi = 0;
    C->error_flag.upload(&zi, 1);
    unsigned int zu = 0;
    C->grid_bar.upload(&zu, 1);
    size_t part = 0, stage = 0;
    for (auto &S : C->sys) {
        part = std::max(part, (size_t)(3 * S->R * partial_blocks(S->plan.Np)));
        stage = std::max(stage, (size_t)(3 * S->R * S->plan.N));
    }
    C->part.alloc(part);
    C->stage.alloc(stage);
    ChainState &cs = C->cs;
    cs.slot_of = C->slot_of.p;
    cs.chain_of = C->chain_of.p;
    cs.T_slot = C->T_slot.p;
    cs.invT_slot = C->invT_slot.p;
    cs.invT64_slot = C->invT64_slot.p;
    cs.sigma_slot = C->sigma_slot.p;
    cs.acc_slot = C->acc_slot.p;
    cs.exch_slot = C->exch_slot.p;
    cs.E_chain = C->E_chain.p;
    cs.M_chain = C->M_chain.p;
    cs.E_win = C->E_win.p;
    cs.sweep_acc = C->sweep_acc.p;
    cs.drift_bits = C->drift_bits.p;
    cs.error_flag = C->error_flag.p;
    std::vector<uint32_t> ids(nc);
    std::iota(ids.begin(), ids.end(), 0u);
    C->chain_id.upload(ids);
    cs.chain_id = C->chain_id.p;

    std::vector<int2> lat;
    for (auto &S : C->sys) lat.push_back(make_int2(S->base, S->R));
    C->lattices.upload(lat);
    CK(cudaHostAlloc((void **)&C->h_flag, sizeof(int), cudaHostAllocDefault));
    *C->h_flag = 0;
    CK(cudaEventCreate(&C->run_e0));
    CK(cudaEventCreate(&C->run_e1));
    C->n_items = 0;
    for (auto &S : C->sys) C->n_items += S->R;
    choose_cluster(*C, 0);
    upload_resident(*C);
    CK(cudaDeviceSynchronize());
    return C.release();
}

// ------------------------------------------------------------ helpers

// Enqueue the copy of the device error flag; after the stream is
// synchronised, raise_flag() turns a set flag into CSMC_ERR_TIMEOUT.
static void queue_flag(Ctx &C) {
    CK(cudaMemcpyAsync(C.h_flag, C.error_flag.p, sizeof(int), cudaMemcpyDeviceToHost, C.st));
}
static void raise_flag(Ctx &C) {
    if (*C.h_flag) {
        *C.h_flag = 0;
        CK(cudaMemset(C.error_flag.p, 0, sizeof(int)));
        throw Error(CSMC_ERR_TIMEOUT, "a bounded device wait gave up (TMA staging or a cluster barrier did not complete)");
    }
}

static void sync_check(Ctx &C) {
    queue_flag(C);
    CK(cudaStreamSynchronize(C.st));
    CK(cudaGetLastError());
    raise_flag(C);
}

static std::vector<int32_t> download_i32(const DevBuf<int32_t> &b) {
    std::vector<int32_t> v(b.n);
    if (b.n) CK(cudaMemcpy(v.data(), b.p, b.n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return v;
}
static std::vector<double> download_f64(const DevBuf<double> &b, size_t n) {
    std::vector<double> v(n);
    if (n) CK(cudaMemcpy(v.data(), b.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    return v;
}

// Apply f(System&, args) with the context's arithmetic type.
template <class F> static void with_args(Ctx &C, System &S, F &&f) {
    if (C.precision == CSMC_FP32) f(S.fa);
    else f(S.da);
}

// A host buffer the device can address directly (pinned or registered host
// memory, mapped into the unified address space), or nullptr.
static const double *device_view(const void *host) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
    return static_cast<const double *>(at.devicePointer);
}

// Slots [first, first+n) of one lattice from / to the FP64 reference layout.
// A host buffer the device can address (pinned or registered host memory)
// is read or written in place by the conversion kernel, whose
// accesses of it are consecutive (two doubles per thread where aligned): one
// launch at the host link's rate, no staging copy.  Pageable host memory goes
// through one bulk copy to or from the device staging buffer and the same
// launch.  Returns after the host buffer has been read (set) or written (get).

static void set_spins_range(Ctx &C, System &S, int first, int n, const double *host) {
    if (n <= 0) return;
    const size_t bytes = (size_t)S.plan.N * 3 * n * sizeof(double);
    const double *src = device_view(host);
    if (!src) {
        CK(cudaMemcpyAsync(C.stage.p, host, bytes, cudaMemcpyHostToDevice, C.st));
        src = C.stage.p;
    }
    with_args(C, S, [&](auto &a) { launch_scatter(a, C.chain_of.p, first, n, src, C.st); });
    CK(cudaStreamSynchronize(C.st));
}

static void get_spins_range(Ctx &C, System &S, int first, int n, double *host) {
    if (n <= 0) return;
    const size_t bytes = (size_t)S.plan.N * 3 * n * sizeof(double);
    double *dst = const_cast<double *>(device_view(host));
    const bool direct = dst != nullptr;
    if (!direct) dst = C.stage.p;
    with_args(C, S, [&](auto &a) { launch_gather(a, C.chain_of.p, first, n, dst, C.st); });
    if (!direct) CK(cudaMemcpyAsync(host, C.stage.p, bytes, cudaMemcpyDeviceToHost, C.st));
    CK(cudaStreamSynchronize(C.st));
}

static void set_spins_slot(Ctx &C, int slot, const double *host) {
    set_spins_range(C, *C.sys[C.sys_of_slot(slot)], slot, 1, host);
}

static void get_spins_slot(Ctx &C, int slot, double *host) {
    get_spins_range(C, *C.sys[C.sys_of_slot(slot)], slot, 1, host);
}

static void set_spins_all(Ctx &C, const double *host) {
    size_t off = 0;
    for (auto &Sp : C.sys) {
        set_spins_range(C, *Sp, Sp->base, Sp->R, host + off);
        off += (size_t)Sp->plan.N * 3 * Sp->R;
    }
}

static void get_spins_all(Ctx &C, double *host) {
    size_t off = 0;
    for (auto &Sp : C.sys) {
        get_spins_range(C, *Sp, Sp->base, Sp->R, host + off);
        off += (size_t)Sp->plan.N * 3 * Sp->R;
    }
}

// chain-indexed device values -> slot-indexed host values
static void chain_to_slot(Ctx &C, const DevBuf<double> &v, double *out) {
    const std::vector<double> x = download_f64(v, C.n_chains);
    const std::vector<int32_t> slot_of = download_i32(C.slot_of);
    for (int c = 0; c < C.n_chains; c++) out[slot_of[c]] = x[c];
}

// ------------------------------------------------------------ sweeps (global path)

struct Launches {
    int64_t n = 0;
};

// One sweep of `what` (0 OR, 1 Metropolis, 2 deterministic) over all replicas
// of every lattice; per_replica issues one launch per replica per class.  The
// constrained Metropolis kinds are one sequential launch per lattice.
static void sweep_global(Ctx &C, int what, int kind, double T_override, bool per_replica, Launches &L) {
    const bool constrained = what == 1 && kind >= CSMC_METROPOLIS_CONSTRAINT;
    for (auto &Sp : C.sys) {
        System &S = *Sp;
        const Plan &P = S.plan;
        with_args(C, S, [&](auto &a) {
            if (constrained) {
                launch_metro_constraint(a, C.cs, S.cons, kind, C.msweep, T_override, C.st);
                L.n++;
                return;
            }
            for (int col = 0; col < P.n_colours; col++) {
                const int64_t st = P.col_start[col], n = P.col_count[col];
                const int groups = per_replica ? S.R : 1;
                for (int g = 0; g < groups; g++) {
                    const int lo = per_replica ? g : 0, cnt = per_replica ? 1 : S.R;
                    if (what == 0) launch_or_colour(a, st, n, lo, cnt, C.st);
                    else if (what == 1) launch_metro_colour(a, C.cs, st, n, lo, cnt, kind, C.msweep, T_override, C.st);
                    else launch_det_colour(a, st, n, lo, cnt, C.st);
                    L.n++;
                }
            }
        });
        if (what == 1) {
            launch_after_metro(C.cs, S.base, S.R, kind, P.N, C.sigma0, C.last_acc.p, C.st);
            L.n++;
        }
    }
    if (what == 1) C.msweep++;
    C.nsweeps++;
}

static void renorm_all(Ctx &C, Launches &L);

// Single precision: renormalise |s| = S when the context's total sweep count
// passed a multiple of renorm_every since `before` (as the resident kernel
// does after each iteration).
static void renorm_check(Ctx &C, Launches &L, uint64_t before) {
    if (C.precision != CSMC_FP32 || C.renorm_every <= 0) return;
    const uint64_t e = (uint64_t)C.renorm_every;
    if (C.nsweeps / e > before / e) renorm_all(C, L);
}

static void energy_all(Ctx &C, Launches &L) {
    for (auto &Sp : C.sys) {
        System &S = *Sp;
        with_args(C, S, [&](auto &a) { launch_energy(a, C.cs, 0, S.R, C.part.p, C.st); });
        L.n += 2;
    }
}
static void magnet_all(Ctx &C, Launches &L) {
    for (auto &Sp : C.sys) {
        System &S = *Sp;
        with_args(C, S, [&](auto &a) { launch_magnet(a, C.cs, 0, S.R, C.part.p, C.st); });
        L.n += 2;
    }
}
static void renorm_all(Ctx &C, Launches &L) {
    if (C.precision != CSMC_FP32) return;
    for (auto &Sp : C.sys) {
        launch_renorm(Sp->fa, 0, Sp->R, C.st);
        L.n++;
    }
}

// ------------------------------------------------------------ run driver

struct Schedule {
    int64_t start, end; // iterations [start, end)
    int64_t t_therm;
    int or_rate, swap_rate, probe_rate, kind;
    bool swap_enabled;
    int64_t dosweep;
    int64_t probe_first, n_probes, cap;
    bool is_probe(int64_t q) const { return probe_rate > 0 && q >= t_therm && q % probe_rate == 0; }
    bool is_metro(int64_t q) const { return q % dosweep == 0; }
    bool is_swap(int64_t q) const { return swap_enabled && is_metro(q) && q % swap_rate == 0; }
    bool need_E(int64_t it) const {
        if (is_swap(it)) return true;
        for (int64_t q = it; q < it + dosweep && q < end; q++)
            if (is_probe(q)) return true;
        return it + dosweep >= end;
    }
};

static int choose_path(Ctx &C, int requested, int kind) {
    if (kind >= CSMC_METROPOLIS_CONSTRAINT) {
        require(requested != CSMC_PATH_RESIDENT, CSMC_ERR_UNSUPPORTED,
                "the constrained Metropolis kinds run on the global path only (sequential proposals per replica)");
        return requested == CSMC_PATH_PER_REPLICA ? requested : CSMC_PATH_GLOBAL;
    }
    if (requested == CSMC_PATH_GLOBAL || requested == CSMC_PATH_PER_REPLICA) return requested;
    bool all = true;
    for (auto &S : C.sys) all = all && S->resident_ok;
    if (requested == CSMC_PATH_RESIDENT) {
        require(all, CSMC_ERR_UNSUPPORTED,
                "resident path needs every replica to fit in shared memory (3 * padded_sites * word size bytes) "
                "and at most 65536 padded sites");
        return CSMC_PATH_RESIDENT;
    }
    return all && !C.global_pref ? CSMC_PATH_RESIDENT : CSMC_PATH_GLOBAL;
}

// Threads per CTA of a group's resident kernel.  `hint` (a multiple of 32)
// forces a size, capped at the kernel's maximum (896 for the specialised
// kernel with scalar couplings and at most diagonal onsite terms, else 512).
// Otherwise the specialised kernel gets the smallest multiple of 32 that gives
// every thread the same number of sites of the largest colour-class part
// between two barriers, and the generic kernel its maximum.  The autotuner's
// block applies to a context of one group.
// The most sites of one colour class any CTA of the group holds.
static int64_t resident_class_sites(const Ctx &C, const Group &G) {
    int64_t n = 32;
    for (int k : G.sys) {
        const System &S = *C.sys[k];
        const Plan &P = S.plan;
        for (int col = 0; col < P.n_colours; col++) {
            if (G.cl > 1)
                for (int q = 0; q < G.cl; q++) n = std::max(n, S.cl_layout.loc_count[(size_t)q * P.n_colours + col]);
            else
                n = std::max(n, P.col_count[col]);
        }
    }
    return n;
}

// Threads per CTA that cover n sites of a colour class in `extra` more rounds
// than the fewest the largest block mx needs, as evenly as whole warps allow.
static int balanced_block(int64_t n, int mx, int extra) {
    const int64_t iters = (n + mx - 1) / mx + extra;
    return (int)std::min<int64_t>(mx, (n + 32 * iters - 1) / (32 * iters) * 32);
}

static int resident_block(Ctx &C, const Group &G, int hint) {
    const ResidentSel sel = resident_selection(C, G);
    int mx = resident_max_threads(sel.fast, sel.bil, sel.ons);
    if (C.size_groups && C.group_block_cap >= 32) mx = std::min(mx, C.group_block_cap);
    if (hint == 0 && C.block_pref > 0 && !C.size_groups) hint = C.block_pref;
    if (hint > 0) {
        require(hint % 32 == 0, CSMC_ERR_INVALID, "resident block must be a multiple of 32");
        return std::min(hint, mx);
    }
    if (!sel.fast) return mx;
    return balanced_block(resident_class_sites(C, G), mx, 0);
}

// The resident kernel for the lattices of a group: the specialised one when
// all of them allow it (with the widest coupling classes among them), else
// the generic one.
static ResidentSel resident_selection(const Ctx &C, const Group &G) {
    ResidentSel sel{true, 0, 0, 4, false, false, G.cl};
    for (int k : G.sys) {
        const System &S = *C.sys[k];
        sel.fast = sel.fast && S.fast_ok;
        sel.bil = std::max(sel.bil, S.bil_class);
        sel.ons = std::max(sel.ons, S.ons_class);
        sel.width = std::max(sel.width, S.plan.W2 <= 4 ? 4 : S.plan.W2 <= 6 ? 6 : 8);
        sel.cub = sel.cub || S.cub;
        sel.qua = sel.qua || S.qua;
    }
    return sel;
}

// Resident CTAs (one replica each) or clusters of a group that fit on the device at once.
static int resident_slots(Ctx &C, const Group &G, int block, size_t *smem_out) {
    size_t smem = 0;
    for (int k : G.sys) smem = std::max(smem, C.sys[k]->resident_smem);
    const ResidentSel sel = resident_selection(C, G);
    const int cap = C.precision == CSMC_FP32 ? resident_capacity<float>(block, smem, sel, C.n_sms)
                                             : resident_capacity<double>(block, smem, sel, C.n_sms);
    require(cap >= 1, CSMC_ERR_UNSUPPORTED, "resident kernel does not fit on the device with this shared memory size");
    if (smem_out) *smem_out = smem;
    return cap;
}

// Is a persistent (cooperative, multi-window) launch possible: one group whose
// replicas are all resident on the device at once.
static bool persistent_fits(Ctx &C, int hint) {
    if (C.groups.size() != 1) return false;
    const Group &G = *C.groups[0];
    return resident_slots(C, G, resident_block(C, G, hint), nullptr) >= G.n_items;
}

// One group's resident launch on stream `st`.
static cudaError_t launch_group(Ctx &C, Group &G, RunDesc rd, int hint, cudaStream_t st) {
    const int block = resident_block(C, G, hint);
    size_t smem = 0;
    const int cap = resident_slots(C, G, block, &smem);
    const ResidentSel sel = resident_selection(C, G);
    // CTAs (one per replica) or clusters (sel.cl CTAs per replica)
    const int grid = std::min(G.n_items, cap) * std::max(sel.cl, 1);
    if (rd.persistent) {
        require(cap >= G.n_items, CSMC_ERR_INVALID, "persistent launch needs every replica resident at once");
        rd.grid_bar = C.grid_bar.p;
        rd.n_blocks = (uint32_t)grid;
        rd.lattices = C.lattices.p;
        rd.n_lattices = (int)C.sys.size();
        rd.k0 = C.k0;
        rd.k1 = C.k1;
        CK(cudaMemsetAsync(C.grid_bar.p, 0, sizeof(unsigned int), st));
    }
    CK(cudaMemsetAsync(G.work_ctr.p, 0, sizeof(int), st));
    return C.precision == CSMC_FP32
               ? launch_resident<float>(C.fres.p, G.items.p, G.n_items, G.work_ctr.p, C.cs, rd, grid, block, smem,
                                        sel, rd.persistent != 0, st)
               : launch_resident<double>(C.dres.p, G.items.p, G.n_items, G.work_ctr.p, C.cs, rd, grid, block, smem,
                                         sel, rd.persistent != 0, st);
}

// One resident launch of every replica (with size groups: one launch per
// group, side by side on the groups' streams, joined back into the context's
// stream).  rd.persistent: a cooperative launch with one CTA (or cluster) per
// replica; returns false, with nothing launched, if the device refuses it.
static bool resident_launch(Ctx &C, RunDesc rd, int hint, Launches &L) {
    auto ev = C.next_kernel_events();
    CK(cudaEventRecord(ev.first, C.st));
    if (C.groups.size() == 1) {
        const cudaError_t e = launch_group(C, *C.groups[0], rd, hint, C.st);
        if (e != cudaSuccess && rd.persistent) {
            cudaGetLastError(); // a refused cooperative launch leaves no sticky error
            C.kev_used--;
            return false;
        }
        CK(e);
        L.n += 1;
    } else {
        require(!rd.persistent, CSMC_ERR_INVALID, "size groups run one launch per window");
        CK(cudaEventRecord(C.fork, C.st));
        for (auto &G : C.groups) {
            CK(cudaStreamWaitEvent(G->st, C.fork, 0));
            CK(launch_group(C, *G, rd, hint, G->st));
            CK(cudaEventRecord(G->done, G->st));
            L.n += 1;
        }
        for (auto &G : C.groups) CK(cudaStreamWaitEvent(C.st, G->done, 0));
    }
    CK(cudaEventRecord(ev.second, C.st));
    return true;
}

static void run(Ctx &C, csmc_run_params *p) {
    require(p != nullptr, CSMC_ERR_INVALID, "params is NULL");
    require(p->n_sweeps >= 0 && p->sweep_start >= 0, CSMC_ERR_INVALID, "negative sweep range");
    require(p->overrelaxation_rate >= 0, CSMC_ERR_INVALID, "overrelaxation_rate must be >= 0");
    require(p->kind >= 0 && p->kind <= CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE, CSMC_ERR_INVALID,
            "unknown Metropolis kind");
    Schedule s;
    s.start = p->sweep_start;
    s.end = p->sweep_start + p->n_sweeps;
    s.t_therm = p->t_thermalization;
    s.or_rate = p->overrelaxation_rate;
    s.swap_rate = p->swap_rate;
    s.probe_rate = p->probe_rate;
    s.kind = p->kind;
    s.dosweep = s.or_rate == 0 ? 1 : s.or_rate;
    bool any_pt = false;
    for (auto &S : C.sys) any_pt = any_pt || S->R > 1;
    s.swap_enabled = s.swap_rate > 0 && any_pt;
    s.probe_first = 0;
    s.n_probes = 0;
    if (s.probe_rate > 0) {
        int64_t lo = std::max(s.t_therm, s.start);
        s.probe_first = (lo + s.probe_rate - 1) / s.probe_rate * s.probe_rate;
        if (s.probe_first < s.end) s.n_probes = (s.end - 1 - s.probe_first) / s.probe_rate + 1;
    }
    const bool want_rec = (p->probe_energy || p->probe_magnetization) && s.n_probes > 0;
    s.cap = want_rec ? std::min<int64_t>(s.n_probes, std::max<int64_t>(p->probe_capacity, 0)) : 0;
    const int n_slots = C.n_chains;
    if (s.cap > 0) {
        if (C.rec_E.n < (size_t)(s.cap * n_slots)) C.rec_E.alloc(s.cap * n_slots);
        if (C.rec_M.n < (size_t)(s.cap * n_slots)) C.rec_M.alloc(s.cap * n_slots);
    }
    double *recE = s.cap > 0 ? C.rec_E.p : nullptr, *recM = s.cap > 0 ? C.rec_M.p : nullptr;
    C.acc_slot.zero(C.st);
    C.exch_slot.zero(C.st);

    const int path = choose_path(C, p->path, p->kind);
    C.reset_kernel_time();
    Launches L;
    cudaEvent_t e0 = C.run_e0, e1 = C.run_e1;
    CK(cudaEventRecord(e0, C.st));

    // the exchange of iteration `it` (every lattice, one launch), followed by
    // probe record kq (kq < 0: none)
    auto exchange = [&](int64_t it, bool do_swap, int64_t kq) {
        launch_exchange(C.cs, C.lattices.p, (int)C.sys.size(), it, s.swap_rate, C.k0, C.k1, do_swap, recE, recM, kq,
                        n_slots, C.st);
        L.n++;
    };
    // probe record index of iteration q, or -1 (no probe, or beyond the capacity)
    auto record_index = [&](int64_t q) -> int64_t {
        if (!s.is_probe(q)) return -1;
        const int64_t kq = (q - s.probe_first) / s.probe_rate;
        return kq < s.cap ? kq : -1;
    };

    if (path == CSMC_PATH_RESIDENT) {
        const int hint = p->resident_block; // threads per CTA asked for (0: automatic)
        require(hint >= 0 && hint % 32 == 0, CSMC_ERR_INVALID, "resident block must be a multiple of 32");
        // windows end at exchange iterations; without exchanges, at most
        // `chunk` iterations per launch.  With exchanges and every replica
        // resident at once, one persistent launch runs up to kWindows windows
        // and the exchanges between them.
        const int64_t chunk = 256, kWindows = 128;
        const int64_t period = s.swap_enabled ? std::lcm((int64_t)s.swap_rate, s.dosweep) : 0;
        bool persistent = s.swap_enabled && C.persistent_on && C.persistent_ok && persistent_fits(C, hint);
        int64_t it = s.start;
        while (it < s.end) {
            if (persistent) {
                const int64_t q1 = (it + period - 1) / period * period;
                const int64_t to = std::min(s.end - 1, q1 + (kWindows - 1) * period);
                RunDesc rd{};
                rd.it0 = it;
                rd.it1 = to + 1;
                rd.t_therm = s.t_therm;
                rd.probe_first = s.probe_first;
                rd.probe_cap = s.cap;
                rd.rec_E = recE;
                rd.rec_M = recM;
                rd.msweep0 = C.msweep;
                rd.or_rate = s.or_rate;
                rd.swap_rate = s.swap_rate;
                rd.probe_rate = s.probe_rate;
                rd.kind = s.kind;
                rd.n_slots = n_slots;
                rd.renorm_every = C.renorm_every;
                rd.sweeps0 = C.nsweeps;
                rd.swap_enabled = 1;
                rd.persistent = 1;
                rd.swap_period = period;
                if (!resident_launch(C, rd, hint, L)) {
                    persistent = false; // the device refused the cooperative launch: one launch per window
                    C.persistent_ok = false;
                    continue;
                }
                for (int64_t q = it; q <= to; q++) {
                    if (s.is_metro(q)) {
                        C.msweep++;
                        C.nsweeps++;
                    }
                    if (s.or_rate != 0) C.nsweeps++;
                }
                it = to + 1;
                continue;
            }
            int64_t to = std::min(s.end, it + chunk) - 1;
            bool ends_swap = false;
            if (s.swap_enabled) {
                for (int64_t q = it; q <= std::min(s.end - 1, it + chunk * std::max(s.swap_rate, 1)); q++)
                    if (s.is_swap(q)) {
                        to = q;
                        ends_swap = true;
                        break;
                    }
                if (!ends_swap) to = s.end - 1;
            }
            RunDesc rd{};
            rd.it0 = it;
            rd.it1 = to + 1;
            rd.t_therm = s.t_therm;
            rd.probe_first = s.probe_first;
            rd.probe_cap = s.cap;
            rd.rec_E = recE;
            rd.rec_M = recM;
            rd.T_override = 0.0;
            rd.msweep0 = C.msweep;
            rd.or_rate = s.or_rate;
            rd.swap_rate = s.swap_rate;
            rd.probe_rate = s.probe_rate;
            rd.kind = s.kind;
            rd.reset_sigma = 0;
            rd.n_slots = n_slots;
            rd.renorm_every = C.renorm_every;
            rd.sweeps0 = C.nsweeps;
            rd.swap_enabled = s.swap_enabled ? 1 : 0;
            resident_launch(C, rd, hint, L);
            for (int64_t q = it; q <= to; q++) {
                if (s.is_metro(q)) {
                    C.msweep++;
                    C.nsweeps++;
                }
                if (s.or_rate != 0) C.nsweeps++;
            }
            // the kernel left |M| of an exchange iteration's probe in M_chain;
            // the record follows the exchange
            if (ends_swap) exchange(to, true, record_index(to));
            it = to + 1;
        }
    } else {
        const bool per_rep = path == CSMC_PATH_PER_REPLICA;
        for (int64_t it = s.start; it < s.end; it++) {
            const uint64_t before = C.nsweeps;
            if (s.or_rate != 0) sweep_global(C, 0, 0, 0.0, per_rep, L);
            if (s.is_metro(it)) {
                sweep_global(C, 1, s.kind, 0.0, per_rep, L);
                if (s.need_E(it)) energy_all(C, L);
            }
            // |M| is per replica, unchanged by the exchange; the probe records
            // by slot after it (monte_carlo.jl:308-349 then :368-370)
            if (s.is_probe(it)) magnet_all(C, L);
            const int64_t kq = record_index(it);
            if (s.is_swap(it) || kq >= 0) exchange(it, s.is_swap(it), kq);
            renorm_check(C, L, before);
        }
    }
    CK(cudaEventRecord(e1, C.st));
    // results into pinned staging, then one synchronisation
    const size_t nrec = (size_t)s.cap * n_slots;
    double *hb = C.host_box(2 * nrec + 2 * (size_t)n_slots);
    double *h_E = hb, *h_M = hb + nrec, *h_acc = hb + 2 * nrec, *h_exch = h_acc + n_slots;
    queue_flag(C);
    if (nrec && p->probe_energy)
        CK(cudaMemcpyAsync(h_E, C.rec_E.p, nrec * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    if (nrec && p->probe_magnetization)
        CK(cudaMemcpyAsync(h_M, C.rec_M.p, nrec * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    if (p->accepted) CK(cudaMemcpyAsync(h_acc, C.acc_slot.p, n_slots * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    if (p->exchanged)
        CK(cudaMemcpyAsync(h_exch, C.exch_slot.p, n_slots * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    CK(cudaStreamSynchronize(C.st));
    CK(cudaGetLastError());
    raise_flag(C);
    C.collect_kernel_time();
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    C.last_ms = ms;
    C.last_launches = L.n;

    if (nrec && p->probe_energy) std::memcpy(p->probe_energy, h_E, nrec * sizeof(double));
    if (nrec && p->probe_magnetization) std::memcpy(p->probe_magnetization, h_M, nrec * sizeof(double));
    if (p->accepted)
        for (int q = 0; q < n_slots; q++) p->accepted[q] += h_acc[q];
    if (p->exchanged)
        for (int q = 0; q < n_slots; q++) p->exchanged[q] += h_exch[q];
    p->n_probes_out = s.cap;
}

static void anneal(Ctx &C, const double *temps, int n_temps, int64_t t_therm, int or_rate, int kind, double sigma0,
                   int path_req, double *accepted) {
    require(n_temps >= 0 && (n_temps == 0 || temps), CSMC_ERR_INVALID, "temperatures missing");
    require(or_rate >= 0, CSMC_ERR_INVALID, "overrelaxation_rate must be >= 0");
    require(kind >= 0 && kind <= CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE, CSMC_ERR_INVALID, "unknown Metropolis kind");
    const int path = choose_path(C, path_req, kind);
    C.sigma0 = sigma0; // also the reset value of the constrained adaptive kind
    C.reset_kernel_time();
    const int n_slots = C.n_chains;
    Launches L;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float total_ms = 0.f;
    const int64_t dosweep = or_rate == 0 ? 1 : or_rate;
    for (int k = 0; k < n_temps; k++) {
        const double T = temps[k];
        require(T > 0, CSMC_ERR_INVALID, "temperatures must be > 0");
        C.acc_slot.zero(C.st);
        CK(cudaEventRecord(e0, C.st));
        if (t_therm > 1) {
            if (path == CSMC_PATH_RESIDENT) {
                RunDesc rd{};
                rd.it0 = 1; // t = 1 .. t_thermalization-1 (monte_carlo.jl:169-182)
                rd.it1 = t_therm;
                rd.t_therm = INT64_MAX;
                rd.T_override = T;
                rd.sigma0 = sigma0;
                rd.msweep0 = C.msweep;
                rd.or_rate = or_rate;
                rd.swap_rate = 0;
                rd.probe_rate = 0;
                rd.kind = kind;
                rd.reset_sigma = 1;
                rd.n_slots = n_slots;
                rd.renorm_every = C.renorm_every;
                rd.sweeps0 = C.nsweeps;
                resident_launch(C, rd, 0, L);
                for (int64_t t = 1; t < t_therm; t++) {
                    if (t % dosweep == 0) {
                        C.msweep++;
                        C.nsweeps++;
                    }
                    if (or_rate != 0) C.nsweeps++;
                }
            } else {
                std::vector<double> sg(n_slots, sigma0);
                CK(cudaMemcpyAsync(C.sigma_slot.p, sg.data(), n_slots * sizeof(double), cudaMemcpyHostToDevice, C.st));
                CK(cudaStreamSynchronize(C.st));
                const bool per_rep = path == CSMC_PATH_PER_REPLICA;
                for (int64_t t = 1; t < t_therm; t++) {
                    const uint64_t before = C.nsweeps;
                    if (or_rate != 0) sweep_global(C, 0, 0, T, per_rep, L);
                    if (t % dosweep == 0) sweep_global(C, 1, kind, T, per_rep, L);
                    renorm_check(C, L, before);
                }
            }
        }
        CK(cudaEventRecord(e1, C.st));
        sync_check(C);
        C.collect_kernel_time();
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        total_ms += ms;
        if (accepted) {
            std::vector<double> a = download_f64(C.acc_slot, n_slots);
            std::copy(a.begin(), a.end(), accepted + (size_t)k * n_slots);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    C.last_ms = total_ms;
    C.last_launches = L.n;
}

// compute_equal_time_correlations of every replica of one lattice (csmc_structure_factor)
template <typename R>
static void structure_factor(Ctx &C, System &S, const SysArgs<R> &a, int dim, const double *positions, int64_t n_k,
                             const double *ks, double *Suv) {
    const Plan &P = S.plan;
    // single precision on the tensor cores (positions padded to whole chunks of sites)
    const bool tensor = sizeof(R) == 4 && C.sf_tensor;
    const int64_t n_pos = tensor ? sf_tc_sites(P.Np) : P.Np;
    std::vector<R> pd((size_t)n_pos * 3, R(0)), kd((size_t)std::max<int64_t>(n_k, 1) * 3, R(0));
    for (int64_t d = 0; d < P.Np; d++) {
        const int64_t i = P.dev2ref[d];
        if (i < 0) continue;
        for (int x = 0; x < dim; x++) pd[(size_t)d * 3 + x] = (R)positions[(size_t)i * dim + x];
    }
    for (int64_t n = 0; n < n_k; n++)
        for (int x = 0; x < dim; x++) kd[(size_t)n * 3 + x] = (R)ks[(size_t)n * dim + x];
    DevBuf<R> dpos, dks;
    DevBuf<double> dout;
    dpos.upload(pd);
    dks.upload(kd);
    dout.alloc((size_t)S.R * std::max<int64_t>(n_k, 1) * 9);
    const int splits = tensor ? sf_tc_splits(n_k, S.R, P.Np, C.n_sms) : 1;
    if (tensor) {
        C.sf_packed.reserve((size_t)sf_tc_packed_floats(P.Np, S.R));
        C.sf_partial.reserve((size_t)sf_tc_partial_floats(n_k, S.R, splits));
    }
    C.reset_kernel_time();
    auto ev = C.next_kernel_events();
    CK(cudaEventRecord(ev.first, C.st));
    if constexpr (sizeof(R) == 4) {
        if (tensor)
            CK(launch_structure_factor_tc(a, dpos.p, dks.p, n_k, C.slot_of.p, S.base, dout.p, C.sf_packed.p,
                                          C.sf_partial.p, splits, C.error_flag.p, C.st));
    }
    if (!tensor) launch_structure_factor<R>(a, dpos.p, dks.p, n_k, C.slot_of.p, S.base, dout.p, C.st);
    CK(cudaEventRecord(ev.second, C.st));
    sync_check(C);
    C.collect_kernel_time();
    C.last_ms = C.last_kernel_ms;
    C.last_launches = 1;
    if (n_k > 0) CK(cudaMemcpy(Suv, dout.p, (size_t)S.R * n_k * 9 * sizeof(double), cudaMemcpyDeviceToHost));
}

static void ensure_exact(Ctx &C, System &S) {
    if (S.exact_ready) return;
    const Plan &P = S.plan;
    const int64_t N = P.N;
    std::vector<int64_t> bs(N * P.N2 + 1), cs(N * P.N3 * 2 + 1), qs(N * P.N4 * 3 + 1);
    std::vector<double> bm(N * P.N2 * 9 + 1), ct(N * P.N3 * 27 + 1), qt(N * P.N4 * 81 + 1), f(N * 3), o(N * 9);
    export_tables(P, bs.data(), bm.data(), cs.data(), ct.data(), qs.data(), qt.data(), f.data(), o.data());
    for (auto &v : bs) v -= 1;
    for (auto &v : cs) v -= 1;
    for (auto &v : qs) v -= 1;
    S.xbs.upload(bs);
    S.xcs.upload(cs);
    S.xqs.upload(qs);
    S.xbm.upload(bm);
    S.xct.upload(ct);
    S.xqt.upload(qt);
    S.xfield.upload(f);
    S.xonsite.upload(o);
    S.exact_ready = true;
}

} // namespace csmc

using namespace csmc;

// The device of the context an entry point works on is made current for the
// call and the caller's device restored on return: a context keeps working
// when its caller has switched devices in between.  ctx_of() pins it.
struct DeviceScope {
    static thread_local DeviceScope *cur;
    DeviceScope *outer;
    int prev = -1;
    DeviceScope() : outer(cur) { cur = this; }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
        cur = outer;
    }
    void pin(int device) {
        int d = -1;
        CK(cudaGetDevice(&d));
        if (d == device) return;
        CK(cudaSetDevice(device));
        if (prev < 0) prev = d;
    }
};
thread_local DeviceScope *DeviceScope::cur = nullptr;

#define API_BEGIN                                                                                                      \
    DeviceScope device_scope_;                                                                                         \
    try {
#define API_END                                                                                                        \
    }                                                                                                                  \
    catch (const Error &e) {                                                                                           \
        g_err = e.what();                                                                                              \
        return e.code;                                                                                                 \
    }                                                                                                                  \
    catch (const std::bad_alloc &) {                                                                                   \
        g_err = "host allocation failed";                                                                              \
        return CSMC_ERR_OOM;                                                                                           \
    }                                                                                                                  \
    catch (const std::exception &e) {                                                                                  \
        g_err = e.what();                                                                                              \
        return CSMC_ERR_INVALID;                                                                                       \
    }                                                                                                                  \
    return CSMC_OK;

static Ctx &ctx_of(void *c) {
    require(c != nullptr, CSMC_ERR_INVALID, "context is NULL");
    Ctx &C = *static_cast<Ctx *>(c);
    if (DeviceScope::cur) DeviceScope::cur->pin(C.device);
    return C;
}

extern "C" {

const char *csmc_last_error(void) { return g_err.c_str(); }
const char *csmc_version(void) { return "csmc 0.1 sm_103a"; }

int csmc_lattice_plan(const csmc_lattice_desc *desc, csmc_lattice_info *info) {
    API_BEGIN
    require(info != nullptr, CSMC_ERR_INVALID, "info is NULL");
    Plan p = make_plan(desc);
    fill_info(p, info);
    API_END
}

int csmc_lattice_tables(const csmc_lattice_desc *desc, int64_t *bs, double *bm, int64_t *cs, double *ct, int64_t *qs,
                        double *qt, double *field, double *onsite) {
    API_BEGIN
    Plan p = make_plan(desc);
    export_tables(p, bs, bm, cs, ct, qs, qt, field, onsite);
    API_END
}

int csmc_lattice_colouring(const csmc_lattice_desc *desc, int32_t *colour_of_site, int64_t *ref_of_device,
                           int64_t *colour_start) {
    API_BEGIN
    Plan p = make_plan(desc);
    if (colour_of_site) std::copy(p.colour_of.begin(), p.colour_of.end(), colour_of_site);
    if (ref_of_device) std::copy(p.dev2ref.begin(), p.dev2ref.end(), ref_of_device);
    if (colour_start) std::copy(p.col_start.begin(), p.col_start.end(), colour_start);
    API_END
}

int csmc_create(const csmc_lattice_desc *desc, int32_t precision, int32_t n_replicas, uint64_t seed, void **out) {
    API_BEGIN
    require(out != nullptr, CSMC_ERR_INVALID, "ctx_out is NULL");
    *out = nullptr;
    *out = create(desc, 1, &n_replicas, precision, seed);
    API_END
}

int csmc_create_batch(const csmc_lattice_desc *descs, int32_t n, const int32_t *reps, int32_t precision, uint64_t seed,
                      void **out) {
    API_BEGIN
    require(out != nullptr && descs != nullptr && reps != nullptr, CSMC_ERR_INVALID, "NULL argument");
    *out = nullptr;
    *out = create(descs, n, reps, precision, seed);
    API_END
}

int csmc_destroy(void *c) {
    API_BEGIN
    if (c) {
        Ctx *C = &ctx_of(c); // its device current: the stream and buffers belong to it
        cudaStreamSynchronize(C->st);
        delete C;
    }
    API_END
}

int csmc_num_slots(void *c, int32_t *n) {
    API_BEGIN
    require(n != nullptr, CSMC_ERR_INVALID, "n_slots is NULL");
    *n = ctx_of(c).n_chains;
    API_END
}

int csmc_lattice_info_of(void *c, int32_t k, csmc_lattice_info *info) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(k >= 0 && k < (int)C.sys.size() && info, CSMC_ERR_INVALID, "bad lattice index");
    fill_info(C.sys[k]->plan, info);
    API_END
}

int csmc_set_spins(void *c, int32_t slot, const double *spins) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(spins != nullptr, CSMC_ERR_INVALID, "spins is NULL");
    set_spins_slot(C, slot, spins);
    CK(cudaGetLastError());
    API_END
}

int csmc_get_spins(void *c, int32_t slot, double *spins) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(spins != nullptr, CSMC_ERR_INVALID, "spins is NULL");
    get_spins_slot(C, slot, spins);
    CK(cudaGetLastError());
    API_END
}

int csmc_set_spins_all(void *c, const double *spins) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(spins != nullptr, CSMC_ERR_INVALID, "spins is NULL");
    set_spins_all(C, spins);
    CK(cudaGetLastError());
    API_END
}

int csmc_get_spins_all(void *c, double *spins) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(spins != nullptr, CSMC_ERR_INVALID, "spins is NULL");
    get_spins_all(C, spins);
    CK(cudaGetLastError());
    API_END
}

int csmc_random_spins(void *c, uint64_t seed) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    for (auto &S : C.sys)
        with_args(C, *S, [&](auto &a) {
            launch_random_spins(a, C.chain_id.p, (uint32_t)seed, (uint32_t)(seed >> 32), C.st);
        });
    sync_check(C);
    API_END
}

int csmc_set_temperatures(void *c, const double *T) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(T != nullptr, CSMC_ERR_INVALID, "T is NULL");
    for (int k = 0; k < C.n_chains; k++) require(T[k] > 0, CSMC_ERR_INVALID, "temperatures must be > 0");
    CK(cudaMemcpy(C.T_slot.p, T, C.n_chains * sizeof(double), cudaMemcpyHostToDevice));
    const std::vector<float> inv = reciprocals(T, C.n_chains);
    CK(cudaMemcpy(C.invT_slot.p, inv.data(), inv.size() * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<double> inv64((size_t)C.n_chains);
    for (int k = 0; k < C.n_chains; k++) inv64[k] = 1.0 / T[k];
    CK(cudaMemcpy(C.invT64_slot.p, inv64.data(), inv64.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<int32_t> ident(C.n_chains);
    std::iota(ident.begin(), ident.end(), 0);
    CK(cudaMemcpy(C.slot_of.p, ident.data(), ident.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(C.chain_of.p, ident.data(), ident.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    API_END
}

int csmc_set_sigma(void *c, const double *sigma) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(sigma != nullptr, CSMC_ERR_INVALID, "sigma is NULL");
    CK(cudaMemcpy(C.sigma_slot.p, sigma, C.n_chains * sizeof(double), cudaMemcpyHostToDevice));
    API_END
}

int csmc_get_sigma(void *c, double *sigma) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(sigma != nullptr, CSMC_ERR_INVALID, "sigma is NULL");
    CK(cudaStreamSynchronize(C.st));
    CK(cudaMemcpy(sigma, C.sigma_slot.p, C.n_chains * sizeof(double), cudaMemcpyDeviceToHost));
    API_END
}

int csmc_set_sigma0(void *c, double sigma0) {
    API_BEGIN
    require(std::isfinite(sigma0) && sigma0 >= 0, CSMC_ERR_INVALID, "sigma0 must be finite and >= 0");
    ctx_of(c).sigma0 = sigma0;
    API_END
}

int csmc_set_constraint(void *c, int32_t lattice, const csmc_constraint *k) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(lattice >= 0 && lattice < (int)C.sys.size(), CSMC_ERR_INVALID, "lattice index out of range");
    System &S = *C.sys[lattice];
    const Plan &P = S.plan;
    ConsArgs a{};
    a.lambda_slot = C.lambda_slot.p;
    std::vector<double> wd, wr;
    if (k) {
        const double vals[7] = {k->g[0], k->g[1], k->g[2], k->q, k->p, k->c0, k->weight};
        for (double v : vals) require(std::isfinite(v), CSMC_ERR_INVALID, "constraint coefficients must be finite");
        a.g[0] = k->g[0];
        a.g[1] = k->g[1];
        a.g[2] = k->g[2];
        a.q = k->q;
        a.p = k->p;
        a.c0 = k->c0;
        a.weight = k->weight;
        if (k->site_weights) {
            wr.assign(k->site_weights, k->site_weights + P.N);
            for (double v : wr) require(std::isfinite(v), CSMC_ERR_INVALID, "site weights must be finite");
            wd.assign((size_t)P.Np, 0.0);
            for (int64_t d = 0; d < P.Np; d++)
                if (P.dev2ref[d] >= 0) wd[d] = wr[P.dev2ref[d]];
        }
    }
    CK(cudaStreamSynchronize(C.st)); // no kernel still reads the old weights
    S.cw.upload(wd);
    S.cw_ref.upload(wr);
    a.w = wd.empty() ? nullptr : S.cw.p;
    S.cons = a;
    API_END
}

int csmc_set_lambda(void *c, const double *lambda) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(lambda != nullptr, CSMC_ERR_INVALID, "lambda is NULL");
    CK(cudaStreamSynchronize(C.st));
    CK(cudaMemcpy(C.lambda_slot.p, lambda, C.n_chains * sizeof(double), cudaMemcpyHostToDevice));
    API_END
}

int csmc_get_lambda(void *c, double *lambda) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(lambda != nullptr, CSMC_ERR_INVALID, "lambda is NULL");
    CK(cudaStreamSynchronize(C.st));
    CK(cudaMemcpy(lambda, C.lambda_slot.p, C.n_chains * sizeof(double), cudaMemcpyDeviceToHost));
    API_END
}

int csmc_get_permutation(void *c, int32_t *replica_of_slot) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(replica_of_slot != nullptr, CSMC_ERR_INVALID, "output is NULL");
    CK(cudaStreamSynchronize(C.st));
    std::vector<int32_t> v = download_i32(C.chain_of);
    std::copy(v.begin(), v.end(), replica_of_slot);
    API_END
}

int csmc_local_field(void *c, int32_t slot, double *H) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(H != nullptr, CSMC_ERR_INVALID, "H is NULL");
    System &S = *C.sys[C.sys_of_slot(slot)];
    const int r = download_i32(C.chain_of)[slot] - S.base;
    with_args(C, S, [&](auto &a) { launch_local_field(a, r, C.stage.p, C.st); });
    CK(cudaMemcpyAsync(H, C.stage.p, S.plan.N * 3 * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    sync_check(C);
    API_END
}

int csmc_energy_diff(void *c, int32_t slot, int64_t n, const int64_t *sites, const double *ns, double *dE) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(n >= 0 && (n == 0 || (sites && ns && dE)), CSMC_ERR_INVALID, "NULL argument");
    System &S = *C.sys[C.sys_of_slot(slot)];
    for (int64_t q = 0; q < n; q++)
        require(sites[q] >= 0 && sites[q] < S.plan.N, CSMC_ERR_INVALID, "site index out of range");
    DevBuf<int64_t> ds;
    DevBuf<double> dn, de;
    ds.upload(sites, n);
    dn.upload(ns, 3 * n);
    de.alloc(n);
    with_args(C, S, [&](auto &a) { launch_energy_diff(a, C.chain_of.p, slot, n, ds.p, dn.p, de.p, C.st); });
    sync_check(C);
    if (n) CK(cudaMemcpy(dE, de.p, n * sizeof(double), cudaMemcpyDeviceToHost));
    API_END
}

} // extern "C"

namespace csmc {

void set_last_error(const char *msg) { g_err = msg; }

int context_device(void *c, int *device) {
    API_BEGIN
    require(device != nullptr, CSMC_ERR_INVALID, "device is NULL");
    *device = ctx_of(c).device;
    API_END
}

// csmc_energy_diff staged through caller-provided device memory (`scratch`,
// laid out as n_max sites | 3*n_max new spins | n_max results): no device
// or host allocation on the success path.
int energy_diff_staged(void *c, int32_t slot, int64_t n, const int64_t *sites, const double *ns, double *dE,
                       void *scratch, int64_t n_max) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(n >= 0 && n <= n_max, CSMC_ERR_INVALID, "n outside 0..capacity");
    require(n == 0 || (sites && ns && dE), CSMC_ERR_INVALID, "NULL argument");
    System &S = *C.sys[C.sys_of_slot(slot)];
    for (int64_t q = 0; q < n; q++)
        require(sites[q] >= 0 && sites[q] < S.plan.N, CSMC_ERR_INVALID, "site index out of range");
    if (n == 0) return CSMC_OK;
    int64_t *d_sites = static_cast<int64_t *>(scratch);
    double *d_ns = reinterpret_cast<double *>(d_sites + n_max);
    double *d_dE = d_ns + 3 * n_max;
    CK(cudaMemcpyAsync(d_sites, sites, n * sizeof(int64_t), cudaMemcpyHostToDevice, C.st));
    CK(cudaMemcpyAsync(d_ns, ns, 3 * n * sizeof(double), cudaMemcpyHostToDevice, C.st));
    with_args(C, S, [&](auto &a) { launch_energy_diff(a, C.chain_of.p, slot, n, d_sites, d_ns, d_dE, C.st); });
    CK(cudaMemcpyAsync(dE, d_dE, n * sizeof(double), cudaMemcpyDeviceToHost, C.st));
    sync_check(C);
    API_END
}

} // namespace csmc

extern "C" {

int csmc_total_energy(void *c, double *E) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(E != nullptr, CSMC_ERR_INVALID, "E is NULL");
    Launches L;
    energy_all(C, L);
    sync_check(C);
    chain_to_slot(C, C.E_chain, E);
    API_END
}

int csmc_magnetization(void *c, double *M) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(M != nullptr, CSMC_ERR_INVALID, "M is NULL");
    Launches L;
    magnet_all(C, L);
    sync_check(C);
    chain_to_slot(C, C.M_chain, M);
    API_END
}

int csmc_metropolis_sweep(void *c, int32_t kind, double *accepted) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(kind >= 0 && kind <= CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE, CSMC_ERR_INVALID, "unknown Metropolis kind");
    Launches L;
    const uint64_t before = C.nsweeps;
    sweep_global(C, 1, kind, 0.0, false, L);
    renorm_check(C, L, before);
    sync_check(C);
    if (accepted) {
        std::vector<double> a = download_f64(C.last_acc, C.n_chains);
        std::copy(a.begin(), a.end(), accepted);
    }
    API_END
}

int csmc_metropolis_sweep_at(void *c, int32_t kind, const double *T, int32_t n_T, double *accepted) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(kind >= 0 && kind <= CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE, CSMC_ERR_INVALID, "unknown Metropolis kind");
    require(T != nullptr && (n_T == 1 || n_T == C.n_chains), CSMC_ERR_INVALID,
            "T must hold one temperature or one per slot");
    for (int k = 0; k < n_T; k++) require(T[k] > 0, CSMC_ERR_INVALID, "temperatures must be > 0");
    Launches L;
    const uint64_t before = C.nsweeps;
    if (n_T == 1) {
        sweep_global(C, 1, kind, T[0], false, L);
    } else { // this sweep at T[slot]; mc.T of every slot and the permutation stay as they are
        const size_t bytes = (size_t)C.n_chains * sizeof(double), fbytes = (size_t)C.n_chains * sizeof(float);
        const std::vector<float> inv = reciprocals(T, C.n_chains);
        CK(cudaMemcpyAsync(C.T_stash.p, C.T_slot.p, bytes, cudaMemcpyDeviceToDevice, C.st));
        CK(cudaMemcpyAsync(C.invT_stash.p, C.invT_slot.p, fbytes, cudaMemcpyDeviceToDevice, C.st));
        CK(cudaMemcpyAsync(C.T_slot.p, T, bytes, cudaMemcpyHostToDevice, C.st));
        CK(cudaMemcpyAsync(C.invT_slot.p, inv.data(), fbytes, cudaMemcpyHostToDevice, C.st));
        sweep_global(C, 1, kind, 0.0, false, L);
        CK(cudaMemcpyAsync(C.T_slot.p, C.T_stash.p, bytes, cudaMemcpyDeviceToDevice, C.st));
        CK(cudaMemcpyAsync(C.invT_slot.p, C.invT_stash.p, fbytes, cudaMemcpyDeviceToDevice, C.st));
        CK(cudaStreamSynchronize(C.st)); // the host copy of the reciprocals is read before it goes
    }
    renorm_check(C, L, before);
    sync_check(C);
    if (accepted) {
        std::vector<double> a = download_f64(C.last_acc, C.n_chains);
        std::copy(a.begin(), a.end(), accepted);
    }
    API_END
}

int csmc_overrelax_sweep(void *c) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    Launches L;
    const uint64_t before = C.nsweeps;
    sweep_global(C, 0, 0, 0.0, false, L);
    renorm_check(C, L, before);
    sync_check(C);
    API_END
}

int csmc_deterministic_sweeps(void *c, int64_t n) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(n >= 0, CSMC_ERR_INVALID, "n_sweeps must be >= 0");
    Launches L;
    for (int64_t k = 0; k < n; k++) {
        const uint64_t before = C.nsweeps;
        sweep_global(C, 2, 0, 0.0, false, L);
        renorm_check(C, L, before);
    }
    sync_check(C);
    API_END
}

int csmc_replay(void *c, int32_t slot, int32_t kind, double T, double *sigma, int64_t n, const int64_t *sites,
                const double *u_phi, const double *u_z, const double *u_acc, uint8_t *accepted) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(C.precision == CSMC_FP64, CSMC_ERR_UNSUPPORTED, "replay needs a CSMC_FP64 context");
    require(kind >= 0 && kind <= CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE, CSMC_ERR_INVALID, "unknown Metropolis kind");
    require(slot >= 0 && slot < C.n_chains, CSMC_ERR_INVALID, "slot out of range");
    require(n >= 0 && (n == 0 || (sites && u_phi && u_z && u_acc && accepted)), CSMC_ERR_INVALID, "NULL argument");
    require(T > 0, CSMC_ERR_INVALID, "T must be > 0");
    System &S = *C.sys[C.sys_of_slot(slot)];
    for (int64_t q = 0; q < n; q++)
        require(sites[q] >= 0 && sites[q] < S.plan.N, CSMC_ERR_INVALID, "site index out of range");
    ensure_exact(C, S);
    const int r = download_i32(C.chain_of)[slot] - S.base;
    DevBuf<int64_t> ds;
    DevBuf<double> dp, dz, da, dsig;
    DevBuf<uint8_t> dacc;
    ds.upload(sites, n);
    dp.upload(u_phi, n);
    dz.upload(u_z, n);
    da.upload(u_acc, n);
    double sg = sigma ? *sigma : 60.0;
    dsig.upload(&sg, 1);
    dacc.alloc(n);
    ExactTables t{};
    t.N = S.plan.N;
    t.N2 = S.plan.N2;
    t.N3 = S.plan.N3;
    t.N4 = S.plan.N4;
    t.bs = S.xbs.p;
    t.cs = S.xcs.p;
    t.qs = S.xqs.p;
    t.bm = S.xbm.p;
    t.ct = S.xct.p;
    t.qt = S.xqt.p;
    t.field = S.xfield.p;
    t.onsite = S.xonsite.p;
    t.ref2dev = S.ref2dev.p;
    t.Np = S.plan.Np;
    t.S = S.plan.desc.S;
    ExactCons k{};
    k.w = S.cw_ref.n ? S.cw_ref.p : nullptr;
    k.g[0] = S.cons.g[0];
    k.g[1] = S.cons.g[1];
    k.g[2] = S.cons.g[2];
    k.q = S.cons.q;
    k.p = S.cons.p;
    k.c0 = S.cons.c0;
    k.weight = S.cons.weight;
    k.lambda = C.lambda_slot.p + slot;
    k.sigma0 = C.sigma0;
    if (n > 0)
        launch_replay(t, k, S.dspins.p + (size_t)r * 3 * S.plan.Np, kind, T, dsig.p, n, ds.p, dp.p, dz.p, da.p,
                      dacc.p, C.st);
    sync_check(C);
    if (n) CK(cudaMemcpy(accepted, dacc.p, n, cudaMemcpyDeviceToHost));
    if (sigma) CK(cudaMemcpy(sigma, dsig.p, sizeof(double), cudaMemcpyDeviceToHost));
    API_END
}

int csmc_run(void *c, csmc_run_params *p) {
    API_BEGIN
    run(ctx_of(c), p);
    API_END
}

int csmc_anneal(void *c, const double *temps, int32_t n_temps, int64_t t_therm, int32_t or_rate, int32_t kind,
                double sigma0, int32_t path, double *accepted) {
    API_BEGIN
    anneal(ctx_of(c), temps, n_temps, t_therm, or_rate, kind, sigma0, path, accepted);
    API_END
}

int csmc_set_cluster_size(void *c, int32_t ranks) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(ranks >= 0, CSMC_ERR_INVALID, "cluster size must be 0, 1, 2 or 4");
    CK(cudaStreamSynchronize(C.st));
    choose_cluster(C, ranks);
    upload_resident(C);
    API_END
}

int csmc_set_size_groups(void *c, int32_t on) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    CK(cudaStreamSynchronize(C.st));
    if (on) make_size_groups(C);
    else choose_cluster(C, 0);
    bool ok = true;
    for (auto &S : C.sys) ok = ok && S->resident_ok;
    upload_resident(C);
    require(ok || !on, CSMC_ERR_UNSUPPORTED, "a lattice of a size group does not fit the resident kernel");
    API_END
}

int csmc_size_groups(void *c, int32_t *n_groups) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(n_groups != nullptr, CSMC_ERR_INVALID, "n_groups is NULL");
    *n_groups = C.size_groups ? (int32_t)C.groups.size() : 0;
    API_END
}

int csmc_cluster_size(void *c, int32_t *ranks) {
    API_BEGIN
    require(ranks != nullptr, CSMC_ERR_INVALID, "ranks is NULL");
    *ranks = ctx_of(c).cl;
    API_END
}

// ------------------------------------------------------------ autotuner

namespace csmc {

// Device state a run changes, copied aside and back so that timing runs leave
// the chain exactly where it was.
struct StateCopy {
    std::vector<std::pair<void *, size_t>> parts;
    DevBuf<unsigned char> buf;
    uint32_t msweep = 0;
    uint64_t nsweeps = 0;
    explicit StateCopy(Ctx &C) {
        for (auto &S : C.sys) {
            if (C.precision == CSMC_FP32) parts.push_back({S->fspins.p, S->fspins.n * sizeof(float)});
            else parts.push_back({S->dspins.p, S->dspins.n * sizeof(double)});
        }
        parts.push_back({C.slot_of.p, C.slot_of.n * sizeof(int32_t)});
        parts.push_back({C.chain_of.p, C.chain_of.n * sizeof(int32_t)});
        for (DevBuf<double> *b : {&C.sigma_slot, &C.acc_slot, &C.exch_slot, &C.E_chain, &C.M_chain, &C.last_acc})
            parts.push_back({b->p, b->n * sizeof(double)});
        parts.push_back({C.sweep_acc.p, C.sweep_acc.n * sizeof(unsigned long long)});
        size_t total = 0;
        for (auto &q : parts) total += (q.second + 255) / 256 * 256;
        buf.alloc(total);
        copy(C, true);
        msweep = C.msweep;
        nsweeps = C.nsweeps;
    }
    void copy(Ctx &C, bool save) {
        size_t off = 0;
        for (auto &q : parts) {
            void *a = buf.p + off;
            CK(cudaMemcpyAsync(save ? a : q.first, save ? q.first : a, q.second, cudaMemcpyDeviceToDevice, C.st));
            off += (q.second + 255) / 256 * 256;
        }
    }
    void restore(Ctx &C) {
        copy(C, false);
        C.msweep = msweep;
        C.nsweeps = nsweeps;
        CK(cudaStreamSynchronize(C.st));
    }
};

// Time the resident kernel's launch configurations on the context's own
// replicas: every cluster size that fits (1, 2, 4) with the balanced block
// size and with the kernel's largest block; keep the fastest.
static void autotune(Ctx &C, const csmc_run_params *p, int n_windows, csmc_tune_entry *out, int capacity,
                     int *n_out) {
    require(p != nullptr && n_windows >= 1, CSMC_ERR_INVALID, "autotune needs run parameters and n_windows >= 1");
    *n_out = 0;
    // a run that asks for the global path has nothing to tune; an automatic
    // run also times the global path against the resident configurations
    if (p->path == CSMC_PATH_GLOBAL || p->path == CSMC_PATH_PER_REPLICA) return;
    // the constrained kinds have a single (sequential) kernel
    if (p->kind >= CSMC_METROPOLIS_CONSTRAINT) return;
    C.global_pref = false;
    bool resident = true;
    for (auto &S : C.sys) resident = resident && S->resident_ok;
    if (!resident && p->path == CSMC_PATH_AUTO) {
        C.global_pref = false;
        return; // the global path is the only one
    }
    require(resident, CSMC_ERR_UNSUPPORTED, "resident path requested but the lattices do not fit it");
    csmc_run_params q = *p;
    q.path = CSMC_PATH_RESIDENT;
    q.resident_block = 0;
    q.probe_energy = q.probe_magnetization = nullptr;
    q.probe_capacity = 0;
    q.accepted = q.exchanged = nullptr;
    const int span = q.swap_rate > 0 ? q.swap_rate : std::max(q.overrelaxation_rate, 1) * 10;
    q.n_sweeps = (int64_t)n_windows * span;
    const bool allow_persistent = C.persistent_on && C.persistent_ok; // csmc_set_persistent(0) is respected
    const bool persistent0 = C.persistent_on;
    StateCopy saved(C);
    struct Cand {
        int cl, block;
        bool persistent;
        double ms;
        bool global = false;
        bool groups = false; // size groups, each with its own launch shape
    };
    std::vector<Cand> cands;
    for (int cl : {1, 2, 4}) {
        try {
            choose_cluster(C, cl);
        } catch (const Error &) {
            continue; // this size does not apply to these lattices
        }
        bool ok = true;
        for (auto &S : C.sys) ok = ok && S->resident_ok;
        if (!ok) continue;
        upload_resident(C);
        C.block_pref = 0;
        const ResidentSel sel = resident_selection(C, *C.groups[0]);
        // the balanced block (fewest rounds per colour class), the balanced
        // blocks of one and two rounds more (fewer warps, each with more
        // registers and less waiting at the class barriers), the largest
        const int balanced = resident_block(C, *C.groups[0], 0),
                  largest = resident_max_threads(sel.fast, sel.bil, sel.ons);
        std::vector<int> blocks{balanced};
        if (sel.fast) {
            const int64_t n = resident_class_sites(C, *C.groups[0]);
            for (int extra : {1, 2}) {
                const int b = balanced_block(n, largest, extra);
                if (b >= 128 && std::find(blocks.begin(), blocks.end(), b) == blocks.end()) blocks.push_back(b);
            }
        }
        if (std::find(blocks.begin(), blocks.end(), largest) == blocks.end()) blocks.push_back(largest);
        for (int block : blocks) {
            for (bool pers : {true, false}) {
                if (pers && !(allow_persistent && C.persistent_ok)) continue;
                C.block_pref = block;
                C.persistent_on = pers;
                run(C, &q); // warm-up (first launch of this configuration)
                saved.restore(C);
                run(C, &q);
                cands.push_back({cl, block, pers && C.persistent_ok, C.last_ms / n_windows});
                saved.restore(C);
            }
        }
    }
    // lattices of very different sizes: size groups side by side, with the
    // groups' CTAs uncapped or capped so that two or three share an SM
    for (bool clusters : {true, false}) {
        if (!make_size_groups(C, clusters)) break;
        bool ok = true;
        for (auto &S : C.sys) ok = ok && S->resident_ok;
        if (!ok) continue;
        upload_resident(C);
        C.block_pref = 0;
        C.persistent_on = persistent0;
        for (int cap : {0, 448, 256}) {
            C.group_block_cap = cap;
            run(C, &q);
            saved.restore(C);
            run(C, &q);
            Cand cg{clusters ? 0 : 1, cap, false, C.last_ms / n_windows};
            cg.groups = true;
            cands.push_back(cg);
            saved.restore(C);
        }
    }
    require(!cands.empty(), CSMC_ERR_UNSUPPORTED, "no resident configuration fits these lattices");
    if (p->path == CSMC_PATH_AUTO) { // the global colour sweeps as one more candidate
        csmc_run_params g = q;
        g.path = CSMC_PATH_GLOBAL;
        run(C, &g);
        saved.restore(C);
        run(C, &g);
        Cand cg{0, 0, false, C.last_ms / n_windows};
        cg.global = true;
        cands.push_back(cg);
        saved.restore(C);
    }
    size_t best = 0;
    for (size_t k = 1; k < cands.size(); k++)
        if (cands[k].ms < cands[best].ms) best = k;
    size_t best_res = cands[best].global ? 0 : best; // resident configuration kept for explicit requests
    for (size_t k = 0; k < cands.size(); k++)
        if (!cands[k].global && cands[k].ms < cands[best_res].ms) best_res = k;
    if (cands[best_res].groups) {
        make_size_groups(C, cands[best_res].cl == 0);
        C.persistent_on = persistent0;
        C.group_block_cap = cands[best_res].block;
        C.block_pref = 0;
    } else {
        choose_cluster(C, cands[best_res].cl);
        C.persistent_on = cands[best_res].persistent;
        C.block_pref = cands[best_res].block;
    }
    upload_resident(C);
    C.global_pref = cands[best].global;
    for (size_t k = 0; k < cands.size() && (int)k < capacity; k++) {
        out[k].path = cands[k].global ? CSMC_PATH_GLOBAL : CSMC_PATH_RESIDENT;
        out[k].cluster = cands[k].groups ? -cands[k].cl : cands[k].cl; // size groups: 0 or -1
        out[k].block = cands[k].block;
        out[k].persistent = cands[k].persistent ? 1 : 0;
        out[k].ms_per_window = cands[k].ms;
        out[k].chosen = k == best ? 1 : 0;
    }
    *n_out = (int)cands.size();
}

} // namespace csmc

int csmc_autotune(void *c, const csmc_run_params *params, int32_t n_windows, csmc_tune_entry *entries,
                  int32_t capacity, int32_t *n_entries) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(n_entries != nullptr && (capacity == 0 || entries != nullptr), CSMC_ERR_INVALID, "entries missing");
    int n = 0;
    CK(cudaStreamSynchronize(C.st));
    autotune(C, params, n_windows, entries, capacity, &n);
    *n_entries = n;
    API_END
}


int csmc_structure_factor(void *c, int32_t lattice, int32_t dim, const double *positions, int64_t n_k,
                          const double *ks, double *Suv) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(lattice >= 0 && lattice < (int)C.sys.size(), CSMC_ERR_INVALID, "bad lattice index");
    require(dim >= 1 && dim <= 3, CSMC_ERR_INVALID, "dim must be 1, 2 or 3");
    require(n_k >= 0 && (n_k == 0 || (positions && ks && Suv)), CSMC_ERR_INVALID, "positions, ks or Suv missing");
    System &S = *C.sys[lattice];
    CK(cudaStreamSynchronize(C.st));
    if (C.precision == CSMC_FP32) structure_factor<float>(C, S, S.fa, dim, positions, n_k, ks, Suv);
    else structure_factor<double>(C, S, S.da, dim, positions, n_k, ks, Suv);
    API_END
}

int csmc_set_tensor_cores(void *c, int32_t on) {
    API_BEGIN
    ctx_of(c).sf_tensor = on != 0;
    API_END
}

int csmc_selftest_timeout(void *c, int32_t which) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(which == 0 || which == 1, CSMC_ERR_INVALID, "which must be 0 (mbarrier) or 1 (grid barrier)");
    CK(cudaStreamSynchronize(C.st));
    CK(cudaMemsetAsync(C.grid_bar.p, 0, sizeof(unsigned int), C.st));
    CK(launch_wait_selftest(which, C.grid_bar.p, C.error_flag.p, C.st));
    sync_check(C); // throws CSMC_ERR_TIMEOUT when the wait gave up, as it must
    throw Error(CSMC_ERR_INVALID, "self-test: a wait that cannot complete reported success");
    API_END
}

int csmc_set_persistent(void *c, int32_t on) {
    API_BEGIN
    ctx_of(c).persistent_on = on != 0;
    API_END
}

int csmc_persistent(void *c, int32_t *on) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(on != nullptr, CSMC_ERR_INVALID, "on is NULL");
    *on = C.persistent_on && C.persistent_ok ? 1 : 0;
    API_END
}

int csmc_set_renormalize(void *c, int32_t every) {
    API_BEGIN
    require(every >= 0, CSMC_ERR_INVALID, "interval must be >= 0");
    ctx_of(c).renorm_every = every;
    API_END
}

int csmc_spin_length_drift(void *c, double *drift) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(drift != nullptr, CSMC_ERR_INVALID, "drift is NULL");
    C.drift_bits.zero(C.st);
    for (auto &S : C.sys) with_args(C, *S, [&](auto &a) { launch_drift(a, C.drift_bits.p, C.st); });
    sync_check(C);
    unsigned int bits = 0;
    CK(cudaMemcpy(&bits, C.drift_bits.p, sizeof(bits), cudaMemcpyDeviceToHost));
    float f;
    std::memcpy(&f, &bits, sizeof(f));
    *drift = f;
    API_END
}

int csmc_set_chain_ids(void *c, const uint32_t *ids) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    require(ids != nullptr, CSMC_ERR_INVALID, "ids is NULL");
    CK(cudaStreamSynchronize(C.st));
    CK(cudaMemcpy(C.chain_id.p, ids, C.n_chains * sizeof(uint32_t), cudaMemcpyHostToDevice));
    API_END
}

int csmc_debug_philox(const uint32_t *ctr, const uint32_t *key, int64_t n, uint32_t *out) {
    API_BEGIN
    require(n >= 0 && (n == 0 || (ctr && key && out)), CSMC_ERR_INVALID, "NULL argument");
    if (n == 0) return CSMC_OK;
    DevBuf<uint32_t> dc, dk, dout;
    dc.upload(ctr, 4 * n);
    dk.upload(key, 2 * n);
    dout.alloc(4 * n);
    launch_philox(dc.p, dk.p, n, dout.p, 0);
    CK(cudaGetLastError());
    CK(cudaMemcpy(out, dout.p, 4 * n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    API_END
}

int csmc_debug_device_allocs(int64_t *count) {
    API_BEGIN
    require(count != nullptr, CSMC_ERR_INVALID, "count is NULL");
    *count = g_device_allocs.load();
    API_END
}

int csmc_last_run_stats(void *c, double *ms, int64_t *launches, double *sweep_kernel_ms,
                        int64_t *sweep_kernel_launches) {
    API_BEGIN
    Ctx &C = ctx_of(c);
    if (ms) *ms = C.last_ms;
    if (launches) *launches = C.last_launches;
    if (sweep_kernel_ms) *sweep_kernel_ms = C.last_kernel_ms;
    if (sweep_kernel_launches) *sweep_kernel_launches = C.last_kernel_launches;
    API_END
}

} // extern "C"
