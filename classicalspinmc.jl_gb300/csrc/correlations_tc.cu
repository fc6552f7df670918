// correlations_tc.cu -- compute_equal_time_correlations (spin_correlations.jl:6-43)
// of every replica of a single-precision lattice on the tensor cores.
//
//   C_a(k) = sum_i cos(k.r_i) s_i,a,   S_a(k) = sum_i sin(k.r_i) s_i,a,
//   Suv[3a+b](k) = (C_a C_b + S_a S_b) / N = Re(S_a(k) conj(S_b(k))) / N.
//
// Two GEMMs, cos and sin phases [n_k x N] times the spins [N x 3R], on
// tcgen05.mma (kind::tf32, FP32 accumulators in tensor memory).  FP32
// accuracy from TF32 operands by splitting each operand x = hi + lo (hi =
// x rounded to TF32, lo = the remainder rounded to TF32): x y ~ hi_x hi_y +
// hi_x lo_y + lo_x hi_y, the dropped lo_x lo_y being ~2^-22 |x y|.
//
// One CTA: 128 wavevectors (the MMA's M) x 64 replicas (N = 192 columns:
// replica-major, x y z), the sites in chunks of 16 (two MMA K-steps of 8).
// Warp-specialised pipeline, synchronised by mbarriers only:
//  * 16 producer warps evaluate each chunk's 128 x 16 phases (range-reduced
//    hardware sincos; the sites' positions read from the packed tiles one
//    chunk ahead) and store their TF32 halves in shared memory in the
//    no-swizzle K-major core-matrix layout (three phase stages; a quarter-warp
//    writes one 128-byte core-matrix column, so the stores are conflict-free;
//    one barrier arrival per warp);
//  * one issuer warp brings each chunk's spins -- split and laid out the same
//    way beforehand by k_sf_pack, one layout for every wavevector tile -- by
//    one bulk copy three chunks ahead (five buffers), and, once the chunk's
//    phases are written, issues its 12 MMAs (cos and sin, three products, two
//    K-steps) and commits them.
// The accumulators (cos sums in TMEM columns 0..191, sin sums in 256..447)
// are read back with tcgen05.ld and turned into the nine products in FP32,
// stored as doubles.  When there are fewer tiles than SMs, a tile's sites are
// split over several CTAs whose partial sums the last of them adds up.
//
// Every wait is bounded (one second of %globaltimer): on a timeout the CTA
// sets the error flag, waits (bounded) for the copies and the MMAs it issued,
// frees its tensor memory and returns.
#include "launch.hpp"

namespace csmc {

namespace {

constexpr int TC_PRODUCERS = 512;                 // 16 warps evaluating phases
constexpr int TC_THREADS = TC_PRODUCERS + 32;      // and one warp issuing copies and MMAs
constexpr int TC_M = 128;                          // wavevectors per CTA (MMA M)
constexpr int TC_R = 64;                           // replicas per CTA
constexpr int TC_N = 3 * TC_R;                     // MMA N: 192 spin columns
constexpr int TC_K = 16;                           // sites per chunk
constexpr int TC_CORES_K = TC_K / 4;               // 16-byte core-matrix columns per chunk (4 TF32 each)
constexpr uint32_t A_BYTES = TC_M * TC_K * 4;      // one A operand (cos or sin, hi or lo): 8 KB
constexpr uint32_t B_BYTES = TC_N * TC_K * 4;      // one B operand (hi or lo): 12 KB
constexpr uint32_t POS_BYTES = TC_K * 16;          // the chunk's site positions, x y z 0 per site
constexpr uint32_t A_STAGE = 4 * A_BYTES;          // cos hi|lo, sin hi|lo of one chunk: 32 KB
constexpr uint32_t B_STAGE = 2 * B_BYTES + POS_BYTES; // spins hi|lo and positions of one chunk
constexpr int TILE_FLOATS = (int)(B_STAGE / 4);    // one chunk of k_sf_pack's output
constexpr int A_STAGES = 3;
constexpr int B_STAGES = 5;
constexpr int B_AHEAD = 3; // a chunk's spins are copied three chunks before its MMAs are issued
constexpr uint32_t PIPE_SMEM = A_STAGES * A_STAGE + B_STAGES * B_STAGE; // 217 KB
// the epilogue's stage of the sums, [384 columns][SPAD] floats over the
// pipeline's buffers: a column of 128 wavevectors padded to 132 floats, so
// that the three components of a replica (columns 3r .. 3r + 2) of one
// wavevector fall in different banks
constexpr int SPAD = TC_M + 4;
constexpr uint32_t STAGE_SMEM = 2 * TC_N * SPAD * 4; // 198 KB
constexpr uint32_t TC_SMEM = PIPE_SMEM > STAGE_SMEM ? PIPE_SMEM : STAGE_SMEM; // one CTA per SM, which
                                                                             // takes all 512 TMEM columns
static_assert(TC_SMEM + 1024 <= 227 * 1024, "shared memory of one CTA (with its static barriers)");
static_assert(TC_SMEM + 1024 < (1u << 18), "descriptor address fields (address / 16, 14 bits) do not carry");
// the copy of chunk c + B_AHEAD reuses the buffer of chunk c + B_AHEAD - B_STAGES,
// whose MMAs the issuer waits for; that chunk must precede c
static_assert(B_STAGES > B_AHEAD, "a spin buffer is refilled only after the MMAs that read it");
constexpr uint32_t TMEM_COLS = 512; // cos 0..191, sin 256..447
constexpr uint32_t SIN_COL = 256;
constexpr uint64_t TC_BUDGET_NS = 1000000000ull;

// Byte offset of element (row, kel) of a [rows x TC_K] K-major operand in
// the no-swizzle core-matrix layout: core matrices of 8 rows x 16 bytes
// (128 contiguous bytes, rows 16 bytes apart), TC_CORES_K of them along K
// (leading byte offset 128), row groups of 8 one after another (stride byte
// offset TC_CORES_K x 128 = 512).
__host__ __device__ constexpr uint32_t core_offset(int row, int kel) {
    return (uint32_t)(((row >> 3) * TC_CORES_K + (kel >> 2)) * 128 + (row & 7) * 16 + (kel & 3) * 4);
}
constexpr uint32_t LBO = 128, SBO = TC_CORES_K * 128;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading and
// stride byte offsets (all >> 4), descriptor version 1 (bits 46-47), no
// swizzle (layout type 0, bits 61-63), base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((LBO >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((SBO >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor (tcgen05.mma kind::tf32): D F32 (bits 4-5 = 1), A and
// B TF32 (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 in
// bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                           ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
// The same rounding (to nearest, ties away from zero, on the magnitude) with
// two integer operations: add half a TF32 unit in the last place to the bits
// and clear the 13 bits below the TF32 mantissa.  For finite x.
__device__ __forceinline__ float tf32_hi(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init_(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// bounded wait for phase `parity` of an mbarrier; false on timeout (the
// timer is read only once the phase is found incomplete)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_test(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    do {
        if (mbar_test(bar, parity)) return true;
    } while (gtimer() - t0 < TC_BUDGET_NS);
    return false;
}

// Single precision sincos of t with the reduction of correlations.cu (Cody
// and Waite, 2 pi in two floats) and the hardware sine and cosine.
__device__ __forceinline__ void sincos_tc(float t, float *s, float *c) {
    const float n = rintf(t * 0.159154943091895336f);
    float r = __fmaf_rn(-n, 6.28318548202514648f, t);
    r = __fmaf_rn(-n, -1.74845553146951305e-7f, r);
    __sincosf(r, s, c);
}

// Buffer index and barrier phase of consecutive chunks in a ring of N
// buffers: chunk c has idx = c % N and phase = (c / N) & 1; next() steps to
// c + 1 (no division on the loops' paths).
template <int N> struct Ring {
    int idx = 0;
    uint32_t phase = 0;
    __device__ __forceinline__ void next() {
        if (++idx == N) {
            idx = 0;
            phase ^= 1u;
        }
    }
};

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[24], int at) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(v[at]), "=r"(v[at + 1]), "=r"(v[at + 2]), "=r"(v[at + 3]), "=r"(v[at + 4]), "=r"(v[at + 5]),
                   "=r"(v[at + 6]), "=r"(v[at + 7])
                 : "r"(taddr));
}

} // namespace

// The spins of every replica of a lattice as the MMA's B operand: for replica
// tile rt (64 replicas) and chunk c (16 device sites), the TF32 halves hi |
// lo of the [192 x 16] K-major tile (column 3 r + a = component a of replica
// r), each in the core-matrix layout, zero beyond the lattice's sites and
// replicas; then the chunk's 16 site positions (x y z 0).  packed holds
// n_rt x n_chunks x TILE_FLOATS floats; pos has 3 floats per device site for
// n_chunks x TC_K sites.
__global__ void k_sf_pack(const float *__restrict__ spins, const float *__restrict__ pos, int64_t Np, int n_rep,
                          int n_chunks, float *__restrict__ packed) {
    // one (chunk, column, site) of replica tile blockIdx.y per thread
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_chunks * TC_N * TC_K) return;
    const int rt = blockIdx.y;
    const int kel = (int)(e % TC_K);
    const int n = (int)((e / TC_K) % TC_N);
    const int c = (int)(e / ((int64_t)TC_K * TC_N));
    const int r = rt * TC_R + n / 3, a = n % 3;
    const int64_t i = (int64_t)c * TC_K + kel;
    float v = 0.f;
    if (r < n_rep && i < Np) v = spins[((int64_t)r * Np + i) * 4 + a];
    const float hi = to_tf32(v), lo = to_tf32(v - hi);
    float *tile = packed + ((int64_t)rt * n_chunks + c) * TILE_FLOATS;
    const uint32_t off = core_offset(n, kel) / 4;
    tile[off] = hi;
    tile[TC_N * TC_K + off] = lo;
    if (n == 0)
        reinterpret_cast<float4 *>(tile + 2 * TC_N * TC_K)[kel] =
            make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.f);
}

// A float widened to double with integer operations (sign kept, exponent
// rebiased by 1023 - 127, mantissa shifted up by 29 bits; infinities and NaNs
// kept; the rare subnormal float becomes a signed zero).  This GPU's FP64
// pipe runs at a small fraction of its FP32 rate, and the epilogue writes
// nine doubles per (wavevector, replica): the conversions stay off it.
__device__ __forceinline__ double widen(float f) {
    const uint32_t u = __float_as_uint(f), e = (u >> 23) & 0xFFu;
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    if (e == 0u) return __longlong_as_double((long long)sign);
    const uint64_t ex = e == 0xFFu ? 0x7FFull : (uint64_t)(e + 896u);
    return __longlong_as_double((long long)(sign | (ex << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29)));
}

// ks: 3 per wavevector; packed: k_sf_pack's tiles; out[slot][k][9].  Grid:
// (splits x wavevector tiles, replica tiles), the split fastest so that a
// tile's CTAs run together.  The sites of a tile are split
// over `splits` CTAs of split_chunks chunks each: with one split the CTA forms
// the products itself; with several, each writes its partial cos and sin sums
// to `partial` ([tile][split][384 columns][128 rows], FP32), and the last of
// the tile's CTAs to finish (counted in tile_ctr, zero before the launch)
// forms the products from all of them.
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_structure_factor_tc(const float *__restrict__ packed, int n_chunks, int split_chunks, int n_rep,
                          const float *__restrict__ ks, int64_t n_k, float inv_n,
                          const int32_t *__restrict__ slot_of, int chain_base, int slot_base,
                          double *__restrict__ out, float *__restrict__ partial, int *__restrict__ tile_ctr,
                          int splits, int *error_flag) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar_b[B_STAGES], bar_full[A_STAGES], bar_mma[A_STAGES];
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail, s_issued, s_last;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool producer = tid < TC_PRODUCERS;
    const int split = (int)(blockIdx.x % splits), kt = (int)(blockIdx.x / splits);
    const int64_t k0 = (int64_t)kt * TC_M;
    const int rt = blockIdx.y;
    const int64_t tile = (int64_t)rt * (gridDim.x / splits) + kt;
    float *const tile_partial = partial ? partial + tile * splits * (2 * TC_N) * TC_M : nullptr;
    unsigned char *const a_st = smem;                       // A_STAGES x (cos hi, cos lo, sin hi, sin lo)
    unsigned char *const b_st = smem + A_STAGES * A_STAGE; // B_STAGES x (spins hi, spins lo, positions)

    if (tid == 0) {
        for (int q = 0; q < B_STAGES; q++) mbar_init_(&bar_b[q], 1);
        for (int q = 0; q < A_STAGES; q++) {
            mbar_init_(&bar_full[q], TC_PRODUCERS / 32); // one arrival per producer warp
            mbar_init_(&bar_mma[q], 1);
        }
        s_fail = 0;
        s_issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) { // the accumulators: 512 columns of tensor memory
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    // this CTA's chunks: [c_begin, c_begin + n_my); loop indices below count from c_begin
    const int c_begin = split * split_chunks;
    const int n_my = max(0, min(n_chunks, c_begin + split_chunks) - c_begin);
    const float *tiles = packed + ((int64_t)rt * n_chunks + c_begin) * TILE_FLOATS;

    if (producer) {
        // row (wavevector) and core-matrix column (4 sites) of this thread: a
        // quarter-warp covers 8 consecutive rows of one column, 128 contiguous bytes
        const int row = 8 * warp + (lane & 7), q4 = lane >> 3;
        const int64_t k = k0 + row;
        float kx = 0.f, ky = 0.f, kz = 0.f;
        if (k < n_k) {
            kx = ks[3 * k];
            ky = ks[3 * k + 1];
            kz = ks[3 * k + 2];
        }
        const uint32_t off = core_offset(row, 4 * q4);
        // this thread's four site positions of a chunk, read from the packed
        // tiles (L2) one chunk ahead, so the phases never wait for the spins' copy
        auto positions = [&](int c, float4 (&p)[4]) {
            const float4 *g = reinterpret_cast<const float4 *>(tiles + (int64_t)c * TILE_FLOATS + 2 * TC_N * TC_K);
#pragma unroll
            for (int e = 0; e < 4; e++) p[e] = __ldg(g + 4 * q4 + e);
        };
        float4 pn[4];
        if (n_my > 0) positions(0, pn);
        Ring<A_STAGES> ra; // chunk c's phase stage
        for (int c = 0; c < n_my; c++, ra.next()) {
            const int s = ra.idx;
            float4 pc[4];
#pragma unroll
            for (int e = 0; e < 4; e++) pc[e] = pn[e];
            if (c + 1 < n_my) positions(c + 1, pn);
            bool ok = true;
            if (c >= A_STAGES) // the MMAs of chunk c - A_STAGES (same stage, previous phase) have read it
                ok = mbar_wait(&bar_mma[s], ra.phase ^ 1u);
            // decided per warp: the warp arrives on the chunk's barrier as one
            if (!__all_sync(0xffffffffu, ok && !*(volatile int *)&s_fail)) {
                s_fail = 1;
                break;
            }
            float hc[4], lc[4], hs[4], ls[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float4 r = pc[e];
                const float t = __fmaf_rn(kz, r.z, __fmaf_rn(ky, r.y, __fmul_rn(kx, r.x)));
                float sv, cv;
                sincos_tc(t, &sv, &cv);
                // hi: the phase rounded to TF32; lo: the exact remainder, of
                // which the MMA reads the TF32 part (|lo| <= 2^-11 |x|, so the
                // pair carries x to ~2^-21 of |x|)
                hc[e] = tf32_hi(cv);
                lc[e] = __fsub_rn(cv, hc[e]);
                hs[e] = tf32_hi(sv);
                ls[e] = __fsub_rn(sv, hs[e]);
            }
            unsigned char *st = a_st + s * A_STAGE;
            *reinterpret_cast<float4 *>(st + 0 * A_BYTES + off) = make_float4(hc[0], hc[1], hc[2], hc[3]);
            *reinterpret_cast<float4 *>(st + 1 * A_BYTES + off) = make_float4(lc[0], lc[1], lc[2], lc[3]);
            *reinterpret_cast<float4 *>(st + 2 * A_BYTES + off) = make_float4(hs[0], hs[1], hs[2], hs[3]);
            *reinterpret_cast<float4 *>(st + 3 * A_BYTES + off) = make_float4(ls[0], ls[1], ls[2], ls[3]);
            // every lane's stores visible to the tensor cores, then the warp counted once
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bar_full[s])) : "memory");
        }
    } else if (lane == 0) { // the issuer
        int copied = -1, landed = -1, issued = 0;
        const uint64_t desc_a0 = smem_desc(smem_addr(a_st)), desc_b0 = smem_desc(smem_addr(b_st));
        Ring<B_STAGES> rcopy; // the spin buffer of the next chunk to copy
        auto copy_chunk = [&](int cc) {
            const int q = rcopy.idx;
            rcopy.next();
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&bar_b[q])),
                         "r"(B_STAGE)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_addr(b_st + q * B_STAGE)),
                "l"(tiles + (int64_t)cc * TILE_FLOATS), "r"(B_STAGE), "r"(smem_addr(&bar_b[q]))
                : "memory");
            copied = cc;
        };
        for (int cc = 0; cc < B_AHEAD && cc < n_my; cc++) copy_chunk(cc);
        Ring<A_STAGES> ra, rj; // chunk c's phase stage; that of chunk j = c + B_AHEAD - B_STAGES
        Ring<B_STAGES> rb;     // chunk c's spin buffer
        for (int c = 0; c < n_my; c++, ra.next(), rb.next()) {
            const int s = ra.idx, q = rb.idx;
            bool ok = true;
            if (c + B_AHEAD < n_my) {
                const int j = c + B_AHEAD - B_STAGES; // the chunk whose buffer the copy reuses
                if (j >= 0) {
                    ok = mbar_wait(&bar_mma[rj.idx], rj.phase);
                    rj.next();
                }
                if (ok) copy_chunk(c + B_AHEAD);
            }
            ok = ok && mbar_wait(&bar_full[s], ra.phase);
            ok = ok && mbar_wait(&bar_b[q], rb.phase);
            if (!ok || *(volatile int *)&s_fail) {
                s_fail = 1;
                break;
            }
            landed = c;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // the operands' descriptors: the stage's base descriptor plus the
            // byte offset / 16 (shared addresses stay below 256 KB, so the
            // 14-bit address field never carries)
            const uint64_t da = desc_a0 + (uint64_t)((s * A_STAGE) >> 4), db = desc_b0 + (uint64_t)((q * B_STAGE) >> 4);
#pragma unroll
            for (int j = 0; j < TC_K / 8; j++) { // K-steps of 8 sites: two core-matrix columns
                const uint64_t kd = (uint64_t)((j * 2 * LBO) >> 4);
                const uint64_t bh = db + kd, bl = db + (B_BYTES >> 4) + kd;
#pragma unroll
                for (int ph = 0; ph < 2; ph++) { // cos, sin
                    const uint64_t ah = da + (uint64_t)(((2 * ph) * A_BYTES) >> 4) + kd;
                    const uint64_t al = da + (uint64_t)(((2 * ph + 1) * A_BYTES) >> 4) + kd;
                    const uint32_t d = tmem + (ph ? SIN_COL : 0u);
                    const uint32_t first = (c == 0 && j == 0) ? 0u : 1u; // accumulate after the first
                    const uint64_t aa[3] = {ah, ah, al}, bb[3] = {bh, bl, bh};
#pragma unroll
                    for (int p = 0; p < 3; p++) {
                        const uint32_t acc = p == 0 ? first : 1u;
                        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                                     "l"(aa[p]), "l"(bb[p]), "r"(IDESC), "r"(acc)
                                     : "memory");
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&bar_mma[s]))
                         : "memory");
            issued = c + 1;
        }
        // after a failure, the copies still in flight land before the CTA exits
        for (int cc = landed + 1; cc <= copied; cc++)
            if (!mbar_wait(&bar_b[cc % B_STAGES], (uint32_t)((cc / B_STAGES) & 1))) break;
        s_issued = issued;
    }
    __syncthreads();
    // the last chunk's MMAs (its commit follows every MMA issued before it)
    const int n_done = s_issued;
    bool ok = !s_fail;
    if (n_done > 0) {
        const int last = n_done - 1;
        const bool w = mbar_wait(&bar_mma[last % A_STAGES], (uint32_t)((last / A_STAGES) & 1));
        ok = ok && w;
    }
    ok = !__syncthreads_or(!ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // The sums of this CTA's sites, TMEM -> the stage in shared memory (the
    // pipeline's buffers, idle now: every copy has landed and every MMA that
    // read them has completed): [384 columns: cos x y z of replica 0 .. 63,
    // then sin][SPAD], FP32.  Warp w reads TMEM lanes 32 (w % 4) .. + 31 (its
    // wavevectors) for replicas 16 (w / 4) .. + 15.
    float *const stage = reinterpret_cast<float *>(smem);
    const bool have = ok && n_done == n_my && n_my > 0;
    if (have && producer) {
        const int lane_base = 32 * (warp & 3), rbase = 16 * (warp >> 2), row = lane_base + lane;
        for (int rg = 0; rg < 16; rg += 8) {
            uint32_t cv[24], sv[24];
            const uint32_t col = (uint32_t)(3 * (rbase + rg));
            const uint32_t ta = tmem + ((uint32_t)lane_base << 16) + col;
            tmem_ld8(ta, cv, 0);
            tmem_ld8(ta + 8, cv, 8);
            tmem_ld8(ta + 16, cv, 16);
            tmem_ld8(ta + SIN_COL, sv, 0);
            tmem_ld8(ta + SIN_COL + 8, sv, 8);
            tmem_ld8(ta + SIN_COL + 16, sv, 16);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int e = 0; e < 24; e++) {
                stage[(col + e) * SPAD + row] = __uint_as_float(cv[e]);
                stage[(TC_N + col + e) * SPAD + row] = __uint_as_float(sv[e]);
            }
        }
    }
    if (!have && tid == 0) atomicExch(error_flag, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    if (!have) return; // block-uniform
    // float4 i of a split's partial sums ([384][128] in global memory): column
    // i / 32, wavevectors 4 (i % 32) .. + 3; in the stage at column * SPAD / 4
    constexpr int STAGE4 = 2 * TC_N * TC_M / 4, Q4 = TC_M / 4, SPAD4 = SPAD / 4;
    float4 *const stage4 = reinterpret_cast<float4 *>(stage);
    if (splits > 1) {
        // this split's sums to the tile's partial buffer, then counted; the
        // last CTA of the tile to finish adds every split's sums, in split
        // order (the same result whichever CTA that is), into its stage
        float4 *const mine = reinterpret_cast<float4 *>(tile_partial) + (int64_t)split * STAGE4;
        for (int i = tid; i < STAGE4; i += blockDim.x) __stcg(mine + i, stage4[(i / Q4) * SPAD4 + i % Q4]);
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = atomicAdd(&tile_ctr[tile], 1) == splits - 1;
        __syncthreads();
        if (!s_last) return; // block-uniform
        __threadfence();
        const float4 *const all = reinterpret_cast<const float4 *>(tile_partial);
        for (int i = tid; i < STAGE4; i += blockDim.x) {
            float4 *const dst = stage4 + (i / Q4) * SPAD4 + i % Q4;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int z = 0; z < splits; z++) {
                const float4 v = z == split ? *dst : __ldcg(all + (int64_t)z * STAGE4 + i);
                acc.x = __fadd_rn(acc.x, v.x);
                acc.y = __fadd_rn(acc.y, v.y);
                acc.z = __fadd_rn(acc.z, v.z);
                acc.w = __fadd_rn(acc.w, v.w);
            }
            *dst = acc;
        }
        __syncthreads();
    }
    // Suv[3a+b] = (C_a C_b + S_a S_b) / N in FP32 (the sums carry FP32
    // accuracy already), stored as doubles.  A replica's 9 x (valid
    // wavevectors) outputs are contiguous: consecutive threads write
    // consecutive doubles.
    const int rows = (int)min((int64_t)TC_M, n_k - k0);
    for (int rl = 0; rl < TC_R; rl++) {
        const int r = rt * TC_R + rl;
        if (r >= n_rep) break;
        double *const o = out + ((int64_t)(slot_of[chain_base + r] - slot_base) * n_k + k0) * 9;
        for (int j = tid; j < 9 * rows; j += blockDim.x) {
            const int row = j / 9, e = j - 9 * row, a = e / 3, b = e - 3 * a;
            const float ca = stage[(3 * rl + a) * SPAD + row], cb = stage[(3 * rl + b) * SPAD + row];
            const float sa = stage[(TC_N + 3 * rl + a) * SPAD + row], sb = stage[(TC_N + 3 * rl + b) * SPAD + row];
            o[j] = widen(__fmul_rn(__fmaf_rn(ca, cb, __fmul_rn(sa, sb)), inv_n));
        }
    }
}


int64_t sf_tc_sites(int64_t Np) { return (Np + TC_K - 1) / TC_K * TC_K; }

// Splits of the sites per tile: the number s <= 8 (and <= the chunks) that
// minimises the launch's waves per unit of work, ceil(tiles s / SMs) / s
// (one CTA per SM); ties go to the smaller s.
int sf_tc_splits(int64_t n_k, int n_rep, int64_t Np, int n_sms) {
    const int64_t tiles = ((n_k + TC_M - 1) / TC_M) * ((n_rep + TC_R - 1) / TC_R);
    const int64_t chunks = sf_tc_sites(Np) / TC_K;
    int best = 1;
    double best_cost = 1e300;
    for (int s = 1; s <= 8 && s <= chunks; s++) {
        const double cost = (double)((tiles * s + n_sms - 1) / n_sms) / s;
        if (cost < best_cost - 1e-12) {
            best_cost = cost;
            best = s;
        }
    }
    return best;
}
// the partial sums and (after them, 16-byte aligned) the per-tile counters
int64_t sf_tc_partial_floats(int64_t n_k, int n_rep, int splits) {
    if (splits <= 1) return 0;
    const int64_t tiles = ((n_k + TC_M - 1) / TC_M) * ((n_rep + TC_R - 1) / TC_R);
    return (int64_t)splits * tiles * (2 * TC_N) * TC_M + (tiles + 3) / 4 * 4;
}
int64_t sf_tc_packed_floats(int64_t Np, int n_rep) {
    return (int64_t)((n_rep + TC_R - 1) / TC_R) * (sf_tc_sites(Np) / TC_K) * TILE_FLOATS;
}

cudaError_t launch_structure_factor_tc(const SysArgs<float> &a, const float *pos, const float *ks, int64_t n_k,
                                       const int32_t *slot_of, int slot_base, double *out, float *packed,
                                       float *partial, int splits, int *error_flag, cudaStream_t st) {
    if (n_k <= 0) return cudaSuccess;
    const int n_rt = (a.n_rep + TC_R - 1) / TC_R;
    const int64_t n_kt = (n_k + TC_M - 1) / TC_M;
    const int64_t n_chunks = sf_tc_sites(a.tb.Np) / TC_K;
    if (n_chunks < 1 || n_chunks * TC_N * TC_K > (int64_t)INT32_MAX || splits < 1 || (splits > 1 && !partial) ||
        (int64_t)splits * n_kt > (int64_t)INT32_MAX || n_rt > 65535)
        return cudaErrorInvalidValue;
    // every split gets at least one chunk (the buffer sized for `splits` covers the rest)
    const int split_chunks = (int)((n_chunks + splits - 1) / splits);
    splits = (int)((n_chunks + split_chunks - 1) / split_chunks);
    const int64_t per_tile = n_chunks * TC_N * TC_K;
    k_sf_pack<<<dim3((unsigned)((per_tile + 255) / 256), (unsigned)n_rt), 256, 0, st>>>(a.spins, pos, a.tb.Np,
                                                                                      a.n_rep, (int)n_chunks, packed);
    cudaError_t e = cudaFuncSetAttribute((const void *)k_structure_factor_tc,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
    if (e != cudaSuccess) return e;
    int *tile_ctr = nullptr;
    if (splits > 1) {
        tile_ctr = reinterpret_cast<int *>(partial + (int64_t)splits * n_kt * n_rt * (2 * TC_N) * TC_M);
        e = cudaMemsetAsync(tile_ctr, 0, sizeof(int) * (size_t)n_kt * n_rt, st);
        if (e != cudaSuccess) return e;
    }
    const dim3 grid((unsigned)(splits * n_kt), (unsigned)n_rt);
    k_structure_factor_tc<<<grid, TC_THREADS, TC_SMEM, st>>>(packed, (int)n_chunks, split_chunks, a.n_rep, ks, n_k,
                                                             (float)(1.0 / (double)a.n_real), slot_of, a.chain_base, slot_base, out,
                                                             splits > 1 ? partial : nullptr, tile_ctr, splits,
                                                             error_flag);
    return cudaGetLastError();
}

} // namespace csmc
