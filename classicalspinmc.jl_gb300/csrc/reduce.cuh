// reduce.cuh -- warp and block reductions shared by the kernels.
#pragma once

namespace csmc {

__device__ __forceinline__ unsigned warp_sum_u(unsigned v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum within a warp in the value's own type (float, double, unsigned), in a
// fixed order; every lane gets the total.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned warp_sum(unsigned v) { return warp_sum_u(v); }

// The FP64 part of a block sum: v is the sum of the calling thread's warp
// (in its own type; lane 0 widens it: FP64 instructions run at a small
// fraction of the FP32 rate on this device, so no lane does more of them
// than it must); the n_warps warps' sums are added by warp 0 (result valid in
// thread 0).  scratch needs n_warps doubles.  Every thread must call it.
template <typename T> __device__ __forceinline__ double block_sum_warps(T v, double *scratch, int n_warps) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) scratch[w] = (double)v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = (int)threadIdx.x < n_warps ? scratch[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;
}

// Sum over a block of NT threads in a fixed order (deterministic); the result
// is valid in thread 0.  scratch needs NT/32 doubles.  Each warp sums in the
// value's type (a float warp sum is 31 single-precision adds; an unsigned one
// is exact), and the warps' sums are added in FP64 -- the FP64 work is per
// warp, not per thread, since FP64 runs at a small fraction of the FP32 rate.
template <int NT, typename T> __device__ __forceinline__ double block_sum(T v, double *scratch) {
    return block_sum_warps(warp_sum(v), scratch, NT / 32);
}

// The same for a block of any multiple of 32 threads (blockDim.x); scratch
// needs blockDim.x/32 doubles.
template <typename T> __device__ __forceinline__ double block_sum_any(T v, double *scratch) {
    return block_sum_warps(warp_sum(v), scratch, (int)(blockDim.x >> 5));
}

// N sums over a block of any multiple of 32 threads at once (one pass
// through shared memory); results valid in thread 0.  scratch needs N x 32
// doubles.  Same order per value as block_sum_any.
template <int N, typename T>
__device__ __forceinline__ void block_sumn_any(const T (&x)[N], double *scratch, double (&out)[N]) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (int)(blockDim.x >> 5);
    T v[N];
#pragma unroll
    for (int q = 0; q < N; q++) v[q] = warp_sum(x[q]);
    __syncthreads();
    if (l == 0) // widened by lane 0 alone
#pragma unroll
        for (int q = 0; q < N; q++) scratch[q * 32 + w] = (double)v[q];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; q++) {
        double t = 0.0;
        if (threadIdx.x < 32) {
            t = l < nw ? scratch[q * 32 + l] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        }
        out[q] = t;
    }
}

} // namespace csmc
