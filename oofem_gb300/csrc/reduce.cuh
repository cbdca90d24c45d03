// Deterministic grid-wide reductions shared by the solver and Newton kernels.
//
// Each block reduces its threads' values in a fixed order (warp shuffles, then
// the warps in index order); the last block to publish its partials sums all
// per-block partials in a fixed order. The result therefore does not depend on
// block scheduling: bitwise reproducible, no floating-point atomics.
#pragma once

#include "internal.cuh"

namespace ogb {
namespace {

template <class T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block reduction of NV values per thread; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV])
{
    __shared__ double red[NV][NTHREADS / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = warp_sum(v[k]);
        if (lane == 0) red[k][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0;
#pragma unroll
            for (int w = 0; w < NTHREADS / 32; ++w) s += red[k][w];
            v[k] = s;
        }
    }
    __syncthreads();
}

// Block reduction of per-thread values of type T: the warp sum stays in T (an
// FP32 warp sum costs no FP64 instruction), the warps are added in FP64 in
// index order. Result valid in thread 0.
template <int NV, class T>
__device__ __forceinline__ void block_sum_t(const T (&v)[NV], double (&out)[NV])
{
    __shared__ double red[NV][NTHREADS / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        T s = warp_sum(v[k]);
        if (lane == 0) red[k][warp] = (double)s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0;
#pragma unroll
            for (int w = 0; w < NTHREADS / 32; ++w) s += red[k][w];
            out[k] = s;
        }
    }
    __syncthreads();
}

// Contiguous row range [lo, hi) of this block: equal shares of n rows, rounded
// up to whole passes of NTHREADS rows (blocks past the end get an empty range).
__device__ __forceinline__ void block_range(int64_t n, int64_t &lo, int64_t &hi)
{
    const int64_t share = (n + gridDim.x - 1) / gridDim.x;
    const int64_t per = (share + NTHREADS - 1) / NTHREADS * NTHREADS;
    lo = (int64_t)blockIdx.x * per;
    hi = lo + per < n ? lo + per : n;
}

// Publish this block's partials and report (to every thread of the block)
// whether it was the last block of the grid to do so.
template <int NV>
__device__ __forceinline__ bool publish_partials(const double (&v)[NV], double *part, unsigned int *count)
{
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) part[(size_t)k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        unsigned int t = atomicAdd(count, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// Run by every thread of the last block: thread t sums partials t, t+256, ...,
// then the fixed-order block reduction; the result does not depend on which
// block finished last. Valid in thread 0; only thread 0 writes the scalars.
template <int NV>
__device__ __forceinline__ void final_sums(const double *part, double (&out)[NV])
{
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = 0;
        const double *pp = part + (size_t)k * gridDim.x;
        // L2 loads (the partials were written by other blocks before their
        // fence and count increment); independent, so a thread's loads are in
        // flight together instead of one L2 round trip per partial
#pragma unroll 8
        for (unsigned b = threadIdx.x; b < gridDim.x; b += NTHREADS) s += __ldcg(pp + b);
        out[k] = s;
    }
    block_sum<NV>(out);
}

}  // namespace
}  // namespace ogb
