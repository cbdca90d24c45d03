// Deterministic exclusive prefix sum over int64 arrays (three-phase block scan).
// Used once per topology by the pattern builders.
#include "internal.cuh"

namespace ogb {

namespace {

constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = NTHREADS * SCAN_ITEMS;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *total)
{
    __shared__ int64_t warp_sums[NTHREADS / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < NTHREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < NTHREADS / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    int64_t base = warp > 0 ? warp_sums[warp - 1] : 0;
    if (total) *total = warp_sums[NTHREADS / 32 - 1];
    int64_t incl = x + base;
    __syncthreads();
    return incl - v;
}

__global__ void __launch_bounds__(NTHREADS) k_tile_sums(const int64_t *in, int64_t n, int64_t *sums)
{
    int64_t t0 = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        int64_t i = t0 + (int64_t)k * NTHREADS + threadIdx.x;
        if (i < n) s += in[i];
    }
    int64_t total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(NTHREADS) k_scan_sums(int64_t *sums, int64_t nt, int64_t *grand)
{
    int64_t carry = 0;
    for (int64_t base = 0; base < nt; base += NTHREADS) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < nt ? sums[i] : 0;
        int64_t total;
        int64_t ex = block_exclusive_scan(v, &total);
        if (i < nt) sums[i] = ex + carry;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(NTHREADS) k_tile_scan(const int64_t *in, int64_t n, const int64_t *sums,
                                                        int64_t *out)
{
    int64_t t0 = (int64_t)blockIdx.x * SCAN_TILE;
    // each thread owns SCAN_ITEMS consecutive items
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        int64_t i = t0 + (int64_t)threadIdx.x * SCAN_ITEMS + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int64_t ex = block_exclusive_scan(s, nullptr) + sums[blockIdx.x];
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        int64_t i = t0 + (int64_t)threadIdx.x * SCAN_ITEMS + k;
        if (i < n) out[i] = ex;
        ex += v[k];
    }
}

}  // namespace

// out[i] = sum_{k<i} in[i]; out may alias in. *total_host (optional) receives the
// grand total (synchronises the stream).
int exclusive_scan_i64(ogb_ctx *ctx, const int64_t *in, int64_t *out, int64_t n, int64_t *total_host)
{
    int64_t nt = ceil_div(n > 0 ? n : 1, SCAN_TILE);
    DBuf<int64_t> sums;
    OGB_CHECK(sums.alloc(nt + 1));
    k_tile_sums<<<(unsigned)nt, NTHREADS, 0, ctx->stream>>>(in, n, sums.p);
    k_scan_sums<<<1, NTHREADS, 0, ctx->stream>>>(sums.p, nt, sums.p + nt);
    k_tile_scan<<<(unsigned)nt, NTHREADS, 0, ctx->stream>>>(in, n, sums.p, out);
    count_launch(ctx, 3);
    OGB_CUDA(cudaGetLastError());
    if (total_host) {
        OGB_CUDA(cudaMemcpyAsync(total_host, sums.p + nt, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
        OGB_CUDA(cudaStreamSynchronize(ctx->stream));
    } else {
        OGB_CUDA(cudaStreamSynchronize(ctx->stream));  // sums is freed on return
    }
    return OGB_OK;
}

}  // namespace ogb
