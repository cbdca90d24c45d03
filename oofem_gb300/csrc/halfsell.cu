// Half-stored FP32 copy of the node-block SELL matrix (the stiffness matrix is
// symmetric: K_ac = K_ca^T), built from the full copy on the device.
//
// For every row a of the full copy (entries: the diagonal block, the blocks of
// the row's other columns, zero padding slots whose column is a itself):
//   upper list  = [diagonal] + [entries with column b > a, in full-row order]
//   lower list  = [(c, k) for entries with column c < a, in full-row order],
//                 k = position of a in row c's upper list, packed c << 6 | k.
// The lower entries of a row are exactly the transposes of upper entries of
// earlier rows (the pattern is symmetric), so every stored block is used twice
// per SpMV and the matrix stream from HBM halves. The SpMV kernel lives with
// the other SpMV forms in solver.cu.
#include "internal.cuh"

namespace ogb {

namespace {

constexpr int LOW_SHIFT = 6;            // k occupies the low six bits of a lower entry
constexpr int MAX_UPPER = 1 << LOW_SHIFT;
constexpr int64_t MAX_ROWS = int64_t(1) << (31 - LOW_SHIFT);

inline unsigned nblk(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, NTHREADS); }

__global__ void k_half_count(int nrows, const int64_t *__restrict__ sl_ptr, const int *__restrict__ sl_width,
                             const int *__restrict__ col, int *__restrict__ nU, int *__restrict__ nL)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows) return;
    const int s = a >> 5, r = a & 31, w = sl_width[s];
    const int *cp = col + sl_ptr[s] + r;
    int u = 1, l = 0;
    for (int k = 0; k < w; ++k) {
        const int c = cp[32 * k];
        u += c > a;
        l += c < a;
    }
    nU[a] = u;
    nL[a] = l;
}

// Slice widths (the longest list of the slice's 32 rows) and slot counts.
__global__ void k_half_slices(int nslices, const int *__restrict__ nU, const int *__restrict__ nL, int *wU, int *wL,
                              int64_t *ptrU, int64_t *ptrL)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > nslices) return;
    if (s == nslices) {
        ptrU[s] = ptrL[s] = 0;
        return;
    }
    int u = 0, l = 0;
    for (int r = 0; r < 32; ++r) {
        u = max(u, nU[s * 32 + r]);
        l = max(l, nL[s * 32 + r]);
    }
    wU[s] = u;
    wL[s] = l;
    ptrU[s] = (int64_t)u * 32;
    ptrL[s] = (int64_t)l * 32;
}

__global__ void k_half_fill(int nrows, const int64_t *__restrict__ sl_ptr, const int *__restrict__ sl_width,
                            const int *__restrict__ col, const int64_t *__restrict__ diag,
                            const int64_t *__restrict__ ptrU, const int *__restrict__ wU,
                            const int64_t *__restrict__ ptrL, const int *__restrict__ wL, int *__restrict__ colU,
                            int64_t *__restrict__ srcU, int *__restrict__ low, int *__restrict__ bad)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows) return;
    const int s = a >> 5, r = a & 31, w = sl_width[s];
    const int64_t base = sl_ptr[s] + r;
    int64_t u = ptrU[s] + r, l = ptrL[s] + r;
    colU[u] = a;
    srcU[u] = diag[a];
    u += 32;
    for (int k = 0; k < w; ++k) {
        const int64_t slot = base + 32 * (int64_t)k;
        const int c = col[slot];
        if (c > a) {
            colU[u] = c;
            srcU[u] = slot;
            u += 32;
        } else if (c < a) {
            // position of a in row c's upper list: its diagonal, then its
            // columns above c in full-row order up to a
            const int sc = c >> 5, rc = c & 31, wc = sl_width[sc];
            const int *cc = col + sl_ptr[sc] + rc;
            int pos = 1, j = 0;
            for (; j < wc; ++j) {
                const int b = cc[32 * j];
                if (b == a) break;
                pos += b > c;
            }
            if (j == wc) *bad = 1;   // a is not a column of row c: the pattern is not symmetric
            low[l] = j == wc ? -1 : (c << LOW_SHIFT) | pos;
            l += 32;
        }
    }
    const int64_t endU = ptrU[s] + r + 32 * (int64_t)wU[s], endL = ptrL[s] + r + 32 * (int64_t)wL[s];
    for (; u < endU; u += 32) {   // zero-valued padding blocks on the row's own column
        colU[u] = a;
        srcU[u] = -1;
    }
    for (; l < endL; l += 32) low[l] = -1;
}

// Upper values from the full FP32 copy (same lane: both slots belong to row a).
template <int ND>
__global__ void k_half_values(int64_t nslots, const int64_t *__restrict__ srcU, const float *__restrict__ full,
                              float *__restrict__ half)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nslots) return;
    const int r = (int)(t & 31);
    const int64_t src = srcU[t];
    float *out = half + (t - r) * (ND * ND) + r;
    if (src < 0) {
#pragma unroll
        for (int e = 0; e < ND * ND; ++e) out[32 * e] = 0.f;
        return;
    }
    const float *in = full + (src - r) * (ND * ND) + r;
#pragma unroll
    for (int e = 0; e < ND * ND; ++e) out[32 * e] = in[32 * e];
}

}  // namespace

int build_half(ogb_ctx *ctx, SellMat &S)
{
    HalfSell &H = S.half;
    H.tried = true;
    H.ok = false;
    H.version = -1;
    const int nslices = S.nslices, nrows = nslices * 32;
    if (nslices <= 0 || (int64_t)nrows >= MAX_ROWS) return OGB_OK;   // the packing does not fit: full copy only
    cudaStream_t st = ctx->stream;
    DBuf<int> nU, nL;
    OGB_CHECK(nU.alloc(nrows));
    OGB_CHECK(nL.alloc(nrows));
    OGB_CHECK(H.sl_ptrU.alloc(nslices + 1));
    OGB_CHECK(H.sl_ptrL.alloc(nslices + 1));
    OGB_CHECK(H.sl_widthU.alloc(nslices));
    OGB_CHECK(H.sl_widthL.alloc(nslices));
    k_half_count<<<nblk(nrows), NTHREADS, 0, st>>>(nrows, S.sl_ptr.p, S.sl_width.p, S.col.p, nU.p, nL.p);
    k_half_slices<<<nblk(nslices + 1), NTHREADS, 0, st>>>(nslices, nU.p, nL.p, H.sl_widthU.p, H.sl_widthL.p,
                                                         H.sl_ptrU.p, H.sl_ptrL.p);
    count_launch(ctx, 2);
    std::vector<int> wU(nslices);
    OGB_CUDA(cudaMemcpyAsync(wU.data(), H.sl_widthU.p, nslices * sizeof(int), cudaMemcpyDeviceToHost, st));
    OGB_CUDA(cudaStreamSynchronize(st));
    for (int w : wU)
        if (w >= MAX_UPPER) return OGB_OK;   // an upper list too long for the packing
    OGB_CHECK(exclusive_scan_i64(ctx, H.sl_ptrU.p, H.sl_ptrU.p, nslices + 1, &H.nslotsU));
    OGB_CHECK(exclusive_scan_i64(ctx, H.sl_ptrL.p, H.sl_ptrL.p, nslices + 1, &H.nslotsL));
    OGB_CHECK(H.colU.alloc(H.nslotsU));
    OGB_CHECK(H.srcU.alloc(H.nslotsU));
    OGB_CHECK(H.low.alloc(H.nslotsL > 0 ? H.nslotsL : 1));
    OGB_CHECK(H.v32.alloc((size_t)H.nslotsU * S.nd * S.nd));
    DBuf<int> bad;
    OGB_CHECK(bad.alloc(1));
    OGB_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    k_half_fill<<<nblk(nrows), NTHREADS, 0, st>>>(nrows, S.sl_ptr.p, S.sl_width.p, S.col.p, S.diag.p, H.sl_ptrU.p,
                                                 H.sl_widthU.p, H.sl_ptrL.p, H.sl_widthL.p, H.colU.p, H.srcU.p,
                                                 H.low.p, bad.p);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    int hbad = 0;
    OGB_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    OGB_CUDA(cudaStreamSynchronize(st));   // the temporaries are freed on return
    H.ok = hbad == 0;                      // an unsymmetric pattern keeps the full copy
    return OGB_OK;
}

int refresh_half(ogb_ctx *ctx, SellMat &S)
{
    HalfSell &H = S.half;
    if (!H.ok) return fail(OGB_E_STATE, "half-stored copy not built");
    if (H.version == S.v32_version) return OGB_OK;
    const int64_t n = H.nslotsU;
    if (S.nd == 3)
        k_half_values<3><<<nblk(n), NTHREADS, 0, ctx->stream>>>(n, H.srcU.p, S.v32.p, H.v32.p);
    else
        k_half_values<2><<<nblk(n), NTHREADS, 0, ctx->stream>>>(n, H.srcU.p, S.v32.p, H.v32.p);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    H.version = S.v32_version;
    return OGB_OK;
}

}  // namespace ogb
