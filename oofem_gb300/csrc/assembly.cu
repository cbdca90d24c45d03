// Deterministic assembly by gathering (K4 matrix, K5 vector).
//
// The reference scatters element matrices into the global matrix inside an
// OpenMP critical section (EngngModel::assemble engngm.C:889-1037 ->
// CompCol::assemble compcol.C:275-316). Here every node block (A,B) of the
// pattern owns the list of (element, a, b) contributions in ascending element
// order, so one thread sums its block in the same order as the serial
// reference loop: no floating-point atomics, bitwise reproducible.
#include "internal.cuh"

namespace ogb {

namespace {

// Also writes the node-block SELL copy (FP64 and FP32) when blk_slot is given:
// every entry of the ND x ND block, with prescribed rows/columns zero and an
// identity diagonal for prescribed DOFs of active nodes.
template <int ND>
__global__ void __launch_bounds__(NTHREADS) k_gather_blocks(
    int64_t nblocks, int nnpe, const int *__restrict__ blk_node, const int *__restrict__ nb_col,
    const int *__restrict__ nb_coloff, const int64_t *__restrict__ cb_ptr, const uint32_t *__restrict__ cb,
    const int *__restrict__ eq, const double *__restrict__ ke, const int64_t *__restrict__ rowptr,
    double *__restrict__ val, const int64_t *__restrict__ blk_slot, double *__restrict__ v64,
    float *__restrict__ v32)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nblocks) return;
    const int A = blk_node[k], B = nb_col[k];
    int ra[ND], cbq[ND];
    int na = 0, nbf = 0;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        ra[d] = eq[(size_t)A * ND + d];
        cbq[d] = eq[(size_t)B * ND + d];
        na += ra[d] > 0;
        nbf += cbq[d] > 0;
    }
    if (na == 0 || nbf == 0) return;
    const int64_t slot = blk_slot ? blk_slot[k] : -1;
    double s[ND][ND];
#pragma unroll
    for (int i = 0; i < ND; ++i)
#pragma unroll
        for (int j = 0; j < ND; ++j) s[i][j] = 0.0;
    const size_t blk = (size_t)ND * ND;
    for (int64_t c = cb_ptr[k]; c < cb_ptr[k + 1]; ++c) {
        uint32_t w = cb[c];
        int e = (int)(w >> 6), a = (int)((w >> 3) & 7u), b = (int)(w & 7u);
        const double *src = ke + (((size_t)e * nnpe + a) * nnpe + b) * blk;
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int j = 0; j < ND; ++j) s[i][j] += src[i * ND + j];
    }
    if (slot >= 0) {
        const int r = (int)(slot & 31);
        const int64_t vb = (slot - r) * (ND * ND) + r;
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int j = 0; j < ND; ++j) {
                double v = (ra[i] > 0 && cbq[j] > 0) ? s[i][j] : ((A == B && i == j) ? 1.0 : 0.0);
                v64[vb + 32 * (i * ND + j)] = v;
                v32[vb + 32 * (i * ND + j)] = (float)v;
            }
    }
    const int off = nb_coloff[k];
#pragma unroll
    for (int i = 0; i < ND; ++i) {
        if (ra[i] <= 0) continue;
        int64_t pos = rowptr[ra[i] - 1] + off;
        int jp = 0;
#pragma unroll
        for (int j = 0; j < ND; ++j) {
            if (cbq[j] <= 0) continue;
            val[pos + jp] = s[i][j];
            ++jp;
        }
    }
}

// f[A] = sum over incident (element, a) in ascending element order of fe[e][a].
template <int ND>
__global__ void __launch_bounds__(NTHREADS) k_gather_nodes(int nnodes, int nnpe, const int64_t *__restrict__ inc_ptr,
                                                           const uint32_t *__restrict__ inc,
                                                           const double *__restrict__ fe, double *__restrict__ f)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nnodes) return;
    double s[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) s[d] = 0.0;
    for (int64_t k = inc_ptr[A]; k < inc_ptr[A + 1]; ++k) {
        uint32_t w = inc[k];
        int e = (int)(w >> 3), a = (int)(w & 7u);
        const double *src = fe + ((size_t)e * nnpe + a) * ND;
#pragma unroll
        for (int d = 0; d < ND; ++d) s[d] += src[d];
    }
#pragma unroll
    for (int d = 0; d < ND; ++d) f[(size_t)A * ND + d] = s[d];
}

// Difference form of the FP32 SELL copy: the diagonal slot of every row
// receives the FP64 block row sum S_A = sum_B K_AB (see k_sell_spmv DIFF);
// padding rows hold one identity block, whose row sum is itself.
template <int ND>
__global__ void __launch_bounds__(NTHREADS) k_sell_rowsum(int nrows, const int64_t *__restrict__ sl_ptr,
                                                          const int *__restrict__ sl_width,
                                                          const int64_t *__restrict__ diag,
                                                          const double *__restrict__ v64, float *__restrict__ v32)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows) return;
    int s = a >> 5, r = a & 31;
    const double *vp = v64 + sl_ptr[s] * (ND * ND) + r;
    double S[ND * ND];
#pragma unroll
    for (int e = 0; e < ND * ND; ++e) S[e] = 0.0;
    for (int k = 0; k < sl_width[s]; ++k)
#pragma unroll
        for (int e = 0; e < ND * ND; ++e) S[e] += vp[(int64_t)k * 32 * ND * ND + 32 * e];
    int64_t slot = diag[a];
    float *out = v32 + (slot - r) * (ND * ND) + r;
#pragma unroll
    for (int e = 0; e < ND * ND; ++e) out[32 * e] = (float)S[e];
}

}  // namespace

int launch_gather_matrix(ogb_model *md, ogb_mtrx *m)
{
    ogb_ctx *ctx = md->ctx;
    unsigned nb = (unsigned)ceil_div(md->nblocks > 0 ? md->nblocks : 1, NTHREADS);
    const int64_t *bs = m->has_sell ? md->blk_slot.p : nullptr;
    double *v64 = m->has_sell ? m->sell.v64.p : nullptr;
    float *v32 = m->has_sell ? m->sell.v32.p : nullptr;
    if (md->ndofpn == 3)
        k_gather_blocks<3><<<nb, NTHREADS, 0, ctx->stream>>>(md->nblocks, md->nnpe, md->blk_node.p, md->nb_col.p,
                                                             md->nb_coloff.p, md->cb_ptr.p, md->cb.p, md->eq.p,
                                                             md->ke.p, m->rowptr.p, m->val.p, bs, v64, v32);
    else
        k_gather_blocks<2><<<nb, NTHREADS, 0, ctx->stream>>>(md->nblocks, md->nnpe, md->blk_node.p, md->nb_col.p,
                                                             md->nb_coloff.p, md->cb_ptr.p, md->cb.p, md->eq.p,
                                                             md->ke.p, m->rowptr.p, m->val.p, bs, v64, v32);
    if (m->has_sell && ctx->mixed_diff) {
        const SellMat &S = m->sell;
        const int nrows = S.nslices * 32;   // instances of a batch interleave active and padding rows
        unsigned nbr = (unsigned)ceil_div(nrows, NTHREADS);
        if (S.nd == 3)
            k_sell_rowsum<3><<<nbr, NTHREADS, 0, ctx->stream>>>(nrows, S.sl_ptr.p, S.sl_width.p, S.diag.p, S.v64.p,
                                                                S.v32.p);
        else
            k_sell_rowsum<2><<<nbr, NTHREADS, 0, ctx->stream>>>(nrows, S.sl_ptr.p, S.sl_width.p, S.diag.p, S.v64.p,
                                                                S.v32.p);
        count_launch(ctx);
    }
    if (m->has_sell) m->sell.v32_version = m->version + 1;   // FP32 copy written together with FP64
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    m->version++;
    return OGB_OK;
}

int launch_gather_vector(ogb_model *md, double *f_node)
{
    ogb_ctx *ctx = md->ctx;
    unsigned nb = (unsigned)ceil_div(md->nnodes, NTHREADS);
    if (md->ndofpn == 3)
        k_gather_nodes<3><<<nb, NTHREADS, 0, ctx->stream>>>(md->nnodes, md->nnpe, md->inc_ptr.p, md->inc.p, md->fe.p,
                                                            f_node);
    else
        k_gather_nodes<2><<<nb, NTHREADS, 0, ctx->stream>>>(md->nnodes, md->nnpe, md->inc_ptr.p, md->inc.p, md->fe.p,
                                                            f_node);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

}  // namespace ogb
