// Sparse matrix-vector product (K6), Jacobi-preconditioned CG (K7) and the
// mixed-precision iterative-refinement loop (K8).
//
// PCG restates IML++ CG (iml/cg.h:22-71) with DiagPreconditioner
// (src/core/iml/diagpre.C:40-67): x0 = incoming x, r = b - A x, stop when
// ||r_k||/||b|| <= tol on the recursively updated residual, ||b|| = 0 -> 1.
// One iteration is three kernels:
//   spmv_dot : q = A p and p.q                -> alpha = rho / p.q
//   update   : x += alpha p, r -= alpha q, z = D^-1 r, r.r, r.z -> convergence, beta
//   p_update : p = z + beta p
// Reductions: each block reduces its rows in a fixed order, the last block to
// finish sums the per-block partials in index order, so every scalar is
// bitwise reproducible. The scalars live on the device; kernels return at
// once when the system is marked done, so the host checks convergence only
// every few iterations and launches are never waited on per iteration.
#include <math.h>

#include "internal.cuh"

namespace ogb {

namespace {

constexpr int GRID_MULT = 8;   // blocks per SM for the vector kernels

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

// Publish this block's partials; returns true only in thread 0 of the last
// block, which alone runs the epilogue (reads and writes of the scalars).
template <int NV>
__device__ __forceinline__ bool publish_partials(const double (&v)[NV], double *part, unsigned int *count)
{
    if (threadIdx.x != 0) return false;
#pragma unroll
    for (int k = 0; k < NV; ++k) part[(size_t)k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(count, 1u);
    return t == gridDim.x - 1;
}

template <int NV>
__device__ __forceinline__ void final_sums(const double *part, double (&out)[NV])
{
    // executed by thread 0 of the last block: fixed index order
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = 0;
        const volatile double *pp = part + (size_t)k * gridDim.x;
        for (unsigned b = 0; b < gridDim.x; ++b) s += pp[b];
        out[k] = s;
    }
}

// ---------------------------------------------------------------- SpMV
// TPR threads per row; a block walks CHUNK rows of a chunk in passes of
// NTHREADS/TPR rows. Row r's entries are read by its TPR lanes in consecutive
// order (coalesced), the partial sums are combined by shuffles.
template <int TPR, class V, class X, bool DOT>
__global__ void __launch_bounds__(NTHREADS) k_spmv(int nchunks, const int64_t *__restrict__ rowptr,
                                                   const int *__restrict__ colind, const V *__restrict__ val,
                                                   const X *__restrict__ x, X *__restrict__ y, double *part,
                                                   unsigned int *count, PcgScal *sc)
{
    if (DOT && sc->done) return;
    constexpr int RPP = NTHREADS / TPR;   // rows per pass
    const int sub = threadIdx.x / TPR, lane = threadIdx.x % TPR;
    double acc[1] = {0.0};
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int r0 = c * CHUNK;
#pragma unroll 1
        for (int rb = 0; rb < CHUNK; rb += RPP) {
            const int row = r0 + rb + sub;
            const int64_t kb = rowptr[row], ke = rowptr[row + 1];
            X s = 0;
            for (int64_t k = kb + lane; k < ke; k += TPR) s += (X)val[k] * __ldg(x + colind[k]);
#pragma unroll
            for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
            if (lane == 0) {
                y[row] = s;
                if (DOT) acc[0] += (double)x[row] * (double)s;
            }
        }
    }
    if (!DOT) return;
    block_sum<1>(acc);
    if (publish_partials<1>(acc, part, count)) {
        double tot[1];
        final_sums<1>(part, tot);
        *count = 0;
        double pq = tot[0];
        sc->pq = pq;
        if (!(pq > 0.0) || !isfinite(pq)) {
            sc->done = 2;   // breakdown
        } else {
            sc->alpha = sc->rho / pq;
        }
    }
}

// r = b - Ax (Ax already in q), z = D^-1 r, p = z; ||b||^2, ||r||^2, r.z.
template <class X>
__global__ void __launch_bounds__(NTHREADS) k_pcg_init(int nchunks, const double *__restrict__ b,
                                                       const X *__restrict__ q, const X *__restrict__ dinv,
                                                       X *__restrict__ r, X *__restrict__ z, X *__restrict__ p,
                                                       double *part, unsigned int *count, PcgScal *sc, double rtol,
                                                       const double *bscale)
{
    double v[3] = {0, 0, 0};
    const double bs = bscale ? *bscale : 1.0;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x)
        for (int i = threadIdx.x; i < CHUNK; i += NTHREADS) {
            int row = c * CHUNK + i;
            double bb = b[row] * bs;
            X rr = (X)bb - q[row];
            X zz = rr * dinv[row];
            r[row] = rr;
            z[row] = zz;
            p[row] = zz;
            v[0] += bb * bb;
            v[1] += (double)rr * (double)rr;
            v[2] += (double)rr * (double)zz;
        }
    block_sum<3>(v);
    if (publish_partials<3>(v, part, count)) {
        double t[3];
        final_sums<3>(part, t);
        *count = 0;
        sc->bnorm2 = t[0];
        sc->rnorm2 = t[1];
        sc->rho = t[2];
        sc->iters = 0;
        double normb = sqrt(t[0]);
        if (normb == 0.0) normb = 1.0;
        if (sc->done == 0) {
            if (sqrt(t[1]) / normb <= rtol) sc->done = 1;
            else if (!isfinite(t[2]) || !(t[2] > 0.0)) sc->done = 2;
        }
    }
}

template <class X>
__global__ void __launch_bounds__(NTHREADS) k_pcg_update(int nchunks, X *__restrict__ x, X *__restrict__ r,
                                                         X *__restrict__ z, const X *__restrict__ p,
                                                         const X *__restrict__ q, const X *__restrict__ dinv,
                                                         double *part, unsigned int *count, PcgScal *sc, double rtol,
                                                         int maxit)
{
    if (sc->done) return;
    const X alpha = (X)sc->alpha;
    double v[2] = {0, 0};
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x)
        for (int i = threadIdx.x; i < CHUNK; i += NTHREADS) {
            int row = c * CHUNK + i;
            x[row] += alpha * p[row];
            X rr = r[row] - alpha * q[row];
            X zz = rr * dinv[row];
            r[row] = rr;
            z[row] = zz;
            v[0] += (double)rr * (double)rr;
            v[1] += (double)rr * (double)zz;
        }
    block_sum<2>(v);
    if (publish_partials<2>(v, part, count)) {
        double t[2];
        final_sums<2>(part, t);
        *count = 0;
        sc->rnorm2 = t[0];
        sc->iters += 1;
        double normb = sqrt(sc->bnorm2);
        if (normb == 0.0) normb = 1.0;
        double resid = sqrt(t[0]) / normb;
        if (resid <= rtol) {
            sc->done = 1;
        } else if (!isfinite(t[1]) || !(t[1] > 0.0)) {
            sc->done = 2;
        } else if (sc->iters >= maxit) {
            sc->done = 4;
        } else {
            sc->beta = t[1] / sc->rho;
            sc->rho_old = sc->rho;
            sc->rho = t[1];
        }
    }
}

template <class X>
__global__ void __launch_bounds__(NTHREADS) k_pcg_pupdate(int n, const X *__restrict__ z, X *__restrict__ p,
                                                          const PcgScal *sc)
{
    if (sc->done) return;
    const X beta = (X)sc->beta;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x)
        p[row] = z[row] + beta * p[row];
}

// D^-1 from the diagonal (DiagPreconditioner::init, diagpre.C:40-56).
template <class X, class V>
__global__ void k_diag_inv(int npad, const int64_t *__restrict__ diagpos, const V *__restrict__ val, X *dinv,
                           PcgScal *sc)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= npad) return;
    int64_t p = diagpos[r];
    double d = p >= 0 ? (double)val[p] : 0.0;
    if (d == 0.0) {
        sc->done = 3;
        dinv[r] = 0;
    } else {
        dinv[r] = (X)(1.0 / d);
    }
}

__global__ void k_to_float(int64_t n, const double *__restrict__ a, float *__restrict__ b)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// r = b - A x in FP64 (x FP64), residual norm partials; used by the refinement loop.
__global__ void __launch_bounds__(NTHREADS) k_residual64(int nchunks, const double *__restrict__ b,
                                                         const double *__restrict__ ax, double *__restrict__ r,
                                                         double *part, unsigned int *count, double *out2)
{
    double v[2] = {0, 0};
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x)
        for (int i = threadIdx.x; i < CHUNK; i += NTHREADS) {
            int row = c * CHUNK + i;
            double rr = b[row] - ax[row];
            r[row] = rr;
            v[0] += rr * rr;
            v[1] += b[row] * b[row];
        }
    block_sum<2>(v);
    if (publish_partials<2>(v, part, count)) {
        double t[2];
        final_sums<2>(part, t);
        *count = 0;
        out2[0] = t[0];
        out2[1] = t[1];
    }
}

// x64 += d32 (solution update in FP64), clears d.
__global__ void k_axpy_update(int n, double *__restrict__ x, float *__restrict__ d, double scale)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += (double)d[i] * scale;
        d[i] = 0.0f;
    }
}

inline int vec_grid(int nchunks) { return nchunks < NUM_SMS * GRID_MULT ? nchunks : NUM_SMS * GRID_MULT; }

template <class V, class X, bool DOT>
int launch_spmv_tpr(ogb_ctx *ctx, int tpr, int nchunks, int64_t nzt, const int64_t *rowptr, const int *colind,
                    const V *val, const X *x, X *y, double *part, unsigned int *count, PcgScal *sc)
{
    int g = vec_grid(nchunks);
    cudaStream_t s = ctx->stream;
    prof_begin(ctx);
    switch (tpr) {
    case 2: k_spmv<2, V, X, DOT><<<g, NTHREADS, 0, s>>>(nchunks, rowptr, colind, val, x, y, part, count, sc); break;
    case 4: k_spmv<4, V, X, DOT><<<g, NTHREADS, 0, s>>>(nchunks, rowptr, colind, val, x, y, part, count, sc); break;
    case 8: k_spmv<8, V, X, DOT><<<g, NTHREADS, 0, s>>>(nchunks, rowptr, colind, val, x, y, part, count, sc); break;
    case 16: k_spmv<16, V, X, DOT><<<g, NTHREADS, 0, s>>>(nchunks, rowptr, colind, val, x, y, part, count, sc); break;
    default: k_spmv<32, V, X, DOT><<<g, NTHREADS, 0, s>>>(nchunks, rowptr, colind, val, x, y, part, count, sc); break;
    }
    if (ctx->prof) {
        // algorithmic bytes: values + column indices + row pointers + x (once) + y
        int64_t n = (int64_t)nchunks * CHUNK;
        prof_end(ctx, (double)nzt * (sizeof(V) + sizeof(int)) + (double)(n + 1) * sizeof(int64_t) +
                          (double)n * sizeof(X) * 2);
    }
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

int ensure_workspace(ogb_mtrx *m, bool mixed)
{
    int np = m->npad;
    int nch = np / CHUNK;
    OGB_CHECK(m->w_x.alloc(np));
    OGB_CHECK(m->w_b.alloc(np));
    OGB_CHECK(m->w_part.alloc((size_t)4 * vec_grid(nch)));
    OGB_CHECK(m->w_scal.alloc(2));
    OGB_CHECK(m->h_scal.alloc(2));
    if (!m->w_count.p) {
        OGB_CHECK(m->w_count.alloc(1));
        OGB_CUDA(cudaMemsetAsync(m->w_count.p, 0, sizeof(unsigned int), m->ctx->stream));
    }
    if (!mixed) {
        OGB_CHECK(m->w_r.alloc(np));
        OGB_CHECK(m->w_z.alloc(np));
        OGB_CHECK(m->w_p.alloc(np));
        OGB_CHECK(m->w_q.alloc(np));
        OGB_CHECK(m->w_dinv.alloc(np));
    } else {
        OGB_CHECK(m->w_r.alloc(np));
        OGB_CHECK(m->w_q.alloc(np));
        OGB_CHECK(m->w_d.alloc(4));
        OGB_CHECK(m->w_r32.alloc(np));
        OGB_CHECK(m->w_z32.alloc(np));
        OGB_CHECK(m->w_p32.alloc(np));
        OGB_CHECK(m->w_q32.alloc(np));
        OGB_CHECK(m->w_dinv32.alloc(np));
        OGB_CHECK(m->w_x32.alloc(np));
    }
    return OGB_OK;
}

int read_scal(ogb_mtrx *m, PcgScal &out)
{
    OGB_CUDA(cudaMemcpyAsync(m->h_scal.p, m->w_scal.p, sizeof(PcgScal), cudaMemcpyDeviceToHost, m->ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(m->ctx->stream));
    out = *m->h_scal.p;
    prof_harvest(m->ctx);
    return OGB_OK;
}

// Generic PCG on (V matrix values, X vectors). b64 is the FP64 right-hand side
// (scaled by *bscale when given), the solution accumulates in x (type X).
template <class V, class X>
int pcg_core(ogb_mtrx *m, const V *val, const double *b64, const double *bscale, X *x, X *r, X *z, X *p, X *q,
             X *dinv, double rtol, int maxit, PcgScal &res)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    const int np = m->npad, nch = np / CHUNK;
    const int g = vec_grid(nch);
    PcgScal *sc = m->w_scal.p;
    OGB_CUDA(cudaMemsetAsync(sc, 0, sizeof(PcgScal), s));
    k_diag_inv<X, V><<<(unsigned)ceil_div(np, NTHREADS), NTHREADS, 0, s>>>(np, m->diagpos.p, val, dinv, sc);
    count_launch(ctx);
    // q = A x0
    OGB_CHECK((launch_spmv_tpr<V, X, false>(ctx, m->spmv_tpr, nch, m->nnz + (m->npad - m->neq), m->rowptr.p, m->colind.p, val, x, q, nullptr,
                                             nullptr, nullptr)));
    k_pcg_init<X><<<g, NTHREADS, 0, s>>>(nch, b64, q, dinv, r, z, p, m->w_part.p, m->w_count.p, sc, rtol, bscale);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    const int batch = 16;
    int it = 0;
    for (;;) {
        OGB_CHECK(read_scal(m, res));
        if (res.done) break;
        if (it >= maxit) break;
        for (int k = 0; k < batch; ++k) {
            OGB_CHECK((launch_spmv_tpr<V, X, true>(ctx, m->spmv_tpr, nch, m->nnz + (m->npad - m->neq), m->rowptr.p, m->colind.p, val, p, q,
                                                    m->w_part.p, m->w_count.p, sc)));
            k_pcg_update<X><<<g, NTHREADS, 0, s>>>(nch, x, r, z, p, q, dinv, m->w_part.p, m->w_count.p, sc, rtol,
                                                   maxit);
            k_pcg_pupdate<X><<<g, NTHREADS, 0, s>>>(np, z, p, sc);
            count_launch(ctx, 2);
        }
        OGB_CUDA(cudaGetLastError());
        it += batch;
    }
    return OGB_OK;
}

}  // namespace

// Threads per row from the mean row length (autotuned default).
int pick_tpr(const ogb_mtrx *m)
{
    double avg = m->neq > 0 ? (double)m->nnz / m->neq : 1.0;
    if (avg <= 6) return 2;
    if (avg <= 14) return 4;
    if (avg <= 40) return 8;
    if (avg <= 100) return 16;
    return 32;
}

int spmv64(ogb_mtrx *m, const double *x, double *y)
{
    return launch_spmv_tpr<double, double, false>(m->ctx, m->spmv_tpr, m->npad / CHUNK, m->nnz + (m->npad - m->neq),
                                                  m->rowptr.p, m->colind.p,
                                                  m->val.p, x, y, nullptr, nullptr, nullptr);
}

static int map_status(const PcgScal &s, ogb_solve_info *info)
{
    int st;
    switch (s.done) {
    case 1: st = OGB_OK; break;
    case 2: st = OGB_E_BREAKDOWN; break;
    case 3: st = OGB_E_ZERODIAG; break;
    default: st = OGB_E_NOTCONV; break;
    }
    if (info) info->status = st;
    return st;
}

// FP64 drop-in solve on padded device vectors (b, x of length npad; padding zero).
int pcg_fp64(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, ogb_solve_info *info)
{
    OGB_CHECK(ensure_workspace(m, false));
    PcgScal res{};
    OGB_CHECK((pcg_core<double, double>(m, m->val.p, b, nullptr, x, m->w_r.p, m->w_z.p, m->w_p.p, m->w_q.p,
                                        m->w_dinv.p, rtol, maxit, res)));
    double normb = sqrt(res.bnorm2);
    if (normb == 0.0) normb = 1.0;
    if (info) {
        info->iterations = res.iters;
        info->outer = 0;
        info->achieved = sqrt(res.rnorm2) / normb;
    }
    map_status(res, info);
    return OGB_OK;
}

// Mixed precision: FP32 matrix + FP32 Jacobi-PCG inner solves inside an FP64
// iterative-refinement loop; the residual f - K u and the update u += d are FP64.
int pcg_mixed(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, ogb_solve_info *info)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    OGB_CHECK(ensure_workspace(m, true));
    const int np = m->npad, nch = np / CHUNK;
    const int64_t ntot = m->nnz + (np - m->neq);
    if (m->val32_version != m->version) {
        OGB_CHECK(m->val32.alloc(ntot));
        k_to_float<<<NUM_SMS * 8, NTHREADS, 0, s>>>(ntot, m->val.p, m->val32.p);
        count_launch(ctx);
        m->val32_version = m->version;
    }
    const double inner_tol = 1e-4;
    int total_inner = 0, outer = 0;
    double achieved = 0.0;
    int status = OGB_E_NOTCONV;
    OGB_CUDA(cudaMemsetAsync(m->w_x32.p, 0, np * sizeof(float), s));
    for (outer = 0; outer < 30; ++outer) {
        // r = b - A x in FP64
        OGB_CHECK(spmv64(m, x, m->w_q.p));
        k_residual64<<<vec_grid(nch), NTHREADS, 0, s>>>(nch, b, m->w_q.p, m->w_r.p, m->w_part.p, m->w_count.p,
                                                         m->w_d.p);
        count_launch(ctx);
        double h2[2];
        OGB_CUDA(cudaMemcpyAsync(h2, m->w_d.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        OGB_CUDA(cudaStreamSynchronize(s));
        double normb = sqrt(h2[1]);
        if (normb == 0.0) normb = 1.0;
        achieved = sqrt(h2[0]) / normb;
        if (achieved <= rtol) { status = OGB_OK; break; }
        if (!isfinite(achieved)) { status = OGB_E_BREAKDOWN; break; }
        if (total_inner >= maxit) break;
        // inner FP32 solve A d = r, d0 = 0, scaled by 1/||r|| to stay in FP32 range
        double inv = 1.0 / sqrt(h2[0]);
        OGB_CUDA(cudaMemcpyAsync(m->w_d.p + 2, &inv, sizeof(double), cudaMemcpyHostToDevice, s));
        PcgScal res{};
        double tol_in = inner_tol;
        if (tol_in < rtol / achieved * 0.5) tol_in = rtol / achieved * 0.5;
        OGB_CHECK((pcg_core<float, float>(m, m->val32.p, m->w_r.p, m->w_d.p + 2, m->w_x32.p, m->w_r32.p,
                                          m->w_z32.p, m->w_p32.p, m->w_q32.p, m->w_dinv32.p, tol_in,
                                          maxit - total_inner, res)));
        total_inner += res.iters;
        if (res.done == 3) { status = OGB_E_ZERODIAG; break; }
        k_axpy_update<<<NUM_SMS * 8, NTHREADS, 0, s>>>(np, x, m->w_x32.p, sqrt(h2[0]));
        count_launch(ctx);
    }
    if (info) {
        info->iterations = total_inner;
        info->outer = outer;
        info->achieved = achieved;
        info->status = status;
    }
    return OGB_OK;
}

int extract_diag(ogb_mtrx *m) { (void)m; return OGB_OK; }

}  // namespace ogb
