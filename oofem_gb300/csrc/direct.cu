// Direct solver: LDL^T factorization of the equation-space matrix and the two
// triangular solves -- the device counterpart of the reference's default linear
// solver, LDLTFactorization (src/core/ldltfact.C:50-63: A.factorized() then
// backSubstitutionWith) on a Skyline matrix (src/core/skyline.C:429-491
// factorized, :248-290 backSubstitutionWith).
//
// What is kept from the reference: the matrix entries it factors (Skyline::
// assemble stores K(i,j) for i <= j only, skyline.C:189-223, so the upper
// triangle of the CSR rows is read), the factor form (unit triangular times a
// diagonal, no pivoting), and the envelope: fill-in of an LDL^T without
// pivoting stays inside each column's profile, which for the full symmetric
// pattern is bounded by the half bandwidth bw = max_i (last column of row i - i).
//
// What is GB300-native: the factor lives in a dense band of n x (bw+1) doubles
// in HBM, column-major (column j holds L(j..j+bw, j), its diagonal slot holds
// d_j), and is computed right-looking in panels of 32 columns -- one CTA
// factors the panel's 32 x 32 diagonal block in shared memory, one thread per
// row below it solves that row against the block (L21 = A21 L11^-T D^-1), then
// a 2-D grid of 32 x 32 tiles applies the panel's rank-32 update to the trailing
// band (shared-memory staged, FP64 FMAs). The solves run in one
// CTA in blocks of 32 equations: one warp resolves the 32 x 32 triangle with
// shuffles, the other warps apply the block to the rows below (forward) or
// reduce the rows below into the block (backward). Every sum has a fixed order,
// so results are bitwise reproducible. The summation order differs from the
// reference's column-by-column Crout loop, so factors agree to rounding.
#include <math.h>

#include "internal.cuh"
#include "reduce.cuh"

namespace ogb {

namespace {

constexpr int PANEL = 32;        // columns per panel
constexpr int PANEL_THREADS = 1024;
constexpr int SOLVE_THREADS = 1024;   // 32 warps: one per column of a 32-equation block

inline unsigned nblk(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, NTHREADS); }

// Half bandwidth of the first n rows: last (sorted) column of each row minus the row.
__global__ void k_ldl_bandwidth(int n, const int64_t *__restrict__ rowptr, const int *__restrict__ colind, int *bw)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t e = rowptr[i + 1];
    if (e <= rowptr[i]) return;
    const int span = colind[e - 1] - i;
    if (span > 0) atomicMax(bw, span);
}

// Band from the upper triangle of the CSR rows: entry (i, j), j >= i, is
// L-column i at offset j - i (the lower triangle K(j, i) of a symmetric matrix).
// One warp per row.
__global__ void k_ldl_fill(int n, int bw, const int64_t *__restrict__ rowptr, const int *__restrict__ colind,
                           const double *__restrict__ val, double *__restrict__ band)
{
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const int i = (int)w;
    const int64_t ld = (int64_t)bw + 1;
    for (int64_t k = rowptr[i] + lane; k < rowptr[i + 1]; k += 32) {
        const int j = colind[k];
        if (j >= i && j < n) band[(int64_t)i * ld + (j - i)] = val[k];
    }
}

// Diagonal block of panel [k0, k1) (P = k1 - k0 <= 32 columns): its lower
// triangle is loaded into shared memory (thread (r, s) of a 32 x 32 CTA owns
// entry (r, s)) and factored in place, column by column: d_j = A(j,j), the
// columns s > j receive A(r, s) -= l_rj A(s, j) (A(s, j) not yet scaled), then
// column j is scaled to l_rj = A(r, j) / d_j. L11 and D go back to the band. A
// zero or non-finite pivot sets *status to the 1-based equation and stops this
// and every later launch.
__global__ void __launch_bounds__(PANEL_THREADS) k_ldl_diag(int n, int bw, double *__restrict__ band, int k0, int k1,
                                                            int *status)
{
    if (*status) return;
    __shared__ double A[PANEL][PANEL + 1];
    __shared__ double lj[PANEL];
    const int64_t ld = (int64_t)bw + 1;
    const int P = k1 - k0;
    const int r = threadIdx.x >> 5, c = threadIdx.x & 31;
    const bool own = r < P && c <= r && r - c <= bw;
    A[r][c] = own ? band[(int64_t)(k0 + c) * ld + (r - c)] : 0.0;
    __syncthreads();
    for (int j = 0; j < P; ++j) {
        const double d = A[j][j];
        if (!(d != 0.0) || !isfinite(d)) {
            if (threadIdx.x == 0) *status = k0 + j + 1;
            return;   // every thread read the same d: a uniform exit
        }
        if (c == j && r > j && r < P) lj[r] = A[r][j] / d;
        __syncthreads();
        if (c > j && r >= c && r < P) A[r][c] -= lj[r] * A[c][j];
        __syncthreads();
        if (c == j && r > j && r < P) A[r][j] = lj[r];
        __syncthreads();
    }
    if (own) band[(int64_t)(k0 + c) * ld + (r - c)] = A[r][c];
}

// Rows below the diagonal block, one thread per row i in [k1, min(n, k1 + bw)):
// y = a L11^-T by forward substitution over the panel columns in order
// (y_j = a_j - sum_{p<j} y_p l_jp), then L(i, j) = y_j / d_j. Entries outside
// the band (i - j > bw) are zero and stay unwritten.
__global__ void __launch_bounds__(NTHREADS) k_ldl_subpanel(int n, int bw, double *__restrict__ band, int k0, int k1,
                                                           const int *status)
{
    if (*status) return;
    __shared__ double L[PANEL][PANEL + 1];
    __shared__ double dd[PANEL];
    const int64_t ld = (int64_t)bw + 1;
    const int P = k1 - k0;
    for (int t = threadIdx.x; t < PANEL * PANEL; t += blockDim.x) {
        const int r = t >> 5, c = t & 31;
        L[r][c] = (r < P && c < r && r - c <= bw) ? band[(int64_t)(k0 + c) * ld + (r - c)] : 0.0;
        if (r == c) dd[r] = r < P ? band[(int64_t)(k0 + r) * ld] : 1.0;
    }
    __syncthreads();
    const int64_t i = (int64_t)k1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t e = min((int64_t)n, (int64_t)k1 + bw);
    if (i >= e) return;
    double y[PANEL];
#pragma unroll
    for (int j = 0; j < PANEL; ++j) {
        const int64_t off = i - (k0 + j);
        y[j] = (j < P && off <= bw) ? band[(int64_t)(k0 + j) * ld + off] : 0.0;
    }
#pragma unroll
    for (int j = 1; j < PANEL; ++j) {
        double s = y[j];
#pragma unroll
        for (int p = 0; p < j; ++p) s -= y[p] * L[j][p];
        y[j] = s;
    }
#pragma unroll
    for (int j = 0; j < PANEL; ++j) {
        const int64_t off = i - (k0 + j);
        if (j < P && off <= bw) band[(int64_t)(k0 + j) * ld + off] = y[j] / dd[j];
    }
}

// Trailing update of panel [k0, k1) on the band rows/columns [k1, e),
// e = min(n, k1 + bw): A(i, c) -= sum_p L(i, p) d_p L(c, p) for c <= i, both
// within the band of the panel column p. Tile (ti, tc) of 32 x 32, lower tiles
// only; the panel rows of the tile are staged in shared memory (Li transposed,
// so the lanes read consecutive words). Lane a takes row i0 + a, so the lanes of
// a warp read and write 32 consecutive entries of one band column.
__global__ void __launch_bounds__(NTHREADS) k_ldl_trailing(int n, int bw, double *__restrict__ band, int k0, int k1,
                                                           const int *status)
{
    if (*status) return;
    const int ti = blockIdx.y, tc = blockIdx.x;
    if (ti < tc) return;
    __shared__ double Li[PANEL][32];       // L(i, p) * d_p, [p][a]
    __shared__ double Lc[32][PANEL + 1];   // L(c, p), [b][p]
    const int64_t ld = (int64_t)bw + 1;
    const int e = (int)min((int64_t)n, (int64_t)k1 + bw);
    const int i0 = k1 + 32 * ti, c0 = k1 + 32 * tc;
    const int P = k1 - k0;
    for (int t = threadIdx.x; t < 32 * PANEL; t += blockDim.x) {
        const int p = t / 32, a = t % 32;
        if (p >= P) {
            Li[p][a] = 0.0;
            Lc[a][p] = 0.0;
            continue;
        }
        const int j = k0 + p;
        const double *cjp = band + (int64_t)j * ld;
        const int i = i0 + a, c = c0 + a;
        Li[p][a] = (i < e && i - j <= bw) ? cjp[i - j] * cjp[0] : 0.0;
        Lc[a][p] = (c < e && c - j <= bw) ? cjp[c - j] : 0.0;
    }
    __syncthreads();
    const int a = threadIdx.x & 31, b0 = threadIdx.x >> 5;
    const int i = i0 + a;
    if (i >= e) return;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int b = b0 + 8 * q;
        const int c = c0 + b;
        if (c >= e || i < c || i - c > bw) continue;
        double s = 0.0;
        for (int p = 0; p < P; ++p) s += Li[p][a] * Lc[b][p];
        band[(int64_t)c * ld + (i - c)] -= s;
    }
}

// x <- (L D L^T)^-1 x, in place, one CTA of 32 warps.
__global__ void __launch_bounds__(SOLVE_THREADS) k_ldl_solve(int n, int bw, const double *__restrict__ band,
                                                             double *__restrict__ x)
{
    __shared__ double yb[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t ld = (int64_t)bw + 1;
    // forward: L y = x (unit lower), blocks of 32 equations in order
    for (int kb = 0; kb < n; kb += 32) {
        const int nbk = min(32, n - kb);
        if (warp == 0) {
            double y = lane < nbk ? x[kb + lane] : 0.0;
            for (int jj = 0; jj < nbk; ++jj) {
                const double yj = __shfl_sync(0xffffffffu, y, jj);
                if (lane > jj && lane < nbk && lane - jj <= bw) y -= band[(int64_t)(kb + jj) * ld + (lane - jj)] * yj;
            }
            if (lane < nbk) {
                x[kb + lane] = y;
                yb[lane] = y;
            }
        }
        __syncthreads();
        const int64_t iend = min((int64_t)n, (int64_t)kb + nbk + bw);
        for (int64_t i = (int64_t)kb + nbk + threadIdx.x; i < iend; i += blockDim.x) {
            double s = 0.0;
            for (int jj = 0; jj < nbk; ++jj) {
                const int64_t off = i - (kb + jj);
                if (off <= bw) s += band[(int64_t)(kb + jj) * ld + off] * yb[jj];
            }
            x[i] -= s;
        }
        __syncthreads();
    }
    // diagonal
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = x[i] / band[i * ld];
    __syncthreads();
    // backward: L^T x = y (unit upper), blocks of 32 equations from the end
    const int last = ((n - 1) / 32) * 32;
    for (int kb = last; kb >= 0; kb -= 32) {
        const int nbk = min(32, n - kb);
        if (warp < nbk) {
            const int64_t j = kb + warp;
            const int64_t iend = min((int64_t)n - 1, j + bw);
            double s = 0.0;
            for (int64_t i = (int64_t)kb + nbk + lane; i <= iend; i += 32) s += band[j * ld + (i - j)] * x[i];
            s = warp_sum(s);
            if (lane == 0) yb[warp] = x[j] - s;
        }
        __syncthreads();
        if (warp == 0) {
            double v = lane < nbk ? yb[lane] : 0.0;
            for (int jj = nbk - 1; jj >= 0; --jj) {
                const double xj = __shfl_sync(0xffffffffu, v, jj);
                if (lane < jj && jj - lane <= bw) v -= band[(int64_t)(kb + lane) * ld + (jj - lane)] * xj;
            }
            if (lane < nbk) x[kb + lane] = v;
        }
        __syncthreads();
    }
}

// ||b - y||^2 and ||b||^2 over the first n rows (y = A x), deterministic.
__global__ void __launch_bounds__(NTHREADS) k_ldl_resid(int64_t n, const double *__restrict__ b,
                                                        const double *__restrict__ y, double *part,
                                                        unsigned int *count, double *out)
{
    int64_t lo, hi;
    block_range(n, lo, hi);
    double v[2] = {0.0, 0.0};
    for (int64_t i = lo + threadIdx.x; i < hi; i += NTHREADS) {
        const double bi = b[i], r = bi - y[i];
        v[0] += r * r;
        v[1] += bi * bi;
    }
    block_sum<2>(v);
    if (publish_partials<2>(v, part, count)) {
        double s[2];
        final_sums<2>(part, s);
        if (threadIdx.x == 0) {
            out[0] = s[0];
            out[1] = s[1];
            *count = 0;
        }
    }
}

}  // namespace

// Factor m's current values (cached per matrix version).
int ldl_factor(ogb_mtrx *m)
{
    LdlFactor &F = m->ldl;
    if (F.version == m->version && F.n == m->neq && F.ok) return OGB_OK;
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    const int n = m->neq;
    F.ok = false;
    OGB_CHECK(F.d_int.alloc(2));
    OGB_CHECK(F.h_int.alloc(2));
    OGB_CUDA(cudaMemsetAsync(F.d_int.p, 0, 2 * sizeof(int), s));
    if (n > 0) {
        k_ldl_bandwidth<<<nblk(n), NTHREADS, 0, s>>>(n, m->rowptr.p, m->colind.p, F.d_int.p);
        count_launch(ctx);
    }
    OGB_CUDA(cudaMemcpyAsync(F.h_int.p, F.d_int.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    const int bw = F.h_int.p[0];
    const int64_t ld = (int64_t)bw + 1;
    const size_t need = (size_t)n * (size_t)ld;
    if (F.band.n < need) {
        size_t freeb = 0, total = 0;
        OGB_CUDA(cudaMemGetInfo(&freeb, &total));
        const size_t have = F.band.n * sizeof(double);
        if (need * sizeof(double) > (freeb + have) / 10 * 9)
            return fail(OGB_E_LIMIT, "direct solver: the band of " + std::to_string(n) + " x " + std::to_string(ld) +
                                         " doubles does not fit in device memory");
    }
    OGB_CHECK(F.band.alloc(need));
    F.n = n;
    F.bw = bw;
    if (n > 0) {
        OGB_CUDA(cudaMemsetAsync(F.band.p, 0, need * sizeof(double), s));
        k_ldl_fill<<<(unsigned)ceil_div((int64_t)n * 32, NTHREADS), NTHREADS, 0, s>>>(n, bw, m->rowptr.p, m->colind.p,
                                                                                        m->val.p, F.band.p);
        count_launch(ctx);
        int *st = F.d_int.p + 1;
        for (int k0 = 0; k0 < n; k0 += PANEL) {
            const int k1 = k0 + PANEL < n ? k0 + PANEL : n;
            k_ldl_diag<<<1, PANEL_THREADS, 0, s>>>(n, bw, F.band.p, k0, k1, st);
            count_launch(ctx);
            const int e = (int)std::min<int64_t>((int64_t)n, (int64_t)k1 + bw);
            if (e > k1) {
                k_ldl_subpanel<<<(unsigned)ceil_div(e - k1, NTHREADS), NTHREADS, 0, s>>>(n, bw, F.band.p, k0, k1, st);
                const unsigned nt = (unsigned)ceil_div(e - k1, 32);
                k_ldl_trailing<<<dim3(nt, nt), NTHREADS, 0, s>>>(n, bw, F.band.p, k0, k1, st);
                count_launch(ctx, 2);
            }
        }
        OGB_CUDA(cudaGetLastError());
    }
    OGB_CUDA(cudaMemcpyAsync(F.h_int.p + 1, F.d_int.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    if (F.h_int.p[1] != 0)
        return fail(OGB_E_ZERODIAG, "direct solver: zero or non-finite pivot at equation " +
                                        std::to_string(F.h_int.p[1]));
    F.version = m->version;
    F.ok = true;
    return OGB_OK;
}

// x = A^-1 b on padded equation-space device vectors (rows >= neq are identity
// rows: copied). The info record gets 0 iterations and the FP64 relative
// residual ||b - A x|| / ||b|| of the result.
int ldl_solve(ogb_mtrx *m, const double *b, double *x, ogb_solve_info *info)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    int r = ldl_factor(m);
    if (r == OGB_E_ZERODIAG) {
        if (info) *info = ogb_solve_info{0, 0, NAN, OGB_E_ZERODIAG};
        return OGB_OK;
    }
    OGB_CHECK(r);
    LdlFactor &F = m->ldl;
    if (x != b) OGB_CUDA(cudaMemcpyAsync(x, b, (size_t)m->npad * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (F.n > 0) {
        k_ldl_solve<<<1, SOLVE_THREADS, 0, s>>>(F.n, F.bw, F.band.p, x);
        count_launch(ctx);
    }
    OGB_CUDA(cudaGetLastError());
    if (info) {
        const int64_t np = m->npad;
        OGB_CHECK(F.y.alloc(np));
        OGB_CHECK(F.part.alloc(2 * (size_t)num_sms()));
        OGB_CHECK(F.cnt.alloc(1));
        OGB_CHECK(F.out.alloc(2));
        OGB_CHECK(F.h_out.alloc(2));
        OGB_CUDA(cudaMemsetAsync(F.cnt.p, 0, sizeof(unsigned int), s));
        OGB_CHECK(spmv64(m, x, F.y.p));
        k_ldl_resid<<<num_sms(), NTHREADS, 0, s>>>(m->neq, b, F.y.p, F.part.p, F.cnt.p, F.out.p);
        count_launch(ctx);
        OGB_CUDA(cudaMemcpyAsync(F.h_out.p, F.out.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        OGB_CUDA(cudaStreamSynchronize(s));
        double nb2 = F.h_out.p[1];
        const double normb = nb2 > 0.0 ? sqrt(nb2) : 1.0;
        info->iterations = 0;
        info->outer = 0;
        info->achieved = sqrt(F.h_out.p[0]) / normb;
        info->status = OGB_OK;
    }
    return OGB_OK;
}

}  // namespace ogb

using namespace ogb;

extern "C" {

int ogb_mtrx_set_solver(ogb_mtrx *m, int lstype)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    if (lstype != OGB_LS_DIRECT && lstype != OGB_LS_IML && lstype != OGB_LS_GPUPCG)
        return fail(OGB_E_ARG, "solver type must be 0 (direct LDL^T), 1 (IML) or 9 (GPU PCG)");
    m->lstype = lstype;
    return OGB_OK;
}

int ogb_ldlt_factorize(ogb_mtrx *m)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    return ldl_factor(m);
}

int ogb_ldlt_bandwidth(ogb_mtrx *m, int *bandwidth)
{
    if (!m || !bandwidth) return fail(OGB_E_ARG, "null argument");
    if (!m->ldl.ok || m->ldl.version != m->version) return fail(OGB_E_STATE, "matrix not factorized");
    *bandwidth = m->ldl.bw;
    return OGB_OK;
}

int ogb_ldlt_solve_dev(ogb_mtrx *m, const double *b, double *x)
{
    if (!m || !b || !x) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    cudaStream_t s = m->ctx->stream;
    OGB_CHECK(m->w_b.alloc(m->npad));
    OGB_CHECK(m->w_x.alloc(m->npad));
    OGB_CUDA(cudaMemcpyAsync(m->w_b.p, b, (size_t)m->neq * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (m->npad > m->neq)
        OGB_CUDA(cudaMemsetAsync(m->w_b.p + m->neq, 0, (size_t)(m->npad - m->neq) * sizeof(double), s));
    ogb_solve_info info{};
    OGB_CHECK(ldl_solve(m, m->w_b.p, m->w_x.p, &info));
    if (info.status != OGB_OK) return fail(info.status, "direct solver: zero or non-finite pivot");
    OGB_CUDA(cudaMemcpyAsync(x, m->w_x.p, (size_t)m->neq * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return OGB_OK;
}

int ogb_ldlt_solve(ogb_mtrx *m, const double *b, double *x)
{
    if (!m || !b || !x) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    cudaStream_t s = m->ctx->stream;
    OGB_CHECK(m->w_b.alloc(m->npad));
    OGB_CHECK(m->w_x.alloc(m->npad));
    OGB_CUDA(cudaMemcpyAsync(m->w_b.p, b, (size_t)m->neq * sizeof(double), cudaMemcpyHostToDevice, s));
    if (m->npad > m->neq)
        OGB_CUDA(cudaMemsetAsync(m->w_b.p + m->neq, 0, (size_t)(m->npad - m->neq) * sizeof(double), s));
    ogb_solve_info info{};
    OGB_CHECK(ldl_solve(m, m->w_b.p, m->w_x.p, &info));
    if (info.status != OGB_OK) return fail(info.status, "direct solver: zero or non-finite pivot");
    OGB_CUDA(cudaMemcpyAsync(x, m->w_x.p, (size_t)m->neq * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

}  // extern "C"
