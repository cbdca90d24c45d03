// Sparse matrix-vector product (K6), Jacobi-preconditioned CG (K7) and the
// mixed-precision loop with FP64 residual replacement (K8).
//
// PCG restates IML++ CG (iml/cg.h:22-71) with DiagPreconditioner
// (src/core/iml/diagpre.C:40-67): x0 = incoming x, r = b - A x, stop when
// ||r_k||/||b|| <= tol on the recursively updated residual, ||b|| = 0 -> 1.
// One iteration is three kernels:
//   spmv_dot : q = A p and p.q                -> alpha = rho / p.q
//   update   : x += alpha p, r -= alpha q, z = D^-1 r, r.r, r.z -> convergence, beta
//   p_update : p = z + beta p
// Reductions: each block reduces its rows in a fixed order, the last block to
// finish sums the per-block partials in a fixed order, so every scalar is
// bitwise reproducible. The scalars live on the device; kernels return at once
// when the system is marked done, so the host looks at them only every few
// iterations and never waits on a single launch.
//
// The operator is either the CSR matrix (drop-in SparseMtrx storage, any
// pattern) or, for matrices assembled from a mesh, the node-block SELL-32 copy
// (one column index per ND x ND block, coalesced k-major block loads), on
// node-space vectors (ND slots per active node, prescribed slots are identity
// rows with zero right-hand side).
//
// Mixed precision (OGB_PREC_MIXED): CG applies the FP32 matrix with FP32
// multiply-adds on FP32 vectors r, z, p, q; only the solution x is FP64
// (x += alpha p, the one FP64 operation per row). Whenever the recursive
// residual has dropped by a factor 10 (or reached the tolerance) it is replaced
// by the true FP64 residual r = b - A64 x64, keeping the search direction
// (reliable updates), so x converges to the solution of the FP64 system;
// convergence is decided on that FP64 residual. On node-block matrices the
// SpMV reads the half-stored FP32 copy (halfsell.cu), the preconditioner is the
// FP32 block Jacobi of the node blocks, and the update and p update are one
// cooperative launch. An FP32 operator not in difference form
// (OGB_OPT_MIXED_DIFF 0) triples the iteration count on the ill-conditioned
// cantilever; accumulating x as an FP32 increment (OGB_OPT_MIXED_X64 0 / 3,
// folded after every batch of iterations) makes an iteration cheaper but the
// solve a few per cent longer there; both stay selectable.
#include <math.h>

#include "internal.cuh"
#include "reduce.cuh"

namespace ogb {

namespace {

constexpr int GRID_MULT = 8;   // blocks per SM for the vector kernels

__device__ __forceinline__ bool halted(const PcgScal *sc) { return sc->done || sc->reliable; }

// Epilogue of the p.q reduction: alpha = rho / p.q (thread 0 of the last block).
__device__ __forceinline__ void finish_pq(double pq, unsigned int *count, PcgScal *sc)
{
    *count = 0;
    sc->pq = pq;
    if (!(pq > 0.0) || !isfinite(pq)) sc->done = 2;
    else sc->alpha = sc->rho / pq;
}

// ---------------------------------------------------------------- CSR SpMV
// TPR threads per row; a block walks CHUNK rows of a chunk in passes of
// NTHREADS/TPR rows; the lanes of a row read its entries in order (coalesced)
// and combine partial sums with shuffles.
template <int TPR, class V, class X, class ACC, bool DOT>
__global__ void __launch_bounds__(NTHREADS) k_spmv(int nchunks, const int64_t *__restrict__ rowptr,
                                                   const int *__restrict__ colind, const V *__restrict__ val,
                                                   const X *__restrict__ x, X *__restrict__ y, double *part,
                                                   unsigned int *count, PcgScal *sc)
{
    if (DOT && halted(sc)) return;
    constexpr int RPP = NTHREADS / TPR;
    const int sub = threadIdx.x / TPR, lane = threadIdx.x % TPR;
    double acc[1] = {0.0};
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int r0 = c * CHUNK;
#pragma unroll 1
        for (int rb = 0; rb < CHUNK; rb += RPP) {
            const int row = r0 + rb + sub;
            const int64_t kb = rowptr[row], ke = rowptr[row + 1];
            ACC s = 0;
            for (int64_t k = kb + lane; k < ke; k += TPR) s += (ACC)val[k] * (ACC)__ldg(x + colind[k]);
#pragma unroll
            for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
            if (lane == 0) {
                y[row] = (X)s;
                if (DOT) acc[0] += (double)x[row] * (double)s;
            }
        }
    }
    if (!DOT) return;
    block_sum<1>(acc);
    if (publish_partials<1>(acc, part, count)) {
        double t[1];
        final_sums<1>(part, t);
        if (threadIdx.x != 0) return;
        finish_pq(t[0], count, sc);
    }
}

// ---------------------------------------------------------------- SELL SpMV
// One warp per slice of 32 node rows, lane r owns row r: for every block k of
// the row it reads the block column and the ND*ND values (each a 128-byte
// coalesced warp load), gathers ND entries of x and accumulates ND outputs.
// DIFF: the values hold the difference form of the operator -- off-diagonal
// blocks K_AB and, in the diagonal slot, the block row sum S_A = sum_B K_AB --
// and the product is (K x)_A = sum_{B != A} K_AB (x_B - x_A) + S_A x_A, which is
// K x exactly but keeps the products small for smooth fields, so FP32 storage
// loses far less on the near-rigid modes that decide CG convergence.
template <int ND, class V, class X, class ACC, bool DOT, bool DIFF, int G>
__global__ void __launch_bounds__(NTHREADS) k_sell_spmv(int nslices, const int64_t *__restrict__ sl_ptr,
                                                        const int *__restrict__ sl_width, const int *__restrict__ col,
                                                        const V *__restrict__ val, const X *__restrict__ x,
                                                        X *__restrict__ y, double *part, unsigned int *count,
                                                        PcgScal *sc)
{
    if (DOT && halted(sc)) return;
    // G = 0: a plain loop over the blocks of the row, unrolled by four.
    // G > 0: blocks are taken in groups of G and the G block columns of the next
    // group are loaded while the current group's gathers and products run, so
    // the column -> x dependency does not stall every block. Which is faster
    // depends on the matrix (its width, the locality of its gathers, its size
    // against L2): sell_autotune times them per matrix and value type.
    const int s = blockIdx.x * (NTHREADS / 32) + (threadIdx.x >> 5);
    const int r = threadIdx.x & 31;
    double dot = 0.0;
    if (s < nslices) {
        const int64_t base = sl_ptr[s];
        const int w = sl_width[s];
        const int arow = s * 32 + r;
        ACC yy[ND], xa[ND];
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            yy[i] = 0;
            xa[i] = DIFF ? (ACC)x[(int64_t)arow * ND + i] : (ACC)0;
        }
        const V *vp = val + base * (ND * ND) + r;
        const int *cp = col + base + r;   // values and columns are streamed once: evict first
        if constexpr (G == 0) {
#pragma unroll 4
            for (int k = 0; k < w; ++k) {
                const int c = __ldcs(cp + 32 * k);
                ACC xb[ND];
#pragma unroll
                for (int j = 0; j < ND; ++j) {
                    xb[j] = (ACC)__ldg(x + (int64_t)c * ND + j);
                    if (DIFF && c != arow) xb[j] -= xa[j];
                }
                const V *vk = vp + (int64_t)k * (32 * ND * ND);
#pragma unroll
                for (int i = 0; i < ND; ++i)
#pragma unroll
                    for (int j = 0; j < ND; ++j) yy[i] += (ACC)__ldcs(vk + 32 * (i * ND + j)) * xb[j];
            }
        } else {
            int cn[G];
#pragma unroll
            for (int g = 0; g < G; ++g) cn[g] = g < w ? __ldcs(cp + 32 * g) : arow;
            for (int k0 = 0; k0 < w; k0 += G) {
                int cc[G];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    cc[g] = cn[g];
                    cn[g] = k0 + G + g < w ? __ldcs(cp + 32 * (k0 + G + g)) : arow;
                }
                ACC xb[G][ND];
#pragma unroll
                for (int g = 0; g < G; ++g)
#pragma unroll
                    for (int j = 0; j < ND; ++j) {
                        xb[g][j] = (ACC)__ldg(x + (int64_t)cc[g] * ND + j);
                        if (DIFF && cc[g] != arow) xb[g][j] -= xa[j];
                    }
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (k0 + g < w) {
                        const V *vk = vp + (int64_t)(k0 + g) * (32 * ND * ND);
#pragma unroll
                        for (int i = 0; i < ND; ++i)
#pragma unroll
                            for (int j = 0; j < ND; ++j) yy[i] += (ACC)__ldcs(vk + 32 * (i * ND + j)) * xb[g][j];
                    }
                }
            }
        }
        const int64_t a = (int64_t)s * 32 + r;
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            y[a * ND + i] = (X)yy[i];
            // p.q in FP64: the product of two FP32 numbers is exact in FP64
            if (DOT) dot += (double)x[a * ND + i] * (double)yy[i];
        }
    }
    if (!DOT) return;
    double acc[1] = {dot};
    block_sum<1>(acc);
    if (publish_partials<1>(acc, part, count)) {
        double t[1];
        final_sums<1>(part, t);
        if (threadIdx.x != 0) return;
        finish_pq(t[0], count, sc);
    }
}

// q = K p from the half-stored FP32 copy (halfsell.cu), fused p.q and alpha.
// Upper pass: the row's diagonal block and its blocks of columns b > a, streamed
// like k_sell_spmv (block columns prefetched G ahead). Lower pass: for every
// column c < a, the block K_ca that row c stored (slot ptrU[c / 32] + 32 k +
// c % 32 of its upper list, the entry packing c << 6 | k) applied transposed,
// K_ac = K_ca^T; the entries are prefetched G ahead.
// The upper values bypass L1 (no reuse within the block) and stay in L2, where
// the lower passes of later rows read them a second and last time (evict-first).
// DIFF: the diagonal slot holds the block row sum and the off-diagonal blocks
// act on x_c - x_a. The sum order is fixed (upper list, then lower list).
// MINB: minimum resident blocks of 256 threads per SM asked of the compiler, which
// bounds the registers per thread (6: 40; 5: 48; 4: 64; 3: 80; 2: 128). EXPL: all
// values of a group of G blocks are loaded into registers before the group's
// products (with G = 3 at 4 blocks per SM the loads of three blocks are in
// flight together: the fastest form on the 3M-DOF cantilever). The sums and
// their order depend on neither: the forms give bitwise equal results.
template <int ND, class X, bool DIFF, int G, int MINB = 4, bool EXPL = false>
__global__ void __launch_bounds__(NTHREADS, MINB) k_half_spmv(int nslices, const int64_t *__restrict__ ptrU,
                                                        const int *__restrict__ wU, const int *__restrict__ colU,
                                                        const float *__restrict__ val, const int64_t *__restrict__ ptrL,
                                                        const int *__restrict__ wL, const int *__restrict__ low,
                                                        const X *__restrict__ x, X *__restrict__ y, double *part,
                                                        unsigned int *count, PcgScal *sc)
{
    if (halted(sc)) return;
    const int s = blockIdx.x * (NTHREADS / 32) + (threadIdx.x >> 5);
    const int r = threadIdx.x & 31;
    // node c's ND entries of x
    auto gather = [&](int c, float (&v)[ND]) {
#pragma unroll
        for (int j = 0; j < ND; ++j) v[j] = (float)__ldg(x + (int64_t)c * ND + j);
    };
    double dot = 0.0;
    if (s < nslices) {
        const int arow = s * 32 + r;
        float yy[ND], xa[ND];
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            yy[i] = 0.f;
            xa[i] = (float)x[(int64_t)arow * ND + i];
        }
        {   // upper pass
            const int64_t base = ptrU[s];
            const int w = wU[s];
            const float *vp = val + base * (ND * ND) + r;
            const int *cp = colU + base + r;
            int cn[G];
#pragma unroll
            for (int g = 0; g < G; ++g) cn[g] = g < w ? __ldcs(cp + 32 * g) : arow;
            for (int k0 = 0; k0 < w; k0 += G) {
                int cc[G];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    cc[g] = cn[g];
                    cn[g] = k0 + G + g < w ? __ldcs(cp + 32 * (k0 + G + g)) : arow;
                }
                float xb[G][ND];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    gather(cc[g], xb[g]);
#pragma unroll
                    for (int j = 0; j < ND; ++j)
                        if (DIFF && cc[g] != arow) xb[g][j] -= xa[j];
                }
                if constexpr (EXPL) {
                    // every value of the group loaded before the products
                    float v[G][ND * ND];
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        const float *vk = vp + (int64_t)(k0 + g) * (32 * ND * ND);
#pragma unroll
                        for (int q = 0; q < ND * ND; ++q) v[g][q] = k0 + g < w ? __ldcg(vk + 32 * q) : 0.f;
                    }
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        if (k0 + g < w) {
#pragma unroll
                            for (int i = 0; i < ND; ++i)
#pragma unroll
                                for (int j = 0; j < ND; ++j) yy[i] += v[g][i * ND + j] * xb[g][j];
                        }
                    }
                } else {
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        if (k0 + g < w) {
                            const float *vk = vp + (int64_t)(k0 + g) * (32 * ND * ND);
#pragma unroll
                            for (int i = 0; i < ND; ++i)
#pragma unroll
                                for (int j = 0; j < ND; ++j) yy[i] += __ldcg(vk + 32 * (i * ND + j)) * xb[g][j];
                        }
                    }
                }
            }
        }
        {   // lower pass
            const int64_t base = ptrL[s];
            const int w = wL[s];
            const int *lp = low + base + r;
            int en[G];
#pragma unroll
            for (int g = 0; g < G; ++g) en[g] = g < w ? __ldcs(lp + 32 * g) : -1;
            for (int k0 = 0; k0 < w; k0 += G) {
                int e[G];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    e[g] = en[g];
                    en[g] = k0 + G + g < w ? __ldcs(lp + 32 * (k0 + G + g)) : -1;
                }
                const float *vk[G];
                float xb[G][ND];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const int c = e[g] >= 0 ? (e[g] >> 6) : arow;
                    const int kk = e[g] >= 0 ? (e[g] & 63) : 0;
                    vk[g] = val + (__ldg(ptrU + (c >> 5)) + 32 * (int64_t)kk) * (ND * ND) + (c & 31);
                    gather(c, xb[g]);
#pragma unroll
                    for (int j = 0; j < ND; ++j)
                        if (DIFF) xb[g][j] -= xa[j];
                }
                if constexpr (EXPL) {
                    float v[G][ND * ND];
#pragma unroll
                    for (int g = 0; g < G; ++g)
#pragma unroll
                        for (int q = 0; q < ND * ND; ++q) v[g][q] = e[g] >= 0 ? __ldcs(vk[g] + 32 * q) : 0.f;
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        if (e[g] >= 0) {
#pragma unroll
                            for (int i = 0; i < ND; ++i)
#pragma unroll
                                for (int j = 0; j < ND; ++j) yy[i] += v[g][j * ND + i] * xb[g][j];
                        }
                    }
                } else {
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        if (e[g] >= 0) {
#pragma unroll
                            for (int i = 0; i < ND; ++i)
#pragma unroll
                                for (int j = 0; j < ND; ++j)
                                    yy[i] += __ldcs(vk[g] + 32 * (j * ND + i)) * xb[g][j];
                        }
                    }
                }
            }
        }
        const int64_t a = (int64_t)s * 32 + r;
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            y[a * ND + i] = (X)yy[i];
            dot += (double)x[a * ND + i] * (double)yy[i];   // exact in FP64
        }
    }
    double acc[1] = {dot};
    block_sum<1>(acc);
    if (publish_partials<1>(acc, part, count)) {
        double t[1];
        final_sums<1>(part, t);
        if (threadIdx.x != 0) return;
        finish_pq(t[0], count, sc);
    }
}

// ---------------------------------------------------------------- vector kernels
// r = b - Ax (Ax in q), z = D^-1 r, p = z; ||b||^2, ||r||^2, r.z.
template <class X>
__global__ void __launch_bounds__(NTHREADS) k_pcg_init(int nchunks, const double *__restrict__ b,
                                                       const X *__restrict__ q, const X *__restrict__ dinv,
                                                       X *__restrict__ r, X *__restrict__ z, X *__restrict__ p,
                                                       double *part, unsigned int *count, PcgScal *sc, double rtol)
{
    double v[3] = {0, 0, 0};
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x)
        for (int i = threadIdx.x; i < CHUNK; i += NTHREADS) {
            int row = c * CHUNK + i;
            double bb = b[row];
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
        if (threadIdx.x != 0) return;
        *count = 0;
        sc->bnorm2 = t[0];
        sc->rnorm2 = t[1];
        sc->rho = t[2];
        sc->iters = 0;
        sc->zcoef = 1.0;
        double normb = sqrt(t[0]);
        if (normb == 0.0) normb = 1.0;
        if (sc->done == 0) {
            if (sqrt(t[1]) / normb <= rtol) sc->done = 1;
            else if (!isfinite(t[2]) || !(t[2] > 0.0)) sc->done = 2;
        }
    }
}

// Mixed update: d += alpha p (FP32 increment), r -= alpha q, z = D^-1 r. Asks
// for an FP64 residual replacement once ||r||^2 fell below drop2 times its value
// at the last one (the context's drop factor, squared) or below the tolerance;
// then rho is left for the replacement.
template <class X, class P>
__global__ void __launch_bounds__(NTHREADS) k_mixed_update(int nchunks, X *__restrict__ d, X *__restrict__ r,
                                                           X *__restrict__ z, const P *__restrict__ p,
                                                           const P *__restrict__ q, const X *__restrict__ dinv,
                                                           double *part, unsigned int *count, PcgScal *sc, int maxit)
{
    if (halted(sc)) return;
    const X alpha = (X)sc->alpha;
    double v[2] = {0, 0};
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x)
        for (int i = threadIdx.x; i < CHUNK; i += NTHREADS) {
            int row = c * CHUNK + i;
            d[row] += alpha * (X)p[row];
            X rr = r[row] - alpha * (X)q[row];
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
        if (threadIdx.x != 0) return;
        *count = 0;
        sc->rnorm2 = t[0];
        sc->iters += 1;
        if (!isfinite(t[0]) || !isfinite(t[1])) {
            sc->done = 2;
        } else if (t[0] <= sc->drop2 * sc->rmax2 || t[0] <= sc->tol2 ||
                   !(t[1] > 0.0) || sc->iters >= maxit || sc->iters >= sc->cycle_end) {
            sc->reliable = 1;
        } else {
            sc->beta = t[1] / sc->rho;
            sc->rho_old = sc->rho;
            sc->rho = t[1];
            sc->zcoef = 1.0;
        }
    }
}

// Residual replacement: r32 = r64, z = D^-1 r32, beta = r.z / rho (0 at the start).
// Plane of entry (i, j) of a symmetric ND x ND block stored as its upper
// triangle, row by row (ND = 3: 00 01 02 11 12 22; ND = 2: 00 01 11).
template <int ND>
__host__ __device__ constexpr int sym_plane(int i, int j)
{
    return i <= j ? i * ND - i * (i - 1) / 2 + (j - i) : j * ND - j * (j - 1) / 2 + (i - j);
}

// Epilogue of the replacement kernels: ||r64||^2, r.z, r.p -> rho, beta, the
// coefficient of z in the next p update and the end of the new cycle.
__device__ __forceinline__ void finish_replace(double (&v)[3], double *part, unsigned int *count, PcgScal *sc,
                                               int first, int orth, int cycle_cap)
{
    block_sum<3>(v);
    if (publish_partials<3>(v, part, count)) {
        double t[3];
        final_sums<3>(part, t);
        if (threadIdx.x != 0) return;
        *count = 0;
        sc->rmax2 = t[0];
        sc->rnorm2 = t[0];
        if (!isfinite(t[1]) || !(t[1] > 0.0)) {
            sc->done = 2;
        } else {
            sc->beta = first ? 0.0 : t[1] / sc->rho;
            // restore r.p = 0 lost by the replacement: p <- p - (r.p / r.z) z before
            // p = z + beta p, i.e. p = (1 - beta*gamma) z + beta p
            double gamma = (orth && !first) ? t[2] / t[1] : 0.0;
            sc->zcoef = 1.0 - sc->beta * gamma;
            sc->rho = t[1];
        }
        sc->reliable = 0;
        // a cycle whose recursive residual no longer falls tenfold still ends
        // after cycle_cap iterations, so the FP64 residual is looked at again
        sc->cycle_end = sc->iters + cycle_cap;
    }
}

template <class X, class P>
__global__ void __launch_bounds__(NTHREADS) k_mixed_replace(int nchunks, const double *__restrict__ r64,
                                                            X *__restrict__ r, X *__restrict__ z,
                                                            const P *__restrict__ p, const X *__restrict__ dinv,
                                                            double *part, unsigned int *count, PcgScal *sc, int first,
                                                            int orth, int cycle_cap)
{
    double v[3] = {0, 0, 0};
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x)
        for (int i = threadIdx.x; i < CHUNK; i += NTHREADS) {
            int row = c * CHUNK + i;
            double r6 = r64[row];
            X rr = (X)r6;
            X zz = rr * dinv[row];
            r[row] = rr;
            z[row] = zz;
            v[0] += r6 * r6;
            v[1] += (double)rr * (double)zz;
            v[2] += (double)rr * (double)p[row];
        }
    finish_replace(v, part, count, sc, first, orth, cycle_cap);
}

// Block-Jacobi form of k_mixed_replace: z_A = B_A^-1 r_A per node (FP32 vectors).
template <int ND, class P>
__global__ void __launch_bounds__(NTHREADS) k_mixed_replace_bj(int64_t nnodes, const double *__restrict__ r64,
                                                               float *__restrict__ r, float *__restrict__ z,
                                                               const P *__restrict__ p, const float *__restrict__ binv,
                                                               double *part, unsigned int *count, PcgScal *sc,
                                                               int first, int orth, int cycle_cap)
{
    double v[3] = {0, 0, 0};
    int64_t lo, hi;
    block_range(nnodes, lo, hi);
    for (int64_t a = lo + threadIdx.x; a < hi; a += NTHREADS) {
        float rr[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const double r6 = r64[a * ND + d];
            rr[d] = (float)r6;
            r[a * ND + d] = rr[d];
            v[0] += r6 * r6;
        }
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            float zz = 0.f;
#pragma unroll
            for (int j = 0; j < ND; ++j) zz = fmaf(binv[sym_plane<ND>(d, j) * nnodes + a], rr[j], zz);
            z[a * ND + d] = zz;
            v[1] += (double)rr[d] * (double)zz;
            v[2] += (double)rr[d] * (double)p[a * ND + d];
        }
    }
    finish_replace(v, part, count, sc, first, orth, cycle_cap);
}

// Inverse of every node's ND x ND diagonal block of the FP64 node-block copy
// (prescribed rows and columns are zero there with a unit diagonal, padding rows
// hold an identity block), stored FP32 as the ND(ND+1)/2 planes of its upper
// triangle, binv[sym_plane(i, j) * nrows + a] (the inverse of a symmetric block
// is symmetric). Cofactor formula in FP64; a singular block reports a zero pivot
// (done = 3).
template <int ND>
__global__ void k_block_inv_sell(int nrows, const int64_t *__restrict__ diag, const double *__restrict__ val,
                                 float *__restrict__ binv, PcgScal *sc)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows) return;
    const int64_t slot = diag[a];
    const int r = (int)(slot & 31);
    const double *vb = val + (slot - r) * (ND * ND) + r;
    double B[ND][ND], C[ND][ND];
#pragma unroll
    for (int i = 0; i < ND; ++i)
#pragma unroll
        for (int j = 0; j < ND; ++j) B[i][j] = vb[32 * (i * ND + j)];
    double det;
    if constexpr (ND == 3) {
        C[0][0] = B[1][1] * B[2][2] - B[1][2] * B[2][1];
        C[0][1] = B[0][2] * B[2][1] - B[0][1] * B[2][2];
        C[0][2] = B[0][1] * B[1][2] - B[0][2] * B[1][1];
        C[1][0] = B[1][2] * B[2][0] - B[1][0] * B[2][2];
        C[1][1] = B[0][0] * B[2][2] - B[0][2] * B[2][0];
        C[1][2] = B[0][2] * B[1][0] - B[0][0] * B[1][2];
        C[2][0] = B[1][0] * B[2][1] - B[1][1] * B[2][0];
        C[2][1] = B[0][1] * B[2][0] - B[0][0] * B[2][1];
        C[2][2] = B[0][0] * B[1][1] - B[0][1] * B[1][0];
        det = B[0][0] * C[0][0] + B[0][1] * C[1][0] + B[0][2] * C[2][0];
    } else {
        C[0][0] = B[1][1];
        C[0][1] = -B[0][1];
        C[1][0] = -B[1][0];
        C[1][1] = B[0][0];
        det = B[0][0] * B[1][1] - B[0][1] * B[1][0];
    }
    const bool ok = det != 0.0 && isfinite(det);
    if (!ok) sc->done = 3;
    const double inv = ok ? 1.0 / det : 0.0;
#pragma unroll
    for (int i = 0; i < ND; ++i)
#pragma unroll
        for (int j = i; j < ND; ++j) binv[(int64_t)sym_plane<ND>(i, j) * nrows + a] = (float)(C[i][j] * inv);
}

template <class X, class P = X>
__global__ void __launch_bounds__(NTHREADS) k_pcg_pupdate(int n, const X *__restrict__ z, P *__restrict__ p,
                                                          const PcgScal *sc)
{
    if (halted(sc)) return;
    const X beta = (X)sc->beta;
    const X zc = (X)sc->zcoef;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x)
        p[row] = (P)(zc * z[row] + beta * (X)p[row]);
}

// ---- FP64 x, r, z, dinv; p, q of type P. Each block owns one contiguous,
// equal share of the rows (no partly filled last wave). MIXED: the
// mixed-precision test (ask for a residual replacement); otherwise the IML
// convergence test.
template <bool MIXED, class P>
__global__ void __launch_bounds__(NTHREADS) k_update4(int64_t n, double *__restrict__ x, double *__restrict__ r,
                                                      double *__restrict__ z, const P *__restrict__ p,
                                                      const P *__restrict__ q, const double *__restrict__ dinv,
                                                      double *part, unsigned int *count, PcgScal *sc, double rtol,
                                                      int maxit)
{
    if (halted(sc)) return;
    const double alpha = sc->alpha;
    int64_t lo, hi;
    block_range(n, lo, hi);
    double v[2] = {0, 0};
#pragma unroll 4
    for (int64_t row = lo + threadIdx.x; row < hi; row += NTHREADS) {
        const double xx = x[row], dd = dinv[row];
        const double pp = (double)p[row], qq = (double)q[row];
        const double rr = r[row] - alpha * qq;
        const double zz = rr * dd;
        x[row] = xx + alpha * pp;
        r[row] = rr;
        z[row] = zz;
        v[0] += rr * rr;
        v[1] += rr * zz;
    }
    block_sum<2>(v);
    if (publish_partials<2>(v, part, count)) {
        double t[2];
        final_sums<2>(part, t);
        if (threadIdx.x != 0) return;
        *count = 0;
        sc->rnorm2 = t[0];
        sc->iters += 1;
        if (MIXED) {
            if (!isfinite(t[0]) || !isfinite(t[1])) {
                sc->done = 2;
            } else if (t[0] <= sc->drop2 * sc->rmax2 || t[0] <= sc->tol2 || !(t[1] > 0.0) || sc->iters >= maxit ||
                       sc->iters >= sc->cycle_end) {
                sc->reliable = 1;
                return;
            }
        } else {
            double normb = sqrt(sc->bnorm2);
            if (normb == 0.0) normb = 1.0;
            if (sqrt(t[0]) / normb <= rtol) { sc->done = 1; return; }
            if (!isfinite(t[1]) || !(t[1] > 0.0)) { sc->done = 2; return; }
            if (sc->iters >= maxit) { sc->done = 4; return; }
        }
        if (sc->done) return;
        sc->beta = t[1] / sc->rho;
        sc->rho_old = sc->rho;
        sc->rho = t[1];
        sc->zcoef = 1.0;
    }
}

// p = zcoef z + beta p, same block ranges.
template <class P>
__global__ void __launch_bounds__(NTHREADS) k_pupdate4(int64_t n, const double *__restrict__ z, P *__restrict__ p,
                                                       const PcgScal *sc)
{
    if (halted(sc)) return;
    const double beta = sc->beta, zc = sc->zcoef;
    int64_t lo, hi;
    block_range(n, lo, hi);
#pragma unroll 4
    for (int64_t row = lo + threadIdx.x; row < hi; row += NTHREADS) p[row] = (P)(zc * z[row] + beta * (double)p[row]);
}

// Epilogue of the mixed update kernels: block sums of r.r and r.z, and in the
// last block the convergence / replacement decision and beta.
__device__ __forceinline__ bool publish_after_sum(double (&v)[2], double *part, unsigned int *count)
{
    block_sum<2>(v);
    return publish_partials<2>(v, part, count);
}

// Run by every thread of the last block; thread 0 writes the scalars.
__device__ __forceinline__ void finish_update32_last(double *part, unsigned int *count, PcgScal *sc, int maxit)
{
    double t[2];
    final_sums<2>(part, t);
    if (threadIdx.x != 0) return;
    *count = 0;
    sc->rnorm2 = t[0];
    sc->iters += 1;
    if (!isfinite(t[0]) || !isfinite(t[1])) {
        sc->done = 2;
    } else if (t[0] <= sc->drop2 * sc->rmax2 || t[0] <= sc->tol2 || !(t[1] > 0.0) || sc->iters >= maxit ||
               sc->iters >= sc->cycle_end) {
        sc->reliable = 1;
    } else {
        sc->beta = t[1] / sc->rho;
        sc->rho_old = sc->rho;
        sc->rho = t[1];
        sc->zcoef = 1.0;
    }
}

__device__ __forceinline__ void finish_update32(double (&v)[2], double *part, unsigned int *count, PcgScal *sc,
                                                int maxit)
{
    if (publish_after_sum(v, part, count)) finish_update32_last(part, count, sc, maxit);
}

// Mixed update with FP32 r, z, dinv, p, q and the FP64 solution x: the FP64
// arithmetic per row is x += alpha p and a quarter of the dot-product sums.
// Each block owns one contiguous, equal share of the rows (no tail of partly
// filled waves).
__global__ void __launch_bounds__(NTHREADS) k_update_rz32(int64_t n, double *__restrict__ x, float *__restrict__ r,
                                                          float *__restrict__ z, const float *__restrict__ p,
                                                          const float *__restrict__ q, const float *__restrict__ dinv,
                                                          double *part, unsigned int *count, PcgScal *sc, int maxit)
{
    if (halted(sc)) return;
    const double alpha = sc->alpha;
    const float af = (float)alpha;
    int64_t lo, hi;
    block_range(n, lo, hi);
    double v[2] = {0.0, 0.0};
    // groups of four rows (t, t+256, t+512, t+768 of the block's range): loads
    // first, FP32 sums within a group, FP64 across groups and in the block sum
    int64_t row = lo + threadIdx.x;
    for (; row + 3 * NTHREADS < hi; row += 4 * NTHREADS) {
        double xx[4];
        float rr[4], pp[4], qq[4], dd[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t i = row + k * NTHREADS;
            xx[k] = x[i];
            rr[k] = r[i];
            pp[k] = p[i];
            qq[k] = q[i];
            dd[k] = dinv[i];
        }
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t i = row + k * NTHREADS;
            rr[k] = fmaf(-af, qq[k], rr[k]);
            const float zz = rr[k] * dd[k];
            x[i] = xx[k] + alpha * (double)pp[k];
            r[i] = rr[k];
            z[i] = zz;
            s0 = fmaf(rr[k], rr[k], s0);
            s1 = fmaf(rr[k], zz, s1);
        }
        v[0] += (double)s0;
        v[1] += (double)s1;
    }
    for (; row < hi; row += NTHREADS) {
        const float rr = fmaf(-af, q[row], r[row]);
        const float zz = rr * dinv[row];
        x[row] += alpha * (double)p[row];
        r[row] = rr;
        z[row] = zz;
        v[0] += (double)(rr * rr);
        v[1] += (double)(rr * zz);
    }
    finish_update32(v, part, count, sc, maxit);
}

// Block-Jacobi form of k_update_rz32 (node-space vectors, ND rows per node):
// z_A = B_A^-1 r_A with the FP32 inverse of node A's ND x ND diagonal block,
// stored as the planes of its upper triangle (coalesced loads). A thread takes
// UNR nodes of the block's node range per pass (nodes a, a + 256, ...), all their
// loads issued before the arithmetic; the grid is one wave of resident blocks.
// XS: the solution accumulator, double (the FP64 solution, x += alpha p) or
// float (the FP32 increment of the current batch of iterations, folded into the
// FP64 solution after each batch; the thread's dot-product terms are then summed
// in FP32 before the FP64 block sums, so no FP64 work is done per node).
// FUSE: the p update of the same iteration follows in this kernel. The blocks
// keep their z in shared memory (zcap nodes; a larger range writes z to memory
// and reads it back), the last block publishes beta and advances *epoch, and
// every other block waits for that advance before p = zcoef z + beta p over its
// own rows. The launch is cooperative (all blocks resident), and the wait is
// bounded: past about a second the block sets done = 5 and returns.
constexpr int DONE_WAIT_TIMEOUT = 5;

template <int ND, class XS, bool FUSE, bool SUM32 = (sizeof(XS) == 4), int UNR = 2>
__global__ void __launch_bounds__(NTHREADS) k_update_bj32(int64_t nnodes, XS *__restrict__ x,
                                                          float *__restrict__ r, float *__restrict__ z,
                                                          float *__restrict__ p, const float *__restrict__ q,
                                                          const float *__restrict__ binv, double *part,
                                                          unsigned int *count, unsigned int *epoch, int zcap,
                                                          PcgScal *sc, int maxit)
{
    extern __shared__ float zs[];
    if (halted(sc)) return;
    constexpr int NSYM = ND * (ND + 1) / 2;
    unsigned int e0 = 0;
    if (FUSE && threadIdx.x == 0) e0 = *(volatile unsigned int *)epoch;
    const double alpha = sc->alpha;
    const float af = (float)alpha;
    int64_t lo, hi;
    block_range(nnodes, lo, hi);
    const bool zsm = FUSE && hi - lo <= zcap;
    double v[2] = {0.0, 0.0};
    float vf[2] = {0.f, 0.f};   // SUM32: the thread's sums in FP32 (no FP64 work per node for them)
    for (int64_t a0 = lo + threadIdx.x; a0 < hi; a0 += (int64_t)UNR * NTHREADS) {
        float rr[UNR][ND], bb[UNR][NSYM], pp[UNR][ND];
        XS xx[UNR][ND];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int64_t a = a0 + (int64_t)u * NTHREADS;
            if (a >= hi) continue;
#pragma unroll
            for (int e = 0; e < NSYM; ++e) bb[u][e] = binv[e * nnodes + a];
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                const int64_t i = a * ND + d;
                rr[u][d] = fmaf(-af, q[i], r[i]);
                xx[u][d] = x[i];
                pp[u][d] = p[i];
            }
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int64_t a = a0 + (int64_t)u * NTHREADS;
            if (a >= hi) continue;
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                const int64_t i = a * ND + d;
                float zz = 0.f;
#pragma unroll
                for (int j = 0; j < ND; ++j) zz = fmaf(bb[u][sym_plane<ND>(d, j)], rr[u][j], zz);
                if constexpr (sizeof(XS) == 8) x[i] = xx[u][d] + alpha * (double)pp[u][d];
                else x[i] = fmaf(af, pp[u][d], xx[u][d]);
                r[i] = rr[u][d];
                if (zsm) zs[(a - lo) * ND + d] = zz;
                else z[i] = zz;
                s0 = fmaf(rr[u][d], rr[u][d], s0);
                s1 = fmaf(rr[u][d], zz, s1);
            }
            if constexpr (!SUM32) {
                v[0] += (double)s0;
                v[1] += (double)s1;
            } else {
                vf[0] += s0;
                vf[1] += s1;
            }
        }
    }
    if constexpr (SUM32) {
        v[0] = (double)vf[0];
        v[1] = (double)vf[1];
    }
    if constexpr (!FUSE) {
        finish_update32(v, part, count, sc, maxit);
    } else {
        if (publish_after_sum(v, part, count)) {
            finish_update32_last(part, count, sc, maxit);
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(epoch, 1u);
            }
        } else if (threadIdx.x == 0) {
            const long long t0 = clock64();
            while (*(volatile unsigned int *)epoch == e0) {
                if (clock64() - t0 > 2000000000LL) {
                    atomicCAS(&sc->done, 0, DONE_WAIT_TIMEOUT);
                    break;
                }
                __nanosleep(100);
            }
            __threadfence();
        }
        __syncthreads();
        // this iteration's scalars, from L2 (written by the last block)
        if (__ldcg(&sc->done) || __ldcg(&sc->reliable)) return;
        const float beta = (float)__ldcg(&sc->beta), zc = (float)__ldcg(&sc->zcoef);
        const int64_t r0 = lo * ND, r1 = hi * ND;
        for (int64_t i = r0 + threadIdx.x; i < r1; i += NTHREADS)
            p[i] = fmaf(zc, zsm ? zs[i - r0] : __ldcg(z + i), beta * p[i]);
    }
}

// p = zcoef z + beta p in FP32, same block ranges.
__global__ void __launch_bounds__(NTHREADS) k_pupdate_f32(int64_t n, const float *__restrict__ z,
                                                          float *__restrict__ p, const PcgScal *sc)
{
    if (halted(sc)) return;
    const float beta = (float)sc->beta, zc = (float)sc->zcoef;
    int64_t lo, hi;
    block_range(n, lo, hi);
#pragma unroll 4
    for (int64_t row = lo + threadIdx.x; row < hi; row += NTHREADS) p[row] = fmaf(zc, z[row], beta * p[row]);
}

// The block-Jacobi update of a node size, solution accumulation and form:
// mode 1 = FP64 solution with FP64 sums per node, 2 = FP64 solution with FP32
// sums per thread, 0 = FP32 increment with FP32 sums per thread, 3 = FP32
// increment with FP64 sums per node.
template <int ND>
const void *bj_update_nd(int mode, bool fuse)
{
    if (mode == 1) return fuse ? (const void *)k_update_bj32<ND, double, true> : (const void *)k_update_bj32<ND, double, false>;
    if (mode == 2)
        return fuse ? (const void *)k_update_bj32<ND, double, true, true> : (const void *)k_update_bj32<ND, double, false, true>;
    if (mode == 3)
        return fuse ? (const void *)k_update_bj32<ND, float, true, false> : (const void *)k_update_bj32<ND, float, false, false>;
    return fuse ? (const void *)k_update_bj32<ND, float, true> : (const void *)k_update_bj32<ND, float, false>;
}

const void *bj_update_fn(int nd, int mode, bool fuse)
{
    return nd == 3 ? bj_update_nd<3>(mode, fuse) : bj_update_nd<2>(mode, fuse);
}

// Launch of bj_update_fn's kernel; xs is the FP64 solution or the FP32 increment
// (the kernel's solution type). The fused form is a cooperative launch, which
// fails instead of starting when the grid cannot be resident at once.
int launch_bj_update(const void *fn, bool coop, int grid, size_t smem, cudaStream_t s, int64_t nnodes, void *xs,
                     float *r, float *z, float *p, const float *q, const float *binv, double *part,
                     unsigned int *count, unsigned int *epoch, int zcap, PcgScal *sc, int maxit)
{
    void *args[] = {&nnodes, &xs, &r, &z, &p, &q, &binv, &part, &count, &epoch, &zcap, &sc, &maxit};
    const cudaError_t e = coop ? cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(NTHREADS), args, smem, s)
                               : cudaLaunchKernel(fn, dim3(grid), dim3(NTHREADS), args, smem, s);
    if (e != cudaSuccess) return cuda_fail(e, coop ? "cooperative launch of the fused block-Jacobi update"
                                                   : "launch of the block-Jacobi update");
    return OGB_OK;
}

// r = b - Ax in FP64, ||r||^2 and ||b||^2 into out2.
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
        if (threadIdx.x != 0) return;
        *count = 0;
        out2[0] = t[0];
        out2[1] = t[1];
    }
}

// x64 += d (FP64 solution update), d = 0.
__global__ void k_fold_increment(int n, double *__restrict__ x, float *__restrict__ d)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += (double)d[i];
        d[i] = 0.0f;
    }
}

// D^-1 from the diagonal (DiagPreconditioner::init, diagpre.C:40-56).
template <class X, class V>
__global__ void k_diag_inv_csr(int n, const int64_t *__restrict__ diagpos, const V *__restrict__ val, X *dinv,
                               PcgScal *sc)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int64_t p = diagpos[r];
    double d = p >= 0 ? (double)val[p] : 0.0;
    if (d == 0.0) {
        sc->done = 3;
        dinv[r] = 0;
    } else {
        dinv[r] = (X)(1.0 / d);
    }
}

template <int ND, class X, class V>
__global__ void k_diag_inv_sell(int nrows, const int64_t *__restrict__ diag, const V *__restrict__ val, X *dinv,
                                PcgScal *sc)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows) return;
    int64_t slot = diag[a];
    int r = (int)(slot & 31);
    const V *vb = val + (slot - r) * (ND * ND) + r;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        double v = (double)vb[32 * (d * ND + d)];
        if (v == 0.0) {
            sc->done = 3;
            dinv[(int64_t)a * ND + d] = 0;
        } else {
            dinv[(int64_t)a * ND + d] = (X)(1.0 / v);
        }
    }
}

__global__ void k_to_float(int64_t n, const double *__restrict__ a, float *__restrict__ b)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_eq_to_ns(int neq, const int *__restrict__ ns_of_eq, const double *__restrict__ xe,
                           double *__restrict__ xn)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < neq) xn[ns_of_eq[e]] = xe[e];
}

__global__ void k_ns_to_eq(int neq, const int *__restrict__ ns_of_eq, const double *__restrict__ xn,
                           double *__restrict__ xe)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < neq) xe[e] = xn[ns_of_eq[e]];
}

inline int vec_grid(int nchunks) { const int g = num_sms() * GRID_MULT; return nchunks < g ? nchunks : g; }
// blocks of the kernels that split the rows into equal contiguous shares
inline int bal_grid(int nchunks) { const int g = num_sms() * 4; return nchunks < g ? nchunks : g; }
inline unsigned nb(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, NTHREADS); }

// ---------------------------------------------------------------- operator
struct Op {
    bool sell = false;
    int64_t n = 0;            // vector length (multiple of CHUNK)
    // CSR
    const int64_t *rowptr = nullptr;
    const int *colind = nullptr;
    const int64_t *diagpos = nullptr;
    int tpr = 8;
    int64_t nzt = 0;
    // SELL
    const SellMat *S = nullptr;
    int nchunks() const { return (int)(n / CHUNK); }
    int spmv_grid() const;
};

// Warps per slice: four for small matrices (fewer than 16 slices per SM, where
// one warp per slice leaves most warp slots empty), else one -- measured on
// GB300 over 1.3k, 10.5k and 31.7k slices of 27-block rows.
inline int sell_split(const SellMat &S)
{
    if (S.force_split) return S.force_split;
    return S.nslices < num_sms() * 16 ? 4 : 1;
}

inline int sell_grid(const SellMat &S)
{
    return (int)ceil_div((int64_t)S.nslices * sell_split(S), NTHREADS / 32);
}

int Op::spmv_grid() const { return sell ? sell_grid(*S) : vec_grid(nchunks()); }

Op make_op(ogb_mtrx *m, bool use_sell)
{
    Op op;
    if (use_sell) {
        m->sell.force_split = m->ctx->spmv_split;
        op.sell = true;
        op.S = &m->sell;
        op.n = m->sell.nns();
        op.nzt = m->nnz;
    } else {
        op.n = m->npad;
        op.rowptr = m->rowptr.p;
        op.colind = m->colind.p;
        op.diagpos = m->diagpos.p;
        op.tpr = m->spmv_tpr;
        op.nzt = m->nnz + (m->npad - m->neq);
    }
    return op;
}

// Split form for matrices with few slices per resident warp: SPLIT warps share
// one slice, warp `part` taking blocks k = part, part + SPLIT, ... (each load
// still a coalesced 128-byte warp load); the parts are added in part order
// through shared memory by the slice's first warp. More, shorter work units
// keep every SM busy to the end instead of a nearly empty last wave. The sum
// order differs from the one-warp forms, so the split is chosen by a fixed
// rule on the slice count (never by timing) and results stay reproducible.
template <int ND, class V, class X, class ACC, bool DOT, bool DIFF, int SPLIT>
__global__ void __launch_bounds__(NTHREADS) k_sell_spmv_split(int nslices, const int64_t *__restrict__ sl_ptr,
                                                              const int *__restrict__ sl_width,
                                                              const int *__restrict__ col, const V *__restrict__ val,
                                                              const X *__restrict__ x, X *__restrict__ y,
                                                              double *part, unsigned int *count, PcgScal *sc)
{
    if (DOT && halted(sc)) return;
    constexpr int WARPS = NTHREADS / 32, SPB = WARPS / SPLIT;
    __shared__ ACC red[WARPS][ND][32];
    const int warp = threadIdx.x >> 5, r = threadIdx.x & 31;
    const int q = warp % SPLIT;
    const int s = blockIdx.x * SPB + warp / SPLIT;
    ACC yy[ND];
#pragma unroll
    for (int i = 0; i < ND; ++i) yy[i] = 0;
    if (s < nslices) {
        const int64_t base = sl_ptr[s];
        const int w = sl_width[s];
        const int arow = s * 32 + r;
        ACC xa[ND];
#pragma unroll
        for (int i = 0; i < ND; ++i) xa[i] = DIFF ? (ACC)x[(int64_t)arow * ND + i] : (ACC)0;
        const V *vp = val + base * (ND * ND) + r;
        const int *cp = col + base + r;
#pragma unroll 2
        for (int k = q; k < w; k += SPLIT) {
            const int c = __ldcs(cp + 32 * k);
            ACC xb[ND];
#pragma unroll
            for (int j = 0; j < ND; ++j) {
                xb[j] = (ACC)__ldg(x + (int64_t)c * ND + j);
                if (DIFF && c != arow) xb[j] -= xa[j];
            }
            const V *vk = vp + (int64_t)k * (32 * ND * ND);
#pragma unroll
            for (int i = 0; i < ND; ++i)
#pragma unroll
                for (int j = 0; j < ND; ++j) yy[i] += (ACC)__ldcs(vk + 32 * (i * ND + j)) * xb[j];
        }
    }
#pragma unroll
    for (int i = 0; i < ND; ++i) red[warp][i][r] = yy[i];
    __syncthreads();
    double dot = 0.0;
    if (q == 0 && s < nslices) {
        const int64_t a = (int64_t)s * 32 + r;
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            ACC t = red[warp][i][r];
#pragma unroll
            for (int p = 1; p < SPLIT; ++p) t += red[warp + p][i][r];
            y[a * ND + i] = (X)t;
            if (DOT) dot += (double)x[a * ND + i] * (double)t;
        }
    }
    if (!DOT) return;
    double acc[1] = {dot};
    block_sum<1>(acc);
    if (publish_partials<1>(acc, part, count)) {
        double t[1];
        final_sums<1>(part, t);
        if (threadIdx.x != 0) return;
        finish_pq(t[0], count, sc);
    }
}

// ---- SELL SpMV with the value and column stream staged by the Tensor Memory
// Accelerator: every warp owns one slice and a TMA_NS-stage shared-memory ring;
// lane 0 issues one bulk copy (cp.async.bulk) of the next TMA_KC blocks' values
// and one of their block columns into a free stage, completing on that stage's
// mbarrier, while the warp computes from the stage that has landed. The copies
// keep many bytes in flight without registers; the products are those of the
// one-warp loop forms, in the same order (identical results). Waits are bounded:
// a stage that does not land sets DS_TIMEOUT, the warp writes NaN (the solve then
// stops on a breakdown) and leaves after a bounded wait for its other copies.
constexpr int TMA_KC = 4, TMA_NS = 2;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bulk global -> shared copy: both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Wait for the phase of `parity` to complete; false after the iteration limit.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    for (int i = 0; i < (1 << 20); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

template <int ND>
__host__ __device__ constexpr int tma_stage_bytes() { return TMA_KC * 32 * (ND * ND * 4 + 4); }
template <int ND>
__host__ __device__ constexpr int tma_smem_bytes() { return (NTHREADS / 32) * TMA_NS * (tma_stage_bytes<ND>() + 8); }

template <int ND, class X, bool DOT, bool DIFF>
__global__ void __launch_bounds__(NTHREADS) k_sell_spmv_tma(int nslices, const int64_t *__restrict__ sl_ptr,
                                                            const int *__restrict__ sl_width,
                                                            const int *__restrict__ col,
                                                            const float *__restrict__ val, const X *__restrict__ x,
                                                            X *__restrict__ y, double *part, unsigned int *count,
                                                            PcgScal *sc, int *status)
{
    if (DOT && halted(sc)) return;
    constexpr int VB = TMA_KC * 32 * ND * ND * 4, STAGE = tma_stage_bytes<ND>();
    extern __shared__ __align__(128) unsigned char tma_smem[];
    const int warp = threadIdx.x >> 5, r = threadIdx.x & 31;
    const int s = blockIdx.x * (NTHREADS / 32) + warp;
    unsigned char *wb = tma_smem + warp * (TMA_NS * STAGE);
    uint64_t *bars = reinterpret_cast<uint64_t *>(tma_smem + (NTHREADS / 32) * TMA_NS * STAGE) + warp * TMA_NS;
    double dot = 0.0;
    if (s < nslices) {
        const int64_t base = sl_ptr[s];
        const int w = sl_width[s];
        const int nch = (w + TMA_KC - 1) / TMA_KC;
        if (r == 0) {
            for (int i = 0; i < TMA_NS; ++i) mbar_init(&bars[i], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncwarp();
        // chunk c: blocks c*KC .. of the slice = one contiguous run of values
        // (slot groups of 32 x ND*ND floats) and of block columns
        auto issue = [&](int c) {
            const int st = c % TMA_NS, kb = min(TMA_KC, w - c * TMA_KC);
            const int64_t slot0 = base + (int64_t)c * TMA_KC * 32;
            mbar_expect_tx(&bars[st], (uint32_t)(kb * 32 * (ND * ND * 4 + 4)));
            bulk_g2s(wb + st * STAGE, val + slot0 * (ND * ND), (uint32_t)(kb * 32 * ND * ND * 4), &bars[st]);
            bulk_g2s(wb + st * STAGE + VB, col + slot0, (uint32_t)(kb * 32 * 4), &bars[st]);
        };
        if (r == 0)
            for (int c = 0; c < TMA_NS && c < nch; ++c) issue(c);
        const int arow = s * 32 + r;
        float yy[ND], xa[ND];
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            yy[i] = 0.f;
            xa[i] = DIFF ? (float)x[(int64_t)arow * ND + i] : 0.f;
        }
        uint32_t par = 0;
        bool ok = true;
        for (int c = 0; c < nch; ++c) {
            const int st = c % TMA_NS, kb = min(TMA_KC, w - c * TMA_KC);
            if (!mbar_wait(&bars[st], (par >> st) & 1u)) {
                ok = false;
                break;
            }
            par ^= 1u << st;
            const float *sv = reinterpret_cast<const float *>(wb + st * STAGE);
            const int *scol = reinterpret_cast<const int *>(wb + st * STAGE + VB);
#pragma unroll 4
            for (int kk = 0; kk < kb; ++kk) {
                const int cc = scol[kk * 32 + r];
                float xb[ND];
#pragma unroll
                for (int j = 0; j < ND; ++j) {
                    xb[j] = (float)__ldg(x + (int64_t)cc * ND + j);
                    if (DIFF && cc != arow) xb[j] -= xa[j];
                }
#pragma unroll
                for (int i = 0; i < ND; ++i)
#pragma unroll
                    for (int j = 0; j < ND; ++j) yy[i] += sv[kk * 32 * ND * ND + (i * ND + j) * 32 + r] * xb[j];
            }
            __syncwarp();
            if (r == 0 && c + TMA_NS < nch) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(c + TMA_NS);
            }
        }
        if (!ok) {
            if (r == 0) {
                atomicCAS(status, DS_OK, DS_TIMEOUT);
                for (int st = 0; st < TMA_NS; ++st) mbar_wait(&bars[st], (par >> st) & 1u);
            }
#pragma unroll
            for (int i = 0; i < ND; ++i) yy[i] = __int_as_float(0x7fc00000);   // NaN: the solve stops
        }
        const int64_t a = (int64_t)s * 32 + r;
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            y[a * ND + i] = (X)yy[i];
            if (DOT) dot += (double)x[a * ND + i] * (double)yy[i];
        }
    }
    if (!DOT) return;
    double acc[1] = {dot};
    block_sum<1>(acc);
    if (publish_partials<1>(acc, part, count)) {
        double t[1];
        final_sums<1>(part, t);
        if (threadIdx.x != 0) return;
        finish_pq(t[0], count, sc);
    }
}

// SELL SpMV loop variants (one warp per slice, the same sum order): 1 = plain
// unrolled loop, 2 / 3 = block columns prefetched in groups of 1 / 4. (Groups of
// two ran at half the speed of both on GB300 and are not offered.)
constexpr int SPMV_VARIANTS = 4;   // 4 = TMA-staged (FP32 values only)
template <class V, class X, class ACC, bool DOT, bool DIFF, int ND>
void launch_sell_nd(cudaStream_t s, int g, const SellMat &S, int variant, const V *val, const X *x, X *y,
                    double *part, unsigned int *count, PcgScal *sc)
{
#define OGB_SELL(G_)                                                                                              \
    k_sell_spmv<ND, V, X, ACC, DOT, DIFF, G_><<<g, NTHREADS, 0, s>>>(S.nslices, S.sl_ptr.p, S.sl_width.p, S.col.p, \
                                                                     val, x, y, part, count, sc)
    switch (variant) {
    case 1: OGB_SELL(0); break;
    case 2: OGB_SELL(1); break;
    default: OGB_SELL(4); break;
    }
#undef OGB_SELL
}

template <int ND, class X, bool DOT, bool DIFF>
void launch_sell_tma(cudaStream_t s, int grid, const SellMat &S, const float *val, const X *x, X *y, double *part,
                     unsigned int *count, PcgScal *sc, int *status)
{
    static bool attr[64] = {};
    set_smem_limit_once((const void *)k_sell_spmv_tma<ND, X, DOT, DIFF>, tma_smem_bytes<ND>(), attr);
    k_sell_spmv_tma<ND, X, DOT, DIFF><<<grid, NTHREADS, tma_smem_bytes<ND>(), s>>>(
        S.nslices, S.sl_ptr.p, S.sl_width.p, S.col.p, val, x, y, part, count, sc, status);
}

template <class V, class X, class ACC, bool DOT, bool DIFF>
void launch_sell(cudaStream_t s, int g, const SellMat &S, int G, const V *val, const X *x, X *y, double *part,
                 unsigned int *count, PcgScal *sc, int *status = nullptr)
{
    (void)g;
    const int split = sell_split(S), grid = sell_grid(S);
    if constexpr (sizeof(V) == 4 && sizeof(ACC) == 4) {
        if (G == 4 && split == 1 && status) {
            if (S.nd == 3) launch_sell_tma<3, X, DOT, DIFF>(s, grid, S, val, x, y, part, count, sc, status);
            else launch_sell_tma<2, X, DOT, DIFF>(s, grid, S, val, x, y, part, count, sc, status);
            return;
        }
    }
    if (G == 4) G = 3;   // no TMA form for FP64 values
#define OGB_SPLIT(ND_, SP_)                                                                                     \
    k_sell_spmv_split<ND_, V, X, ACC, DOT, DIFF, SP_><<<grid, NTHREADS, 0, s>>>(S.nslices, S.sl_ptr.p, S.sl_width.p, \
                                                                                S.col.p, val, x, y, part, count, sc)
    if (split == 2) {
        if (S.nd == 3) OGB_SPLIT(3, 2);
        else OGB_SPLIT(2, 2);
        return;
    }
    if (split == 4) {
        if (S.nd == 3) OGB_SPLIT(3, 4);
        else OGB_SPLIT(2, 4);
        return;
    }
#undef OGB_SPLIT
    if (S.nd == 3) launch_sell_nd<V, X, ACC, DOT, DIFF, 3>(s, grid, S, G, val, x, y, part, count, sc);
    else launch_sell_nd<V, X, ACC, DOT, DIFF, 2>(s, grid, S, G, val, x, y, part, count, sc);
}

// SELL SpMV variant for value type V: the context's forced choice, else the
// matrix's tuned one (the plain loop until tuned).
template <class V>
int sell_group(const ogb_ctx *ctx, const SellMat &S)
{
    if (ctx->spmv_group) return ctx->spmv_group;
    const int v = S.group[sizeof(V) == 4 ? 1 : 0];
    return v ? v : 1;
}

// Autotuner: times every SELL SpMV variant of this matrix and value type in the
// form the solve launches (fused p.q, on scratch scalars `sc`, whose `done`
// must be 0) -- one warm-up and three timed launches each, CUDA events on the
// context stream -- and keeps the fastest. Runs once per matrix structure and
// value type, outside graph capture; x and y are scratch vectors.
template <class V, class X, class ACC, bool DIFF>
int sell_autotune(ogb_ctx *ctx, const Op &op, const V *val, const X *x, X *y, double *part, unsigned int *count,
                  PcgScal *sc)
{
    if (!op.sell || ctx->spmv_group) return OGB_OK;
    SellMat &S = const_cast<SellMat &>(*op.S);
    int &slot = S.group[sizeof(V) == 4 ? 1 : 0];
    if (slot) return OGB_OK;
    if (sell_split(S) > 1) {   // the split form has one loop variant
        slot = 1;
        return OGB_OK;
    }
    cudaStream_t s = ctx->stream;
    const int g = op.spmv_grid();
    OGB_CUDA(cudaMemsetAsync(sc, 0, sizeof(PcgScal), s));
    cudaEvent_t e0, e1;
    OGB_CUDA(cudaEventCreate(&e0));
    OGB_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    int best_v = 1;
    for (int v = 1; v <= SPMV_VARIANTS; ++v) {
        // the scratch scalars are cleared before every launch: an epilogue that
        // met p.q <= 0 on the scratch vectors would otherwise mark them done and
        // turn the following launches into no-ops
        cudaMemsetAsync(sc, 0, sizeof(PcgScal), s);
        if (v == 4 && sizeof(V) != 4) break;   // the TMA form exists for FP32 values only
        launch_sell<V, X, ACC, true, DIFF>(s, g, S, v, val, x, y, part, count, sc, ctx->status.p);
        cudaEventRecord(e0, s);
        for (int k = 0; k < 3; ++k) {
            cudaMemsetAsync(sc, 0, sizeof(PcgScal), s);
            launch_sell<V, X, ACC, true, DIFF>(s, g, S, v, val, x, y, part, count, sc, ctx->status.p);
        }
        cudaEventRecord(e1, s);
        count_launch(ctx, 4);
        cudaError_t e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_fail(e, "SpMV autotune");
        }
        // a later form must win by 2 % to replace an earlier one: near-ties keep
        // the simpler form, and the choice does not flip with timing noise
        if (v == 1 || ms < 0.98f * best) {
            best = ms;
            best_v = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    slot = best_v;
    return OGB_OK;
}

template <class V, class X, bool DOT, class ACC = V, bool DIFF = false>
int apply_op(ogb_ctx *ctx, const Op &op, const V *val, const X *x, X *y, double *part, unsigned int *count,
             PcgScal *sc)
{
    cudaStream_t s = ctx->stream;
    const int g = op.spmv_grid();
    double bytes;
    prof_begin(ctx);
    if (op.sell) {
        const SellMat &S = *op.S;
        launch_sell<V, X, ACC, DOT, DIFF>(s, g, S, sell_group<V>(ctx, S), val, x, y, part, count, sc, ctx->status.p);
        // algorithmic bytes: every stored value and block column once (the SELL
        // padding slots are not counted), x once and y once
        bytes = (double)op.nzt * sizeof(V) + (double)op.nzt / (S.nd * S.nd) * sizeof(int) +
                (double)op.n * sizeof(X) * 2;
    } else {
        const int nch = op.nchunks();
        switch (op.tpr) {
        case 2: k_spmv<2, V, X, ACC, DOT><<<g, NTHREADS, 0, s>>>(nch, op.rowptr, op.colind, val, x, y, part, count, sc); break;
        case 4: k_spmv<4, V, X, ACC, DOT><<<g, NTHREADS, 0, s>>>(nch, op.rowptr, op.colind, val, x, y, part, count, sc); break;
        case 8: k_spmv<8, V, X, ACC, DOT><<<g, NTHREADS, 0, s>>>(nch, op.rowptr, op.colind, val, x, y, part, count, sc); break;
        case 16: k_spmv<16, V, X, ACC, DOT><<<g, NTHREADS, 0, s>>>(nch, op.rowptr, op.colind, val, x, y, part, count, sc); break;
        default: k_spmv<32, V, X, ACC, DOT><<<g, NTHREADS, 0, s>>>(nch, op.rowptr, op.colind, val, x, y, part, count, sc); break;
        }
        bytes = (double)op.nzt * (sizeof(V) + sizeof(int)) + (double)(op.n + 1) * sizeof(int64_t) +
                (double)op.n * sizeof(X) * 2;
    }
    prof_end(ctx, bytes);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

// q = K p through the half-stored FP32 copy, fused p.q (mixed solves).
// Half-stored SpMV forms: groups of 8 blocks, 1 = 4 resident blocks per SM (64
// registers), 2 = 3 blocks (80), 3 = 2 blocks (128); every value of the group
// loaded before its products: 4 = groups of 4 at 3 blocks per SM (80), 5 =
// groups of 3 at 4 blocks (64), 6 = groups of 2 at 5 blocks (48). The
// autotuner times them in HALF_ORDER (the first is kept unless a later one is
// 2 % faster).
constexpr int HALF_FORMS = 6;
constexpr int HALF_ORDER[HALF_FORMS] = {5, 6, 4, 1, 2, 3};

template <int ND, class X, bool DIFF>
int launch_half(cudaStream_t s, int form, const SellMat &S, const X *x, X *y, double *part, unsigned int *count,
                PcgScal *sc)
{
    const HalfSell &H = S.half;
    const int grid = (int)ceil_div(S.nslices, NTHREADS / 32);
#define OGB_HALF_ARGS S.nslices, H.sl_ptrU.p, H.sl_widthU.p, H.colU.p, H.v32.p, H.sl_ptrL.p, H.sl_widthL.p, H.low.p, \
                      x, y, part, count, sc
    if (form == 2) k_half_spmv<ND, X, DIFF, 8, 3><<<grid, NTHREADS, 0, s>>>(OGB_HALF_ARGS);
    else if (form == 3) k_half_spmv<ND, X, DIFF, 8, 2><<<grid, NTHREADS, 0, s>>>(OGB_HALF_ARGS);
    else if (form == 4) k_half_spmv<ND, X, DIFF, 4, 3, true><<<grid, NTHREADS, 0, s>>>(OGB_HALF_ARGS);
    else if (form == 5) k_half_spmv<ND, X, DIFF, 3, 4, true><<<grid, NTHREADS, 0, s>>>(OGB_HALF_ARGS);
    else if (form == 6) k_half_spmv<ND, X, DIFF, 2, 5, true><<<grid, NTHREADS, 0, s>>>(OGB_HALF_ARGS);
    else k_half_spmv<ND, X, DIFF, 8, 4><<<grid, NTHREADS, 0, s>>>(OGB_HALF_ARGS);
#undef OGB_HALF_ARGS
    return OGB_OK;
}

// Time the half-stored forms once per matrix (scratch scalars; three launches
// each after a warm-up launch); a later form must be 2 % faster to be chosen.
template <class X, bool DIFF>
int half_autotune(ogb_ctx *ctx, const Op &op, const X *x, X *y, double *part, unsigned int *count, PcgScal *sc)
{
    SellMat &S = const_cast<SellMat &>(*op.S);
    if (S.half.form) return OGB_OK;
    cudaStream_t s = ctx->stream;
    cudaEvent_t e0, e1;
    OGB_CUDA(cudaEventCreate(&e0));
    OGB_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    int best_f = HALF_ORDER[0];
    for (int fi = 0; fi < HALF_FORMS; ++fi) {
        const int f = HALF_ORDER[fi];
        auto launch = [&]() {
            cudaMemsetAsync(sc, 0, sizeof(PcgScal), s);
            return S.nd == 3 ? launch_half<3, X, DIFF>(s, f, S, x, y, part, count, sc)
                             : launch_half<2, X, DIFF>(s, f, S, x, y, part, count, sc);
        };
        OGB_CHECK(launch());
        cudaEventRecord(e0, s);
        for (int k = 0; k < 3; ++k) OGB_CHECK(launch());
        cudaEventRecord(e1, s);
        count_launch(ctx, 4);
        cudaError_t e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_fail(e, "half-stored SpMV autotune");
        }
        if (fi == 0 || ms < 0.98f * best) {
            best = ms;
            best_f = f;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    S.half.form = best_f;
    return OGB_OK;
}

template <class X, bool DIFF>
int apply_half(ogb_ctx *ctx, const Op &op, const X *x, X *y, double *part, unsigned int *count, PcgScal *sc)
{
    const SellMat &S = *op.S;
    const int form = ctx->half_form ? ctx->half_form : (S.half.form ? S.half.form : HALF_ORDER[0]);
    cudaStream_t s = ctx->stream;
    prof_begin(ctx);
    OGB_CHECK((S.nd == 3 ? launch_half<3, X, DIFF>(s, form, S, x, y, part, count, sc)
                         : launch_half<2, X, DIFF>(s, form, S, x, y, part, count, sc)));
    // algorithmic bytes: the upper values (the diagonal blocks and half of the
    // off-diagonal ones) with their block columns, one 4-byte entry per lower
    // block, x once and y once; padding slots not counted
    const double nd2 = (double)S.nd * S.nd, blocks = (double)op.nzt / nd2, rows = (double)S.nact;
    const double up = 0.5 * (blocks + rows), lo = 0.5 * (blocks - rows);
    prof_end(ctx, up * nd2 * sizeof(float) + up * sizeof(int) + lo * sizeof(int) + (double)op.n * sizeof(X) * 2);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

template <class X, class V>
int launch_diag_inv(ogb_ctx *ctx, const Op &op, const V *val, X *dinv, PcgScal *sc)
{
    cudaStream_t s = ctx->stream;
    if (op.sell) {
        int nrows = op.S->nslices * 32;
        if (op.S->nd == 3) k_diag_inv_sell<3, X, V><<<nb(nrows), NTHREADS, 0, s>>>(nrows, op.S->diag.p, val, dinv, sc);
        else k_diag_inv_sell<2, X, V><<<nb(nrows), NTHREADS, 0, s>>>(nrows, op.S->diag.p, val, dinv, sc);
    } else {
        k_diag_inv_csr<X, V><<<nb(op.n), NTHREADS, 0, s>>>((int)op.n, op.diagpos, val, dinv, sc);
    }
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

template <class X>
__global__ void k_fill_one(int64_t n, X *__restrict__ v)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = (X)1;
}

// The preconditioner's diagonal: D^-1 (lsprecond 1, DiagPreconditioner) or the
// identity (lsprecond 0, VoidPreconditioner: plain CG, z = r).
template <class X, class V>
int launch_prec_diag(ogb_mtrx *m, const Op &op, const V *val, X *dinv, PcgScal *sc)
{
    if (m->precond == 0) {
        k_fill_one<X><<<num_sms() * 8, NTHREADS, 0, m->ctx->stream>>>(op.n, dinv);
        count_launch(m->ctx);
        OGB_CUDA(cudaGetLastError());
        return OGB_OK;
    }
    return launch_diag_inv<X, V>(m->ctx, op, val, dinv, sc);
}

int ensure_workspace(ogb_mtrx *m, const Op &op, bool mixed)
{
    const int64_t n = op.n;
    int gmax = op.spmv_grid() > vec_grid(op.nchunks()) ? op.spmv_grid() : vec_grid(op.nchunks());
    OGB_CHECK(m->w_part.alloc((size_t)4 * gmax));
    OGB_CHECK(m->w_scal.alloc(2));
    OGB_CHECK(m->h_scal.alloc(2));
    OGB_CHECK(m->w_d.alloc(4));
    if (!m->w_count.p) {
        OGB_CHECK(m->w_count.alloc(1));
        OGB_CUDA(cudaMemsetAsync(m->w_count.p, 0, sizeof(unsigned int), m->ctx->stream));
    }
    if (true) {
        OGB_CHECK(m->w_r.alloc(n));
        OGB_CHECK(m->w_z.alloc(n));
        OGB_CHECK(m->w_p.alloc(n));
        OGB_CHECK(m->w_q.alloc(n));
        OGB_CHECK(m->w_dinv.alloc(n));
    }
    if (mixed) {
        OGB_CHECK(m->n_r64.alloc(n));
        OGB_CHECK(m->n_q64.alloc(n));
        OGB_CHECK(m->w_r32.alloc(n));
        OGB_CHECK(m->w_z32.alloc(n));
        OGB_CHECK(m->w_p32.alloc(n));
        OGB_CHECK(m->w_q32.alloc(n));
        OGB_CHECK(m->w_dinv32.alloc(n));
        OGB_CHECK(m->n_d32.alloc(n));
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

constexpr int BATCH = 16;

// One batch of PCG iterations recorded as a CUDA graph and replayed until the
// device-side scalars say the system is done. With profiling on, the SpMV
// launches of the batch are bracketed by event nodes owned by the graph; their
// times are added after every replay (the host waits for each batch anyway).
struct IterGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaEvent_t> ev;
    double bytes = 0.0;
    ~IterGraph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    template <class F>
    int capture(ogb_ctx *ctx, F &&launch_batch)
    {
        cudaGraph_t g = nullptr;
        ctx->capture_events = &ev;
        ctx->capture_bytes = 0.0;
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            ctx->capture_events = nullptr;
            return cuda_fail(e, "cudaStreamBeginCapture");
        }
        int r = launch_batch();
        cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
        ctx->capture_events = nullptr;
        bytes = ctx->capture_bytes;
        if (r != OGB_OK) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        return OGB_OK;
    }
    int launch(ogb_ctx *ctx)
    {
        OGB_CUDA(cudaGraphLaunch(exec, ctx->stream));
        return OGB_OK;
    }
    // after the stream is synchronized
    void harvest(ogb_ctx *ctx)
    {
        if (!ctx->prof) return;
        for (size_t k = 0; k + 1 < ev.size(); k += 2) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev[k], ev[k + 1]) == cudaSuccess) {
                ctx->prof_ms += ms;
                ctx->prof_count++;
            } else {
                cudaGetLastError();   // a failed query must not leak into the next error check
            }
        }
        ctx->prof_bytes += bytes;
    }
};

// FP64 PCG (drop-in semantics) on op-space vectors b (read), x (initial guess, updated).
int pcg64_core(ogb_mtrx *m, const Op &op, const double *val, const double *b, double *x, double rtol, int maxit,
               PcgScal &res)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    const int nch = op.nchunks(), g = vec_grid(nch), gb = bal_grid(nch);
    PcgScal *sc = m->w_scal.p;
    double *r = m->w_r.p, *z = m->w_z.p, *p = m->w_p.p, *q = m->w_q.p, *dinv = m->w_dinv.p;
    OGB_CUDA(cudaMemsetAsync(sc, 0, sizeof(PcgScal), s));
    OGB_CHECK((sell_autotune<double, double, double, false>(ctx, op, val, p, q, m->w_part.p, m->w_count.p, sc + 1)));
    OGB_CHECK((launch_prec_diag<double, double>(m, op, val, dinv, sc)));
    OGB_CHECK((apply_op<double, double, false>(ctx, op, val, x, q, nullptr, nullptr, nullptr)));
    k_pcg_init<double><<<g, NTHREADS, 0, s>>>(nch, b, q, dinv, r, z, p, m->w_part.p, m->w_count.p, sc, rtol);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    auto batch = [&]() -> int {
        for (int k = 0; k < BATCH; ++k) {
            ctx->prof_sample = k == BATCH / 2 || !ctx->capture_events;   // time one mid-batch SpMV per replay
            OGB_CHECK((apply_op<double, double, true>(ctx, op, val, p, q, m->w_part.p, m->w_count.p, sc)));
            ctx->prof_sample = true;
            k_update4<false, double><<<gb, NTHREADS, 0, s>>>(op.n, x, r, z, p, q, dinv, m->w_part.p, m->w_count.p,
                                                            sc, rtol, maxit);
            k_pupdate4<double><<<gb, NTHREADS, 0, s>>>(op.n, z, p, sc);
            count_launch(ctx, 2);
        }
        OGB_CUDA(cudaGetLastError());
        return OGB_OK;
    };
    IterGraph graph;
    if (ctx->use_graphs) OGB_CHECK(graph.capture(ctx, batch));
    int it = 0;
    for (;;) {
        OGB_CHECK(read_scal(m, res));
        if (ctx->use_graphs && it > 0) graph.harvest(ctx);
        if (res.done || it >= maxit) break;
        if (ctx->use_graphs) {
            OGB_CHECK(graph.launch(ctx));
            count_launch(ctx, 3 * BATCH);
        } else {
            OGB_CHECK(batch());
        }
        it += BATCH;
    }
    return OGB_OK;
}

// ---------------------------------------------------------------- IC-preconditioned CG
// IML CG (iml/cg.h:22-71) with z = M^-1 r from the incomplete-Cholesky factor
// (icprec.cu): x += alpha p, r -= alpha q, test ||r|| / ||b||; z = M^-1 r;
// rho = r.z, beta = rho / rho_1 (none in the first iteration); p = z + beta p;
// q = A p, alpha = rho / p.q.
__global__ void __launch_bounds__(NTHREADS) k_ic_init(int64_t n, const double *__restrict__ b,
                                                      const double *__restrict__ q, double *__restrict__ r,
                                                      double *part, unsigned int *count, PcgScal *sc, double rtol)
{
    int64_t lo, hi;
    block_range(n, lo, hi);
    double v[2] = {0, 0};
    for (int64_t row = lo + threadIdx.x; row < hi; row += NTHREADS) {
        const double bb = b[row], rr = bb - q[row];
        r[row] = rr;
        v[0] += bb * bb;
        v[1] += rr * rr;
    }
    block_sum<2>(v);
    if (publish_partials<2>(v, part, count)) {
        double t[2];
        final_sums<2>(part, t);
        if (threadIdx.x != 0) return;
        *count = 0;
        sc->bnorm2 = t[0];
        sc->rnorm2 = t[1];
        double normb = sqrt(t[0]);
        if (normb == 0.0) normb = 1.0;
        if (sqrt(t[1]) / normb <= rtol) sc->done = 1;
    }
}

__global__ void __launch_bounds__(NTHREADS) k_ic_rz(int64_t n, const double *__restrict__ r,
                                                    const double *__restrict__ z, double *part, unsigned int *count,
                                                    PcgScal *sc)
{
    if (halted(sc)) return;
    int64_t lo, hi;
    block_range(n, lo, hi);
    double v[1] = {0};
    for (int64_t row = lo + threadIdx.x; row < hi; row += NTHREADS) v[0] += r[row] * z[row];
    block_sum<1>(v);
    if (publish_partials<1>(v, part, count)) {
        double t[1];
        final_sums<1>(part, t);
        if (threadIdx.x != 0) return;
        *count = 0;
        if (!isfinite(t[0]) || !(t[0] > 0.0)) {
            sc->done = 2;
            return;
        }
        sc->beta = sc->iters == 0 ? 0.0 : t[0] / sc->rho;
        sc->rho = t[0];
        sc->zcoef = 1.0;
    }
}

__global__ void __launch_bounds__(NTHREADS) k_ic_xr(int64_t n, double *__restrict__ x, double *__restrict__ r,
                                                    const double *__restrict__ p, const double *__restrict__ q,
                                                    double *part, unsigned int *count, PcgScal *sc, double rtol,
                                                    int maxit)
{
    if (halted(sc)) return;
    const double alpha = sc->alpha;
    int64_t lo, hi;
    block_range(n, lo, hi);
    double v[1] = {0};
    for (int64_t row = lo + threadIdx.x; row < hi; row += NTHREADS) {
        x[row] += alpha * p[row];
        const double rr = r[row] - alpha * q[row];
        r[row] = rr;
        v[0] += rr * rr;
    }
    block_sum<1>(v);
    if (publish_partials<1>(v, part, count)) {
        double t[1];
        final_sums<1>(part, t);
        if (threadIdx.x != 0) return;
        *count = 0;
        sc->rnorm2 = t[0];
        sc->iters += 1;
        double normb = sqrt(sc->bnorm2);
        if (normb == 0.0) normb = 1.0;
        if (sqrt(t[0]) / normb <= rtol) sc->done = 1;
        else if (!isfinite(t[0])) sc->done = 2;
        else if (sc->iters >= maxit) sc->done = 4;
    }
}

int pcg_ic_core(ogb_mtrx *m, const Op &op, const double *b, double *x, double rtol, int maxit, PcgScal &res)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    const int gb = bal_grid(op.nchunks());
    PcgScal *sc = m->w_scal.p;
    double *r = m->w_r.p, *z = m->w_z.p, *p = m->w_p.p, *q = m->w_q.p;
    OGB_CHECK(build_ic(m));
    OGB_CUDA(cudaMemsetAsync(sc, 0, sizeof(PcgScal), s));
    OGB_CUDA(cudaMemsetAsync(p, 0, op.n * sizeof(double), s));
    OGB_CHECK((apply_op<double, double, false>(ctx, op, m->val.p, x, q, nullptr, nullptr, nullptr)));
    k_ic_init<<<gb, NTHREADS, 0, s>>>(op.n, b, q, r, m->w_part.p, m->w_count.p, sc, rtol);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    // iterations per captured graph (two cluster launches for the triangular
    // solves and four vector/SpMV launches each)
    const int nb_it = BATCH;
    auto batch = [&]() -> int {
        for (int k = 0; k < nb_it; ++k) {
            OGB_CHECK(launch_ic_solve(m, r, z, sc));
            k_ic_rz<<<gb, NTHREADS, 0, s>>>(op.n, r, z, m->w_part.p, m->w_count.p, sc);
            k_pupdate4<double><<<gb, NTHREADS, 0, s>>>(op.n, z, p, sc);
            count_launch(ctx, 2);
            OGB_CHECK((apply_op<double, double, true>(ctx, op, m->val.p, p, q, m->w_part.p, m->w_count.p, sc)));
            k_ic_xr<<<gb, NTHREADS, 0, s>>>(op.n, x, r, p, q, m->w_part.p, m->w_count.p, sc, rtol, maxit);
            count_launch(ctx);
        }
        OGB_CUDA(cudaGetLastError());
        return OGB_OK;
    };
    IterGraph graph;
    if (ctx->use_graphs) OGB_CHECK(graph.capture(ctx, batch));
    for (int it = 0;; it += nb_it) {
        OGB_CHECK(read_scal(m, res));
        if (ctx->use_graphs && it > 0) graph.harvest(ctx);
        if (res.done || it >= maxit) break;
        if (ctx->use_graphs) OGB_CHECK(graph.launch(ctx));
        else OGB_CHECK(batch());
    }
    return OGB_OK;
}

// Mixed precision with FP64 residual replacement (see file header). X is the
// type of the Krylov vectors: float keeps everything but the residual and the
// solution in FP32 (the solution increment d is folded into x64 at every
// replacement); double keeps r, z, p, q and x in FP64 while the matrix stays
// FP32 and the SpMV multiplies and accumulates in FP32.
template <class X, class P>
int pcg_mixed_core(ogb_mtrx *m, const Op &op, const double *v64, const float *v32, const double *b, double *x,
                   double rtol, int maxit, ogb_solve_info *info, bool *stalled)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    const int nch = op.nchunks(), g = vec_grid(nch), gb = bal_grid(nch);
    // grid of the block-Jacobi update and p update: one wave of the update kernel's
    // resident blocks per SM (its occupancy, queried once), or the option's count;
    // each block takes an equal contiguous share of the nodes
    // (the fused form is a cooperative launch: at most its occupancy per SM)
    const bool fuse = ctx->fused_update && op.sell;
    const void *ufn = op.sell ? bj_update_fn(op.S->nd, ctx->mixed_x64 ? (ctx->mixed_sum32 ? 2 : 1) : (ctx->mixed_sum32 ? 0 : 3), fuse)
                              : nullptr;
    // (at most the occupancy, and no more blocks per SM than give each block about
    // 2,048 nodes: below that the per-block reductions and the grid-wide wait
    // outweigh the bandwidth of more blocks)
    int upd_bps = ctx->upd_bps;
    if (op.sell) {
        int occ = 0;
        const cudaError_t oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ufn, NTHREADS, 0);
        if (oe != cudaSuccess) return cuda_fail(oe, "occupancy of the block-Jacobi update");
        if (occ < 1) occ = 1;
        if (!upd_bps) {
            const int64_t by_size = (op.n / op.S->nd) / ((int64_t)num_sms() * 2048);
            upd_bps = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(occ, 8), by_size));
        }
        if (fuse && upd_bps > occ) upd_bps = occ;
    }
    const int gu = upd_bps ? (nch < num_sms() * upd_bps ? nch : num_sms() * upd_bps) : gb;
    const int n = (int)op.n;
    constexpr bool F32 = sizeof(X) == 4;
    PcgScal *sc = m->w_scal.p;
    X *r, *z, *dinv, *d;
    P *p, *q;
    if constexpr (F32) {
        r = m->w_r32.p; z = m->w_z32.p; dinv = m->w_dinv32.p; d = m->n_d32.p;
    } else {
        r = m->w_r.p; z = m->w_z.p; dinv = m->w_dinv.p; d = x;
    }
    if constexpr (sizeof(P) == 4) {
        p = m->w_p32.p; q = m->w_q32.p;
    } else {
        p = m->w_p.p; q = m->w_q.p;
    }
    double *r64 = m->n_r64.p, *q64 = m->n_q64.p;
    OGB_CUDA(cudaMemsetAsync(sc, 0, sizeof(PcgScal), s));
    if constexpr (F32) OGB_CUDA(cudaMemsetAsync(d, 0, n * sizeof(X), s));
    OGB_CUDA(cudaMemsetAsync(p, 0, n * sizeof(P), s));
    // Jacobi from the FP64 diagonal blocks (the FP32 copy may hold row sums there)
    OGB_CHECK((launch_prec_diag<X, double>(m, op, v64, dinv, sc)));
    // block Jacobi (FP32 inverses of the node diagonal blocks) in place of the
    // scalar one for node-block operators with FP32 vectors
    const bool bj = F32 && ctx->mixed_bj && op.sell && m->precond == 1;
    const int nd = op.sell ? op.S->nd : 1;
    const int64_t nnodes = op.n / nd;
    float *binv = nullptr;
    if (bj) {
        OGB_CHECK(m->w_binv32.alloc((size_t)nnodes * (nd * (nd + 1) / 2)));
        binv = m->w_binv32.p;
        const int nrows = (int)nnodes;
        if (nd == 3) k_block_inv_sell<3><<<nb(nrows), NTHREADS, 0, s>>>(nrows, op.S->diag.p, v64, binv, sc);
        else k_block_inv_sell<2><<<nb(nrows), NTHREADS, 0, s>>>(nrows, op.S->diag.p, v64, binv, sc);
        count_launch(ctx);
    }
    m->last_bj = bj;
    // fused form: z of the block's nodes in shared memory when they fit in 48 KB
    // without lowering the resident blocks below the grid
    int zcap = 0;
    size_t zbytes = 0;
    if (bj && fuse) {
        if (!m->w_epoch.p) {
            OGB_CHECK(m->w_epoch.alloc(1));
            OGB_CUDA(cudaMemsetAsync(m->w_epoch.p, 0, sizeof(unsigned int), s));
        }
        const int64_t share = (nnodes + gu - 1) / gu;
        const int64_t per = (share + NTHREADS - 1) / NTHREADS * NTHREADS;
        const size_t bytes = (size_t)per * nd * sizeof(float);
        if (bytes <= 48 * 1024) {
            int occz = 0;
            OGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occz, ufn, NTHREADS, bytes));
            if ((int64_t)occz * num_sms() >= gu) {
                zcap = (int)per;
                zbytes = bytes;
            }
        }
    }
    const bool diff = op.sell && ctx->mixed_diff;
    // the half-stored FP32 copy for large node-block matrices (one warp per slice)
    bool half = false;
    if constexpr (sizeof(P) == 4) {
        if (op.sell && !ctx->spmv_group &&
            (ctx->spmv_half == 2 || (ctx->spmv_half == 1 && sell_split(*op.S) == 1))) {
            SellMat &S = const_cast<SellMat &>(*op.S);
            if (!S.half.tried) OGB_CHECK(build_half(ctx, S));
            if (S.half.ok) {
                OGB_CHECK(refresh_half(ctx, S));
                half = true;
            }
        }
    }
    m->last_half = half;
    if (half) {
        if constexpr (sizeof(P) == 4) {
            if (!ctx->half_form) {
                if (diff) OGB_CHECK((half_autotune<P, true>(ctx, op, p, q, m->w_part.p, m->w_count.p, sc + 1)));
                else OGB_CHECK((half_autotune<P, false>(ctx, op, p, q, m->w_part.p, m->w_count.p, sc + 1)));
            }
        }
    } else if (diff) {
        OGB_CHECK((sell_autotune<float, P, float, true>(ctx, op, v32, p, q, m->w_part.p, m->w_count.p, sc + 1)));
    } else {
        OGB_CHECK((sell_autotune<float, P, float, false>(ctx, op, v32, p, q, m->w_part.p, m->w_count.p, sc + 1)));
    }
    int iters = 0, replacements = 0, status = OGB_E_NOTCONV, since_mark = 0, longest = 0;
    double mark = INFINITY;
    *stalled = false;
    double achieved = 0.0;
    bool first = true;
    PcgScal res{};
    auto batch = [&]() -> int {
        for (int k = 0; k < BATCH; ++k) {
            ctx->prof_sample = k == BATCH / 2 || !ctx->capture_events;   // time one mid-batch SpMV per replay
            if (half) {
                if constexpr (sizeof(P) == 4) {
                    if (diff) OGB_CHECK((apply_half<P, true>(ctx, op, p, q, m->w_part.p, m->w_count.p, sc)));
                    else OGB_CHECK((apply_half<P, false>(ctx, op, p, q, m->w_part.p, m->w_count.p, sc)));
                }
            } else if (diff) {
                OGB_CHECK((apply_op<float, P, true, float, true>(ctx, op, v32, p, q, m->w_part.p, m->w_count.p, sc)));
            } else {
                OGB_CHECK((apply_op<float, P, true, float>(ctx, op, v32, p, q, m->w_part.p, m->w_count.p, sc)));
            }
            ctx->prof_sample = true;
            if constexpr (F32) {
                if (bj) {
                    void *xs = ctx->mixed_x64 ? (void *)x : (void *)d;
                    OGB_CHECK(launch_bj_update(ufn, fuse, gu, zbytes, s, nnodes, xs, r, z, p, q, binv, m->w_part.p,
                                               m->w_count.p, m->w_epoch.p, zcap, sc, maxit));
                    if (!fuse) k_pupdate_f32<<<gu, NTHREADS, 0, s>>>(op.n, z, p, sc);
                } else if (ctx->mixed_x64) {
                    k_update_rz32<<<gb, NTHREADS, 0, s>>>(op.n, x, r, z, p, q, dinv, m->w_part.p, m->w_count.p, sc,
                                                           maxit);
                    k_pupdate_f32<<<gb, NTHREADS, 0, s>>>(op.n, z, p, sc);
                } else {
                    k_mixed_update<X, P><<<g, NTHREADS, 0, s>>>(nch, d, r, z, p, q, dinv, m->w_part.p, m->w_count.p,
                                                                sc, maxit);
                    k_pcg_pupdate<X, P><<<g, NTHREADS, 0, s>>>(n, z, p, sc);
                }
            } else {
                k_update4<true, P><<<gb, NTHREADS, 0, s>>>(op.n, d, r, z, p, q, dinv, m->w_part.p, m->w_count.p, sc,
                                                          rtol, maxit);
                k_pupdate4<P><<<gb, NTHREADS, 0, s>>>(op.n, z, p, sc);
            }
            count_launch(ctx, bj && fuse ? 1 : 2);
        }
        if constexpr (F32) {
            if (!ctx->mixed_x64) {
                // fold the FP32 increment of these iterations into the FP64 solution
                k_fold_increment<<<num_sms() * 8, NTHREADS, 0, s>>>(n, x, d);
                count_launch(ctx);
            }
        }
        OGB_CUDA(cudaGetLastError());
        return OGB_OK;
    };
    IterGraph graph;
    if (ctx->use_graphs) OGB_CHECK(graph.capture(ctx, batch));
    for (;;) {
        // FP64 residual of the current x64 (not sampled by the kernel timing, which
        // measures the FP32 operator of the iterations)
        ctx->prof_sample = false;
        const int rres = apply_op<double, double, false>(ctx, op, v64, x, q64, nullptr, nullptr, nullptr);
        ctx->prof_sample = true;
        OGB_CHECK(rres);
        k_residual64<<<g, NTHREADS, 0, s>>>(nch, b, q64, r64, m->w_part.p, m->w_count.p, m->w_d.p);
        count_launch(ctx);
        double h2[2];
        OGB_CUDA(cudaMemcpyAsync(h2, m->w_d.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        OGB_CUDA(cudaStreamSynchronize(s));
        double normb = sqrt(h2[1]);
        if (normb == 0.0) normb = 1.0;
        achieved = sqrt(h2[0]) / normb;
        if (achieved <= rtol) { status = OGB_OK; break; }
        if (!isfinite(achieved)) { status = OGB_E_BREAKDOWN; break; }
        if (iters >= maxit) break;
        // stagnation: the FP32 operator no longer brings the FP64 residual down
        // (six replacement cycles without halving it, or a breakdown of the
        // FP32 recurrences); the caller finishes the solve in FP64
        if (!(achieved < 0.5 * mark)) {
            if (++since_mark >= 6 || replacements > 400) {
                *stalled = true;
                break;
            }
        } else {
            mark = achieved;
            since_mark = 0;
        }
        if (first) {
            // the recursive residual below half the target asks for an FP64 check
            double th[2] = {0.25 * rtol * rtol * normb * normb, ctx->mixed_drop * ctx->mixed_drop};
            OGB_CUDA(cudaMemcpyAsync(&sc->tol2, th, 2 * sizeof(double), cudaMemcpyHostToDevice, s));
            OGB_CUDA(cudaStreamSynchronize(s));
        }
        // replacement: r = r64, z = D^-1 r, beta; then p = z + beta p
        // cycle cap: unbounded for the first cycle, then twice the longest cycle so far (at least 512)
        const int cap = first ? (maxit < (1 << 29) ? maxit : (1 << 29)) : (2 * longest > 512 ? 2 * longest : 512);
        if constexpr (F32) {
            if (bj) {
                if (nd == 3)
                    k_mixed_replace_bj<3, P><<<g, NTHREADS, 0, s>>>(nnodes, r64, r, z, p, binv, m->w_part.p,
                                                                     m->w_count.p, sc, first ? 1 : 0,
                                                                     ctx->mixed_orth ? 1 : 0, cap);
                else
                    k_mixed_replace_bj<2, P><<<g, NTHREADS, 0, s>>>(nnodes, r64, r, z, p, binv, m->w_part.p,
                                                                     m->w_count.p, sc, first ? 1 : 0,
                                                                     ctx->mixed_orth ? 1 : 0, cap);
            }
        }
        if (!bj)
            k_mixed_replace<X, P><<<g, NTHREADS, 0, s>>>(nch, r64, r, z, p, dinv, m->w_part.p, m->w_count.p, sc,
                                                         first ? 1 : 0, ctx->mixed_orth ? 1 : 0, cap);
        k_pcg_pupdate<X, P><<<g, NTHREADS, 0, s>>>(n, z, p, sc);
        count_launch(ctx, 2);
        first = false;
        ++replacements;
        // iterations on the FP32 operator until the next replacement is due
        for (int nb = 0;; ++nb) {
            OGB_CHECK(read_scal(m, res));
            if (ctx->use_graphs && nb > 0) graph.harvest(ctx);
            if (res.done || res.reliable) break;
            if (ctx->use_graphs) {
                OGB_CHECK(graph.launch(ctx));
                count_launch(ctx, (bj && fuse ? 2 : 3) * BATCH + (F32 && !ctx->mixed_x64 ? 1 : 0));
            } else {
                OGB_CHECK(batch());
            }
        }
        longest = res.iters - iters > longest ? res.iters - iters : longest;
        iters = res.iters;
        if (res.done == DONE_WAIT_TIMEOUT)
            return fail(OGB_E_CUDA, "fused block-Jacobi update: the blocks did not all arrive within the wait limit");
        if (res.done == 3) { status = OGB_E_ZERODIAG; break; }
        if (res.done == 2) {   // FP32 recurrences broke down: finish in FP64
            *stalled = true;
            break;
        }
        if constexpr (F32) {
            if (!ctx->mixed_x64) {
                // fold the FP32 increment into the FP64 solution
                k_fold_increment<<<num_sms() * 8, NTHREADS, 0, s>>>(n, x, d);
                count_launch(ctx);
            }
        }
    }
    if (info) {
        info->iterations = iters;
        info->outer = replacements;
        info->achieved = achieved;
        info->status = status;
    }
    return OGB_OK;
}

bool sell_current(const ogb_mtrx *m) { return m->has_sell && m->sell.v32_version == m->version; }

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
    Op op = make_op(m, false);
    return apply_op<double, double, false>(m->ctx, op, m->val.p, x, y, nullptr, nullptr, nullptr);
}

static int map_status(int done)
{
    switch (done) {
    case 1: return OGB_OK;
    case 2: return OGB_E_BREAKDOWN;
    case 3: return OGB_E_ZERODIAG;
    default: return OGB_E_NOTCONV;
    }
}

// Operator-space copies of b and x: node space for the SELL operator, the
// padded equation space (b, x themselves) for CSR.
static int to_op_space(ogb_mtrx *m, const Op &op, const double *b, double *x, const double **bo, double **xo)
{
    if (!op.sell) {
        *bo = b;
        *xo = x;
        return OGB_OK;
    }
    cudaStream_t s = m->ctx->stream;
    OGB_CHECK(m->n_b.alloc(op.n));
    OGB_CHECK(m->n_x.alloc(op.n));
    OGB_CUDA(cudaMemsetAsync(m->n_b.p, 0, op.n * sizeof(double), s));
    OGB_CUDA(cudaMemsetAsync(m->n_x.p, 0, op.n * sizeof(double), s));
    k_eq_to_ns<<<nb(m->neq), NTHREADS, 0, s>>>(m->neq, m->sell.ns_of_eq.p, b, m->n_b.p);
    k_eq_to_ns<<<nb(m->neq), NTHREADS, 0, s>>>(m->neq, m->sell.ns_of_eq.p, x, m->n_x.p);
    count_launch(m->ctx, 2);
    *bo = m->n_b.p;
    *xo = m->n_x.p;
    return OGB_OK;
}

static int from_op_space(ogb_mtrx *m, const Op &op, double *x)
{
    if (!op.sell) return OGB_OK;
    k_ns_to_eq<<<nb(m->neq), NTHREADS, 0, m->ctx->stream>>>(m->neq, m->sell.ns_of_eq.p, m->n_x.p, x);
    count_launch(m->ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

// FP64 drop-in solve on padded equation-space device vectors (padding zero).
int pcg_fp64(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, ogb_solve_info *info)
{
    if (m->precond == 4 || m->precond == 2) {   // IC / ILU: equation space, CSR operator
        Op op = make_op(m, false);
        OGB_CHECK(ensure_workspace(m, op, false));
        PcgScal res{};
        OGB_CHECK(pcg_ic_core(m, op, b, x, rtol, maxit, res));
        double normb = sqrt(res.bnorm2);
        if (normb == 0.0) normb = 1.0;
        if (info) {
            info->iterations = res.iters;
            info->outer = 0;
            info->achieved = sqrt(res.rnorm2) / normb;
            info->status = map_status(res.done);
        }
        return OGB_OK;
    }
    const bool use_sell = sell_current(m);
    Op op = make_op(m, use_sell);
    OGB_CHECK(ensure_workspace(m, op, false));
    const double *bo;
    double *xo;
    OGB_CHECK(to_op_space(m, op, b, x, &bo, &xo));
    PcgScal res{};
    OGB_CHECK(pcg64_core(m, op, use_sell ? m->sell.v64.p : m->val.p, bo, xo, rtol, maxit, res));
    OGB_CHECK(from_op_space(m, op, x));
    double normb = sqrt(res.bnorm2);
    if (normb == 0.0) normb = 1.0;
    if (info) {
        info->iterations = res.iters;
        info->outer = 0;
        info->achieved = sqrt(res.rnorm2) / normb;
        info->status = map_status(res.done);
    }
    return OGB_OK;
}

int pcg_mixed(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, ogb_solve_info *info)
{
    ogb_ctx *ctx = m->ctx;
    if (m->precond == 4 || m->precond == 2)
        return fail(OGB_E_ARG, "the IC and ILU preconditioners run in FP64 only");
    const bool use_sell = sell_current(m);
    Op op = make_op(m, use_sell);
    OGB_CHECK(ensure_workspace(m, op, true));
    const double *v64;
    const float *v32;
    if (use_sell) {
        v64 = m->sell.v64.p;
        v32 = m->sell.v32.p;
    } else {
        const int64_t ntot = m->nnz + (m->npad - m->neq);
        if (m->val32_version != m->version) {
            OGB_CHECK(m->val32.alloc(ntot));
            k_to_float<<<num_sms() * 8, NTHREADS, 0, ctx->stream>>>(ntot, m->val.p, m->val32.p);
            count_launch(ctx);
            m->val32_version = m->version;
        }
        v64 = m->val.p;
        v32 = m->val32.p;
    }
    const double *bo;
    double *xo;
    OGB_CHECK(to_op_space(m, op, b, x, &bo, &xo));
    ogb_solve_info mi{};
    bool stalled = false;
    if (m->ctx->mixed_vec32)
        OGB_CHECK((pcg_mixed_core<float, float>(m, op, v64, v32, bo, xo, rtol, maxit, &mi, &stalled)));
    else if (m->ctx->mixed_p32)
        OGB_CHECK((pcg_mixed_core<double, float>(m, op, v64, v32, bo, xo, rtol, maxit, &mi, &stalled)));
    else
        OGB_CHECK((pcg_mixed_core<double, double>(m, op, v64, v32, bo, xo, rtol, maxit, &mi, &stalled)));
    if (stalled && mi.status != OGB_OK && mi.iterations < maxit) {
        // the FP32 operator cannot reach this tolerance on this matrix: continue
        // from the current solution with the FP64 drop-in PCG (same test on ||b||)
        PcgScal res{};
        OGB_CHECK(pcg64_core(m, op, v64, bo, xo, rtol, maxit - mi.iterations, res));
        double normb = sqrt(res.bnorm2);
        if (normb == 0.0) normb = 1.0;
        mi.iterations += res.iters;
        mi.achieved = sqrt(res.rnorm2) / normb;
        mi.status = map_status(res.done);
    }
    if (info) *info = mi;
    OGB_CHECK(from_op_space(m, op, x));
    return OGB_OK;
}

int extract_diag(ogb_mtrx *m) { (void)m; return OGB_OK; }

}  // namespace ogb

// ---------------------------------------------------------------------------
// Allocation-free Jacobi-PCG (ogb_pcg_solve_noalloc).
//
// For callers that must not allocate device memory once they are running --
// for example an application that reserves the GPU's memory for its own pool
// at start-up, or a time-stepping loop in which a cudaMalloc/cudaFree (cudaFree
// synchronizes the whole device) would stall every stream. The caller passes
// the CSR matrix, b and x in device memory; the solver's work vectors live in
// the file-scope array below, which every GPU that loads this library holds
// until the process exits. All calls share it: a call clears what must start at
// zero, and two calls that overlap on the GPU (different streams or threads)
// race on it.
namespace ogb {
namespace {

constexpr int NOALLOC_MAX_ROWS = 1 << 17;           // 131,072 equations
constexpr int NOALLOC_GRID = 304;                   // fixed grid (2 x 152 SMs of a GB300): sizes the static partials
constexpr size_t NOALLOC_DOUBLES = (size_t)5 * NOALLOC_MAX_ROWS + 4 * NOALLOC_GRID + 16;

// r, z, p, q, dinv (NOALLOC_MAX_ROWS each), reduction partials, the PcgScal
// record and the last-block counter: about 5.2 MB.
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

struct NoallocView {
    double *r, *z, *p, *q, *dinv, *part;
    PcgScal *sc;
    unsigned int *count;
};

__host__ __device__ inline NoallocView noalloc_view(double *base)
{
    NoallocView v;
    v.r = base;
    v.z = base + NOALLOC_MAX_ROWS;
    v.p = base + 2 * (size_t)NOALLOC_MAX_ROWS;
    v.q = base + 3 * (size_t)NOALLOC_MAX_ROWS;
    v.dinv = base + 4 * (size_t)NOALLOC_MAX_ROWS;
    v.part = base + 5 * (size_t)NOALLOC_MAX_ROWS;
    v.sc = reinterpret_cast<PcgScal *>(v.part + 4 * NOALLOC_GRID);
    v.count = reinterpret_cast<unsigned int *>(v.sc + 1);
    return v;
}

// D^-1 by a binary search for the diagonal of each (sorted) row.
__global__ void k_na_diag(int n, const int64_t *__restrict__ rowptr, const int *__restrict__ colind,
                          const double *__restrict__ val, double *scratch)
{
    NoallocView w = noalloc_view(scratch);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int64_t lo = rowptr[i], hi = rowptr[i + 1] - 1;
        double d = 0.0;
        while (lo <= hi) {
            int64_t mid = (lo + hi) >> 1;
            int c = colind[mid];
            if (c < i) lo = mid + 1;
            else if (c > i) hi = mid - 1;
            else { d = val[mid]; break; }
        }
        if (d == 0.0) {
            w.sc->done = 3;
            w.dinv[i] = 0.0;
        } else {
            w.dinv[i] = 1.0 / d;
        }
    }
}

// y = A x (8 lanes per row); with DOT also x.y -> alpha = rho / p.q.
template <bool DOT>
__global__ void __launch_bounds__(NTHREADS) k_na_spmv(int n, const int64_t *__restrict__ rowptr,
                                                      const int *__restrict__ colind, const double *__restrict__ val,
                                                      const double *x, double *y, double *scratch)
{
    NoallocView w = noalloc_view(scratch);
    if (DOT && w.sc->done) return;
    const int sub = threadIdx.x >> 3, lane = threadIdx.x & 7;
    double acc[1] = {0.0};
    for (int64_t rb = (int64_t)blockIdx.x * (NTHREADS / 8); rb < n; rb += (int64_t)gridDim.x * (NTHREADS / 8)) {
        const int64_t row = rb + sub;
        double s = 0.0;
        if (row < n)
            for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += 8) s += val[k] * x[colind[k]];
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, 8);
        if (lane == 0 && row < n) {
            y[row] = s;
            if (DOT) acc[0] += x[row] * s;
        }
    }
    if (!DOT) return;
    block_sum<1>(acc);
    if (publish_partials<1>(acc, w.part, w.count)) {
        double t[1];
        final_sums<1>(w.part, t);
        if (threadIdx.x != 0) return;
        finish_pq(t[0], w.count, w.sc);
    }
}

__global__ void __launch_bounds__(NTHREADS) k_na_init(int n, const double *__restrict__ b, double *scratch,
                                                      double rtol)
{
    NoallocView w = noalloc_view(scratch);
    double v[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double rr = b[i] - w.q[i];
        double zz = rr * w.dinv[i];
        w.r[i] = rr;
        w.z[i] = zz;
        w.p[i] = zz;
        v[0] += b[i] * b[i];
        v[1] += rr * rr;
        v[2] += rr * zz;
    }
    block_sum<3>(v);
    if (publish_partials<3>(v, w.part, w.count)) {
        double t[3];
        final_sums<3>(w.part, t);
        if (threadIdx.x != 0) return;
        *w.count = 0;
        PcgScal *sc = w.sc;
        sc->bnorm2 = t[0];
        sc->rnorm2 = t[1];
        sc->rho = t[2];
        double normb = sqrt(t[0]);
        if (normb == 0.0) normb = 1.0;
        if (sc->done == 0) {
            if (sqrt(t[1]) / normb <= rtol) sc->done = 1;
            else if (!isfinite(t[2]) || !(t[2] > 0.0)) sc->done = 2;
        }
    }
}

__global__ void __launch_bounds__(NTHREADS) k_na_update(int n, double *__restrict__ x, double *scratch, double rtol,
                                                        int maxit)
{
    NoallocView w = noalloc_view(scratch);
    PcgScal *sc = w.sc;
    if (sc->done) return;
    const double alpha = sc->alpha;
    double v[2] = {0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * w.p[i];
        double rr = w.r[i] - alpha * w.q[i];
        double zz = rr * w.dinv[i];
        w.r[i] = rr;
        w.z[i] = zz;
        v[0] += rr * rr;
        v[1] += rr * zz;
    }
    block_sum<2>(v);
    if (publish_partials<2>(v, w.part, w.count)) {
        double t[2];
        final_sums<2>(w.part, t);
        if (threadIdx.x != 0) return;
        *w.count = 0;
        sc->rnorm2 = t[0];
        sc->iters += 1;
        double normb = sqrt(sc->bnorm2);
        if (normb == 0.0) normb = 1.0;
        if (sqrt(t[0]) / normb <= rtol) sc->done = 1;
        else if (!isfinite(t[1]) || !(t[1] > 0.0)) sc->done = 2;
        else if (sc->iters >= maxit) sc->done = 4;
        else {
            sc->beta = t[1] / sc->rho;
            sc->rho = t[1];
        }
    }
}

__global__ void __launch_bounds__(NTHREADS) k_na_pupdate(int n, double *scratch)
{
    NoallocView w = noalloc_view(scratch);
    if (w.sc->done) return;
    const double beta = w.sc->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w.p[i] = w.z[i] + beta * w.p[i];
}

// Device address of g_noalloc_scratch on the current device, looked up on every
// call (cheap; in host code the symbol's name is only a host-side stand-in, and
// a cached address would go stale after a device reset).
int noalloc_scratch(double **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    *out = static_cast<double *>(p);
    return OGB_OK;
}

}  // namespace
}  // namespace ogb

extern "C" int ogb_pcg_solve_noalloc(int n, const int64_t *rowptr, const int *colind, const double *val,
                                     const double *b, double *x, double rtol, int maxit, void *stream,
                                     ogb_solve_info *info)
{
    using namespace ogb;
    if (n < 0 || (n > 0 && (!rowptr || !colind || !val || !b || !x)))
        return fail(OGB_E_ARG, "ogb_pcg_solve_noalloc: null device pointer or negative size");
    if (n > NOALLOC_MAX_ROWS)
        return fail(OGB_E_LIMIT, "ogb_pcg_solve_noalloc: " + std::to_string(n) + " equations exceed its fixed maximum of " +
                                     std::to_string(NOALLOC_MAX_ROWS) + "; use ogb_pcg_solve");
    double *base = nullptr;
    OGB_CHECK(noalloc_scratch(&base));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    NoallocView w = noalloc_view(base);
    // the scalars and the last-block counter must start at zero
    OGB_CUDA(cudaMemsetAsync(w.sc, 0, sizeof(PcgScal) + sizeof(double), s));
    const int gv = NOALLOC_GRID;
    k_na_diag<<<gv, NTHREADS, 0, s>>>(n, rowptr, colind, val, base);
    k_na_spmv<false><<<gv, NTHREADS, 0, s>>>(n, rowptr, colind, val, x, w.q, base);
    k_na_init<<<gv, NTHREADS, 0, s>>>(n, b, base, rtol);
    OGB_CUDA(cudaGetLastError());
    PcgScal h{};
    for (int it = 0;; it += BATCH) {
        OGB_CUDA(cudaMemcpyAsync(&h, w.sc, sizeof(PcgScal), cudaMemcpyDeviceToHost, s));
        OGB_CUDA(cudaStreamSynchronize(s));
        if (h.done || it >= maxit) break;
        for (int k = 0; k < BATCH; ++k) {
            k_na_spmv<true><<<gv, NTHREADS, 0, s>>>(n, rowptr, colind, val, w.p, w.q, base);
            k_na_update<<<gv, NTHREADS, 0, s>>>(n, x, base, rtol, maxit);
            k_na_pupdate<<<gv, NTHREADS, 0, s>>>(n, base);
        }
        OGB_CUDA(cudaGetLastError());
    }
    double normb = sqrt(h.bnorm2);
    if (normb == 0.0) normb = 1.0;
    int st = map_status(h.done);
    if (info) {
        info->iterations = h.iters;
        info->outer = 0;
        info->achieved = sqrt(h.rnorm2) / normb;
        info->status = st;
    }
    if (st != OGB_OK)
        set_error(st == OGB_E_ZERODIAG ? "zero diagonal detected"
                  : st == OGB_E_BREAKDOWN ? "PCG breakdown (rho or p'q not positive/finite)"
                                          : "PCG did not converge within maxit");
    return st;
}
