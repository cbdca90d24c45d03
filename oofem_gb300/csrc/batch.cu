// Batched Jacobi-PCG: many independent meshes (instances) and several load
// cases per mesh (right-hand sides) advanced together, one set of launches per
// CG iteration for the whole batch.
//
// Every (instance, right-hand side) pair runs its own IML CG (iml/cg.h:22-71,
// DiagPreconditioner diagpre.C:60-67) with its own scalars and convergence
// test; a pair that has converged is masked out and its solution no longer
// changes, so each pair's result is that of a separate FP64 drop-in solve. The
// matrix is streamed once per iteration for all right-hand sides: vectors are
// node-space, right-hand sides interleaved (entry (row, c) at row * NR + c).
//
// Instances start on 1024-node-row boundaries of the node-block storage, so
// every reduction unit -- a SpMV block of 256 node rows, a vector block of 256
// scalar rows -- belongs to one instance. Each instance has its own completion
// counter: the last block of an instance to publish its partials sums that
// instance's partials in a fixed order and updates its pairs' scalars. Sums do
// not depend on block scheduling (bitwise reproducible, no floating-point
// atomics), and the per-instance epilogues run in parallel across the grid.
//
// Mixed precision (FP32 matrix and vectors, FP64 residual replacements) keeps
// the solution as an FP32 increment of the current batch of captured
// iterations, folded into the FP64 solution after each batch, and, for two DOFs
// per node, preconditions with the 2 x 2 node-block inverses.
#include <math.h>

#include <functional>
#include <vector>

#include <memory>

#include "internal.cuh"
#include "reduce.cuh"

namespace ogb {

namespace {

struct BatchScal {
    double bnorm2, rho, pq, rnorm2, alpha, beta;
    double mark;   // mixed precision: FP64 residual^2 at the last halving
    double rrep;   // mixed precision: FP64 residual^2 at the last replacement (the drop test's reference)
    int done;      // 0 running, 1 converged, 2 breakdown, 3 zero pivot, 4 iteration limit, 5 stalled (mixed)
    int iters;
    int pause;     // mixed precision: waits for the next FP64 residual replacement
    int since;     // mixed precision: replacements since the FP64 residual last halved
    int repl;      // mixed precision: replaced in the last replacement pass, p update pending
    int pad_;
};

constexpr int RPT = 4;                       // scalar rows per thread in the vector kernels
constexpr int UNIT = RPT * NTHREADS;         // scalar rows per vector block (1024)
constexpr int SPMV_SLICES = NTHREADS / 32;   // slices (of 32 node rows) per SpMV block
constexpr int MAXNR = 4;
constexpr int BBATCH = 16;                   // iterations per captured graph

// Publish the block sums v (valid in thread 0) for block `unit`; true in every
// thread of the block that completed its instance (count reaches its units).
template <int NV>
__device__ __forceinline__ bool publish_inst(const double (&v)[NV], double *part, int64_t unit, unsigned int *cnt,
                                             int64_t inst_units)
{
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) part[unit * NV + k] = v[k];
        __threadfence();
        const unsigned int t = atomicAdd(cnt, 1u);
        s_last = ((int64_t)t == inst_units - 1);
    }
    __syncthreads();
    return s_last;
}

// Fixed-order sums of the partials of units [u0, u1): thread t takes units
// u0+t, u0+t+256, ..., then the fixed-order block reduction. Valid in thread 0.
template <int NV>
__device__ __forceinline__ void inst_sums(const double *part, int64_t u0, int64_t u1, double (&out)[NV])
{
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = 0.0;
#pragma unroll 4
    for (int64_t u = u0 + threadIdx.x; u < u1; u += NTHREADS)
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] += __ldcg(part + u * NV + k);
    block_sum<NV>(out);
}

// Instance skip test (the same for every block of the instance within one
// launch). mode 1: no pair of the instance is running (all converged, failed or
// waiting for a residual replacement); mode 2: every pair is finished; mode 3:
// no pair waits for a residual replacement.
template <int NR>
__device__ __forceinline__ bool inst_skip(const BatchScal *sc, int inst, int mode)
{
    bool all = true;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        const BatchScal &q = sc[inst * NR + c];
        if (mode == 3) all = all && !(q.done == 0 && q.pause != 0);
        else all = all && (q.done != 0 || (mode == 1 && q.pause != 0));
    }
    return all;
}
template <int NR>
__device__ __forceinline__ bool pair_running(const BatchScal &q)
{
    return q.done == 0 && q.pause == 0;
}

// The W entries of one node row of an interleaved vector (W = ND x NR values,
// the row starting at a multiple of W): 16-byte loads when W is a multiple of 4
// floats, 8-byte loads when even (the row start is then aligned to them), else
// single loads -- fewer gather instructions per block.
template <int W>
__device__ __forceinline__ void gather_row(const float *__restrict__ src, float (&dst)[W])
{
    if constexpr (W % 4 == 0) {
#pragma unroll
        for (int j = 0; j < W; j += 4) {
            const float4 v = __ldg(reinterpret_cast<const float4 *>(src + j));
            dst[j] = v.x; dst[j + 1] = v.y; dst[j + 2] = v.z; dst[j + 3] = v.w;
        }
    } else if constexpr (W % 2 == 0) {
#pragma unroll
        for (int j = 0; j < W; j += 2) {
            const float2 v = __ldg(reinterpret_cast<const float2 *>(src + j));
            dst[j] = v.x; dst[j + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int j = 0; j < W; ++j) dst[j] = __ldg(src + j);
    }
}

template <int W>
__device__ __forceinline__ void gather_row(const double *__restrict__ src, double (&dst)[W])
{
    if constexpr (W % 2 == 0) {
#pragma unroll
        for (int j = 0; j < W; j += 2) {
            const double2 v = __ldg(reinterpret_cast<const double2 *>(src + j));
            dst[j] = v.x; dst[j + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int j = 0; j < W; ++j) dst[j] = __ldg(src + j);
    }
}

// q = K p for all right-hand sides: matrix values V, vectors X, products and
// sums in V. DOT: also p.q per pair (block sums in V per warp, FP64 above) and
// alpha for running pairs. DIFF: the FP32 difference form (the diagonal slot
// holds the block row sum, off-diagonal products act on x_B - x_A). skip: the
// inst_skip mode (0 = never). Block columns are prefetched one group ahead.
// EXPL: all values of a group are loaded before its products (more loads in
// flight per warp; same products in the same order).
template <int ND, int NR, bool DOT, class V, class X, bool DIFF, bool EXPL = false>
__global__ void __launch_bounds__(NTHREADS) k_bspmv(int nslices, const int64_t *__restrict__ sl_ptr,
                                                    const int *__restrict__ sl_width, const int *__restrict__ col,
                                                    const V *__restrict__ val, const X *__restrict__ x,
                                                    X *__restrict__ y, double *part, unsigned int *cnt,
                                                    BatchScal *sc, const int *__restrict__ unit_inst,
                                                    const int64_t *__restrict__ unit_ptr, int skip)
{
    if (skip && inst_skip<NR>(sc, unit_inst[blockIdx.x], skip)) return;
    constexpr int W = ND * NR;               // vector entries per node row
    // blocks per prefetch group: FP64 products are bound by the FP64 pipe and
    // gain nothing from the extra registers of deeper prefetch
    constexpr int G = sizeof(V) == 8 ? 1 : 4;
    const int s = blockIdx.x * SPMV_SLICES + (threadIdx.x >> 5);
    const int r = threadIdx.x & 31;
    V dot[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) dot[c] = 0;
    if (s < nslices) {
        const int64_t base = sl_ptr[s];
        const int w = sl_width[s];
        const int arow = s * 32 + r;
        V yy[ND][NR], xa[W];
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int c = 0; c < NR; ++c) yy[i][c] = 0;
#pragma unroll
        for (int j = 0; j < W; ++j) xa[j] = DIFF ? (V)x[(int64_t)arow * W + j] : (V)0;
        const V *vp = val + base * (ND * ND) + r;
        const int *cp = col + base + r;
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
            V xb[G][W];
#pragma unroll
            for (int g = 0; g < G; ++g) {
                gather_row<W>(x + (int64_t)cc[g] * W, xb[g]);
                if (DIFF && cc[g] != arow)
#pragma unroll
                    for (int j = 0; j < W; ++j) xb[g][j] -= xa[j];
            }
            if constexpr (EXPL) {
                // every value of the group loaded before the group's products
                V vv[G][ND * ND];
#pragma unroll
                for (int g = 0; g < G; ++g)
#pragma unroll
                    for (int q = 0; q < ND * ND; ++q)
                        vv[g][q] = k0 + g < w ? __ldcs(vp + (int64_t)(k0 + g) * (32 * ND * ND) + 32 * q) : (V)0;
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (k0 + g < w) {
#pragma unroll
                        for (int i = 0; i < ND; ++i)
#pragma unroll
                            for (int j = 0; j < ND; ++j)
#pragma unroll
                                for (int c = 0; c < NR; ++c)
                                    yy[i][c] = fma(vv[g][i * ND + j], xb[g][j * NR + c], yy[i][c]);
                    }
                }
            } else {
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (k0 + g < w) {
                        const V *vk = vp + (int64_t)(k0 + g) * (32 * ND * ND);
#pragma unroll
                        for (int i = 0; i < ND; ++i)
#pragma unroll
                            for (int j = 0; j < ND; ++j) {
                                const V v = __ldcs(vk + 32 * (i * ND + j));
#pragma unroll
                                for (int c = 0; c < NR; ++c) yy[i][c] = fma(v, xb[g][j * NR + c], yy[i][c]);
                            }
                    }
                }
            }
        }
        const int64_t a = (int64_t)s * 32 + r;
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                y[(a * ND + i) * NR + c] = (X)yy[i][c];
                if (DOT) dot[c] = fma((V)x[(a * ND + i) * NR + c], yy[i][c], dot[c]);
            }
    }
    if (!DOT) return;
    const int inst = unit_inst[blockIdx.x];
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
    double bs[NR];
    block_sum_t<NR, V>(dot, bs);
    if (!publish_inst<NR>(bs, part, blockIdx.x, cnt + inst, u1 - u0)) return;
    double t[NR];
    inst_sums<NR>(part, u0, u1, t);
    if (threadIdx.x != 0) return;
    cnt[inst] = 0;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        BatchScal &q = sc[inst * NR + c];
        if (!pair_running<NR>(q)) continue;
        q.pq = t[c];
        if (!(t[c] > 0.0) || !isfinite(t[c])) q.done = sizeof(V) == 4 ? 5 : 2;   // FP32: the FP64 pass takes over
        else q.alpha = q.rho / t[c];
    }
}

// r = b - q, z = p = D^-1 r; per pair ||b||^2, ||r||^2, r.z and the initial test.
template <int NR>
__global__ void __launch_bounds__(NTHREADS) k_binit(const double *__restrict__ b, const double *__restrict__ q,
                                                    const double *__restrict__ dinv, double *__restrict__ r,
                                                    double *__restrict__ z, double *__restrict__ p, double *part,
                                                    unsigned int *cnt, BatchScal *sc,
                                                    const int *__restrict__ unit_inst,
                                                    const int64_t *__restrict__ unit_ptr, double rtol)
{
    double v[3 * NR];
#pragma unroll
    for (int k = 0; k < 3 * NR; ++k) v[k] = 0.0;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int64_t row = (int64_t)blockIdx.x * UNIT + j * NTHREADS + threadIdx.x;
        const double di = dinv[row];
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            const int64_t k = row * NR + c;
            const double bb = b[k];
            const double rr = bb - q[k];
            const double zz = rr * di;
            r[k] = rr;
            z[k] = zz;
            p[k] = zz;
            v[c] += bb * bb;
            v[NR + c] += rr * rr;
            v[2 * NR + c] += rr * zz;
        }
    }
    const int inst = unit_inst[blockIdx.x];
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
    block_sum<3 * NR>(v);
    if (!publish_inst<3 * NR>(v, part, blockIdx.x, cnt + inst, u1 - u0)) return;
    double t[3 * NR];
    inst_sums<3 * NR>(part, u0, u1, t);
    if (threadIdx.x != 0) return;
    cnt[inst] = 0;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        BatchScal &s = sc[inst * NR + c];
        s.bnorm2 = t[c];
        s.rnorm2 = t[NR + c];
        s.rho = t[2 * NR + c];
        s.iters = 0;
        double normb = sqrt(t[c]);
        if (normb == 0.0) normb = 1.0;
        if (s.done == 0) {
            if (sqrt(t[NR + c]) / normb <= rtol) s.done = 1;
            else if (!isfinite(t[2 * NR + c]) || !(t[2 * NR + c] > 0.0)) s.done = 2;
        }
    }
}

// x += alpha p, r -= alpha q, z = D^-1 r for running pairs; per pair ||r||^2,
// r.z, the convergence test of cg.h:63-66 and beta.
template <int NR>
__global__ void __launch_bounds__(NTHREADS) k_bupdate(double *__restrict__ x, double *__restrict__ r,
                                                      double *__restrict__ z, const double *__restrict__ p,
                                                      const double *__restrict__ q, const double *__restrict__ dinv,
                                                      double *part, unsigned int *cnt, BatchScal *sc,
                                                      const int *__restrict__ unit_inst,
                                                      const int64_t *__restrict__ unit_ptr, double rtol, int maxit)
{
    const int inst = unit_inst[blockIdx.x];
    if (inst_skip<NR>(sc, inst, 1)) return;
    bool run[NR];
    double alpha[NR], v[2 * NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        run[c] = sc[inst * NR + c].done == 0;   // converged pairs keep their solution
        alpha[c] = sc[inst * NR + c].alpha;
        v[c] = 0.0;
        v[NR + c] = 0.0;
    }
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int64_t row = (int64_t)blockIdx.x * UNIT + j * NTHREADS + threadIdx.x;
        const double di = dinv[row];
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            if (!run[c]) continue;
            const int64_t k = row * NR + c;
            x[k] = fma(alpha[c], p[k], x[k]);
            const double rr = fma(-alpha[c], q[k], r[k]);
            const double zz = rr * di;
            r[k] = rr;
            z[k] = zz;
            v[c] += rr * rr;
            v[NR + c] += rr * zz;
        }
    }
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
    block_sum<2 * NR>(v);
    if (!publish_inst<2 * NR>(v, part, blockIdx.x, cnt + inst, u1 - u0)) return;
    double t[2 * NR];
    inst_sums<2 * NR>(part, u0, u1, t);
    if (threadIdx.x != 0) return;
    cnt[inst] = 0;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        BatchScal &s = sc[inst * NR + c];
        if (s.done) continue;
        s.rnorm2 = t[c];
        s.iters += 1;
        double normb = sqrt(s.bnorm2);
        if (normb == 0.0) normb = 1.0;
        if (sqrt(t[c]) / normb <= rtol) s.done = 1;
        else if (!isfinite(t[NR + c]) || !(t[NR + c] > 0.0)) s.done = 2;
        else if (s.iters >= maxit) s.done = 4;
        else {
            s.beta = t[NR + c] / s.rho;
            s.rho = t[NR + c];
        }
    }
}

template <int NR>
__global__ void __launch_bounds__(NTHREADS) k_bpupdate(const double *__restrict__ z, double *__restrict__ p,
                                                       const BatchScal *sc, const int *__restrict__ unit_inst)
{
    const int inst = unit_inst[blockIdx.x];
    if (inst_skip<NR>(sc, inst, 1)) return;
    bool run[NR];
    double beta[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        run[c] = sc[inst * NR + c].done == 0;
        beta[c] = sc[inst * NR + c].beta;
    }
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int64_t row = (int64_t)blockIdx.x * UNIT + j * NTHREADS + threadIdx.x;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            if (!run[c]) continue;
            const int64_t k = row * NR + c;
            p[k] = fma(beta[c], p[k], z[k]);
        }
    }
}

// Inverse of the point diagonal of every node row (padding rows hold identity),
// from the FP64 values, stored as T.
template <int ND, class T>
__global__ void k_bdiag(int nrows, const int64_t *__restrict__ diag, const double *__restrict__ val,
                        T *__restrict__ dinv, int *zero_diag)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows) return;
    const int64_t slot = diag[a];
    const int r = (int)(slot & 31);
    const double *vb = val + (slot - r) * (ND * ND) + r;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
        const double v = vb[32 * (d * ND + d)];
        if (v == 0.0) {
            atomicExch(zero_diag, 1);
            dinv[(int64_t)a * ND + d] = 0;
        } else {
            dinv[(int64_t)a * ND + d] = (T)(1.0 / v);
        }
    }
}

// Block Jacobi for two DOFs per node: node a's 2 x 2 diagonal block inverted in
// FP64, row d of the inverse stored (FP32) with node row 2a + d. The blocks of
// prescribed DOFs hold a unit diagonal with zeroed couplings (identity rows).
__global__ void k_bbinv2(int nrows, const int64_t *__restrict__ diag, const double *__restrict__ val,
                         float2 *__restrict__ binv, int *zero_diag)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows) return;
    const int64_t slot = diag[a];
    const int r = (int)(slot & 31);
    const double *vb = val + (slot - r) * 4 + r;
    const double d00 = vb[0], d01 = vb[32], d10 = vb[64], d11 = vb[96];
    const double det = d00 * d11 - d01 * d10;
    if (!(det != 0.0) || !isfinite(det)) {
        atomicExch(zero_diag, 1);
        binv[2 * (int64_t)a] = make_float2(0.f, 0.f);
        binv[2 * (int64_t)a + 1] = make_float2(0.f, 0.f);
        return;
    }
    const double inv = 1.0 / det;
    binv[2 * (int64_t)a] = make_float2((float)(d11 * inv), (float)(-d01 * inv));
    binv[2 * (int64_t)a + 1] = make_float2((float)(-d10 * inv), (float)(d00 * inv));
}

// z of one row from the preconditioner: the scalar inverse diagonal, or (BJ2)
// the row of its node's 2 x 2 block inverse applied to the node's two residual
// entries (the partner row is the neighbouring lane: node rows 2a, 2a + 1 sit
// on an even and the following odd lane). Called by every lane of the warp.
template <bool BJ2>
__device__ __forceinline__ float bprecond(float rf, const float *__restrict__ dinv, const float2 *__restrict__ binv,
                                         int64_t row)
{
    if constexpr (!BJ2) {
        return rf * dinv[row];
    } else {
        const float ro = __shfl_xor_sync(0xffffffffu, rf, 1);
        const bool odd = row & 1;
        const float r0 = odd ? ro : rf, r1 = odd ? rf : ro;
        const float2 b = binv[row];
        return fmaf(b.y, r1, b.x * r0);
    }
}

// ---- mixed precision: FP32 matrix (difference form) and FP32 r, z, p, q per
// pair, FP64 solution x. A pair whose recursive residual has dropped by the drop
// factor since its last replacement, or reached half the tolerance, or the
// iteration limit, pauses in the update; after the current batch of captured
// iterations its true residual b - K64 x is formed in FP64 and replaces r, z and
// the CG scalars (reliable update), convergence being decided on it only, and
// p = z + beta p continues the recurrence. Running pairs are not touched by a
// replacement.
// FP64 residual replacement (reliable update) of the pairs that paused -- their
// recursive FP32 residual dropped by the drop factor since their last
// replacement, or reached half the tolerance, or the FP32 recurrences ended --
// and of every pair at init: r = b - K64 x (FP64, stored FP32), z = D^-1 r; per
// pair ||b||^2 (init), ||r||^2 and r.z; the convergence test on the FP64
// residual; for pairs that go on, beta = r.z / rho of the last iteration (0 at
// init) for the pending p = z + beta p (k_bpupdate32 in replacement mode).
// Pairs that are still running are left alone: their p already holds this
// iteration's update, so replacing their r and z would break the recurrence.
template <int NR, bool BJ2 = false>
__global__ void __launch_bounds__(NTHREADS) k_breplace(const double *__restrict__ b, const double *__restrict__ q64,
                                                       const float *__restrict__ dinv,
                                                       const float2 *__restrict__ binv, float *__restrict__ r,
                                                       float *__restrict__ z, double *part, unsigned int *cnt,
                                                       BatchScal *sc, const int *__restrict__ unit_inst,
                                                       const int64_t *__restrict__ unit_ptr, double rtol, int maxit,
                                                       int init)
{
    const int inst = unit_inst[blockIdx.x];
    if (inst_skip<NR>(sc, inst, init ? 2 : 3)) return;
    bool live[NR];
    double v[3 * NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        const BatchScal &s = sc[inst * NR + c];
        live[c] = s.done == 0 && (init || s.pause);
        v[c] = 0.0;
        v[NR + c] = 0.0;
        v[2 * NR + c] = 0.0;
    }
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int64_t row = (int64_t)blockIdx.x * UNIT + j * NTHREADS + threadIdx.x;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            if (!live[c]) continue;   // the same for the whole warp (one instance)
            const int64_t k = row * NR + c;
            const double bb = b[k];
            const double r6 = bb - q64[k];
            const float rf = (float)r6;
            const float zf = bprecond<BJ2>(rf, dinv, binv, row);
            r[k] = rf;
            z[k] = zf;
            v[c] += bb * bb;
            v[NR + c] += r6 * r6;
            v[2 * NR + c] += (double)(rf * zf);
        }
    }
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
    block_sum<3 * NR>(v);
    if (!publish_inst<3 * NR>(v, part, blockIdx.x, cnt + inst, u1 - u0)) return;
    double t[3 * NR];
    inst_sums<3 * NR>(part, u0, u1, t);
    if (threadIdx.x != 0) return;
    cnt[inst] = 0;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        BatchScal &s = sc[inst * NR + c];
        if (s.done || !(init || s.pause)) continue;
        if (init) {
            s.bnorm2 = t[c];
            s.iters = 0;
            s.mark = t[NR + c];
            s.since = 0;
        }
        double normb = sqrt(s.bnorm2);
        if (normb == 0.0) normb = 1.0;
        s.rnorm2 = t[NR + c];
        const double rz = t[2 * NR + c];
        // stagnation: six replacements without halving the FP64 residual, or an
        // FP32 breakdown, hand the pair to the FP64 pass
        if (!init) {
            if (t[NR + c] < 0.25 * s.mark) {
                s.mark = t[NR + c];
                s.since = 0;
            } else {
                ++s.since;
            }
        }
        if (sqrt(t[NR + c]) / normb <= rtol) s.done = 1;
        else if (!isfinite(t[NR + c])) s.done = 2;
        else if (s.iters >= maxit) s.done = 4;
        else if (!isfinite(rz) || !(rz > 0.0) || s.since >= 6) s.done = 5;
        else {
            s.beta = init ? 0.0 : rz / s.rho;
            s.rho = rz;
            s.rrep = t[NR + c];
            s.pause = 0;
            s.repl = 1;
        }
    }
}

// x64 += alpha p, r -= alpha q, z = D^-1 r for running pairs (FP32 but x);
// per pair ||r||^2 and r.z (FP32 per thread and warp, FP64 above), the pause
// test and beta.
template <int NR, bool BJ2 = false, class XS = double>
__global__ void __launch_bounds__(NTHREADS) k_bupdate32(XS *__restrict__ x, float *__restrict__ r,
                                                        float *__restrict__ z, const float *__restrict__ p,
                                                        const float *__restrict__ q, const float *__restrict__ dinv,
                                                        const float2 *__restrict__ binv,
                                                        double *part, unsigned int *cnt, BatchScal *sc,
                                                        const int *__restrict__ unit_inst,
                                                        const int64_t *__restrict__ unit_ptr, double rtol, int maxit,
                                                        double drop2)
{
    const int inst = unit_inst[blockIdx.x];
    if (inst_skip<NR>(sc, inst, 1)) return;
    bool run[NR];
    double alpha[NR];
    float v[2 * NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        const BatchScal &s = sc[inst * NR + c];
        run[c] = pair_running<NR>(s);
        alpha[c] = s.alpha;
        v[c] = 0.f;
        v[NR + c] = 0.f;
    }
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int64_t row = (int64_t)blockIdx.x * UNIT + j * NTHREADS + threadIdx.x;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            if (!run[c]) continue;   // the same for the whole warp (one instance)
            const int64_t k = row * NR + c;
            const float pp = p[k];
            if constexpr (sizeof(XS) == 8) x[k] = fma(alpha[c], (double)pp, x[k]);
            else x[k] = fmaf((float)alpha[c], pp, x[k]);   // FP32 increment of the current batch
            const float rr = fmaf(-(float)alpha[c], q[k], r[k]);
            const float zz = bprecond<BJ2>(rr, dinv, binv, row);
            r[k] = rr;
            z[k] = zz;
            v[c] = fmaf(rr, rr, v[c]);
            v[NR + c] = fmaf(rr, zz, v[NR + c]);
        }
    }
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
    double bs[2 * NR];
    block_sum_t<2 * NR, float>(v, bs);
    if (!publish_inst<2 * NR>(bs, part, blockIdx.x, cnt + inst, u1 - u0)) return;
    double t[2 * NR];
    inst_sums<2 * NR>(part, u0, u1, t);
    if (threadIdx.x != 0) return;
    cnt[inst] = 0;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        BatchScal &s = sc[inst * NR + c];
        if (!pair_running<NR>(s)) continue;
        s.rnorm2 = t[c];
        s.iters += 1;
        s.repl = 0;
        double normb = sqrt(s.bnorm2);
        if (normb == 0.0) normb = 1.0;
        const double half = 0.5 * rtol * normb;
        // pause for an FP64 replacement once the recursive residual has dropped by
        // the drop factor since the last one (or reached half the tolerance); rho
        // stays that of this iteration's direction for the continuation
        if (!isfinite(t[c]) || !isfinite(t[NR + c])) s.done = 5;
        else if (t[c] <= half * half || t[c] <= drop2 * s.rrep || !(t[NR + c] > 0.0) || s.iters >= maxit)
            s.pause = 1;
        else {
            s.beta = t[NR + c] / s.rho;
            s.rho = t[NR + c];
        }
    }
}

// p = z + beta p: mode 0 for the running pairs of an iteration, mode 1 for the
// pairs a replacement pass just restarted (k_breplace's beta; 0 at init).
template <int NR>
__global__ void __launch_bounds__(NTHREADS) k_bpupdate32(const float *__restrict__ z, float *__restrict__ p,
                                                         const BatchScal *sc, const int *__restrict__ unit_inst,
                                                         int mode)
{
    const int inst = unit_inst[blockIdx.x];
    if (mode == 0 && inst_skip<NR>(sc, inst, 1)) return;
    bool run[NR];
    float beta[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        const BatchScal &s = sc[inst * NR + c];
        run[c] = mode == 0 ? pair_running<NR>(s) : (s.repl != 0 && s.done == 0);
        beta[c] = (float)s.beta;
    }
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int64_t row = (int64_t)blockIdx.x * UNIT + j * NTHREADS + threadIdx.x;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            if (!run[c]) continue;
            const int64_t k = row * NR + c;
            p[k] = fmaf(beta[c], p[k], z[k]);
        }
    }
}

// x64 += d, d = 0: the FP32 increment of a batch of iterations folded into the
// FP64 solution.
__global__ void k_bfold(int64_t n, double *__restrict__ x, float *__restrict__ d)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += (double)d[i];
        d[i] = 0.f;
    }
}

// x = 0 for the pairs that ended stalled with a residual above their starting
// one (or not finite): their FP64 pass must not start from diverged iterates.
template <int NR>
__global__ void __launch_bounds__(NTHREADS) k_bzero_diverged(double *__restrict__ x, const BatchScal *sc,
                                                              const int *__restrict__ unit_inst)
{
    const int inst = unit_inst[blockIdx.x];
    bool zero[NR];
    bool any = false;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        const BatchScal &s = sc[inst * NR + c];
        zero[c] = s.done == 5 && !(s.rnorm2 <= s.bnorm2);
        any = any || zero[c];
    }
    if (!any) return;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int64_t row = (int64_t)blockIdx.x * UNIT + j * NTHREADS + threadIdx.x;
#pragma unroll
        for (int c = 0; c < NR; ++c)
            if (zero[c]) x[row * NR + c] = 0.0;
    }
}

struct BatchWork {
    DBuf<int> vinst, sinst, zero;
    DBuf<int64_t> vptr, sptr;
    DBuf<BatchScal> sc;
    DBuf<double> part, r, z, p, q, dinv, q64;
    DBuf<float> r32, z32, p32, q32, dinv32;
    DBuf<float2> binv2;   // block Jacobi rows (two DOFs per node)
    DBuf<float> d32;      // FP32 solution increment of the current batch (batch_x64 off)
    DBuf<unsigned int> cnt;
};

// Captures `iteration` BBATCH times into an executable graph (exec stays null
// when graphs are off).
template <class F>
int capture_batch(ogb_ctx *ctx, F &&iteration, cudaGraphExec_t &exec)
{
    exec = nullptr;
    if (!ctx->use_graphs) return OGB_OK;
    cudaGraph_t g = nullptr;
    OGB_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < BBATCH; ++k) iteration();
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return OGB_OK;
}

struct ExecGuard {
    cudaGraphExec_t e = nullptr;
    ~ExecGuard()
    {
        if (e) cudaGraphExecDestroy(e);
    }
};

template <int ND, int NR>
int run_batch(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, bool mixed,
              std::vector<BatchScal> &res)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    const SellMat &S = m->sell;
    const int ninst = S.ninst, npair = ninst * NR;
    const int64_t nrows = S.nns();   // scalar rows
    const int nvu = (int)(nrows / UNIT);
    const int nsu = (int)ceil_div(S.nslices, SPMV_SLICES);
    std::vector<int> vinst(nvu), sinst(nsu);
    std::vector<int64_t> vptr(ninst + 1), sptr(ninst + 1);
    for (int i = 0; i <= ninst; ++i) {
        vptr[i] = S.inst_row_base[i] * ND / UNIT;            // 1024 * ND / 1024: exact
        sptr[i] = S.inst_row_base[i] / (32 * SPMV_SLICES);   // 1024 / 256: exact
    }
    for (int i = 0; i < ninst; ++i) {
        for (int64_t u = vptr[i]; u < vptr[i + 1]; ++u) vinst[u] = i;
        for (int64_t u = sptr[i]; u < sptr[i + 1]; ++u) sinst[u] = i;
    }
    BatchWork w;
    const int64_t nv = nrows * NR;
    OGB_CHECK(w.vinst.alloc(nvu));
    OGB_CHECK(w.sinst.alloc(nsu));
    OGB_CHECK(w.vptr.alloc(ninst + 1));
    OGB_CHECK(w.sptr.alloc(ninst + 1));
    OGB_CHECK(w.sc.alloc(npair));
    OGB_CHECK(w.zero.alloc(1));
    OGB_CHECK(w.part.alloc((size_t)nvu * 3 * NR));
    OGB_CHECK(w.cnt.alloc(ninst));
    if (mixed) {
        OGB_CHECK(w.r32.alloc(nv));
        OGB_CHECK(w.z32.alloc(nv));
        OGB_CHECK(w.p32.alloc(nv));
        OGB_CHECK(w.q32.alloc(nv));
        OGB_CHECK(w.dinv32.alloc(nrows));
        OGB_CHECK(w.q64.alloc(nv));
    } else {
        OGB_CHECK(w.r.alloc(nv));
        OGB_CHECK(w.z.alloc(nv));
        OGB_CHECK(w.p.alloc(nv));
        OGB_CHECK(w.q.alloc(nv));
        OGB_CHECK(w.dinv.alloc(nrows));
    }
    OGB_CUDA(cudaMemcpyAsync(w.vinst.p, vinst.data(), nvu * sizeof(int), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(w.sinst.p, sinst.data(), nsu * sizeof(int), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(w.vptr.p, vptr.data(), (ninst + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(w.sptr.p, sptr.data(), (ninst + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemsetAsync(w.sc.p, 0, npair * sizeof(BatchScal), st));
    OGB_CUDA(cudaMemsetAsync(w.zero.p, 0, sizeof(int), st));
    OGB_CUDA(cudaMemsetAsync(w.cnt.p, 0, ninst * sizeof(unsigned int), st));
    const int nr = S.nslices * 32;
    const unsigned gd = (unsigned)ceil_div(nr, NTHREADS);
    // FP64 K x for every unfinished pair (the initial residual; the replacements)
    // skip 2: every unfinished pair (FP64 path, init); skip 3: instances with a paused pair
    auto residual_spmv = [&](double *q64, int skip) {
        k_bspmv<ND, NR, false, double, double, false><<<nsu, NTHREADS, 0, st>>>(
            S.nslices, S.sl_ptr.p, S.sl_width.p, S.col.p, S.v64.p, x, q64, nullptr, nullptr, w.sc.p, w.sinst.p,
            w.sptr.p, skip);
    };
    std::function<void()> iteration;
    // mixed preconditioner: FP32 block Jacobi of the 2 x 2 node blocks (two DOFs
    // per node) where the option allows it, else the scalar diagonal
    const bool bj2 = mixed && ND == 2 && ctx->mixed_bj;
    auto replace = [&, bj2](int init) {
        if (bj2)
            k_breplace<NR, true><<<nvu, NTHREADS, 0, st>>>(b, w.q64.p, w.dinv32.p, w.binv2.p, w.r32.p, w.z32.p,
                                                           w.part.p, w.cnt.p, w.sc.p, w.vinst.p, w.vptr.p, rtol, maxit,
                                                           init);
        else
            k_breplace<NR><<<nvu, NTHREADS, 0, st>>>(b, w.q64.p, w.dinv32.p, nullptr, w.r32.p, w.z32.p, w.part.p,
                                                     w.cnt.p, w.sc.p, w.vinst.p, w.vptr.p, rtol, maxit, init);
    };
    if (mixed) {
        m->last_bj = bj2;
        if (bj2) {
            OGB_CHECK(w.binv2.alloc(nrows));
            k_bbinv2<<<gd, NTHREADS, 0, st>>>(nr, S.diag.p, S.v64.p, w.binv2.p, w.zero.p);
        } else {
            k_bdiag<ND, float><<<gd, NTHREADS, 0, st>>>(nr, S.diag.p, S.v64.p, w.dinv32.p, w.zero.p);
        }
        residual_spmv(w.q64.p, 2);
        // p starts at zero: the init pass's p = z + 0 p is z
        OGB_CUDA(cudaMemsetAsync(w.p32.p, 0, nv * sizeof(float), st));
        replace(1);
        k_bpupdate32<NR><<<nvu, NTHREADS, 0, st>>>(w.z32.p, w.p32.p, w.sc.p, w.vinst.p, 1);
        const bool diff = ctx->mixed_diff;
        const double drop2 = ctx->mixed_drop * ctx->mixed_drop;
        // one iteration: q = K p (FP32), the updates (pairs whose recursive residual
        // dropped by the drop factor pause), p = z + beta p for the running pairs
        // FP32 SpMV form, timed once per matrix (the launches recompute q, p.q and
        // alpha of the same p: no state changes)
        auto spmv32 = [&, diff](int form) {
#define OGB_BSPMV_ARGS S.nslices, S.sl_ptr.p, S.sl_width.p, S.col.p, S.v32.p, w.p32.p, w.q32.p, w.part.p, w.cnt.p, \
                       w.sc.p, w.sinst.p, w.sptr.p, 1
            if (diff && form == 2) k_bspmv<ND, NR, true, float, float, true, true><<<nsu, NTHREADS, 0, st>>>(OGB_BSPMV_ARGS);
            else if (diff) k_bspmv<ND, NR, true, float, float, true><<<nsu, NTHREADS, 0, st>>>(OGB_BSPMV_ARGS);
            else if (form == 2) k_bspmv<ND, NR, true, float, float, false, true><<<nsu, NTHREADS, 0, st>>>(OGB_BSPMV_ARGS);
            else k_bspmv<ND, NR, true, float, float, false><<<nsu, NTHREADS, 0, st>>>(OGB_BSPMV_ARGS);
#undef OGB_BSPMV_ARGS
        };
        SellMat &Sm = const_cast<SellMat &>(S);
        if (ctx->batch_form) Sm.bform32 = ctx->batch_form;
        if (!Sm.bform32) {
            cudaEvent_t e0, e1;
            OGB_CUDA(cudaEventCreate(&e0));
            OGB_CUDA(cudaEventCreate(&e1));
            float best = 0.f;
            for (int f = 1; f <= 2; ++f) {
                spmv32(f);
                cudaEventRecord(e0, st);
                for (int k = 0; k < 3; ++k) spmv32(f);
                cudaEventRecord(e1, st);
                count_launch(ctx, 4);
                float ms = 0.f;
                cudaError_t e = cudaEventSynchronize(e1);
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess) {
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    return cuda_fail(e, "batched SpMV autotune");
                }
                if (f == 1 || ms < 0.98f * best) {
                    best = ms;
                    Sm.bform32 = f;
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        }
        const int bform = Sm.bform32;
        // with kernel timing on, one more launch of the chosen form on the first
        // search directions is timed when every pair is running (no instance
        // skipped): the launch recomputes q, p.q and alpha of the same p, so the
        // solve is unchanged. Algorithmic bytes: every stored value and block
        // column once (padding slots not counted), p read and q written once per
        // right-hand side
        if (ctx->prof) {
            std::vector<BatchScal> s0(npair);
            OGB_CUDA(cudaMemcpyAsync(s0.data(), w.sc.p, npair * sizeof(BatchScal), cudaMemcpyDeviceToHost, st));
            OGB_CUDA(cudaStreamSynchronize(st));
            bool all = true;
            for (const auto &q : s0) all = all && q.done == 0;
            if (all) {
                prof_begin(ctx);
                spmv32(bform);
                prof_end(ctx, (double)m->nnz * sizeof(float) + (double)m->nnz / (ND * ND) * sizeof(int) +
                                  2.0 * NR * (double)nrows * sizeof(float));
                count_launch(ctx);
            }
        }
        // solution accumulation: FP64 every iteration, or an FP32 increment folded
        // into the FP64 solution after every batch of BBATCH iterations (before any
        // FP64 residual replacement reads x)
        const bool x64 = ctx->batch_x64;
        if (!x64) {
            OGB_CHECK(w.d32.alloc(nv));
            OGB_CUDA(cudaMemsetAsync(w.d32.p, 0, nv * sizeof(float), st));
        }
        auto calls = std::make_shared<int>(0);
        iteration = [&, drop2, bform, bj2, x64, calls]() {
            spmv32(bform);
            if (bj2 && x64)
                k_bupdate32<NR, true><<<nvu, NTHREADS, 0, st>>>(x, w.r32.p, w.z32.p, w.p32.p, w.q32.p, w.dinv32.p,
                                                                w.binv2.p, w.part.p, w.cnt.p, w.sc.p, w.vinst.p,
                                                                w.vptr.p, rtol, maxit, drop2);
            else if (bj2)
                k_bupdate32<NR, true, float><<<nvu, NTHREADS, 0, st>>>(w.d32.p, w.r32.p, w.z32.p, w.p32.p, w.q32.p,
                                                                       w.dinv32.p, w.binv2.p, w.part.p, w.cnt.p, w.sc.p,
                                                                       w.vinst.p, w.vptr.p, rtol, maxit, drop2);
            else if (x64)
                k_bupdate32<NR><<<nvu, NTHREADS, 0, st>>>(x, w.r32.p, w.z32.p, w.p32.p, w.q32.p, w.dinv32.p, nullptr,
                                                          w.part.p, w.cnt.p, w.sc.p, w.vinst.p, w.vptr.p, rtol, maxit,
                                                          drop2);
            else
                k_bupdate32<NR, false, float><<<nvu, NTHREADS, 0, st>>>(w.d32.p, w.r32.p, w.z32.p, w.p32.p, w.q32.p,
                                                                        w.dinv32.p, nullptr, w.part.p, w.cnt.p, w.sc.p,
                                                                        w.vinst.p, w.vptr.p, rtol, maxit, drop2);
            k_bpupdate32<NR><<<nvu, NTHREADS, 0, st>>>(w.z32.p, w.p32.p, w.sc.p, w.vinst.p, 0);
            if (!x64 && ++*calls % BBATCH == 0) k_bfold<<<num_sms() * 4, NTHREADS, 0, st>>>(nv, x, w.d32.p);
        };
    } else {
        k_bdiag<ND, double><<<gd, NTHREADS, 0, st>>>(nr, S.diag.p, S.v64.p, w.dinv.p, w.zero.p);
        residual_spmv(w.q.p, 2);
        k_binit<NR><<<nvu, NTHREADS, 0, st>>>(b, w.q.p, w.dinv.p, w.r.p, w.z.p, w.p.p, w.part.p, w.cnt.p, w.sc.p,
                                              w.vinst.p, w.vptr.p, rtol);
        iteration = [&]() {
            k_bspmv<ND, NR, true, double, double, false><<<nsu, NTHREADS, 0, st>>>(
                S.nslices, S.sl_ptr.p, S.sl_width.p, S.col.p, S.v64.p, w.p.p, w.q.p, w.part.p, w.cnt.p, w.sc.p,
                w.sinst.p, w.sptr.p, 1);
            k_bupdate<NR><<<nvu, NTHREADS, 0, st>>>(x, w.r.p, w.z.p, w.p.p, w.q.p, w.dinv.p, w.part.p, w.cnt.p, w.sc.p,
                                                    w.vinst.p, w.vptr.p, rtol, maxit);
            k_bpupdate<NR><<<nvu, NTHREADS, 0, st>>>(w.z.p, w.p.p, w.sc.p, w.vinst.p);
        };
    }
    count_launch(ctx, 3);
    OGB_CUDA(cudaGetLastError());
    ExecGuard graph;
    OGB_CHECK(capture_batch(ctx, iteration, graph.e));
    int zero = 0;
    OGB_CUDA(cudaMemcpyAsync(&zero, w.zero.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    res.resize(npair);
    for (int it = 0;;) {
        OGB_CUDA(cudaMemcpyAsync(res.data(), w.sc.p, npair * sizeof(BatchScal), cudaMemcpyDeviceToHost, st));
        OGB_CUDA(cudaStreamSynchronize(st));
        if (zero) {
            for (auto &s : res) s.done = 3;
            break;
        }
        bool all = true, paused = false;
        for (auto &s : res) {
            all = all && s.done;
            paused = paused || (s.done == 0 && s.pause != 0);
        }
        if (all || it > maxit + 2 * BBATCH) break;
        if (mixed && paused) {
            // FP64 replacement of the pairs that paused during the last batch of
            // iterations (instances without one skip every kernel): residual, r, z,
            // beta, and their p = z + beta p
            residual_spmv(w.q64.p, 3);
            replace(0);
            k_bpupdate32<NR><<<nvu, NTHREADS, 0, st>>>(w.z32.p, w.p32.p, w.sc.p, w.vinst.p, 1);
            count_launch(ctx, 3);
            OGB_CUDA(cudaGetLastError());
            continue;
        }
        if (graph.e) {
            OGB_CUDA(cudaGraphLaunch(graph.e, st));
        } else {
            for (int k = 0; k < BBATCH; ++k) iteration();
        }
        count_launch(ctx, 3 * BBATCH + (mixed && !ctx->batch_x64 ? 1 : 0));
        OGB_CUDA(cudaGetLastError());
        it += BBATCH;
    }
    if (mixed) {
        // a pair whose FP32 iterates diverged restarts its FP64 pass from zero
        k_bzero_diverged<NR><<<nvu, NTHREADS, 0, st>>>(x, w.sc.p, w.vinst.p);
        count_launch(ctx);
        OGB_CUDA(cudaGetLastError());
    }
    return OGB_OK;
}

// Node-space right-hand side of load case c: b[(act*nd + d) * nr + c] = f_ext - f_int at free DOFs.
__global__ void k_brhs(int n, int nd, int nr, int c, const int *__restrict__ eq, const int *__restrict__ act,
                       const double *__restrict__ fext, const double *__restrict__ fint, double *__restrict__ b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || eq[i] <= 0) return;
    const int64_t row = (int64_t)act[i / nd] * nd + i % nd;
    b[row * nr + c] = (fext ? fext[i] : 0.0) - fint[i];
}

// u[i] = x[(act*nd + d) * nr + c] at free DOFs (prescribed values already in u).
__global__ void k_bscatter(int n, int nd, int nr, int c, const int *__restrict__ eq, const int *__restrict__ act,
                           const double *__restrict__ x, double *__restrict__ u)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || eq[i] <= 0) return;
    const int64_t row = (int64_t)act[i / nd] * nd + i % nd;
    u[i] = x[row * nr + c];
}

__global__ void k_bu_from_bc(int n, const int *__restrict__ eq, const double *__restrict__ bcval,
                             double *__restrict__ u)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) u[i] = eq[i] < 0 ? bcval[i] : 0.0;
}

// StructuralEngngModel::computeReaction (structengngmodel.C:183-201)
__global__ void k_breactions(int n, const int *__restrict__ eq, const double *__restrict__ fint,
                             const double *__restrict__ fext, double *__restrict__ reac)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) reac[i] = eq[i] < 0 ? fint[i] - (fext ? fext[i] : 0.0) : 0.0;
}

inline unsigned nblk(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, NTHREADS); }
// Column c of a column-major equation-space block <-> node space with nr interleaved columns.
__global__ void k_eq_to_ns_col(int neq, const int *__restrict__ ns_of_eq, int nr, int c, const double *__restrict__ xe,
                               double *__restrict__ xn)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < neq) xn[(int64_t)ns_of_eq[e] * nr + c] = xe[e];
}

__global__ void k_ns_to_eq_col(int neq, const int *__restrict__ ns_of_eq, int nr, int c, const double *__restrict__ xn,
                               double *__restrict__ xe)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < neq) xe[e] = xn[(int64_t)ns_of_eq[e] * nr + c];
}


}  // namespace

int batch_pcg(ogb_mtrx *m, int nrhs, const double *b, double *x, double rtol, int maxit, int precision, int *iters,
              double *achieved, int *status)
{
    if (m->precond != 1) return fail(OGB_E_ARG, "batched solves use the diagonal preconditioner (lsprecond 1)");
    if (!m->has_sell) return fail(OGB_E_STATE, "batched solves need a matrix built from a model");
    if (nrhs < 1 || nrhs > MAXNR) return fail(OGB_E_ARG, "nrhs must be 1..4");
    if (precision != OGB_PREC_FP64 && precision != OGB_PREC_MIXED) return fail(OGB_E_ARG, "unknown precision");
    const bool mixed = precision == OGB_PREC_MIXED;
    if (mixed && m->sell.v32_version != m->version)
        return fail(OGB_E_STATE, "the FP32 copy of the matrix is not current (assemble through the model)");
    std::vector<BatchScal> res;
    int r = OGB_E_ARG;
    const int nd = m->sell.nd;
#define OGB_BATCH_CASE(ND_, NR_) \
    if (nd == ND_ && nrhs == NR_) r = run_batch<ND_, NR_>(m, b, x, rtol, maxit, mx, out);
    auto run = [&](bool mx, std::vector<BatchScal> &out) {
        OGB_BATCH_CASE(3, 1) OGB_BATCH_CASE(3, 2) OGB_BATCH_CASE(3, 3) OGB_BATCH_CASE(3, 4)
        OGB_BATCH_CASE(2, 1) OGB_BATCH_CASE(2, 2) OGB_BATCH_CASE(2, 3) OGB_BATCH_CASE(2, 4)
    };
#undef OGB_BATCH_CASE
    run(mixed, res);
    if (r != OGB_OK) return r;
    bool stalled = false;
    int used = 0;
    for (const auto &q : res) {
        stalled = stalled || q.done == 5;
        used = q.iters > used ? q.iters : used;
    }
    if (stalled && used < maxit) {
        // pairs the FP32 operator cannot bring to the tolerance continue from their
        // current solution in an FP64 pass; converged pairs stop at its first test
        std::vector<BatchScal> res64;
        run(false, res64);
        if (r != OGB_OK) return r;
        for (size_t k = 0; k < res.size(); ++k)
            if (res[k].done == 5) {
                const int it = res[k].iters;
                res[k] = res64[k];
                res[k].iters += it;
            }
    }
    int worst = OGB_OK;
    for (size_t k = 0; k < res.size(); ++k) {
        const BatchScal &s = res[k];
        double normb = sqrt(s.bnorm2);
        if (normb == 0.0) normb = 1.0;
        const int code = s.done == 1                 ? OGB_OK
                         : s.done == 2 || s.done == 5 ? OGB_E_BREAKDOWN
                         : s.done == 3               ? OGB_E_ZERODIAG
                                                     : OGB_E_NOTCONV;
        if (iters) iters[k] = s.iters;
        if (achieved) achieved[k] = sqrt(s.rnorm2) / normb;
        if (status) status[k] = code;
        if (code != OGB_OK && worst == OGB_OK) worst = code;
    }
    return worst;
}

// SparseLinearSystemNM::solve(A, B, X) (sparselinsystemnm.h:91) on a matrix
// assembled from a model: B and X are device, column-major neq x nrhs, X holds
// the initial guesses and receives the solutions. Columns go through the
// batched solve four at a time; per column, the iteration count and achieved
// residual are the largest over the instances and the status the first failure.
int pcg_solve_multi(ogb_mtrx *m, int nrhs, const double *B, double *X, double rtol, int maxit, int precision,
                    int *iters, double *achieved, int *status)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    if (!(m->has_sell && m->sell.v32_version == m->version))
        return fail(OGB_E_STATE, "node-block copy not current");
    const int neq = m->neq, ninst = m->sell.ninst;
    int worst = OGB_OK;
    for (int c0 = 0; c0 < nrhs; c0 += MAXNR) {
        const int nr = nrhs - c0 < MAXNR ? nrhs - c0 : MAXNR;
        const int64_t nv = m->sell.nns() * nr;
        DBuf<double> b, x;
        OGB_CHECK(b.alloc(nv));
        OGB_CHECK(x.alloc(nv));
        OGB_CUDA(cudaMemsetAsync(b.p, 0, nv * sizeof(double), s));
        OGB_CUDA(cudaMemsetAsync(x.p, 0, nv * sizeof(double), s));
        for (int c = 0; c < nr; ++c) {
            k_eq_to_ns_col<<<nblk(neq), NTHREADS, 0, s>>>(neq, m->sell.ns_of_eq.p, nr, c, B + (size_t)(c0 + c) * neq, b.p);
            k_eq_to_ns_col<<<nblk(neq), NTHREADS, 0, s>>>(neq, m->sell.ns_of_eq.p, nr, c, X + (size_t)(c0 + c) * neq, x.p);
        }
        count_launch(ctx, 2 * nr);
        std::vector<int> it(ninst * nr), st(ninst * nr);
        std::vector<double> ac(ninst * nr);
        int r = batch_pcg(m, nr, b.p, x.p, rtol, maxit, precision, it.data(), ac.data(), st.data());
        if (r != OGB_OK && r != OGB_E_NOTCONV && r != OGB_E_BREAKDOWN && r != OGB_E_ZERODIAG) return r;
        if (r != OGB_OK && worst == OGB_OK) worst = r;
        for (int c = 0; c < nr; ++c) {
            k_ns_to_eq_col<<<nblk(neq), NTHREADS, 0, s>>>(neq, m->sell.ns_of_eq.p, nr, c, x.p, X + (size_t)(c0 + c) * neq);
            int imax = 0, scode = OGB_OK;
            double amax = 0.0;
            for (int i = 0; i < ninst; ++i) {
                const int k = i * nr + c;
                imax = it[k] > imax ? it[k] : imax;
                amax = ac[k] > amax ? ac[k] : amax;
                if (st[k] != OGB_OK && scode == OGB_OK) scode = st[k];
            }
            if (iters) iters[c0 + c] = imax;
            if (achieved) achieved[c0 + c] = amax;
            if (status) status[c0 + c] = scode;
        }
        count_launch(ctx, nr);
        OGB_CUDA(cudaGetLastError());
        OGB_CUDA(cudaStreamSynchronize(s));   // b and x are freed at the end of the chunk
    }
    return worst;
}

// LinearStatic (linearstatic.C:177-253) for every instance and load case of a
// batch at once: one stiffness assembly, nrhs internal-force evaluations of
// the prescribed fields, one batched solve, nrhs scatters (and reactions).
// bcval, load, u_nodes, reacs: device, nrhs consecutive node vectors.
int batch_linear_static(ogb_model *md, ogb_mtrx *m, int nrhs, const double *bcval, const double *load, double rtol,
                        int maxit, int precision, double *u_nodes, double *reacs, int *iters, double *achieved,
                        int *status,
                        int (*assemble)(ogb_model *, ogb_mtrx *), int (*forces)(ogb_model *, const double *, double *))
{
    ogb_ctx *ctx = md->ctx;
    cudaStream_t s = ctx->stream;
    const int nd = md->ndofpn, n = md->nnodes * nd;
    OGB_CHECK(assemble(md, m));
    const int64_t nv = m->sell.nns() * nrhs;
    DBuf<double> b, x;
    OGB_CHECK(b.alloc(nv));
    OGB_CHECK(x.alloc(nv));
    OGB_CHECK(md->v_fnode.alloc(n));
    OGB_CUDA(cudaMemsetAsync(b.p, 0, nv * sizeof(double), s));
    OGB_CUDA(cudaMemsetAsync(x.p, 0, nv * sizeof(double), s));
    for (int c = 0; c < nrhs; ++c) {
        double *u = u_nodes + (size_t)c * n;
        k_bu_from_bc<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, bcval + (size_t)c * n, u);
        count_launch(ctx);
        OGB_CHECK(forces(md, u, md->v_fnode.p));
        k_brhs<<<nblk(n), NTHREADS, 0, s>>>(n, nd, nrhs, c, md->eq.p, md->act.p, load ? load + (size_t)c * n : nullptr,
                                            md->v_fnode.p, b.p);
        count_launch(ctx);
    }
    OGB_CUDA(cudaGetLastError());
    OGB_CHECK(check_device_status(ctx, "assembly"));
    int r = batch_pcg(m, nrhs, b.p, x.p, rtol, maxit, precision, iters, achieved, status);
    if (r != OGB_OK && r != OGB_E_NOTCONV && r != OGB_E_BREAKDOWN && r != OGB_E_ZERODIAG) return r;
    for (int c = 0; c < nrhs; ++c) {
        double *u = u_nodes + (size_t)c * n;
        k_bscatter<<<nblk(n), NTHREADS, 0, s>>>(n, nd, nrhs, c, md->eq.p, md->act.p, x.p, u);
        count_launch(ctx);
        if (reacs) {
            OGB_CHECK(forces(md, u, md->v_fnode.p));
            k_breactions<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, md->v_fnode.p,
                                                      load ? load + (size_t)c * n : nullptr, reacs + (size_t)c * n);
            count_launch(ctx);
        }
    }
    OGB_CUDA(cudaGetLastError());
    OGB_CUDA(cudaStreamSynchronize(s));   // b and x are freed on return
    return r;
}

}  // namespace ogb
