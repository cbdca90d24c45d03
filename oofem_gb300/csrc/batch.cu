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
#include <math.h>

#include <vector>

#include "internal.cuh"
#include "reduce.cuh"

namespace ogb {

namespace {

struct BatchScal {
    double bnorm2, rho, pq, rnorm2, alpha, beta;
    int done, iters;   // done: 0 running, 1 converged, 2 breakdown, 3 zero pivot, 4 iteration limit
};

constexpr int UNIT = NTHREADS;               // scalar rows per vector block
constexpr int SPMV_SLICES = NTHREADS / 32;   // slices (of 32 node rows) per SpMV block
constexpr int MAXNR = 4;
constexpr int BBATCH = 16;                   // iterations per captured graph

// Block sums of NV values, published for block `unit`; true in every thread of
// the block that completed its instance (count reaches the instance's units).
template <int NV>
__device__ __forceinline__ bool publish_inst(double (&v)[NV], double *part, int64_t unit, unsigned int *cnt,
                                             int64_t inst_units)
{
    block_sum<NV>(v);
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
    for (int64_t u = u0 + threadIdx.x; u < u1; u += NTHREADS)
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] += __ldcg(part + u * NV + k);
    block_sum<NV>(out);
}

// q = K p for all right-hand sides; with DOT, also p.q per pair and alpha.
template <int ND, int NR, bool DOT>
__global__ void __launch_bounds__(NTHREADS) k_bspmv(int nslices, const int64_t *__restrict__ sl_ptr,
                                                    const int *__restrict__ sl_width, const int *__restrict__ col,
                                                    const double *__restrict__ val, const double *__restrict__ x,
                                                    double *__restrict__ y, double *part, unsigned int *cnt,
                                                    BatchScal *sc, const int *__restrict__ unit_inst,
                                                    const int64_t *__restrict__ unit_ptr)
{
    const int s = blockIdx.x * SPMV_SLICES + (threadIdx.x >> 5);
    const int r = threadIdx.x & 31;
    double acc[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) acc[c] = 0.0;
    if (s < nslices) {
        const int64_t base = sl_ptr[s];
        const int w = sl_width[s];
        double yy[ND][NR];
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int c = 0; c < NR; ++c) yy[i][c] = 0.0;
        const double *vp = val + base * (ND * ND) + r;
        const int *cp = col + base + r;
        for (int k = 0; k < w; ++k) {
            const int cc = __ldcs(cp + 32 * k);
            double xb[ND * NR];
            const double *xp = x + (int64_t)cc * (ND * NR);
#pragma unroll
            for (int j = 0; j < ND * NR; ++j) xb[j] = __ldg(xp + j);
            const double *vk = vp + (int64_t)k * (32 * ND * ND);
#pragma unroll
            for (int i = 0; i < ND; ++i)
#pragma unroll
                for (int j = 0; j < ND; ++j) {
                    const double v = __ldcs(vk + 32 * (i * ND + j));
#pragma unroll
                    for (int c = 0; c < NR; ++c) yy[i][c] = fma(v, xb[j * NR + c], yy[i][c]);
                }
        }
        const int64_t a = (int64_t)s * 32 + r;
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int c = 0; c < NR; ++c) {
                y[(a * ND + i) * NR + c] = yy[i][c];
                if (DOT) acc[c] = fma(x[(a * ND + i) * NR + c], yy[i][c], acc[c]);
            }
    }
    if (!DOT) return;
    const int inst = unit_inst[blockIdx.x];
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
    if (!publish_inst<NR>(acc, part, blockIdx.x, cnt + inst, u1 - u0)) return;
    double t[NR];
    inst_sums<NR>(part, u0, u1, t);
    if (threadIdx.x != 0) return;
    cnt[inst] = 0;
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        BatchScal &q = sc[inst * NR + c];
        if (q.done) continue;
        q.pq = t[c];
        if (!(t[c] > 0.0) || !isfinite(t[c])) q.done = 2;
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
    const int64_t row = (int64_t)blockIdx.x * UNIT + threadIdx.x;
    double v[3 * NR];
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
        v[c] = bb * bb;
        v[NR + c] = rr * rr;
        v[2 * NR + c] = rr * zz;
    }
    const int inst = unit_inst[blockIdx.x];
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
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
    const int64_t row = (int64_t)blockIdx.x * UNIT + threadIdx.x;
    const int inst = unit_inst[blockIdx.x];
    const double di = dinv[row];
    double v[2 * NR];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        v[c] = 0.0;
        v[NR + c] = 0.0;
        const int done = sc[inst * NR + c].done;
        const double alpha = sc[inst * NR + c].alpha;
        if (done) continue;   // converged pairs keep their solution
        const int64_t k = row * NR + c;
        x[k] = fma(alpha, p[k], x[k]);
        const double rr = fma(-alpha, q[k], r[k]);
        const double zz = rr * di;
        r[k] = rr;
        z[k] = zz;
        v[c] = rr * rr;
        v[NR + c] = rr * zz;
    }
    const int64_t u0 = unit_ptr[inst], u1 = unit_ptr[inst + 1];
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
    const int64_t row = (int64_t)blockIdx.x * UNIT + threadIdx.x;
    const int inst = unit_inst[blockIdx.x];
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        const int done = sc[inst * NR + c].done;
        const double beta = sc[inst * NR + c].beta;
        if (done) continue;
        const int64_t k = row * NR + c;
        p[k] = fma(beta, p[k], z[k]);
    }
}

// Inverse of the point diagonal of every node row (padding rows hold identity).
template <int ND>
__global__ void k_bdiag(int nrows, const int64_t *__restrict__ diag, const double *__restrict__ val,
                        double *__restrict__ dinv, int *zero_diag)
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
            dinv[(int64_t)a * ND + d] = 0.0;
        } else {
            dinv[(int64_t)a * ND + d] = 1.0 / v;
        }
    }
}

struct BatchWork {
    DBuf<int> vinst, sinst, zero;
    DBuf<int64_t> vptr, sptr;
    DBuf<BatchScal> sc;
    DBuf<double> part, r, z, p, q, dinv;
    DBuf<unsigned int> cnt;
};

template <int ND, int NR>
int run_batch(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, std::vector<BatchScal> &res)
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
        vptr[i] = S.inst_row_base[i] * ND / UNIT;            // 1024 * ND / 256: exact
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
    OGB_CHECK(w.r.alloc(nv));
    OGB_CHECK(w.z.alloc(nv));
    OGB_CHECK(w.p.alloc(nv));
    OGB_CHECK(w.q.alloc(nv));
    OGB_CHECK(w.dinv.alloc(nrows));
    OGB_CHECK(w.cnt.alloc(ninst));
    OGB_CUDA(cudaMemcpyAsync(w.vinst.p, vinst.data(), nvu * sizeof(int), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(w.sinst.p, sinst.data(), nsu * sizeof(int), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(w.vptr.p, vptr.data(), (ninst + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(w.sptr.p, sptr.data(), (ninst + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemsetAsync(w.sc.p, 0, npair * sizeof(BatchScal), st));
    OGB_CUDA(cudaMemsetAsync(w.zero.p, 0, sizeof(int), st));
    OGB_CUDA(cudaMemsetAsync(w.cnt.p, 0, ninst * sizeof(unsigned int), st));
    const int nr = S.nslices * 32;
    k_bdiag<ND><<<(unsigned)ceil_div(nr, NTHREADS), NTHREADS, 0, st>>>(nr, S.diag.p, S.v64.p, w.dinv.p, w.zero.p);
    k_bspmv<ND, NR, false><<<nsu, NTHREADS, 0, st>>>(S.nslices, S.sl_ptr.p, S.sl_width.p, S.col.p, S.v64.p, x, w.q.p,
                                                     nullptr, nullptr, nullptr, nullptr, nullptr);
    k_binit<NR><<<nvu, NTHREADS, 0, st>>>(b, w.q.p, w.dinv.p, w.r.p, w.z.p, w.p.p, w.part.p, w.cnt.p, w.sc.p,
                                          w.vinst.p, w.vptr.p, rtol);
    count_launch(ctx, 3);
    OGB_CUDA(cudaGetLastError());
    auto iteration = [&]() {
        k_bspmv<ND, NR, true><<<nsu, NTHREADS, 0, st>>>(S.nslices, S.sl_ptr.p, S.sl_width.p, S.col.p, S.v64.p, w.p.p,
                                                        w.q.p, w.part.p, w.cnt.p, w.sc.p, w.sinst.p, w.sptr.p);
        k_bupdate<NR><<<nvu, NTHREADS, 0, st>>>(x, w.r.p, w.z.p, w.p.p, w.q.p, w.dinv.p, w.part.p, w.cnt.p, w.sc.p,
                                                w.vinst.p, w.vptr.p, rtol, maxit);
        k_bpupdate<NR><<<nvu, NTHREADS, 0, st>>>(w.z.p, w.p.p, w.sc.p, w.vinst.p);
    };
    // BBATCH iterations per host check, replayed from a captured graph
    cudaGraphExec_t exec = nullptr;
    struct ExecGuard {
        cudaGraphExec_t &e;
        ~ExecGuard()
        {
            if (e) cudaGraphExecDestroy(e);
        }
    } guard{exec};
    if (ctx->use_graphs) {
        cudaGraph_t g = nullptr;
        OGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < BBATCH; ++k) iteration();
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    }
    int zero = 0;
    OGB_CUDA(cudaMemcpyAsync(&zero, w.zero.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    res.resize(npair);
    for (int it = 0;; it += BBATCH) {
        OGB_CUDA(cudaMemcpyAsync(res.data(), w.sc.p, npair * sizeof(BatchScal), cudaMemcpyDeviceToHost, st));
        OGB_CUDA(cudaStreamSynchronize(st));
        if (zero) {
            for (auto &s : res) s.done = 3;
            break;
        }
        bool all = true;
        for (auto &s : res) all = all && s.done;
        if (all || it >= maxit) break;
        if (exec) {
            OGB_CUDA(cudaGraphLaunch(exec, st));
        } else {
            for (int k = 0; k < BBATCH; ++k) iteration();
        }
        count_launch(ctx, 3 * BBATCH);
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

}  // namespace

int batch_pcg_fp64(ogb_mtrx *m, int nrhs, const double *b, double *x, double rtol, int maxit, int *iters,
                   double *achieved, int *status)
{
    if (!m->has_sell) return fail(OGB_E_STATE, "batched solves need a matrix built from a model");
    if (nrhs < 1 || nrhs > MAXNR) return fail(OGB_E_ARG, "nrhs must be 1..4");
    std::vector<BatchScal> res;
    int r = OGB_E_ARG;
    const int nd = m->sell.nd;
#define OGB_BATCH_CASE(ND_, NR_) \
    if (nd == ND_ && nrhs == NR_) r = run_batch<ND_, NR_>(m, b, x, rtol, maxit, res);
    OGB_BATCH_CASE(3, 1) OGB_BATCH_CASE(3, 2) OGB_BATCH_CASE(3, 3) OGB_BATCH_CASE(3, 4)
    OGB_BATCH_CASE(2, 1) OGB_BATCH_CASE(2, 2) OGB_BATCH_CASE(2, 3) OGB_BATCH_CASE(2, 4)
#undef OGB_BATCH_CASE
    if (r != OGB_OK) return r;
    int worst = OGB_OK;
    for (size_t k = 0; k < res.size(); ++k) {
        const BatchScal &s = res[k];
        double normb = sqrt(s.bnorm2);
        if (normb == 0.0) normb = 1.0;
        const int code = s.done == 1   ? OGB_OK
                         : s.done == 2 ? OGB_E_BREAKDOWN
                         : s.done == 3 ? OGB_E_ZERODIAG
                                       : OGB_E_NOTCONV;
        if (iters) iters[k] = s.iters;
        if (achieved) achieved[k] = sqrt(s.rnorm2) / normb;
        if (status) status[k] = code;
        if (code != OGB_OK && worst == OGB_OK) worst = code;
    }
    return worst;
}

// LinearStatic (linearstatic.C:177-253) for every instance and load case of a
// batch at once: one stiffness assembly, nrhs internal-force evaluations of
// the prescribed fields, one batched solve, nrhs scatters (and reactions).
// bcval, load, u_nodes, reacs: device, nrhs consecutive node vectors.
int batch_linear_static(ogb_model *md, ogb_mtrx *m, int nrhs, const double *bcval, const double *load, double rtol,
                        int maxit, double *u_nodes, double *reacs, int *iters, double *achieved, int *status,
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
    int r = batch_pcg_fp64(m, nrhs, b.p, x.p, rtol, maxit, iters, achieved, status);
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
