// Newton-Raphson step of NonLinearStatic on the GPU.
//
// Restates NRSolver::solve (src/core/nrsolver.C:204-402) for the setting
// NonLinearStatic uses with `controlmode 1 manrmsteps 1` (full Newton, the
// tangent assembled before the first residual and again in every later
// iteration, no line search, no initial guess) and NRSolver::checkConvergence
// with DOF grouping (nrsolver.C:593-790): per DOF id d,
//   forceErr_d = sqrt( sum_free(d) rhs^2 / (sum_free(d) RT^2 + eNorm_d) ),
// absolute when the denominator is below 1e-6; converged when every group is
// <= rtolf, never at iteration 0 with a non-zero error. eNorm_d is the sum of
// squared element internal-force entries with DOF id d (engngm.C:1398-1401).
// Everything but the handful of group sums stays on the device; the host reads
// 3*ndofpn doubles per iteration to take the convergence decision.
#include <math.h>

#include <vector>

#include "internal.cuh"
#include "reduce.cuh"

namespace ogb {

namespace {

inline unsigned nblk(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, NTHREADS); }
inline int nr_grid() { return num_sms() * 4; }

__global__ void k_nr_assemble_u(int n, const int *__restrict__ eq, const double *__restrict__ X,
                                const double *__restrict__ bcval, double *__restrict__ u)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) u[i] = eq[i] > 0 ? X[eq[i] - 1] : bcval[i];
}

// rhs = RT - F at free DOFs (written to the equation-space vector b), and the
// per-DOF-id sums of rhs^2 and RT^2 over free DOFs.
template <int ND>
__global__ void __launch_bounds__(NTHREADS) k_nr_rhs(int nnodes, const int *__restrict__ eq,
                                                     const double *__restrict__ load, const double *__restrict__ fint,
                                                     double *__restrict__ b, double *part, unsigned int *count,
                                                     double *out)
{
    double v[2 * ND];
#pragma unroll
    for (int k = 0; k < 2 * ND; ++k) v[k] = 0.0;
    for (int A = blockIdx.x * blockDim.x + threadIdx.x; A < nnodes; A += gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const int i = A * ND + d;
            const int q = eq[i];
            if (q > 0) {
                const double rt = load ? load[i] : 0.0;
                const double r = rt - fint[i];
                b[q - 1] = r;
                v[d] += r * r;
                v[ND + d] += rt * rt;
            }
        }
    }
    block_sum<2 * ND>(v);
    if (publish_partials<2 * ND>(v, part, count)) {
        double t[2 * ND];
        final_sums<2 * ND>(part, t);
        if (threadIdx.x != 0) return;
        *count = 0;
#pragma unroll
        for (int k = 0; k < 2 * ND; ++k) out[k] = t[k];
    }
}

// eNorm_d = sum over all element force entries with DOF id d of fe^2.
template <int ND>
__global__ void __launch_bounds__(NTHREADS) k_nr_enorm(int64_t nentries, const double *__restrict__ fe, double *part,
                                                       unsigned int *count, double *out)
{
    double v[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) v[d] = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nentries;
         k += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const double f = fe[k * ND + d];
            v[d] += f * f;
        }
    }
    block_sum<ND>(v);
    if (publish_partials<ND>(v, part, count)) {
        double t[ND];
        final_sums<ND>(part, t);
        if (threadIdx.x != 0) return;
        *count = 0;
#pragma unroll
        for (int d = 0; d < ND; ++d) out[d] = t[d];
    }
}

__global__ void k_nr_add(int n, double *__restrict__ X, const double *__restrict__ dX)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) X[i] += dX[i];
}

__global__ void k_nr_reactions(int n, const int *__restrict__ eq, const double *__restrict__ fint,
                               const double *__restrict__ load, double *__restrict__ reac)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) reac[i] = eq[i] < 0 ? fint[i] - (load ? load[i] : 0.0) : 0.0;
}

// Prescribed increment since the last converged step: du = bcval - bcprev at
// prescribed DOFs, 0 at free ones.
__global__ void k_nr_prescribed_increment(int n, const int *__restrict__ eq, const double *__restrict__ bcval,
                                          const double *__restrict__ bcprev, double *__restrict__ du)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) du[i] = eq[i] < 0 ? bcval[i] - bcprev[i] : 0.0;
}

// fe[e][a] = sum_b K_e[a][b] du[conn[e][b]] from the element matrices of the last
// stiffness evaluation (node-block layout ke[e][a][b][i][j]); one thread per (e, a).
template <int ND>
__global__ void __launch_bounds__(NTHREADS) k_nr_ke_times(int nelem, int nnpe, const double *__restrict__ ke,
                                                          const int *__restrict__ conn, const double *__restrict__ du,
                                                          double *__restrict__ fe)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nelem * nnpe) return;
    const int64_t e = t / nnpe;
    const int a = (int)(t % nnpe);
    double f[ND];
#pragma unroll
    for (int i = 0; i < ND; ++i) f[i] = 0.0;
    const double *kb = ke + (size_t)t * nnpe * ND * ND;
    for (int b = 0; b < nnpe; ++b) {
        const int B = conn[e * nnpe + b];
        double u[ND];
#pragma unroll
        for (int j = 0; j < ND; ++j) u[j] = du[(int64_t)B * ND + j];
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int j = 0; j < ND; ++j) f[i] += kb[(b * ND + i) * ND + j] * u[j];
    }
#pragma unroll
    for (int i = 0; i < ND; ++i) fe[(size_t)t * ND + i] = f[i];
}

// b[eq-1] = -f at free DOFs.
__global__ void k_nr_neg_free(int n, const int *__restrict__ eq, const double *__restrict__ f, double *__restrict__ b)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && eq[i] > 0) b[eq[i] - 1] = -f[i];
}

// ---- batched Newton: independent instances, each with its own convergence test
// u from the node-space solution X (free DOFs) and the prescribed values.
__global__ void k_nrb_assemble_u(int n, int nd, const int *__restrict__ eq, const int *__restrict__ act,
                                 const double *__restrict__ X, const double *__restrict__ bcval, double *__restrict__ u)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) u[i] = eq[i] > 0 ? X[(int64_t)act[i / nd] * nd + i % nd] : bcval[i];
}

// Per instance and DOF id: sum_free rhs^2, sum_free RT^2 (nodes of the instance)
// and eNorm (element force entries of the instance). Grid (GX, ninst); the last
// block of an instance sums its GX partials in order.
template <int ND>
__global__ void __launch_bounds__(NTHREADS) k_nrb_sums(const int *__restrict__ node_start,
                                                       const int *__restrict__ elem_start, int nnpe,
                                                       const int *__restrict__ eq, const double *__restrict__ load,
                                                       const double *__restrict__ fint, const double *__restrict__ fe,
                                                       double *part, unsigned int *cnt, double *out)
{
    const int inst = blockIdx.y;
    double v[3 * ND];
#pragma unroll
    for (int k = 0; k < 3 * ND; ++k) v[k] = 0.0;
    const int stride = gridDim.x * blockDim.x;
    for (int A = node_start[inst] + blockIdx.x * blockDim.x + threadIdx.x; A < node_start[inst + 1]; A += stride) {
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const int i = A * ND + d;
            if (eq[i] > 0) {
                const double rt = load ? load[i] : 0.0;
                const double r = rt - fint[i];
                v[d] += r * r;
                v[ND + d] += rt * rt;
            }
        }
    }
    const int64_t k0 = (int64_t)elem_start[inst] * nnpe, k1 = (int64_t)elem_start[inst + 1] * nnpe;
    for (int64_t k = k0 + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += stride) {
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const double f = fe[k * ND + d];
            v[2 * ND + d] += f * f;
        }
    }
    block_sum<3 * ND>(v);
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 3 * ND; ++k) part[((size_t)inst * gridDim.x + blockIdx.x) * 3 * ND + k] = v[k];
        __threadfence();
        s_last = atomicAdd(cnt + inst, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last || threadIdx.x != 0) return;
    __threadfence();
    double t[3 * ND];
#pragma unroll
    for (int k = 0; k < 3 * ND; ++k) t[k] = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b)
#pragma unroll
        for (int k = 0; k < 3 * ND; ++k) t[k] += __ldcg(part + ((size_t)inst * gridDim.x + b) * 3 * ND + k);
#pragma unroll
    for (int k = 0; k < 3 * ND; ++k) out[(size_t)inst * 3 * ND + k] = t[k];
    cnt[inst] = 0;
}

// Node-space right-hand side: b = RT - F at free DOFs of running instances
// (scale -1 and no load: b = -F, for the initial guess), 0 elsewhere.
__global__ void k_nrb_rhs(int n, int nd, const int *__restrict__ eq, const int *__restrict__ act,
                          const int *__restrict__ node_inst, const int *__restrict__ active,
                          const double *__restrict__ load, const double *__restrict__ f, double *__restrict__ b)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || eq[i] <= 0) return;
    const int A = i / nd;
    b[(int64_t)act[A] * nd + i % nd] = active[node_inst[A]] ? (load ? load[i] : 0.0) - f[i] : 0.0;
}

__global__ void k_nrb_add(int64_t n, double *__restrict__ X, const double *__restrict__ dX)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) X[i] += dX[i];
}

}  // namespace

int nr_ensure(ogb_model *md)
{
    if (!md->nr_X.p) {
        OGB_CHECK(md->nr_X.alloc(md->neq > 0 ? md->neq : 1));
        OGB_CUDA(cudaMemsetAsync(md->nr_X.p, 0, (size_t)(md->neq > 0 ? md->neq : 1) * sizeof(double), md->ctx->stream));
    }
    OGB_CHECK(md->nr_part.alloc((size_t)8 * nr_grid()));
    if (!md->nr_count.p) {
        OGB_CHECK(md->nr_count.alloc(1));
        OGB_CUDA(cudaMemsetAsync(md->nr_count.p, 0, sizeof(unsigned int), md->ctx->stream));
    }
    OGB_CHECK(md->nr_out.alloc(16));
    OGB_CHECK(md->h_nr_out.alloc(16));
    const size_t n = (size_t)md->nnodes * md->ndofpn;
    if (!md->nr_bcprev.p) {
        OGB_CHECK(md->nr_bcprev.alloc(n));
        OGB_CUDA(cudaMemsetAsync(md->nr_bcprev.p, 0, n * sizeof(double), md->ctx->stream));
    }
    OGB_CHECK(md->nr_du.alloc(n));
    return OGB_OK;
}

// NRSolver's re-assembly test before the linear solve of iteration nite
// (nrsolver.C:285-290, mCalcStiffBeforeRes on): never at nite 0 (the tangent of
// the start of the step serves), then every manrmsteps-th iteration; modified
// Newton (manrmsteps 0) keeps the start-of-step tangent.
static bool nr_reassemble(const ogb_model *md, int nite)
{
    return nite > 0 && md->nr_manrm > 0 && nite % md->nr_manrm == 0;
}

// One NonLinearStatic step. bcval/load: this step's total prescribed values and
// nodal loads (device, nnodes*ndofpn). On success the material state is
// committed; u_node and reac (device, optional) receive the converged field.
int nonlinear_step(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf, int maxiter,
                   double lin_rtol, int precision, double *u_node, double *reac, int *iterations,
                   ogb_solve_info *lin_info, int (*assemble)(ogb_model *, ogb_mtrx *),
                   int (*forces)(ogb_model *, const double *, double *),
                   int (*solve)(ogb_mtrx *, double, int, int, ogb_solve_info *))
{
    ogb_ctx *ctx = md->ctx;
    cudaStream_t s = ctx->stream;
    const int nd = md->ndofpn, nn = md->nnodes, n = nn * nd;
    OGB_CHECK(nr_ensure(md));
    OGB_CHECK(md->v_fnode.alloc(n));
    OGB_CHECK(m->w_b.alloc(m->npad));
    OGB_CHECK(m->w_x.alloc(m->npad));
    // DOF groups in use (free DOFs per DOF id)
    std::vector<int> nfree(nd, 0);
    for (int i = 0; i < n; ++i)
        if (md->h_eq[i] > 0) nfree[i % nd]++;
    // tangent at the start of the step (temp state == committed state)
    OGB_CHECK(assemble(md, m));
    ogb_solve_info last{};
    if (md->initial_guess == 1) {
        // IG_Tangent (nlinearstatic.C:532-544): X += K^-1 (-sum_e K_e du_p)
        k_nr_prescribed_increment<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, bcval, md->nr_bcprev.p, md->nr_du.p);
        const int64_t nt = (int64_t)md->nelem * md->nnpe;
        if (nd == 3)
            k_nr_ke_times<3><<<nblk(nt), NTHREADS, 0, s>>>(md->nelem, md->nnpe, md->ke.p, md->conn.p, md->nr_du.p,
                                                           md->fe.p);
        else
            k_nr_ke_times<2><<<nblk(nt), NTHREADS, 0, s>>>(md->nelem, md->nnpe, md->ke.p, md->conn.p, md->nr_du.p,
                                                           md->fe.p);
        count_launch(ctx, 2);
        OGB_CHECK(launch_gather_vector(md, md->v_fnode.p));
        OGB_CUDA(cudaMemsetAsync(m->w_b.p, 0, (size_t)m->npad * sizeof(double), s));
        k_nr_neg_free<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, md->v_fnode.p, m->w_b.p);
        OGB_CUDA(cudaMemsetAsync(m->w_x.p, 0, (size_t)m->npad * sizeof(double), s));
        count_launch(ctx);
        OGB_CUDA(cudaGetLastError());
        int r = solve(m, lin_rtol, 1000000, precision, &last);
        md->lin_solves++;
        md->lin_iters += last.iterations;
        if (r != OGB_OK) {
            if (iterations) *iterations = 0;
            return r;
        }
        k_nr_add<<<nblk(md->neq), NTHREADS, 0, s>>>(md->neq, md->nr_X.p, m->w_x.p);
        count_launch(ctx);
    }
    double *out = md->nr_out.p;
    int nite = 0;
    for (;;) {
        k_nr_assemble_u<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, md->nr_X.p, bcval, u_node);
        count_launch(ctx);
        OGB_CHECK(forces(md, u_node, md->v_fnode.p));   // updates the temp material state
        OGB_CUDA(cudaMemsetAsync(m->w_b.p, 0, (size_t)m->npad * sizeof(double), s));
        if (nd == 3) {
            k_nr_rhs<3><<<nr_grid(), NTHREADS, 0, s>>>(nn, md->eq.p, load, md->v_fnode.p, m->w_b.p, md->nr_part.p,
                                                     md->nr_count.p, out);
            k_nr_enorm<3><<<nr_grid(), NTHREADS, 0, s>>>((int64_t)md->nelem * md->nnpe, md->fe.p, md->nr_part.p,
                                                       md->nr_count.p, out + 6);
        } else {
            k_nr_rhs<2><<<nr_grid(), NTHREADS, 0, s>>>(nn, md->eq.p, load, md->v_fnode.p, m->w_b.p, md->nr_part.p,
                                                     md->nr_count.p, out);
            k_nr_enorm<2><<<nr_grid(), NTHREADS, 0, s>>>((int64_t)md->nelem * md->nnpe, md->fe.p, md->nr_part.p,
                                                       md->nr_count.p, out + 4);
        }
        count_launch(ctx, 2);
        OGB_CUDA(cudaGetLastError());
        OGB_CUDA(cudaMemcpyAsync(md->h_nr_out.p, out, 3 * nd * sizeof(double), cudaMemcpyDeviceToHost, s));
        OGB_CUDA(cudaStreamSynchronize(s));
        OGB_CHECK(check_device_status(ctx, "nonlinear step"));
        const double *h = md->h_nr_out.p;
        bool converged = true;
        for (int d = 0; d < nd; ++d) {
            if (!nfree[d]) continue;
            const double fe2 = h[d], rt2 = h[nd + d], en = h[2 * nd + d];
            const double den = rt2 + en;
            const double err = den >= 1e-6 ? sqrt(fe2 / den) : sqrt(fe2);
            if (!isfinite(err) || err > rtolf * 1e20) {
                if (iterations) *iterations = nite;
                return fail(OGB_E_BREAKDOWN, "NRSolver divergence: residual out of range");
            }
            if (err > rtolf) converged = false;
            if (err > 0.0 && nite == 0) converged = false;
        }
        if (converged) break;
        if (nite >= maxiter) {
            if (iterations) *iterations = nite;
            return fail(OGB_E_NOTCONV, "NRSolver: maximum number of iterations reached without convergence");
        }
        if (nr_reassemble(md, nite)) OGB_CHECK(assemble(md, m));   // tangent from the current temp state
        OGB_CUDA(cudaMemsetAsync(m->w_x.p, 0, (size_t)m->npad * sizeof(double), s));
        int r = solve(m, lin_rtol, 1000000, precision, &last);
        md->lin_solves++;
        md->lin_iters += last.iterations;
        if (r != OGB_OK) {
            if (iterations) *iterations = nite;
            return r;
        }
        k_nr_add<<<nblk(md->neq), NTHREADS, 0, s>>>(md->neq, md->nr_X.p, m->w_x.p);
        count_launch(ctx);
        ++nite;
    }
    OGB_CHECK(ogb_model_commit_state(md));
    OGB_CUDA(cudaMemcpyAsync(md->nr_bcprev.p, bcval, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (reac) {
        k_nr_reactions<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, md->v_fnode.p, load, reac);
        count_launch(ctx);
    }
    OGB_CUDA(cudaGetLastError());
    if (iterations) *iterations = nite;
    if (lin_info) *lin_info = last;
    return OGB_OK;
}

// NonLinearStatic steps of independent instances advanced together (a batch of
// separate runs): one internal-force evaluation, one tangent assembly and one
// batched PCG per Newton iteration for all instances, while every instance
// keeps its own NRSolver convergence test (DOF-grouped, as nonlinear_step) and
// stops iterating -- zero right-hand side, zero increment -- once converged.
// iterations[i]: Newton iterations of instance i. Returns OGB_OK when every
// instance converged; the state is committed only then.
int nonlinear_step_batch(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf,
                         int maxiter, double lin_rtol, int precision, double *u_node, double *reac, int *iterations,
                         int (*assemble)(ogb_model *, ogb_mtrx *), int (*forces)(ogb_model *, const double *, double *))
{
    ogb_ctx *ctx = md->ctx;
    cudaStream_t s = ctx->stream;
    const int nd = md->ndofpn, nn = md->nnodes, n = nn * nd;
    const int ninst = (int)md->inst_start.size() - 1;
    if (!m->has_sell || m->sell.ninst != ninst) return fail(OGB_E_STATE, "matrix not built from this batch");
    if ((int)md->inst_elem_start.size() != ninst + 1)
        return fail(OGB_E_STATE, "batched Newton needs each instance's elements contiguous and in instance order");
    OGB_CHECK(nr_ensure(md));
    OGB_CHECK(md->v_fnode.alloc(n));
    const int64_t nv = m->sell.nns();
    if (md->nrb_X.p && md->nrb_X.n != (size_t)nv)
        return fail(OGB_E_STATE, "restored batched Newton solution does not fit this matrix");
    if (!md->nrb_X.p) {
        OGB_CHECK(md->nrb_X.alloc(nv));
        OGB_CUDA(cudaMemsetAsync(md->nrb_X.p, 0, nv * sizeof(double), s));
    }
    OGB_CHECK(md->nrb_b.alloc(nv));
    OGB_CHECK(md->nrb_x.alloc(nv));
    OGB_CHECK(md->nrb_out.alloc((size_t)ninst * 3 * nd));
    constexpr int GX = 16;
    OGB_CHECK(md->nr_part.alloc((size_t)ninst * GX * 3 * nd));
    if (!md->nrb_cnt.p) {
        OGB_CHECK(md->nrb_cnt.alloc(ninst));
        OGB_CUDA(cudaMemsetAsync(md->nrb_cnt.p, 0, ninst * sizeof(unsigned int), s));
    }
    OGB_CHECK(md->nrb_active.alloc(ninst));
    if (!md->d_node_inst.p) {
        std::vector<int> ni(nn);
        for (int i = 0; i < ninst; ++i)
            for (int A = md->inst_start[i]; A < md->inst_start[i + 1]; ++A) ni[A] = i;
        OGB_CHECK(md->d_node_inst.alloc(nn));
        OGB_CHECK(md->d_inst_start.alloc(ninst + 1));
        OGB_CHECK(md->d_inst_elem_start.alloc(ninst + 1));
        OGB_CUDA(cudaMemcpyAsync(md->d_node_inst.p, ni.data(), nn * sizeof(int), cudaMemcpyHostToDevice, s));
        OGB_CUDA(cudaMemcpyAsync(md->d_inst_start.p, md->inst_start.data(), (ninst + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, s));
        OGB_CUDA(cudaMemcpyAsync(md->d_inst_elem_start.p, md->inst_elem_start.data(), (ninst + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, s));
        OGB_CUDA(cudaStreamSynchronize(s));
    }
    // free DOFs per (instance, DOF id): which groups enter the test
    std::vector<int> nfree((size_t)ninst * nd, 0);
    for (int i = 0; i < ninst; ++i)
        for (int A = md->inst_start[i]; A < md->inst_start[i + 1]; ++A)
            for (int d = 0; d < nd; ++d)
                if (md->h_eq[(size_t)A * nd + d] > 0) nfree[(size_t)i * nd + d]++;
    std::vector<int> active(ninst, 1), nite(ninst, 0);
    std::vector<double> h((size_t)ninst * 3 * nd);
    std::vector<int> pit(ninst), pst(ninst);
    std::vector<double> pac(ninst);
    auto solve_batch = [&]() -> int {
        OGB_CUDA(cudaMemsetAsync(md->nrb_x.p, 0, nv * sizeof(double), s));
        int r = batch_pcg(m, 1, md->nrb_b.p, md->nrb_x.p, lin_rtol, 1000000, precision, pit.data(), pac.data(),
                          pst.data());
        md->lin_solves++;
        for (int i = 0; i < ninst; ++i) md->lin_iters += pit[i];
        if (r != OGB_OK) return r;
        k_nrb_add<<<nblk(nv), NTHREADS, 0, s>>>(nv, md->nrb_X.p, md->nrb_x.p);
        count_launch(ctx);
        return OGB_OK;
    };
    auto upload_active = [&]() -> int {
        OGB_CUDA(cudaMemcpyAsync(md->nrb_active.p, active.data(), ninst * sizeof(int), cudaMemcpyHostToDevice, s));
        return OGB_OK;
    };
    OGB_CHECK(assemble(md, m));   // tangent at the start of the step
    if (md->initial_guess == 1) {
        k_nr_prescribed_increment<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, bcval, md->nr_bcprev.p, md->nr_du.p);
        const int64_t nt = (int64_t)md->nelem * md->nnpe;
        if (nd == 3)
            k_nr_ke_times<3><<<nblk(nt), NTHREADS, 0, s>>>(md->nelem, md->nnpe, md->ke.p, md->conn.p, md->nr_du.p,
                                                           md->fe.p);
        else
            k_nr_ke_times<2><<<nblk(nt), NTHREADS, 0, s>>>(md->nelem, md->nnpe, md->ke.p, md->conn.p, md->nr_du.p,
                                                           md->fe.p);
        count_launch(ctx, 2);
        OGB_CHECK(launch_gather_vector(md, md->v_fnode.p));
        OGB_CHECK(upload_active());
        OGB_CUDA(cudaMemsetAsync(md->nrb_b.p, 0, nv * sizeof(double), s));
        k_nrb_rhs<<<nblk(n), NTHREADS, 0, s>>>(n, nd, md->eq.p, md->act.p, md->d_node_inst.p, md->nrb_active.p,
                                               nullptr, md->v_fnode.p, md->nrb_b.p);
        count_launch(ctx);
        OGB_CHECK(solve_batch());
    }
    int status = OGB_OK;
    for (int it = 0;; ++it) {
        k_nrb_assemble_u<<<nblk(n), NTHREADS, 0, s>>>(n, nd, md->eq.p, md->act.p, md->nrb_X.p, bcval, u_node);
        count_launch(ctx);
        OGB_CHECK(forces(md, u_node, md->v_fnode.p));
        dim3 grid(GX, ninst);
        if (nd == 3)
            k_nrb_sums<3><<<grid, NTHREADS, 0, s>>>(md->d_inst_start.p, md->d_inst_elem_start.p, md->nnpe, md->eq.p,
                                                    load, md->v_fnode.p, md->fe.p, md->nr_part.p, md->nrb_cnt.p,
                                                    md->nrb_out.p);
        else
            k_nrb_sums<2><<<grid, NTHREADS, 0, s>>>(md->d_inst_start.p, md->d_inst_elem_start.p, md->nnpe, md->eq.p,
                                                    load, md->v_fnode.p, md->fe.p, md->nr_part.p, md->nrb_cnt.p,
                                                    md->nrb_out.p);
        count_launch(ctx);
        OGB_CUDA(cudaGetLastError());
        OGB_CUDA(cudaMemcpyAsync(h.data(), md->nrb_out.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        OGB_CUDA(cudaStreamSynchronize(s));
        OGB_CHECK(check_device_status(ctx, "batched nonlinear step"));
        bool any = false;
        for (int i = 0; i < ninst; ++i) {
            if (!active[i]) continue;
            bool conv = true;
            for (int d = 0; d < nd; ++d) {
                if (!nfree[(size_t)i * nd + d]) continue;
                const double *hi = h.data() + (size_t)i * 3 * nd;
                const double den = hi[nd + d] + hi[2 * nd + d];
                const double err = den >= 1e-6 ? sqrt(hi[d] / den) : sqrt(hi[d]);
                if (!isfinite(err) || err > rtolf * 1e20) {
                    for (int k = 0; k < ninst; ++k)
                        if (iterations) iterations[k] = nite[k];
                    return fail(OGB_E_BREAKDOWN, "NRSolver divergence in instance " + std::to_string(i));
                }
                if (err > rtolf || (err > 0.0 && nite[i] == 0)) conv = false;
            }
            if (conv) active[i] = 0;
            else if (nite[i] >= maxiter) status = OGB_E_NOTCONV;
            else any = true;
        }
        if (status != OGB_OK || !any) break;
        if (nr_reassemble(md, it)) OGB_CHECK(assemble(md, m));   // tangent from the current temp state
        OGB_CHECK(upload_active());
        OGB_CUDA(cudaMemsetAsync(md->nrb_b.p, 0, nv * sizeof(double), s));
        k_nrb_rhs<<<nblk(n), NTHREADS, 0, s>>>(n, nd, md->eq.p, md->act.p, md->d_node_inst.p, md->nrb_active.p, load,
                                               md->v_fnode.p, md->nrb_b.p);
        count_launch(ctx);
        OGB_CHECK(solve_batch());
        for (int i = 0; i < ninst; ++i)
            if (active[i]) ++nite[i];
    }
    if (iterations)
        for (int i = 0; i < ninst; ++i) iterations[i] = nite[i];
    if (status != OGB_OK) return fail(status, "NRSolver: maximum number of iterations reached without convergence");
    OGB_CHECK(ogb_model_commit_state(md));
    OGB_CUDA(cudaMemcpyAsync(md->nr_bcprev.p, bcval, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (reac) {
        k_nr_reactions<<<nblk(n), NTHREADS, 0, s>>>(n, md->eq.p, md->v_fnode.p, load, reac);
        count_launch(ctx);
    }
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

}  // namespace ogb
