// C ABI of liboofem_gb300 (declared in include/oofem_gb300.h): handle
// management, host<->device staging, and the LinearStatic driver sequence.
#include <math.h>
#include <string.h>

#include <atomic>

#include <algorithm>
#include <string>
#include <vector>

#include "internal.cuh"

namespace ogb {

static thread_local std::string g_last_error;
}  // namespace ogb
extern "C" void ogb_ctx_free_impl(ogb_ctx *ctx);
namespace ogb {
static void ctx_free(ogb_ctx *ctx) { ogb_ctx_free_impl(ctx); }

void ctx_release(ogb_ctx *ctx)
{
    if (--ctx->refs == 0 && ctx->closing) ctx_free(ctx);
}

void set_error(const std::string &msg) { g_last_error = msg; }

int num_sms()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    const int slot = dev >= 0 && dev < 64 ? dev : 0;
    int n = cache[slot].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    cache[slot].store(n, std::memory_order_relaxed);
    return n;
}

int fail(int code, const std::string &msg)
{
    set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return OGB_E_CUDA;
}

int check_device_status(ogb_ctx *ctx, const char *where)
{
    OGB_CUDA(cudaMemcpyAsync(ctx->h_status.p, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(ctx->stream));
    int s = *ctx->h_status.p;
    if (s == DS_OK) return OGB_OK;
    OGB_CUDA(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->stream));
    std::string w(where);
    switch (s) {
    case DS_LIMIT: return fail(OGB_E_LIMIT, w + ": a per-node/per-row capacity was exceeded");
    case DS_PATTERN: return fail(OGB_E_PATTERN, w + ": location outside the sparsity pattern");
    case DS_NEGVOL: return fail(OGB_E_MESH, w + ": negative volume (tetrahedron with detJ <= 0)");
    case DS_TIMEOUT: return fail(OGB_E_CUDA, w + ": a bulk copy into shared memory did not complete in time");
    }
    return fail(OGB_E_STATE, w + ": device error");
}

static cudaEvent_t take_event(ogb_ctx *ctx)
{
    if (ctx->ev_pool.empty()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        return e;
    }
    cudaEvent_t e = ctx->ev_pool.back();
    ctx->ev_pool.pop_back();
    return e;
}

void prof_begin(ogb_ctx *ctx)
{
    if (!ctx->prof || !ctx->prof_sample) return;
    if (ctx->capture_events) {   // inside a graph capture: the graph owns its events
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        // inside a capture only an external record becomes a timestamp node
        cudaEventRecordWithFlags(e, ctx->stream, cudaEventRecordExternal);
        ctx->capture_events->push_back(e);
        return;
    }
    cudaEvent_t e = take_event(ctx);
    if (!e) return;
    cudaEventRecord(e, ctx->stream);
    ctx->ev_pending.push_back(e);
}

void prof_end(ogb_ctx *ctx, double bytes)
{
    if (!ctx->prof || !ctx->prof_sample) return;
    if (ctx->capture_events) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        cudaEventRecordWithFlags(e, ctx->stream, cudaEventRecordExternal);
        ctx->capture_events->push_back(e);
        ctx->capture_bytes += bytes;
        return;
    }
    if (ctx->ev_pending.size() % 2 == 0) return;
    cudaEvent_t e = take_event(ctx);
    if (!e) {
        ctx->ev_pool.push_back(ctx->ev_pending.back());
        ctx->ev_pending.pop_back();
        return;
    }
    cudaEventRecord(e, ctx->stream);
    ctx->ev_pending.push_back(e);
    ctx->pending_bytes += bytes;
    ctx->prof_count++;
}

// Sum the elapsed time of completed start/stop pairs (call after a stream sync).
void prof_harvest(ogb_ctx *ctx)
{
    size_t n = ctx->ev_pending.size() & ~(size_t)1;
    for (size_t k = 0; k < n; k += 2) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ctx->ev_pending[k], ctx->ev_pending[k + 1]) == cudaSuccess) ctx->prof_ms += ms;
        else cudaGetLastError();   // a failed query must not leak into the next error check
        ctx->ev_pool.push_back(ctx->ev_pending[k]);
        ctx->ev_pool.push_back(ctx->ev_pending[k + 1]);
    }
    ctx->ev_pending.erase(ctx->ev_pending.begin(), ctx->ev_pending.begin() + n);
    ctx->prof_bytes += ctx->pending_bytes;
    ctx->pending_bytes = 0.0;
}

namespace {

__global__ void k_u_from_bc(int n, const int *eq, const double *bcval, double *u)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) u[i] = eq[i] < 0 ? bcval[i] : 0.0;
}

// b[eq-1] = f_ext - f_int at free DOFs; padding untouched (zero).
__global__ void k_build_rhs(int n, const int *eq, const double *fext, const double *fint, double *b)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && eq[i] > 0) b[eq[i] - 1] = (fext ? fext[i] : 0.0) - fint[i];
}

__global__ void k_scatter_solution(int n, const int *eq, const double *x, double *u)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && eq[i] > 0) u[i] = x[eq[i] - 1];
}

// StructuralEngngModel::computeReaction (structengngmodel.C:183-201): internal
// minus external forces at prescribed DOFs.
__global__ void k_reactions(int n, const int *eq, const double *fint, const double *fext, double *reac)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) reac[i] = eq[i] < 0 ? fint[i] - (fext ? fext[i] : 0.0) : 0.0;
}

__global__ void k_commit_state(int64_t ngp_total, const int *emat, const double *mats, int ngp, double *state)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ngp_total) return;
    int e = (int)(t / ngp);
    int kind = (int)mats[8 * emat[e]];
    double *st = state + t * NSTATE;
    if (kind == OGB_MAT_MISES) {
        for (int i = 0; i < 7; ++i) st[i] = st[8 + i];
    } else if (kind == OGB_MAT_IDM1) {
        st[0] = st[8];
        st[1] = st[9];
    }
}

__global__ void k_gp_state(int64_t ngp_total, const int *emat, const double *mats, int ngp, const double *state,
                           double *out4)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ngp_total) return;
    int e = (int)(t / ngp);
    int kind = (int)mats[8 * emat[e]];
    const double *st = state + t * NSTATE;
    double k = 0, w = 0, le = 0;
    if (kind == OGB_MAT_MISES) {
        k = st[6];
    } else if (kind == OGB_MAT_IDM1) {
        k = st[0];
        w = st[1];
        le = st[2];
    }
    out4[t * 4 + 0] = k;
    out4[t * 4 + 1] = w;
    out4[t * 4 + 2] = le;
    out4[t * 4 + 3] = 0.0;
}

inline unsigned nb(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, NTHREADS); }

// General inverse (Gauss-Jordan, partial pivoting), n <= 6.
void inv_n(int n, const double *A, double *Ai)
{
    double M[6][12];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 2 * n; ++j) M[i][j] = j < n ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
        if (p != c)
            for (int j = 0; j < 2 * n; ++j) std::swap(M[c][j], M[p][j]);
        double piv = M[c][c];
        for (int j = 0; j < 2 * n; ++j) M[c][j] /= piv;
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = M[r][c];
            if (f != 0.0)
                for (int j = 0; j < 2 * n; ++j) M[r][j] -= f * M[c][j];
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Ai[i * n + j] = M[i][j + n];
}

// IsotropicLinearElasticMaterial::initTangents (isolinearelasticmaterial.C:80-88):
// D = 2G I_dev6 + K I6(x)I6; plane stress = inverse of the (xx,yy,xy) block of
// the 3-D compliance (linearelasticmaterial.C:62-79).
void isotropic_D(int etype, double E, double nu, double *D)
{
    double G = E / (2.0 * (1. + nu));
    double K = E / (3.0 * (1. - 2. * nu));
    double D6[36];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double idev = (i < 3 && j < 3) ? (i == j ? 2. / 3. : -1. / 3.) : (i == j ? 0.5 : 0.0);
            double ii = (i < 3 && j < 3) ? 1.0 : 0.0;
            D6[i * 6 + j] = 2 * G * idev + K * ii;
        }
    if (etype != OGB_PLANESTRESS2D) {
        memcpy(D, D6, sizeof(D6));
        return;
    }
    double C[36], R[9];
    inv_n(6, D6, C);
    const int idx[3] = {0, 1, 5};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i * 3 + j] = C[idx[i] * 6 + idx[j]];
    memset(D, 0, 36 * sizeof(double));
    inv_n(3, R, D);
}

int upload_padded(ogb_mtrx *m, const double *src, double *dst, bool from_host)
{
    cudaStream_t s = m->ctx->stream;
    OGB_CUDA(cudaMemcpyAsync(dst, src, (size_t)m->neq * sizeof(double),
                             from_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    if (m->npad > m->neq)
        OGB_CUDA(cudaMemsetAsync(dst + m->neq, 0, (size_t)(m->npad - m->neq) * sizeof(double), s));
    return OGB_OK;
}

int solve_padded(ogb_mtrx *m, double rtol, int maxit, int precision, ogb_solve_info *info)
{
    ogb_solve_info tmp{};
    ogb_solve_info *inf = info ? info : &tmp;
    int r = m->lstype == OGB_LS_DIRECT          ? ldl_solve(m, m->w_b.p, m->w_x.p, inf)
            : precision == OGB_PREC_MIXED ? pcg_mixed(m, m->w_b.p, m->w_x.p, rtol, maxit, inf)
                                          : pcg_fp64(m, m->w_b.p, m->w_x.p, rtol, maxit, inf);
    if (r != OGB_OK) return r;
    if (inf->status != OGB_OK) {
        const char *why = m->lstype == OGB_LS_DIRECT    ? "direct solver: zero or non-finite pivot"
                          : inf->status == OGB_E_ZERODIAG ? "zero diagonal detected"
                          : inf->status == OGB_E_BREAKDOWN ? "PCG breakdown (rho or p'q not positive/finite)"
                                                          : "PCG did not converge within maxit";
        set_error(why);
    }
    return inf->status;
}

int ensure_solver_vectors(ogb_mtrx *m)
{
    OGB_CHECK(m->w_x.alloc(m->npad));
    OGB_CHECK(m->w_b.alloc(m->npad));
    return OGB_OK;
}

}  // namespace
}  // namespace ogb

using namespace ogb;

extern "C" {

const char *ogb_last_error(void) { return g_last_error.c_str(); }

int ogb_version(void) { return 1; }

int ogb_ctx_create(int device, ogb_ctx **out)
{
    if (!out) return fail(OGB_E_ARG, "null output");
    OGB_CUDA(cudaSetDevice(device));
    ogb_ctx *c = new ogb_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    int r = c->status.alloc(1);
    if (r == OGB_OK) r = c->h_status.alloc(1);
    if (r != OGB_OK) {
        delete c;
        return r;
    }
    OGB_CUDA(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
    *out = c;
    return OGB_OK;
}

void ogb_ctx_free_impl(ogb_ctx *ctx)
{
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    prof_harvest(ctx);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->ev_pending) cudaEventDestroy(e);
    ctx->status.release();
    ctx->h_status.release();
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// A context outlives its matrices and models: destroying it while some are
// alive only marks it; the last child to go frees it.
int ogb_ctx_destroy(ogb_ctx *ctx)
{
    if (!ctx) return OGB_OK;
    if (ctx->refs > 0) {
        ctx->closing = true;
        return OGB_OK;
    }
    ogb_ctx_free_impl(ctx);
    return OGB_OK;
}

void *ogb_ctx_stream(ogb_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int ogb_ctx_synchronize(ogb_ctx *ctx)
{
    if (!ctx) return fail(OGB_E_ARG, "null context");
    OGB_CUDA(cudaStreamSynchronize(ctx->stream));
    return OGB_OK;
}

int64_t ogb_ctx_kernel_launches(ogb_ctx *ctx) { return ctx ? ctx->launches : 0; }

int ogb_ctx_set_option(ogb_ctx *ctx, int option, int64_t value)
{
    if (!ctx) return fail(OGB_E_ARG, "null context");
    switch (option) {
    case OGB_OPT_MIXED_VEC32: ctx->mixed_vec32 = value != 0; return OGB_OK;
    case OGB_OPT_MIXED_DIFF: ctx->mixed_diff = value != 0; return OGB_OK;
    case OGB_OPT_MIXED_ORTH: ctx->mixed_orth = value != 0; return OGB_OK;
    case OGB_OPT_MIXED_P32: ctx->mixed_p32 = value != 0; return OGB_OK;
    case OGB_OPT_MIXED_X64:
        if (value < 0 || value > 3) return fail(OGB_E_ARG, "OGB_OPT_MIXED_X64 must be 0, 1, 2 or 3");
        ctx->mixed_x64 = value == 1 || value == 2;
        ctx->mixed_sum32 = value == 0 || value == 2;
        return OGB_OK;
    case OGB_OPT_SPMV_VARIANT:
        if (value < 0 || value > 6) return fail(OGB_E_ARG, "SpMV variant must be 0 (tuned) or 1..6");
        ctx->spmv_group = value >= 5 ? 1 : (int)value;
        ctx->spmv_split = value == 0 ? 0 : value == 5 ? 2 : value == 6 ? 4 : 1;
        return OGB_OK;
    case OGB_OPT_SPMV_HALF:
        if (value < 0 || value > 2) return fail(OGB_E_ARG, "half-stored SpMV option must be 0, 1 or 2");
        ctx->spmv_half = (int)value;
        return OGB_OK;
    case OGB_OPT_MIXED_BLOCK_JACOBI: ctx->mixed_bj = value != 0; return OGB_OK;
    case OGB_OPT_UPDATE_BLOCKS:
        if (value < 0 || value > 8) return fail(OGB_E_ARG, "update blocks per SM must be 0 (default) or 1..8");
        ctx->upd_bps = (int)value;
        return OGB_OK;
    case OGB_OPT_HALF_FORM:
        if (value < 0 || value > 6) return fail(OGB_E_ARG, "half-stored SpMV form must be 0 (timed) or 1..6");
        ctx->half_form = (int)value;
        return OGB_OK;
    case OGB_OPT_FUSED_UPDATE: ctx->fused_update = value != 0; return OGB_OK;
    case OGB_OPT_BATCH_X64: ctx->batch_x64 = value != 0; return OGB_OK;
    case OGB_OPT_BATCH_FORM:
        if (value < 0 || value > 2) return fail(OGB_E_ARG, "batched SpMV form must be 0 (timed), 1 or 2");
        ctx->batch_form = (int)value;
        return OGB_OK;
    case OGB_OPT_TANGENT_TC:
        if (value < 0 || value > 2) return fail(OGB_E_ARG, "tensor-core tangent option must be 0, 1 or 2");
        ctx->tangent_tc = (int)value;
        return OGB_OK;
    case OGB_OPT_MIXED_DROP_PPM:
        if (value <= 0 || value >= 1000000) return fail(OGB_E_ARG, "drop factor must be in (0,1)");
        ctx->mixed_drop = value * 1e-6;
        return OGB_OK;
    }
    return fail(OGB_E_ARG, "unknown option");
}

int ogb_ctx_profile_enable(ogb_ctx *ctx, int enable)
{
    if (!ctx) return fail(OGB_E_ARG, "null context");
    OGB_CUDA(cudaStreamSynchronize(ctx->stream));
    prof_harvest(ctx);
    ctx->prof = enable != 0;
    return OGB_OK;
}

int ogb_ctx_profile_read(ogb_ctx *ctx, double *total_ms, int64_t *launches, double *bytes)
{
    if (!ctx) return fail(OGB_E_ARG, "null context");
    OGB_CUDA(cudaStreamSynchronize(ctx->stream));
    prof_harvest(ctx);
    if (total_ms) *total_ms = ctx->prof_ms;
    if (launches) *launches = ctx->prof_count;
    if (bytes) *bytes = ctx->prof_bytes;
    ctx->prof_ms = 0.0;
    ctx->prof_bytes = 0.0;
    ctx->prof_count = 0;
    return OGB_OK;
}

// ------------------------------------------------------------------ matrix
int ogb_mtrx_create(ogb_ctx *ctx, ogb_mtrx **out)
{
    if (!ctx || !out) return fail(OGB_E_ARG, "null argument");
    ogb_mtrx *m = new ogb_mtrx();
    m->ctx = ctx;
    m->st_ptr.assign(1, 0);
    ctx->refs++;
    *out = m;
    return OGB_OK;
}

int ogb_mtrx_destroy(ogb_mtrx *m)
{
    if (!m) return OGB_OK;
    ogb_ctx *ctx = m->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete m;
    ctx_release(ctx);
    return OGB_OK;
}

int ogb_mtrx_build_structure(ogb_mtrx *m, int neq, int nelem, const int64_t *loc_ptr, const int *loc)
{
    if (!m || neq < 0 || nelem < 0 || (nelem > 0 && (!loc_ptr || !loc))) return fail(OGB_E_ARG, "bad argument");
    for (int e = 0; e < nelem; ++e) {
        if (loc_ptr[e + 1] < loc_ptr[e]) return fail(OGB_E_ARG, "loc_ptr not monotone");
    }
    for (int64_t k = 0; k < (nelem > 0 ? loc_ptr[nelem] : 0); ++k)
        if (loc[k] < 0 || loc[k] > neq) return fail(OGB_E_ARG, "location outside 0..neq");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    int64_t zero_ptr = 0;
    OGB_CHECK(build_loc_pattern(m, neq, nelem, nelem > 0 ? loc_ptr : &zero_ptr, loc));
    m->spmv_tpr = pick_tpr(m);
    m->st_ptr.assign(1, 0);
    return OGB_OK;
}

int ogb_mtrx_neq(ogb_mtrx *m, int *neq)
{
    if (!m || !neq) return fail(OGB_E_ARG, "null argument");
    *neq = m->neq;
    return OGB_OK;
}

int ogb_mtrx_nnz(ogb_mtrx *m, int64_t *nnz)
{
    if (!m || !nnz) return fail(OGB_E_ARG, "null argument");
    *nnz = m->nnz;
    return OGB_OK;
}

int ogb_mtrx_pattern(ogb_mtrx *m, int64_t *rowptr, int *colind)
{
    if (!m || !rowptr || !colind) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    cudaStream_t s = m->ctx->stream;
    OGB_CUDA(cudaMemcpyAsync(rowptr, m->rowptr.p, (m->neq + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaMemcpyAsync(colind, m->colind.p, m->nnz * sizeof(int), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

int ogb_mtrx_values(ogb_mtrx *m, double *val)
{
    if (!m || !val) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaMemcpyAsync(val, m->val.p, m->nnz * sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(m->ctx->stream));
    return OGB_OK;
}

int ogb_mtrx_zero(ogb_mtrx *m)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaMemsetAsync(m->val.p, 0, m->nnz * sizeof(double), m->ctx->stream));
    m->version++;
    return OGB_OK;
}

int ogb_mtrx_assemble_begin(ogb_mtrx *m)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    m->st_ptr.assign(1, 0);
    m->st_loc.clear();
    m->st_keoff.clear();
    m->st_ke.clear();
    return OGB_OK;
}

int ogb_mtrx_assemble(ogb_mtrx *m, int n, const int *loc, const double *ke)
{
    if (!m || n < 0 || (n > 0 && (!loc || !ke))) return fail(OGB_E_ARG, "bad argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    for (int i = 0; i < n; ++i)
        if (loc[i] < 0 || loc[i] > m->neq) return fail(OGB_E_ARG, "location outside 0..neq");
    m->st_keoff.push_back((int64_t)m->st_ke.size());
    m->st_loc.insert(m->st_loc.end(), loc, loc + n);
    m->st_ptr.push_back((int64_t)m->st_loc.size());
    m->st_ke.insert(m->st_ke.end(), ke, ke + (size_t)n * n);
    return OGB_OK;
}

int ogb_mtrx_assemble_end(ogb_mtrx *m)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    return staged_assemble(m);
}

int ogb_mtrx_times(ogb_mtrx *m, const double *x, double *y)
{
    if (!m || !x || !y) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    OGB_CHECK(ensure_solver_vectors(m));
    OGB_CHECK(upload_padded(m, x, m->w_x.p, true));
    OGB_CHECK(spmv64(m, m->w_x.p, m->w_b.p));
    OGB_CUDA(cudaMemcpyAsync(y, m->w_b.p, m->neq * sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(m->ctx->stream));
    return OGB_OK;
}

int ogb_mtrx_times_dev(ogb_mtrx *m, const double *x, double *y)
{
    if (!m || !x || !y) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CHECK(ensure_solver_vectors(m));
    OGB_CHECK(upload_padded(m, x, m->w_x.p, false));
    OGB_CHECK(spmv64(m, m->w_x.p, m->w_b.p));
    OGB_CUDA(cudaMemcpyAsync(y, m->w_b.p, m->neq * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream));
    return OGB_OK;
}

static int locate(ogb_mtrx *m, int i, int j, int64_t *pos)
{
    if (i < 1 || j < 1 || i > m->neq || j > m->neq) return fail(OGB_E_ARG, "index out of range");
    int64_t rp[2];
    cudaStream_t s = m->ctx->stream;
    OGB_CUDA(cudaMemcpyAsync(rp, m->rowptr.p + (i - 1), 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    std::vector<int> cols(rp[1] - rp[0]);
    OGB_CUDA(cudaMemcpyAsync(cols.data(), m->colind.p + rp[0], cols.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    auto it = std::lower_bound(cols.begin(), cols.end(), j - 1);
    if (it == cols.end() || *it != j - 1) return fail(OGB_E_PATTERN, "entry not in the sparsity pattern");
    *pos = rp[0] + (it - cols.begin());
    return OGB_OK;
}

int ogb_mtrx_at(ogb_mtrx *m, int i, int j, double *value)
{
    if (!m || !value) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    int64_t p;
    int r = locate(m, i, j, &p);
    if (r == OGB_E_PATTERN) {   // SparseMtrx::at of a structural zero reads 0
        *value = 0.0;
        return OGB_OK;
    }
    OGB_CHECK(r);
    OGB_CUDA(cudaMemcpyAsync(value, m->val.p + p, sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(m->ctx->stream));
    return OGB_OK;
}

int ogb_mtrx_set_at(ogb_mtrx *m, int i, int j, double value)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    int64_t p;
    OGB_CHECK(locate(m, i, j, &p));
    OGB_CUDA(cudaMemcpyAsync(m->val.p + p, &value, sizeof(double), cudaMemcpyHostToDevice, m->ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(m->ctx->stream));
    m->version++;
    return OGB_OK;
}

int ogb_mtrx_spmv_forms(ogb_mtrx *m, int *fp64_form, int *fp32_form, int *warps_per_slice)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    const bool sell = m->has_sell;
    if (fp64_form) *fp64_form = sell ? m->sell.group[0] : 0;
    if (fp32_form)
        *fp32_form = sell ? (m->last_half ? 8 + 10 * (m->ctx->half_form ? m->ctx->half_form : m->sell.half.form)
                                          : m->sell.group[1])
                          : 0;
    if (warps_per_slice) *warps_per_slice = sell ? (m->sell.force_split ? m->sell.force_split
                                                    : (m->sell.nslices < num_sms() * 16 ? 4 : 1)) : 0;
    return OGB_OK;
}

int ogb_mtrx_mixed_block_jacobi(ogb_mtrx *m, int *used)
{
    if (!m || !used) return fail(OGB_E_ARG, "null argument");
    *used = m->last_bj ? 1 : 0;
    return OGB_OK;
}

int ogb_mtrx_set_preconditioner(ogb_mtrx *m, int type)
{
    if (!m) return fail(OGB_E_ARG, "null argument");
    if (type == 3) return fail(OGB_E_ARG, "the threshold ILU of compressed rows (lsprecond 3) is not built");
    if (type != 0 && type != 1 && type != 2 && type != 4) return fail(OGB_E_ARG, "unknown preconditioner type");
    m->precond = type;
    return OGB_OK;
}

int ogb_mtrx_version(ogb_mtrx *m, int64_t *version)
{
    if (!m || !version) return fail(OGB_E_ARG, "null argument");
    *version = m->version;
    return OGB_OK;
}

// ------------------------------------------------------------------ solver
int ogb_pcg_solve(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, int precision,
                  ogb_solve_info *info)
{
    if (!m || !b || !x) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    OGB_CHECK(ensure_solver_vectors(m));
    OGB_CHECK(upload_padded(m, b, m->w_b.p, true));
    OGB_CHECK(upload_padded(m, x, m->w_x.p, true));
    int r = solve_padded(m, rtol, maxit, precision, info);
    OGB_CUDA(cudaMemcpyAsync(x, m->w_x.p, m->neq * sizeof(double), cudaMemcpyDeviceToHost, m->ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(m->ctx->stream));
    return r;
}

int ogb_pcg_solve_dev(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, int precision,
                      ogb_solve_info *info)
{
    if (!m || !b || !x) return fail(OGB_E_ARG, "null argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CHECK(ensure_solver_vectors(m));
    OGB_CHECK(upload_padded(m, b, m->w_b.p, false));
    OGB_CHECK(upload_padded(m, x, m->w_x.p, false));
    int r = solve_padded(m, rtol, maxit, precision, info);
    OGB_CUDA(cudaMemcpyAsync(x, m->w_x.p, m->neq * sizeof(double), cudaMemcpyDeviceToDevice, m->ctx->stream));
    return r;
}

int ogb_pcg_solve_multi_dev(ogb_mtrx *m, int nrhs, const double *B, double *X, double rtol, int maxit,
                            int precision, int *iterations, double *achieved, int *status)
{
    if (!m || !B || !X || nrhs < 0) return fail(OGB_E_ARG, "bad argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    if (nrhs == 0) return OGB_OK;
    if (m->has_sell && m->sell.v32_version == m->version && m->precond == 1 && m->lstype != OGB_LS_DIRECT)
        return pcg_solve_multi(m, nrhs, B, X, rtol, maxit, precision, iterations, achieved, status);
    // no current node-block copy (location-array matrix, or values changed
    // through set_at): the reference's column loop (sparselinsystemnm.C:47-69)
    int worst = OGB_OK;
    for (int c = 0; c < nrhs; ++c) {
        ogb_solve_info info{};
        int r = ogb_pcg_solve_dev(m, B + (size_t)c * m->neq, X + (size_t)c * m->neq, rtol, maxit, precision, &info);
        if (r != OGB_OK && r != OGB_E_NOTCONV && r != OGB_E_BREAKDOWN && r != OGB_E_ZERODIAG) return r;
        if (iterations) iterations[c] = info.iterations;
        if (achieved) achieved[c] = info.achieved;
        if (status) status[c] = r;
        if (r != OGB_OK && worst == OGB_OK) worst = r;
    }
    return worst;
}

int ogb_pcg_solve_multi(ogb_mtrx *m, int nrhs, const double *B, double *X, double rtol, int maxit, int precision,
                        int *iterations, double *achieved, int *status)
{
    if (!m || !B || !X || nrhs < 0) return fail(OGB_E_ARG, "bad argument");
    if (!m->has_structure) return fail(OGB_E_STATE, "no structure");
    OGB_CUDA(cudaSetDevice(m->ctx->device));
    const size_t n = (size_t)m->neq * nrhs;
    if (n == 0) return OGB_OK;
    cudaStream_t s = m->ctx->stream;
    DBuf<double> dB, dX;
    OGB_CHECK(dB.alloc(n));
    OGB_CHECK(dX.alloc(n));
    OGB_CUDA(cudaMemcpyAsync(dB.p, B, n * sizeof(double), cudaMemcpyHostToDevice, s));
    OGB_CUDA(cudaMemcpyAsync(dX.p, X, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int r = ogb_pcg_solve_multi_dev(m, nrhs, dB.p, dX.p, rtol, maxit, precision, iterations, achieved, status);
    if (r != OGB_OK && r != OGB_E_NOTCONV && r != OGB_E_BREAKDOWN && r != OGB_E_ZERODIAG) return r;
    OGB_CUDA(cudaMemcpyAsync(X, dX.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return r;
}

// ------------------------------------------------------------------ element backend
int ogb_model_create(ogb_ctx *ctx, int etype, int nnodes, const double *coords, int nelem, const int *conn,
                     const int *elem_mat, int nmat, const double *mats, double thickness, const uint8_t *bc_mask,
                     ogb_model **out)
{
    if (!ctx || !out || !coords || !conn || !elem_mat || !mats || !bc_mask || nnodes <= 0 || nelem <= 0 || nmat <= 0)
        return fail(OGB_E_ARG, "bad argument");
    if (etype != OGB_LSPACE && etype != OGB_PLANESTRESS2D && etype != OGB_LTRSPACE)
        return fail(OGB_E_ARG, "unknown element type");
    const int nnpe = etype == OGB_LSPACE ? 8 : 4;
    const int ndofpn = etype == OGB_PLANESTRESS2D ? 2 : 3;
    if ((int64_t)nelem >= (1LL << 26)) return fail(OGB_E_LIMIT, "more than 2^26 elements");
    for (int64_t k = 0; k < (int64_t)nelem * nnpe; ++k)
        if (conn[k] < 0 || conn[k] >= nnodes) return fail(OGB_E_ARG, "connectivity outside 0..nnodes-1");
    bool nonlinear = false;
    for (int i = 0; i < nmat; ++i) {
        int kind = (int)mats[8 * i];
        if (kind != OGB_MAT_ISOLE && kind != OGB_MAT_MISES && kind != OGB_MAT_IDM1)
            return fail(OGB_E_ARG, "unknown material kind");
        if (kind != OGB_MAT_ISOLE) {
            if (etype == OGB_PLANESTRESS2D)
                return fail(OGB_E_ARG, "misesmat/idm1 are supported for 3-D elements only");
            nonlinear = true;
        }
    }
    for (int e = 0; e < nelem; ++e)
        if (elem_mat[e] < 0 || elem_mat[e] >= nmat) return fail(OGB_E_ARG, "element material out of range");
    OGB_CUDA(cudaSetDevice(ctx->device));
    ogb_model *md = new ogb_model();
    md->ctx = ctx;
    md->etype = etype;
    md->nnodes = nnodes;
    md->nelem = nelem;
    md->nnpe = nnpe;
    md->ndofpn = ndofpn;
    md->ndim = etype == OGB_PLANESTRESS2D ? 2 : 3;
    md->ngp = etype == OGB_LSPACE ? 8 : (etype == OGB_PLANESTRESS2D ? 4 : 1);
    md->nstress = etype == OGB_PLANESTRESS2D ? 3 : 6;
    md->nmat = nmat;
    md->thickness = thickness;
    md->nonlinear = nonlinear;
    // a1: equation numbering (engngm.C:469-530, masterdof.C:105-120)
    md->h_eq.resize((size_t)nnodes * ndofpn);
    int neq = 0, npeq = 0;
    for (size_t k = 0; k < md->h_eq.size(); ++k) md->h_eq[k] = bc_mask[k] ? -(++npeq) : ++neq;
    md->neq = neq;
    md->npeq = npeq;
    md->inst_start = {0, nnodes};
    std::vector<double> D((size_t)nmat * 36, 0.0);
    for (int i = 0; i < nmat; ++i) isotropic_D(etype, mats[8 * i + 1], mats[8 * i + 2], &D[(size_t)36 * i]);
    cudaStream_t s = ctx->stream;
    int r = OGB_OK;
    auto up = [&](auto &buf, const auto *src, size_t n) {
        if (r != OGB_OK) return;
        r = buf.alloc(n);
        if (r == OGB_OK) {
            cudaError_t e = cudaMemcpyAsync(buf.p, src, n * sizeof(*src), cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync");
        }
    };
    up(md->coords, coords, (size_t)nnodes * md->ndim);
    up(md->conn, conn, (size_t)nelem * nnpe);
    up(md->emat, elem_mat, (size_t)nelem);
    up(md->mats, mats, (size_t)nmat * 8);
    up(md->Dmat, D.data(), D.size());
    up(md->eq, md->h_eq.data(), md->h_eq.size());
    size_t ngpt = (size_t)nelem * md->ngp;
    if (r == OGB_OK) r = md->ke.alloc((size_t)nelem * nnpe * nnpe * ndofpn * ndofpn);
    if (r == OGB_OK) r = md->fe.alloc((size_t)nelem * nnpe * ndofpn);
    if (r == OGB_OK) r = md->gp_stress.alloc(ngpt * md->nstress);
    if (r == OGB_OK) r = md->gp_strain.alloc(ngpt * md->nstress);
    if (r == OGB_OK && nonlinear) {
        r = md->state.alloc(ngpt * NSTATE);
        if (r == OGB_OK) {
            cudaError_t e = cudaMemsetAsync(md->state.p, 0, ngpt * NSTATE * sizeof(double), s);
            if (e != cudaSuccess) r = cuda_fail(e, "cudaMemsetAsync");
        }
    }
    if (r == OGB_OK) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = cuda_fail(e, "model upload");
    }
    if (r != OGB_OK) {
        delete md;
        return r;
    }
    ctx->refs++;
    *out = md;
    return OGB_OK;
}

int ogb_model_destroy(ogb_model *md)
{
    if (!md) return OGB_OK;
    ogb_ctx *ctx = md->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete md;
    ctx_release(ctx);
    return OGB_OK;
}

int ogb_model_neq(ogb_model *md, int *neq, int *npeq)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    if (neq) *neq = md->neq;
    if (npeq) *npeq = md->npeq;
    return OGB_OK;
}

int ogb_model_equations(ogb_model *md, int *eq)
{
    if (!md || !eq) return fail(OGB_E_ARG, "null argument");
    memcpy(eq, md->h_eq.data(), md->h_eq.size() * sizeof(int));
    return OGB_OK;
}

int ogb_model_build_matrix(ogb_model *md, ogb_mtrx *m)
{
    if (!md || !m) return fail(OGB_E_ARG, "null argument");
    if (md->ctx != m->ctx) return fail(OGB_E_ARG, "model and matrix on different contexts");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    OGB_CHECK(build_model_pattern(md, m));
    OGB_CHECK(build_sell(md, m));
    m->spmv_tpr = pick_tpr(m);
    md->bound = m;
    return OGB_OK;
}

// Element tangents of a mixed-precision Newton step (md->mixed_tangent) may run
// on the tensor cores (split BF16, FP32 accuracy) instead of the FP64 CUDA cores:
// OGB_OPT_TANGENT_TC 1 always, 2 when the first such assembly of the model timed
// the tensor-core kernel faster (each kernel once after a warm-up launch, CUDA
// events), 0 (default) never. FP64 solves always use the FP64 kernel.
static int element_tangents(ogb_model *md)
{
    ogb_ctx *ctx = md->ctx;
    const bool isotropic_hex = md->etype == OGB_LSPACE && !md->nonlinear;   // the cheaper isotropic FP64 form
    if (!md->mixed_tangent || ctx->tangent_tc == 0 || isotropic_hex) {
        md->last_tangent_tc = false;
        return launch_elem_stiffness(md);
    }
    if (ctx->tangent_tc == 2 && md->tc_choice == 0) {
        cudaStream_t s = ctx->stream;
        cudaEvent_t ev[4];
        for (auto &e : ev) OGB_CUDA(cudaEventCreate(&e));
        OGB_CHECK(launch_elem_stiffness(md));
        OGB_CHECK(launch_elem_stiffness_tc(md));
        OGB_CUDA(cudaEventRecord(ev[0], s));
        OGB_CHECK(launch_elem_stiffness(md));
        OGB_CUDA(cudaEventRecord(ev[1], s));
        OGB_CHECK(launch_elem_stiffness_tc(md));
        OGB_CUDA(cudaEventRecord(ev[2], s));
        OGB_CUDA(cudaEventSynchronize(ev[2]));
        float t64 = 0.f, ttc = 0.f;
        OGB_CUDA(cudaEventElapsedTime(&t64, ev[0], ev[1]));
        OGB_CUDA(cudaEventElapsedTime(&ttc, ev[1], ev[2]));
        for (auto &e : ev) cudaEventDestroy(e);
        OGB_CHECK(check_device_status(ctx, "tensor-core element stiffness"));
        md->tc_ms[0] = t64;
        md->tc_ms[1] = ttc;
        md->tc_choice = ttc < t64 ? 1 : 2;
        md->last_tangent_tc = md->tc_choice == 1;
        // the last launch was the tensor-core one: its element matrices are current
        return md->tc_choice == 1 ? OGB_OK : launch_elem_stiffness(md);
    }
    const bool tc = ctx->tangent_tc == 1 || md->tc_choice == 1;
    md->last_tangent_tc = tc;
    return tc ? launch_elem_stiffness_tc(md) : launch_elem_stiffness(md);
}

static int assemble_stiffness_async(ogb_model *md, ogb_mtrx *m)
{
    if (md->bound != m || !m->has_structure)
        return fail(OGB_E_STATE, "matrix was not built from this model (ogb_model_build_matrix)");
    OGB_CHECK(element_tangents(md));
    OGB_CHECK(launch_gather_matrix(md, m));
    return OGB_OK;
}

int ogb_model_assemble_tangent(ogb_model *md, ogb_mtrx *m, int precision)
{
    if (!md || !m) return fail(OGB_E_ARG, "null argument");
    if (precision != OGB_PREC_FP64 && precision != OGB_PREC_MIXED) return fail(OGB_E_ARG, "unknown precision");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    md->mixed_tangent = precision == OGB_PREC_MIXED;
    const int r = assemble_stiffness_async(md, m);
    md->mixed_tangent = false;
    OGB_CHECK(r);
    return check_device_status(md->ctx, "assemble tangent");
}

int ogb_model_assemble_stiffness(ogb_model *md, ogb_mtrx *m)
{
    if (!md || !m) return fail(OGB_E_ARG, "null argument");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    OGB_CHECK(assemble_stiffness_async(md, m));
    return check_device_status(md->ctx, "element stiffness");
}

static int internal_forces_async(ogb_model *md, const double *u_dev, double *f_dev)
{
    if (!md->inc.p) {
        OGB_CHECK(build_incidence(md->ctx, md->nnodes, md->nelem, md->nnpe, md->conn.p, md->inc_ptr, md->inc));
    }
    OGB_CHECK(launch_elem_internal_forces(md, u_dev));
    OGB_CHECK(launch_gather_vector(md, f_dev));
    return OGB_OK;
}

int ogb_model_internal_forces_dev(ogb_model *md, const double *u, double *f)
{
    if (!md || !u || !f) return fail(OGB_E_ARG, "null argument");
    OGB_CHECK(internal_forces_async(md, u, f));
    return OGB_OK;
}

int ogb_model_internal_forces(ogb_model *md, const double *u, double *f)
{
    if (!md || !u || !f) return fail(OGB_E_ARG, "null argument");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    size_t n = (size_t)md->nnodes * md->ndofpn;
    OGB_CHECK(md->v_unode.alloc(n));
    OGB_CHECK(md->v_fnode.alloc(n));
    cudaStream_t s = md->ctx->stream;
    OGB_CUDA(cudaMemcpyAsync(md->v_unode.p, u, n * sizeof(double), cudaMemcpyHostToDevice, s));
    OGB_CHECK(internal_forces_async(md, md->v_unode.p, md->v_fnode.p));
    OGB_CUDA(cudaMemcpyAsync(f, md->v_fnode.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    return check_device_status(md->ctx, "internal forces");
}

int ogb_model_gp_stress(ogb_model *md, double *stress, double *strain)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    size_t n = (size_t)md->nelem * md->ngp * md->nstress;
    cudaStream_t s = md->ctx->stream;
    if (stress) OGB_CUDA(cudaMemcpyAsync(stress, md->gp_stress.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (strain) OGB_CUDA(cudaMemcpyAsync(strain, md->gp_strain.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

int ogb_model_commit_state(ogb_model *md)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    if (!md->nonlinear) return OGB_OK;
    int64_t n = (int64_t)md->nelem * md->ngp;
    k_commit_state<<<nb(n), NTHREADS, 0, md->ctx->stream>>>(n, md->emat.p, md->mats.p, md->ngp, md->state.p);
    count_launch(md->ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

int ogb_model_gp_state(ogb_model *md, double *state4)
{
    if (!md || !state4) return fail(OGB_E_ARG, "null argument");
    int64_t n = (int64_t)md->nelem * md->ngp;
    if (!md->nonlinear) {
        memset(state4, 0, n * 4 * sizeof(double));
        return OGB_OK;
    }
    DBuf<double> tmp;
    OGB_CHECK(tmp.alloc(n * 4));
    k_gp_state<<<nb(n), NTHREADS, 0, md->ctx->stream>>>(n, md->emat.p, md->mats.p, md->ngp, md->state.p, tmp.p);
    count_launch(md->ctx);
    OGB_CUDA(cudaMemcpyAsync(state4, tmp.p, n * 4 * sizeof(double), cudaMemcpyDeviceToHost, md->ctx->stream));
    OGB_CUDA(cudaStreamSynchronize(md->ctx->stream));
    return OGB_OK;
}

static int nr_assemble(ogb_model *md, ogb_mtrx *m) { return assemble_stiffness_async(md, m); }
static int nr_forces(ogb_model *md, const double *u, double *f) { return internal_forces_async(md, u, f); }
static int nr_solve(ogb_mtrx *m, double rtol, int maxit, int precision, ogb_solve_info *info)
{
    return solve_padded(m, rtol, maxit, precision, info);
}

int ogb_model_reset_state(ogb_model *md)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    cudaStream_t s = md->ctx->stream;
    if (md->nr_X.p) OGB_CUDA(cudaMemsetAsync(md->nr_X.p, 0, md->nr_X.n * sizeof(double), s));
    if (md->nr_bcprev.p) OGB_CUDA(cudaMemsetAsync(md->nr_bcprev.p, 0, md->nr_bcprev.n * sizeof(double), s));
    if (md->nrb_X.p) OGB_CUDA(cudaMemsetAsync(md->nrb_X.p, 0, md->nrb_X.n * sizeof(double), s));
    md->lin_solves = md->lin_iters = 0;
    if (md->state.p) OGB_CUDA(cudaMemsetAsync(md->state.p, 0, md->state.n * sizeof(double), s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

namespace {
// Header of a state checkpoint; the arrays follow it in this order: GP state,
// free-DOF Newton solution (neq), last prescribed values (nnodes x ndofpn),
// batched Newton solution (nrb_len). All doubles.
struct StateHeader {
    char magic[8];
    int32_t format, etype, nnodes, nelem, ngp, ndofpn, neq, nstate;
    int64_t state_len, nrb_len;
};
constexpr char STATE_MAGIC[8] = {'O', 'G', 'B', 'S', 'T', 'A', 'T', 'E'};
constexpr int32_t STATE_FORMAT = 1;

StateHeader state_header(const ogb_model *md)
{
    StateHeader h{};
    memcpy(h.magic, STATE_MAGIC, 8);
    h.format = STATE_FORMAT;
    h.etype = md->etype;
    h.nnodes = md->nnodes;
    h.nelem = md->nelem;
    h.ngp = md->ngp;
    h.ndofpn = md->ndofpn;
    h.neq = md->neq;
    h.nstate = NSTATE;
    h.state_len = md->state.p ? (int64_t)md->nelem * md->ngp * NSTATE : 0;
    h.nrb_len = md->nrb_X.p ? (int64_t)md->nrb_X.n : 0;
    return h;
}

size_t state_bytes(const StateHeader &h)
{
    return sizeof(StateHeader) +
           sizeof(double) * (size_t)(h.state_len + h.neq + (int64_t)h.nnodes * h.ndofpn + h.nrb_len);
}
}  // namespace

int ogb_model_state_bytes(ogb_model *md, size_t *bytes)
{
    if (!md || !bytes) return fail(OGB_E_ARG, "null argument");
    *bytes = state_bytes(state_header(md));
    return OGB_OK;
}

int ogb_model_save_state(ogb_model *md, void *buf, size_t bytes)
{
    if (!md || !buf) return fail(OGB_E_ARG, "null argument");
    const StateHeader h = state_header(md);
    if (bytes < state_bytes(h)) return fail(OGB_E_ARG, "state buffer too small");
    cudaStream_t s = md->ctx->stream;
    char *p = static_cast<char *>(buf);
    memcpy(p, &h, sizeof h);
    double *d = reinterpret_cast<double *>(p + sizeof h);
    auto put = [&](const DBuf<double> &src, size_t n) -> int {
        if (n == 0) return OGB_OK;
        if (src.p) OGB_CUDA(cudaMemcpyAsync(d, src.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        else memset(d, 0, n * sizeof(double));
        d += n;
        return OGB_OK;
    };
    OGB_CHECK(put(md->state, (size_t)h.state_len));
    OGB_CHECK(put(md->nr_X, (size_t)h.neq));
    OGB_CHECK(put(md->nr_bcprev, (size_t)h.nnodes * h.ndofpn));
    OGB_CHECK(put(md->nrb_X, (size_t)h.nrb_len));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

int ogb_model_restore_state(ogb_model *md, const void *buf, size_t bytes)
{
    if (!md || !buf) return fail(OGB_E_ARG, "null argument");
    if (bytes < sizeof(StateHeader)) return fail(OGB_E_ARG, "state blob shorter than its header");
    StateHeader h;
    memcpy(&h, buf, sizeof h);
    const StateHeader mine = state_header(md);
    if (memcmp(h.magic, STATE_MAGIC, 8) != 0 || h.format != STATE_FORMAT)
        return fail(OGB_E_ARG, "not a state checkpoint of this library");
    if (h.etype != mine.etype || h.nnodes != mine.nnodes || h.nelem != mine.nelem || h.ngp != mine.ngp ||
        h.ndofpn != mine.ndofpn || h.neq != mine.neq || h.nstate != mine.nstate || h.state_len != mine.state_len)
        return fail(OGB_E_ARG, "state checkpoint of another mesh or material model");
    if (h.nrb_len < 0 || bytes < state_bytes(h)) return fail(OGB_E_ARG, "state blob truncated");
    cudaStream_t s = md->ctx->stream;
    OGB_CHECK(nr_ensure(md));
    const double *d = reinterpret_cast<const double *>(static_cast<const char *>(buf) + sizeof h);
    auto get = [&](DBuf<double> &dst, size_t n) -> int {
        if (n == 0) return OGB_OK;
        OGB_CHECK(dst.alloc(n));
        OGB_CUDA(cudaMemcpyAsync(dst.p, d, n * sizeof(double), cudaMemcpyHostToDevice, s));
        d += n;
        return OGB_OK;
    };
    OGB_CHECK(get(md->state, (size_t)h.state_len));
    OGB_CHECK(get(md->nr_X, (size_t)h.neq));
    OGB_CHECK(get(md->nr_bcprev, (size_t)h.nnodes * h.ndofpn));
    if (h.nrb_len > 0) {
        if (md->nrb_X.p && md->nrb_X.n != (size_t)h.nrb_len) md->nrb_X.release();
        OGB_CHECK(get(md->nrb_X, (size_t)h.nrb_len));
    }
    OGB_CUDA(cudaStreamSynchronize(s));   // the blob is the caller's: copies done before return
    return OGB_OK;
}

int ogb_model_tangent_kernel(ogb_model *md, int *tensor_cores, double *ms_fp64, double *ms_tc)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    if (tensor_cores) *tensor_cores = md->last_tangent_tc ? 1 : 0;
    if (ms_fp64) *ms_fp64 = md->tc_ms[0];
    if (ms_tc) *ms_tc = md->tc_ms[1];
    return OGB_OK;
}

int ogb_model_solver_stats(ogb_model *md, int64_t *solves, int64_t *iterations)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    if (solves) *solves = md->lin_solves;
    if (iterations) *iterations = md->lin_iters;
    return OGB_OK;
}

int ogb_model_set_initial_guess(ogb_model *md, int type)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    if (type != 0 && type != 1) return fail(OGB_E_ARG, "initial guess must be 0 (IG_None) or 1 (IG_Tangent)");
    md->initial_guess = type;
    return OGB_OK;
}

int ogb_model_set_nr_mode(ogb_model *md, int manrmsteps)
{
    if (!md) return fail(OGB_E_ARG, "null argument");
    if (manrmsteps < 0) return fail(OGB_E_ARG, "manrmsteps < 0");
    md->nr_manrm = manrmsteps;
    return OGB_OK;
}

int ogb_nonlinear_step_dev(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf,
                           int maxiter, double lin_rtol, int precision, double *u_node, double *reac, int *iterations)
{
    if (!md || !m || !bcval || !u_node) return fail(OGB_E_ARG, "null argument");
    if (md->bound != m) OGB_CHECK(ogb_model_build_matrix(md, m));
    if (!md->inc.p)
        OGB_CHECK(build_incidence(md->ctx, md->nnodes, md->nelem, md->nnpe, md->conn.p, md->inc_ptr, md->inc));
    md->mixed_tangent = precision == OGB_PREC_MIXED;
    const int r = nonlinear_step(md, m, bcval, load, rtolf, maxiter, lin_rtol, precision, u_node, reac, iterations,
                                 nullptr, nr_assemble, nr_forces, nr_solve);
    md->mixed_tangent = false;
    return r;
}

int ogb_nonlinear_step(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf, int maxiter,
                       double lin_rtol, int precision, double *u_node, double *reac, int *iterations)
{
    if (!md || !m || !bcval || !u_node) return fail(OGB_E_ARG, "null argument");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    const size_t n = (size_t)md->nnodes * md->ndofpn;
    cudaStream_t s = md->ctx->stream;
    OGB_CHECK(md->v_bcval.alloc(n));
    OGB_CHECK(md->v_load.alloc(n));
    OGB_CHECK(md->v_unode.alloc(n));
    OGB_CHECK(md->v_reac.alloc(n));
    OGB_CUDA(cudaMemcpyAsync(md->v_bcval.p, bcval, n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (load) OGB_CUDA(cudaMemcpyAsync(md->v_load.p, load, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int r = ogb_nonlinear_step_dev(md, m, md->v_bcval.p, load ? md->v_load.p : nullptr, rtolf, maxiter, lin_rtol,
                                   precision, md->v_unode.p, reac ? md->v_reac.p : nullptr, iterations);
    if (r != OGB_OK) return r;
    OGB_CUDA(cudaMemcpyAsync(u_node, md->v_unode.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (reac) OGB_CUDA(cudaMemcpyAsync(reac, md->v_reac.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

int ogb_model_set_instances(ogb_model *md, int ninst, const int *node_start)
{
    if (!md || !node_start || ninst < 1) return fail(OGB_E_ARG, "bad argument");
    if (md->bound) return fail(OGB_E_STATE, "instances must be declared before the matrix is built");
    if (node_start[0] != 0 || node_start[ninst] != md->nnodes)
        return fail(OGB_E_ARG, "node_start must run from 0 to nnodes");
    for (int i = 0; i < ninst; ++i)
        if (node_start[i + 1] <= node_start[i]) return fail(OGB_E_ARG, "instances must be non-empty and ordered");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    std::vector<int> conn((size_t)md->nelem * md->nnpe);
    OGB_CUDA(cudaMemcpy(conn.data(), md->conn.p, conn.size() * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int> inst_of(md->nnodes);
    for (int i = 0; i < ninst; ++i)
        for (int A = node_start[i]; A < node_start[i + 1]; ++A) inst_of[A] = i;
    // element ranges: recorded when the elements of each instance are contiguous
    // and in instance order (as for concatenated meshes); the batched Newton
    // step needs them
    std::vector<int> elem_start(ninst + 1, 0);
    bool ordered = true;
    int prev = 0;
    for (int e = 0; e < md->nelem; ++e) {
        const int i0 = inst_of[conn[(size_t)e * md->nnpe]];
        for (int a = 1; a < md->nnpe; ++a)
            if (inst_of[conn[(size_t)e * md->nnpe + a]] != i0)
                return fail(OGB_E_MESH, "element " + std::to_string(e) + " couples two instances");
        if (i0 < prev) ordered = false;
        for (int i = prev + 1; i <= i0; ++i) elem_start[i] = e;
        prev = i0 > prev ? i0 : prev;
    }
    for (int i = prev + 1; i <= ninst; ++i) elem_start[i] = md->nelem;
    md->inst_start.assign(node_start, node_start + ninst + 1);
    md->inst_elem_start.clear();
    if (ordered) md->inst_elem_start = elem_start;
    return OGB_OK;
}

int ogb_batch_nonlinear_step_dev(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf,
                                 int maxiter, double lin_rtol, int precision, double *u_node, double *reac,
                                 int *iterations)
{
    if (!md || !m || !bcval || !u_node) return fail(OGB_E_ARG, "null argument");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    if (md->bound != m) OGB_CHECK(ogb_model_build_matrix(md, m));
    if (!md->inc.p)
        OGB_CHECK(build_incidence(md->ctx, md->nnodes, md->nelem, md->nnpe, md->conn.p, md->inc_ptr, md->inc));
    md->mixed_tangent = precision == OGB_PREC_MIXED;
    const int r = nonlinear_step_batch(md, m, bcval, load, rtolf, maxiter, lin_rtol, precision, u_node, reac,
                                       iterations, nr_assemble, nr_forces);
    md->mixed_tangent = false;
    return r;
}

int ogb_batch_nonlinear_step(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf,
                             int maxiter, double lin_rtol, int precision, double *u_node, double *reac,
                             int *iterations)
{
    if (!md || !m || !bcval || !u_node) return fail(OGB_E_ARG, "null argument");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    const size_t n = (size_t)md->nnodes * md->ndofpn;
    cudaStream_t s = md->ctx->stream;
    OGB_CHECK(md->v_bcval.alloc(n));
    OGB_CHECK(md->v_load.alloc(n));
    OGB_CHECK(md->v_unode.alloc(n));
    OGB_CHECK(md->v_reac.alloc(n));
    OGB_CUDA(cudaMemcpyAsync(md->v_bcval.p, bcval, n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (load) OGB_CUDA(cudaMemcpyAsync(md->v_load.p, load, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int r = ogb_batch_nonlinear_step_dev(md, m, md->v_bcval.p, load ? md->v_load.p : nullptr, rtolf, maxiter, lin_rtol,
                                         precision, md->v_unode.p, reac ? md->v_reac.p : nullptr, iterations);
    if (r != OGB_OK) return r;
    OGB_CUDA(cudaMemcpyAsync(u_node, md->v_unode.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (reac) OGB_CUDA(cudaMemcpyAsync(reac, md->v_reac.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

int ogb_batch_linear_static_dev(ogb_model *md, ogb_mtrx *m, int nrhs, const double *bcval, const double *load,
                                double rtol, int maxit, int precision, double *u_nodes, double *reacs, int *iters,
                                double *achieved, int *status)
{
    if (!md || !m || !bcval || !u_nodes) return fail(OGB_E_ARG, "null argument");
    if (nrhs < 1 || nrhs > 4) return fail(OGB_E_ARG, "nrhs must be 1..4");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    if (md->bound != m) OGB_CHECK(ogb_model_build_matrix(md, m));
    return batch_linear_static(md, m, nrhs, bcval, load, rtol, maxit, precision, u_nodes, reacs, iters, achieved,
                               status, nr_assemble, nr_forces);
}

int ogb_batch_linear_static(ogb_model *md, ogb_mtrx *m, int nrhs, const double *bcval, const double *load,
                            double rtol, int maxit, int precision, double *u_nodes, double *reacs, int *iters,
                            double *achieved, int *status)
{
    if (!md || !m || !bcval || !u_nodes) return fail(OGB_E_ARG, "null argument");
    if (nrhs < 1 || nrhs > 4) return fail(OGB_E_ARG, "nrhs must be 1..4");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    const size_t n = (size_t)md->nnodes * md->ndofpn * nrhs;
    cudaStream_t s = md->ctx->stream;
    DBuf<double> d_bc, d_load, d_u, d_reac;
    OGB_CHECK(d_bc.alloc(n));
    OGB_CHECK(d_u.alloc(n));
    if (load) OGB_CHECK(d_load.alloc(n));
    if (reacs) OGB_CHECK(d_reac.alloc(n));
    OGB_CUDA(cudaMemcpyAsync(d_bc.p, bcval, n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (load) OGB_CUDA(cudaMemcpyAsync(d_load.p, load, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int r = ogb_batch_linear_static_dev(md, m, nrhs, d_bc.p, load ? d_load.p : nullptr, rtol, maxit, precision, d_u.p,
                                        reacs ? d_reac.p : nullptr, iters, achieved, status);
    if (r != OGB_OK && r != OGB_E_NOTCONV && r != OGB_E_BREAKDOWN && r != OGB_E_ZERODIAG) return r;
    OGB_CUDA(cudaMemcpyAsync(u_nodes, d_u.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (reacs) OGB_CUDA(cudaMemcpyAsync(reacs, d_reac.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return r;
}

int ogb_linear_static_dev(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtol, int maxit,
                          int precision, double *u_node, double *reac, ogb_solve_info *info)
{
    if (!md || !m || !bcval || !u_node) return fail(OGB_E_ARG, "null argument");
    ogb_ctx *ctx = md->ctx;
    cudaStream_t s = ctx->stream;
    const int n = md->nnodes * md->ndofpn;
    if (md->bound != m) OGB_CHECK(ogb_model_build_matrix(md, m));
    OGB_CHECK(md->v_fnode.alloc(n));
    OGB_CHECK(ensure_solver_vectors(m));
    // K (K1 + K4)
    OGB_CHECK(assemble_stiffness_async(md, m));
    // prescribed displacement field and its internal forces (linearstatic.C:224-230)
    k_u_from_bc<<<nb(n), NTHREADS, 0, s>>>(n, md->eq.p, bcval, u_node);
    count_launch(ctx);
    OGB_CHECK(internal_forces_async(md, u_node, md->v_fnode.p));
    OGB_CUDA(cudaMemsetAsync(m->w_b.p, 0, m->npad * sizeof(double), s));
    OGB_CUDA(cudaMemsetAsync(m->w_x.p, 0, m->npad * sizeof(double), s));
    k_build_rhs<<<nb(n), NTHREADS, 0, s>>>(n, md->eq.p, load, md->v_fnode.p, m->w_b.p);
    count_launch(ctx);
    OGB_CHECK(check_device_status(ctx, "assembly"));
    int r = solve_padded(m, rtol, maxit, precision, info);
    k_scatter_solution<<<nb(n), NTHREADS, 0, s>>>(n, md->eq.p, m->w_x.p, u_node);
    count_launch(ctx);
    if (reac) {
        OGB_CHECK(internal_forces_async(md, u_node, md->v_fnode.p));
        k_reactions<<<nb(n), NTHREADS, 0, s>>>(n, md->eq.p, md->v_fnode.p, load, reac);
        count_launch(ctx);
    }
    OGB_CUDA(cudaGetLastError());
    return r;
}

int ogb_linear_static(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtol, int maxit,
                      int precision, double *u_node, double *reac, ogb_solve_info *info)
{
    if (!md || !m || !bcval || !u_node) return fail(OGB_E_ARG, "null argument");
    OGB_CUDA(cudaSetDevice(md->ctx->device));
    const size_t n = (size_t)md->nnodes * md->ndofpn;
    cudaStream_t s = md->ctx->stream;
    OGB_CHECK(md->v_bcval.alloc(n));
    OGB_CHECK(md->v_load.alloc(n));
    OGB_CHECK(md->v_unode.alloc(n));
    OGB_CHECK(md->v_reac.alloc(n));
    OGB_CUDA(cudaMemcpyAsync(md->v_bcval.p, bcval, n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (load) OGB_CUDA(cudaMemcpyAsync(md->v_load.p, load, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int r = ogb_linear_static_dev(md, m, md->v_bcval.p, load ? md->v_load.p : nullptr, rtol, maxit, precision,
                                  md->v_unode.p, reac ? md->v_reac.p : nullptr, info);
    if (r != OGB_OK && r != OGB_E_NOTCONV && r != OGB_E_BREAKDOWN && r != OGB_E_ZERODIAG) return r;
    OGB_CUDA(cudaMemcpyAsync(u_node, md->v_unode.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (reac) OGB_CUDA(cudaMemcpyAsync(reac, md->v_reac.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return r;
}

}  // extern "C"
