// Internal declarations shared by the CUDA translation units of liboofem_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/oofem_gb300.h"

namespace ogb {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define OGB_CUDA(call)                                              \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return ::ogb::cuda_fail(_e, #call);  \
    } while (0)

#define OGB_CHECK(call)                       \
    do {                                      \
        int _r = (call);                      \
        if (_r != OGB_OK) return _r;          \
    } while (0)

// Rows of every system are processed in chunks of CHUNK rows; systems are
// padded to a multiple of CHUNK with identity rows so that every chunk belongs
// to one system and block-level reductions stay deterministic.
constexpr int CHUNK = 1024;
constexpr int NTHREADS = 256;
// Multiprocessor count of the current device (queried once per device; 152 on a
// GB300). Grids of the vector and reduction kernels are multiples of it.
int num_sms();

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------- device buffers
template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        if (count <= n && p) return OGB_OK;
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; n = 0; return cuda_fail(e, "cudaMalloc"); }
        n = count;
        return OGB_OK;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DBuf() { release(); }
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
};

// Pinned host staging buffer.
template <class T>
struct HBuf {
    T *p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        if (count <= n && p) return OGB_OK;
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMallocHost((void **)&p, count * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; n = 0; return cuda_fail(e, "cudaMallocHost"); }
        n = count;
        return OGB_OK;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
    ~HBuf() { release(); }
    HBuf() = default;
    HBuf(const HBuf &) = delete;
    HBuf &operator=(const HBuf &) = delete;
};

// Device-side status word written by kernels instead of trapping.
enum DevStatus : int {
    DS_OK = 0,
    DS_LIMIT = 1,      // a fixed per-row / per-node capacity was exceeded
    DS_PATTERN = 2,    // an assembled location is missing from the pattern
    DS_NEGVOL = 3,     // tetrahedron with detJ <= 0 (fei3dtetlin.C:146)
    DS_TIMEOUT = 4,    // an asynchronous copy did not complete within the wait limit
};

// Per-system PCG scalars (one record per right-hand side / instance).
struct PcgScal {
    double bnorm2;    // ||b||^2
    double rho;       // r.z of the current iteration
    double rho_old;
    double pq;        // p.q
    double rnorm2;    // ||r||^2
    double alpha, beta;
    double rmax2;     // ||r||^2 at the last FP64 residual replacement (mixed)
    double tol2;      // (rtol ||b||)^2 (mixed)
    double drop2;     // replacement threshold: ||r||^2 <= drop2 * rmax2 (mixed)
    double zcoef;     // p = zcoef z + beta p (1 except right after a replacement)
    int done;         // 1 converged, 2 breakdown, 3 zero diagonal, 4 max iterations,
                      // 5 a device-wide wait of a fused update timed out
    int iters;
    int reliable;     // mixed: an FP64 residual replacement is due
    int cycle_end;    // mixed: iteration count at which the current cycle ends at the latest
};

// Node-block SELL-32 storage: rows = active nodes (>= 1 free DOF) in node
// order, ND x ND blocks, 32 rows per slice, blocks of a slice stored k-major so
// that lane r of a warp reads row r's k-th block with coalesced loads.
//   slot(s, k, r)   = sl_ptr[s] + 32 k + r                (column index array)
//   value(slot, e)  = (slot - r) * ND*ND + 32 e + r        (e = i*ND + j)
// Half-stored FP32 copy of a symmetric node-block SELL matrix. Row a keeps its
// diagonal block and the blocks of its columns b > a as a SELL-32 of its own
// (the upper part); for its columns c < a it keeps a list entry (c << 6 | k),
// k the position of a in row c's upper list, and reads K_ac as the transpose of
// the block K_ca stored there. The upper values stream from HBM once; the
// transposed reads come back to the same blocks shortly after (on structured
// meshes a warp's lanes read neighbouring blocks together) and hit L2. Slots
// are laid out as in the full copy: slot = sl_ptr[s] + 32 k + r, values at
// (slot - r) * ND*ND + 32 e + r.
struct HalfSell {
    bool ok = false;
    bool tried = false;          // built or found unsuitable for this structure
    int64_t nslotsU = 0, nslotsL = 0;
    DBuf<int64_t> sl_ptrU, sl_ptrL;   // nslices + 1
    DBuf<int> sl_widthU, sl_widthL;   // nslices
    DBuf<int> colU;                   // nslotsU (padding: the row itself)
    DBuf<int64_t> srcU;               // slot of the same block in the full copy (-1: padding)
    DBuf<int> low;                    // nslotsL: c << 6 | k (-1: padding)
    DBuf<float> v32;                  // nslotsU * ND*ND
    int64_t version = -1;             // full-copy v32_version these values were taken from
    int form = 0;                     // SpMV form chosen by the autotuner (0 = not yet)
    void reset()
    {
        ok = tried = false;
        version = -1;
        form = 0;
    }
};

struct SellMat {
    int nd = 0;
    int nact = 0;           // active node rows
    int nslices = 0;        // padded to a multiple of 32 slices
    int64_t nslots = 0;
    DBuf<int64_t> sl_ptr;   // nslices+1
    DBuf<int> sl_width;     // blocks per row of each slice
    DBuf<int> col;          // nslots
    DBuf<int64_t> diag;     // slot of the diagonal block of each row (nslices*32)
    DBuf<double> v64;       // nslots * ND*ND
    DBuf<float> v32;
    int64_t v32_version = -1;
    DBuf<int> ns_of_eq;     // node-space index of equation e (0-based)
    int ninst = 1;          // independent instances (block-diagonal batch)
    int group[2] = {0, 0};  // tuned SpMV variant for FP64 / FP32 values (0 = not yet)
    int force_split = 0;    // warps per slice forced by OGB_OPT_SPMV_VARIANT 5 / 6 (0 = rule)
    int bform32 = 0;        // batched FP32 SpMV form timed for this matrix: 1 plain, 2 values of a group first
    std::vector<int64_t> inst_row_base;   // first node-space row of each instance (+ total)
    HalfSell half;                        // half-stored FP32 copy (built on first use)
    int64_t nns() const { return (int64_t)nslices * 32 * nd; }
};

// Incomplete-Cholesky factor of the IML solver's IC preconditioner (icprec.cu):
// forward rows (entries of the transposed columns), backward rows (each row's
// own column below the diagonal), the diagonal, and both level schedules.
struct IcFactor {
    int64_t version = -1;
    int kind = 0;   // 4 incomplete Cholesky, 2 ILU (lsprecond)
    int n = 0;
    DBuf<int64_t> fptr, bptr;
    DBuf<int> fcol, bcol, frows, brows;
    DBuf<double> fval, bval, diag, work;
    std::vector<int> flev, blev;   // level starts into frows / brows
    DBuf<int> d_flev, d_blev;      // the same on the device
};

// LDL^T factor of the direct solver (direct.cu): dense band of n x (bw+1)
// doubles, column j holds L(j..j+bw, j) with d_j in its diagonal slot.
struct LdlFactor {
    int64_t version = -1;   // matrix version the factor belongs to
    bool ok = false;
    int n = 0, bw = 0;      // equations, half bandwidth
    DBuf<double> band;
    DBuf<int> d_int;        // [0] half bandwidth, [1] 1-based equation of a zero pivot
    HBuf<int> h_int;
    DBuf<double> y, part, out;   // residual check of a solve
    DBuf<unsigned int> cnt;
    HBuf<double> h_out;
};

// Instances of a batch start on multiples of INST_ALIGN node-space rows.
constexpr int INST_ALIGN = 1024;

}  // namespace ogb

// ---------------------------------------------------------------- handles
struct ogb_ctx {
    int device = 0;
    int refs = 0;          // live matrices/models created on this context
    bool closing = false;  // ogb_ctx_destroy called while refs > 0
    cudaStream_t stream = nullptr;
    int64_t launches = 0;
    // kernel timing (SpMV launches), see ogb_ctx_profile_enable
    bool prof = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<cudaEvent_t> ev_pending;   // start/stop pairs
    double prof_ms = 0.0, prof_bytes = 0.0, pending_bytes = 0.0;
    int64_t prof_count = 0;
    bool mixed_vec32 = true;    // mixed solve with FP32 Krylov vectors (see solver.cu)
    bool use_graphs = true;     // replay PCG iteration batches as CUDA graphs
    std::vector<cudaEvent_t> *capture_events = nullptr;   // profiling events recorded into a graph
    double capture_bytes = 0.0;
    bool prof_sample = true;    // inside a captured batch only the first SpMV is bracketed
    bool mixed_diff = true;     // FP32 operator in difference form (see solver.cu)
    bool mixed_orth = false;    // restore r.p = 0 after a residual replacement
    bool mixed_p32 = false;     // mixed solve keeps p and q = K p in FP32 (x, r, z FP64)
    bool mixed_x64 = true;      // with FP32 vectors: update the FP64 solution directly
    bool mixed_sum32 = false;   // ... with the update's dot-product terms summed per thread in FP32
    int spmv_group = 0;         // SELL SpMV loop variant forced (1..4) or 0 = tuned per matrix
    int spmv_half = 1;          // half-stored FP32 copy in mixed solves: 0 never, 1 one-warp-per-slice matrices, 2 always
    int half_form = 0;          // half-stored SpMV form forced (1..3) or 0 = timed per matrix
    int upd_bps = 0;            // blocks per SM of the block-Jacobi update and p update (0 = its occupancy)
    bool fused_update = true;   // block-Jacobi update and p update in one cooperative launch
    int batch_form = 0;         // batched FP32 SpMV form forced (1, 2) or 0 = timed per matrix
    bool batch_x64 = false;     // batched mixed solves: FP64 solution every iteration (else FP32 increment per batch)
    int spmv_split = 0;         // warps per slice forced (1, 2, 4) or 0 = the slice-count rule
    double mixed_drop = 0.1;    // residual drop between FP64 replacements
    bool mixed_bj = true;       // mixed solves on node-block operators: block-Jacobi preconditioner
    int tangent_tc = 0;         // mixed Newton tangents on tensor cores: 0 never, 1 always, 2 when timed faster
    ogb::DBuf<int> status;           // device status word
    ogb::HBuf<int> h_status;
};

struct ogb_mtrx {
    ogb_ctx *ctx = nullptr;
    int neq = 0;          // equations
    int npad = 0;         // rows incl. identity padding (multiple of CHUNK)
    int64_t nnz = 0;      // pattern entries of the neq real rows
    int64_t version = 0;
    bool has_structure = false;
    ogb::DBuf<int64_t> rowptr;   // npad+1
    ogb::DBuf<int> colind;       // nnz + (npad-neq)
    ogb::DBuf<double> val;       // same length
    ogb::DBuf<float> val32;      // FP32 copy for the mixed-precision solve
    int64_t val32_version = -1;
    ogb::DBuf<int64_t> diagpos;  // position of (r,r) per row (npad)
    // drop-in staging (SparseMtrx::assemble from host element loops)
    std::vector<int64_t> st_ptr;     // per staged matrix: offset into st_loc
    std::vector<int> st_loc;
    std::vector<int64_t> st_keoff;   // per staged matrix: offset into st_ke
    std::vector<double> st_ke;
    // solver workspace
    ogb::DBuf<double> w_r, w_z, w_p, w_q, w_dinv, w_x, w_b, w_part, w_d;
    ogb::DBuf<float> w_r32, w_z32, w_p32, w_q32, w_dinv32, w_x32;
    ogb::DBuf<float> w_binv32;   // block-Jacobi inverses of the node diagonal blocks (upper-triangle planes)
    bool last_bj = false;        // the last mixed solve used the block-Jacobi preconditioner
    ogb::DBuf<ogb::PcgScal> w_scal;
    ogb::HBuf<ogb::PcgScal> h_scal;
    ogb::DBuf<unsigned int> w_count;
    ogb::DBuf<unsigned int> w_epoch;             // fused update: advanced once per iteration by its last block
    int spmv_tpr = 8;    // threads per row of the CSR SpMV (autotuned)
    // node-block copy used by the solver when the matrix was built from a model
    bool has_sell = false;
    ogb::SellMat sell;
    ogb::DBuf<double> n_b, n_x, n_r64, n_q64;   // node-space FP64 vectors
    ogb::DBuf<float> n_d32;                      // mixed: solution increment since the last replacement
    bool last_half = false;                      // the last mixed solve used the half-stored FP32 copy
    int precond = 1;                             // IML preconditioner type: 0 none, 1 diagonal, 2 ILU, 4 incomplete Cholesky
    ogb::IcFactor ic;
    int lstype = OGB_LS_GPUPCG;                  // linear solver: OGB_LS_DIRECT factors (direct.cu), else PCG
    ogb::LdlFactor ldl;
};

struct ogb_model {
    ogb_ctx *ctx = nullptr;
    int etype = 0, nnodes = 0, nelem = 0, nnpe = 0, ndofpn = 0, ndim = 0, ngp = 0, nstress = 0;
    int nmat = 0;
    double thickness = 1.0;
    int neq = 0, npeq = 0;
    std::vector<int> h_eq;
    ogb::DBuf<double> coords, mats, Dmat;
    ogb::DBuf<int> conn, emat, eq;
    // node -> (element << 3 | local node), sorted by element
    ogb::DBuf<int64_t> inc_ptr;
    ogb::DBuf<uint32_t> inc;
    // node adjacency (node blocks) of the pattern
    ogb::DBuf<int64_t> nb_ptr;
    ogb::DBuf<int> nb_col, nb_coloff, blk_node;
    int64_t nblocks = 0;
    // contributions per node block: (element << 6 | a << 3 | b), sorted by element
    ogb::DBuf<int64_t> cb_ptr;
    ogb::DBuf<uint32_t> cb;
    ogb::DBuf<int64_t> node_rowbase;   // CSR position of the first row of each node
    ogb::DBuf<int> node_rowlen;
    ogb::DBuf<int> act;                // active-node index per node (-1: all DOFs prescribed)
    ogb::DBuf<int64_t> blk_slot;       // SELL slot per node block (-1: none)
    // element buffers
    ogb::DBuf<double> ke;       // nelem x nnpe x nnpe x ndofpn x ndofpn
    ogb::DBuf<double> fe;       // nelem x nnpe x ndofpn
    ogb::DBuf<double> state;    // nelem x ngp x NSTATE
    ogb::DBuf<double> gp_stress, gp_strain;
    // linear-static work vectors
    ogb::DBuf<double> v_unode, v_fnode, v_bcval, v_load, v_b, v_x, v_reac;
    ogb_mtrx *bound = nullptr;
    bool nonlinear = false;
    std::vector<int> inst_start;   // first node of each instance (+ nnodes); {0, nnodes} for one mesh
    std::vector<int> inst_elem_start;   // first element of each instance (+ nelem) when contiguous, else empty
    ogb::DBuf<int> d_inst_start, d_inst_elem_start, d_node_inst;
    ogb::DBuf<double> nrb_X, nrb_b, nrb_x, nrb_out;   // batched Newton: node-space solution, increment
    ogb::DBuf<unsigned int> nrb_cnt;
    ogb::DBuf<int> nrb_active;
    // Newton driver
    ogb::DBuf<double> nr_X, nr_part, nr_out;
    ogb::DBuf<double> nr_bcprev, nr_du;   // prescribed values of the last converged step; increment
    int initial_guess = 0;                 // NonLinearStatic initialGuess: 0 IG_None, 1 IG_Tangent
    int nr_manrm = 1;                      // NRSolver manrmsteps: 0 modified Newton, k re-assembles when nite % k == 0
    int64_t lin_solves = 0, lin_iters = 0;  // linear solves of the Newton drivers and their PCG iterations
    bool mixed_tangent = false;   // inside a mixed-precision Newton step: tangents may run on tensor cores
    int tc_choice = 0;            // tensor-core tangent timing: 0 not yet, 1 tensor cores faster, 2 FP64 faster
    bool last_tangent_tc = false; // the last element tangents came from the tensor-core kernel
    float tc_ms[2] = {0.f, 0.f};  // timed FP64 and tensor-core element stiffness (ms)
    ogb::DBuf<unsigned int> nr_count;
    ogb::HBuf<double> h_nr_out;
};

namespace ogb {

constexpr int NSTATE = 24;

// Raise a kernel's dynamic shared-memory limit once per device (the attribute
// belongs to the device the call is made on). `done` is the caller's flag table.
inline cudaError_t set_smem_limit_once(const void *kernel, int bytes, bool (&done)[64])
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

// --------------------------------------------------------------- launchers
// scan.cu
int exclusive_scan_i64(ogb_ctx *ctx, const int64_t *in, int64_t *out, int64_t n, int64_t *total_host);

// pattern.cu
int build_incidence(ogb_ctx *ctx, int nnodes, int nelem, int nnpe, const int *conn,
                    DBuf<int64_t> &inc_ptr, DBuf<uint32_t> &inc);
int build_model_pattern(ogb_model *md, ogb_mtrx *m);
int build_loc_pattern(ogb_mtrx *m, int neq, int nelem, const int64_t *loc_ptr_h, const int *loc_h);
int staged_assemble(ogb_mtrx *m);
int pad_matrix_rows(ogb_mtrx *m);
int build_sell(ogb_model *md, ogb_mtrx *m);
// halfsell.cu: the half-stored FP32 copy of m->sell (half.ok stays false when the
// matrix does not fit its index packing); refresh_half copies the current FP32
// values into it.
int build_half(ogb_ctx *ctx, SellMat &S);
// icprec.cu: the IC factor of m (host, cached per matrix version) and z = M^-1 r
// (device, level-scheduled; kernels skip once sc reports done).
int build_ic(ogb_mtrx *m);
int launch_ic_solve(ogb_mtrx *m, const double *r, double *z, const PcgScal *sc);
int refresh_half(ogb_ctx *ctx, SellMat &S);

// element.cu
int launch_elem_stiffness(ogb_model *md);
// Split-BF16 tensor-core element stiffness (FP32 accuracy) for mixed-precision tangents.
int launch_elem_stiffness_tc(ogb_model *md);
int launch_elem_internal_forces(ogb_model *md, const double *u_node);
int launch_isotropic_tables(ogb_model *md);

// assembly.cu
int launch_gather_matrix(ogb_model *md, ogb_mtrx *m);
int launch_gather_vector(ogb_model *md, double *f_node);

// solver.cu
int spmv64(ogb_mtrx *m, const double *x, double *y);
int pcg_fp64(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, ogb_solve_info *info);
int pcg_mixed(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit, ogb_solve_info *info);
int extract_diag(ogb_mtrx *m);
int pick_tpr(const ogb_mtrx *m);

// direct.cu: LDL^T factor of m (cached per version) and x = A^-1 b on padded
// equation-space device vectors (info: 0 iterations, FP64 relative residual).
int ldl_factor(ogb_mtrx *m);
int ldl_solve(ogb_mtrx *m, const double *b, double *x, ogb_solve_info *info);

// newton.cu
int nr_ensure(ogb_model *md);   // Newton work buffers; nr_X and nr_bcprev zeroed on first allocation
int nonlinear_step(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf, int maxiter,
                   double lin_rtol, int precision, double *u_node, double *reac, int *iterations,
                   ogb_solve_info *lin_info, int (*assemble)(ogb_model *, ogb_mtrx *),
                   int (*forces)(ogb_model *, const double *, double *),
                   int (*solve)(ogb_mtrx *, double, int, int, ogb_solve_info *));

// batch.cu
int batch_pcg(ogb_mtrx *m, int nrhs, const double *b, double *x, double rtol, int maxit, int precision, int *iters,
              double *achieved, int *status);
int pcg_solve_multi(ogb_mtrx *m, int nrhs, const double *B, double *X, double rtol, int maxit, int precision,
                    int *iters, double *achieved, int *status);
int batch_linear_static(ogb_model *md, ogb_mtrx *m, int nrhs, const double *bcval, const double *load, double rtol,
                        int maxit, int precision, double *u_nodes, double *reacs, int *iters, double *achieved,
                        int *status,
                        int (*assemble)(ogb_model *, ogb_mtrx *), int (*forces)(ogb_model *, const double *, double *));

int nonlinear_step_batch(ogb_model *md, ogb_mtrx *m, const double *bcval, const double *load, double rtolf,
                         int maxiter, double lin_rtol, int precision, double *u_node, double *reac, int *iterations,
                         int (*assemble)(ogb_model *, ogb_mtrx *), int (*forces)(ogb_model *, const double *, double *));

// helpers in capi.cu
inline void count_launch(ogb_ctx *ctx, int n = 1) { ctx->launches += n; }
int check_device_status(ogb_ctx *ctx, const char *where);
void ctx_release(ogb_ctx *ctx);
// profiling helpers (capi.cu)
void prof_begin(ogb_ctx *ctx);
void prof_end(ogb_ctx *ctx, double bytes);
void prof_harvest(ogb_ctx *ctx);

}  // namespace ogb
