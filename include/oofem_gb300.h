/*
 * oofem_gb300 -- GB300-native (sm_103a) structural hot path of OOFEM behind a C ABI.
 *
 * Plain C types only (pointers, sizes, int status codes); no exception crosses
 * this boundary. Every call returns OGB_OK (0) or a negative OGB_E* code; the
 * message of the last failure on the calling thread is ogb_last_error().
 *
 * Conventions (follow the reference):
 *   - element types: OGB_LSPACE (8-node hex, 2x2x2 Gauss), OGB_PLANESTRESS2D
 *     (4-node quad, 2x2 Gauss, thickness), OGB_LTRSPACE (4-node tet, 1 point).
 *   - element node order as FEI3dHexaLin / FEI2dQuadLin / FEI3dTetLin
 *     (src/core/fei3dhexalin.C:45-63, fei2dquadlin.C:60-72, fei3dtetlin.C:45-55).
 *   - equation numbers: nodes in input order, DOFs in node order (u,v[,w]);
 *     free DOFs 1..neq, prescribed DOFs -1..-npeq (engngm.C:469-530,
 *     masterdof.C:105-120). Location arrays are 1-based, 0 = prescribed.
 *   - CSR (row pointers int64, column indices int32, 0-based, sorted) of the full
 *     symmetric pattern == CompCol colptr/rowind (compcol.C:174-272).
 *   - Voigt order xx,yy,zz,yz,zx,xy (3-D) / xx,yy,xy (plane stress).
 *   - material table: rows of 8 doubles {kind, E, nu, sig0, H, e0, gf, 0},
 *     kind OGB_MAT_ISOLE / OGB_MAT_MISES / OGB_MAT_IDM1.
 *   - "host" entry points take host pointers and copy; "_dev" entry points take
 *     device pointers of the library's device and never copy to the host.
 *
 * Streams: every handle owns one CUDA stream (ogb_ctx_stream); calls are
 * asynchronous on it unless they return host data.
 */
#ifndef OOFEM_GB300_H
#define OOFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define OGB_API __attribute__((visibility("default")))
#else
#define OGB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define OGB_OK 0
#define OGB_E_ARG -1        /* bad argument / size mismatch */
#define OGB_E_CUDA -2       /* CUDA runtime error */
#define OGB_E_STATE -3      /* call out of order (e.g. no structure yet) */
#define OGB_E_PATTERN -4    /* location outside the sparsity pattern */
#define OGB_E_NOTCONV -5    /* solver did not converge (CR_DIVERGED_ITS) */
#define OGB_E_BREAKDOWN -6  /* PCG breakdown: rho or p'q <= 0 or not finite */
#define OGB_E_ZERODIAG -7   /* zero diagonal (DiagPreconditioner::init error) */
#define OGB_E_MESH -8       /* invalid mesh (e.g. negative tet volume) */
#define OGB_E_LIMIT -9      /* a fixed capacity of the library was exceeded */

#define OGB_LSPACE 1
#define OGB_PLANESTRESS2D 2
#define OGB_LTRSPACE 3

#define OGB_MAT_ISOLE 1
#define OGB_MAT_MISES 2
#define OGB_MAT_IDM1 3

/* Precision of a solve. FP64 is the drop-in (IML CG + DiagPreconditioner
 * semantics); MIXED stores and applies an FP32 matrix inside an FP64
 * iterative-refinement loop whose residual is evaluated in FP64. */
#define OGB_PREC_FP64 0
#define OGB_PREC_MIXED 1

typedef struct ogb_ctx ogb_ctx;       /* device + stream */
typedef struct ogb_mtrx ogb_mtrx;     /* GPU compressed sparse matrix (SparseMtrx) */
typedef struct ogb_model ogb_model;   /* GPU element backend for one mesh */

/* ---- library / context ---------------------------------------------------- */
OGB_API const char *ogb_last_error(void);
OGB_API int ogb_version(void);
/* Create a context on CUDA device `device` with its own non-blocking stream. */
OGB_API int ogb_ctx_create(int device, ogb_ctx **out);
OGB_API int ogb_ctx_destroy(ogb_ctx *ctx);
OGB_API void *ogb_ctx_stream(ogb_ctx *ctx);                 /* cudaStream_t */
OGB_API int ogb_ctx_synchronize(ogb_ctx *ctx);
/* Number of kernels this library launched on the context since creation. */
OGB_API int64_t ogb_ctx_kernel_launches(ogb_ctx *ctx);
/* Tuning options of a context (no reference counterpart):
 *   OGB_OPT_MIXED_VEC32 (0/1): mixed solves keep the CG vectors in FP32 instead
 *   of FP64 (default 1). */
#define OGB_OPT_MIXED_VEC32 1
/*   OGB_OPT_MIXED_DIFF (0/1): FP32 operator stored in difference form (default 1).
 *   OGB_OPT_MIXED_ORTH (0/1): restore r.p = 0 after an FP64 residual replacement.
 *   OGB_OPT_MIXED_DROP_PPM: residual drop factor between replacements, in 1e-6
 *   units (default 100000 = 0.1). */
#define OGB_OPT_MIXED_DIFF 2
#define OGB_OPT_MIXED_ORTH 3
#define OGB_OPT_MIXED_DROP_PPM 4
/*   OGB_OPT_MIXED_P32 (0/1): mixed solves keep p and q = K p in FP32 only. */
#define OGB_OPT_MIXED_P32 5
/*   OGB_OPT_MIXED_X64 (0..3): with FP32 vectors, accumulate the solution in
 *   FP64 every iteration (1; 2: the same with the update's r.r and r.z terms
 *   summed per thread in FP32 before the FP64 block sums), or as an FP32
 *   increment folded into the FP64 solution after every 16 iterations and at
 *   each residual replacement (0: terms summed per thread in FP32; 3: summed
 *   per node in FP64). Single-matrix solves only (batched solves: see
 *   OGB_OPT_BATCH_X64). */
#define OGB_OPT_MIXED_X64 6
/*   OGB_OPT_SPMV_VARIANT: node-block SpMV form, 1 = plain unrolled loop,
 *   2 / 3 = block columns loaded 1 / 4 blocks ahead, 4 = values and columns
 *   staged through shared memory by bulk asynchronous copies (FP32 values; FP64
 *   uses form 3), 5 / 6 = each slice shared by 2 / 4 warps; 0 (default) = warps
 *   per slice from the slice count, loop form timed once per matrix and value
 *   type by the built-in autotuner. */
#define OGB_OPT_SPMV_VARIANT 7
/*   OGB_OPT_SPMV_HALF (0/1/2, default 1): mixed solves keep the FP32 operator
 *   of a node-block matrix half-stored: the diagonal and upper blocks of each
 *   row, the lower blocks read as transposes of the upper blocks of earlier rows
 *   (the matrix is symmetric), which halves the matrix stream of every FP32
 *   SpMV. 1 = for matrices large enough for one warp per slice, 2 = for every
 *   node-block matrix, 0 = never. A forced OGB_OPT_SPMV_VARIANT uses the full
 *   copy. The sum order differs from the full copy's (results agree to FP32
 *   rounding of the operator, not bitwise). */
#define OGB_OPT_SPMV_HALF 8
/*   OGB_OPT_MIXED_BLOCK_JACOBI (0/1, default 1): mixed solves on a matrix
 *   assembled from a model precondition with the FP32 inverses of the node
 *   ND x ND diagonal blocks (block Jacobi) where the diagonal preconditioner
 *   (lsprecond 1) is selected; 0 keeps the scalar diagonal. FP64 solves always
 *   use the reference's scalar DiagPreconditioner. */
#define OGB_OPT_MIXED_BLOCK_JACOBI 9
/*   OGB_OPT_HALF_FORM (0..6, default 0): loop form of the half-stored SpMV:
 *   groups of 8 blocks with the registers per thread bounded for 4 (1), 3 (2)
 *   or 2 (3) resident blocks of 256 threads per SM, or every value of a group
 *   loaded before its products with groups of 4 at 3 blocks per SM (4), of 3 at
 *   4 (5), of 2 at 5 (6); 0 = timed once per matrix by the built-in autotuner.
 *   The forms give bitwise equal results. */
#define OGB_OPT_HALF_FORM 12
/*   OGB_OPT_UPDATE_BLOCKS (0..8, default 0): blocks per SM of the block-Jacobi
 *   vector update of mixed solves; 0 = one wave of the kernel's resident blocks
 *   (its occupancy), fewer when that would leave a block fewer than about 2,048
 *   nodes. */
#define OGB_OPT_UPDATE_BLOCKS 13
/*   OGB_OPT_TANGENT_TC (0/1/2, default 0): element tangents of mixed-precision
 *   Newton steps (ogb_nonlinear_step, ogb_batch_nonlinear_step with
 *   OGB_PREC_MIXED) on the tensor cores: K_e = sum B^T D B dV as split-BF16
 *   products accumulated in FP32, the upper triangle mirrored (FP32 accuracy);
 *   0 = FP64 CUDA cores, 1 = tensor cores, 2 = whichever kernel the first such
 *   assembly of the model timed faster. An FP32-accurate tangent annihilates the
 *   element rigid-body modes only to about 1e-7 of its entries: on meshes whose
 *   stiffness spans more than about seven decades that perturbs the tangent
 *   beyond what the Newton iteration and the CG solve tolerate, hence off by
 *   default. FP64 steps and LinearStatic always use the FP64 element kernels. */
#define OGB_OPT_TANGENT_TC 11
/*   OGB_OPT_FUSED_UPDATE (0/1, default 1): mixed solves with the block-Jacobi
 *   preconditioner run the vector update and the p update of an iteration as
 *   one cooperative launch (z stays in shared memory; the blocks wait for the
 *   iteration's beta with a bounded wait). Same arithmetic and sum order as the
 *   two-launch form: bitwise equal iterates. */
#define OGB_OPT_FUSED_UPDATE 14
/*   OGB_OPT_BATCH_FORM (0..2, default 0): FP32 SpMV of batched mixed solves:
 *   1 = values loaded among the products, 2 = every value of a group of blocks
 *   loaded before the group's products; 0 = timed once per matrix. Bitwise equal
 *   results. */
#define OGB_OPT_BATCH_FORM 15
/*   OGB_OPT_BATCH_X64 (0/1, default 0): batched mixed solves accumulate the
 *   solution in FP64 every iteration (1) or as an FP32 increment folded into
 *   the FP64 solution after every 16 iterations (0: 24 fewer bytes per row and
 *   no FP64 work per iteration; the same iteration counts on the RVE batch). */
#define OGB_OPT_BATCH_X64 16
OGB_API int ogb_ctx_set_option(ogb_ctx *ctx, int option, int64_t value);
/* Kernel timing: when enabled, SpMV launches (the dominant kernel of the solve)
 * are bracketed by CUDA events on the context stream -- every launch outside CUDA
 * graphs, the ninth of each replayed 16-iteration batch inside them, not the FP64
 * residual products of mixed solves; ogb_ctx_profile_read
 * returns the summed device time (ms), the launch count and the algorithmic
 * bytes of those launches (values + column indices + row pointers + x + y),
 * and resets the counters. No reference counterpart (instrumentation). */
OGB_API int ogb_ctx_profile_enable(ogb_ctx *ctx, int enable);
OGB_API int ogb_ctx_profile_read(ogb_ctx *ctx, double *total_ms, int64_t *launches, double *bytes);

/* ---- sparse matrix: replaces SparseMtrx (src/core/sparsemtrx.h:62-303) ------ */
/* CTOR<SparseMtrx,T> / classFactory.createSparseMtrx (classfactory.h:125,149). */
OGB_API int ogb_mtrx_create(ogb_ctx *ctx, ogb_mtrx **out);
OGB_API int ogb_mtrx_destroy(ogb_mtrx *m);
/* SparseMtrx::buildInternalStructure (sparsemtrx.h:198; CompCol compcol.C:174-272):
 * pattern from element location arrays (1-based, 0 = skip), element e owning
 * loc[loc_ptr[e] .. loc_ptr[e+1]). Host pointers. Values are zeroed. */
OGB_API int ogb_mtrx_build_structure(ogb_mtrx *m, int neq, int nelem, const int64_t *loc_ptr,
                             const int *loc);
OGB_API int ogb_mtrx_neq(ogb_mtrx *m, int *neq);
OGB_API int ogb_mtrx_nnz(ogb_mtrx *m, int64_t *nnz);
/* Copy the pattern out (host buffers of neq+1 and nnz entries). */
OGB_API int ogb_mtrx_pattern(ogb_mtrx *m, int64_t *rowptr, int *colind);
/* Copy the values out (host, nnz doubles, CSR order). */
OGB_API int ogb_mtrx_values(ogb_mtrx *m, double *val);
/* SparseMtrx::zero (sparsemtrx.h:254). */
OGB_API int ogb_mtrx_zero(ogb_mtrx *m);
/* SparseMtrx::assembleBegin (sparsemtrx.h:234). */
OGB_API int ogb_mtrx_assemble_begin(ogb_mtrx *m);
/* SparseMtrx::assemble(loc, mat) (sparsemtrx.h:220; CompCol::assemble compcol.C:275-316):
 * stage one n x n element matrix; `ke_colmajor` is FloatMatrix storage (column-major).
 * Host pointers, copied; applied in call order at ogb_mtrx_assemble_end. */
OGB_API int ogb_mtrx_assemble(ogb_mtrx *m, int n, const int *loc, const double *ke_colmajor);
/* SparseMtrx::assembleEnd (sparsemtrx.h:236; called by EngngModel::assemble,
 * engngm.C:1035-1036): adds every staged element matrix on the device in a fixed
 * order (deterministic, no floating-point atomics). */
OGB_API int ogb_mtrx_assemble_end(ogb_mtrx *m);
/* SparseMtrx::times (sparsemtrx.h:137): y = A x, host vectors of neq. */
OGB_API int ogb_mtrx_times(ogb_mtrx *m, const double *x, double *y);
OGB_API int ogb_mtrx_times_dev(ogb_mtrx *m, const double *x_dev, double *y_dev);
/* SparseMtrx::at(i,j) (sparsemtrx.h:265-267), 1-based; read and scale-in-place
 * (NRSolver::applyConstraintsToStiffness does at(i,i) *= 1e6, nrsolver.C:501-503). */
OGB_API int ogb_mtrx_at(ogb_mtrx *m, int i, int j, double *value);
OGB_API int ogb_mtrx_set_at(ogb_mtrx *m, int i, int j, double value);
/* Preconditioner of the solves on this matrix, numbered as the IML solver's
 * `lsprecond` (IMLSolver::initializeFrom, src/core/iml/imlsolver.C:78-94):
 * 0 = none (VoidPreconditioner, plain CG), 1 = diagonal (DiagPreconditioner,
 * the default here), 2 = ILU by columns (CompCol_ILUPreconditioner,
 * src/core/iml/iluprecond.C), 4 = incomplete Cholesky
 * (CompCol_ICPreconditioner, src/core/iml/icprecond.C). For 2 and 4 the
 * reference's factorization loop runs on the host once per matrix version and
 * the two triangular solves run level by level on the device (FP64 only,
 * equation-space CSR operator). 3 (threshold ILU of a DynCompRow matrix) gives
 * OGB_E_ARG. Batched solves (ogb_batch_*) use the diagonal preconditioner only. */
OGB_API int ogb_mtrx_set_preconditioner(ogb_mtrx *m, int type);
/* Node-block SpMV forms in use for this matrix (0 = not tuned yet, or no
 * node-block copy): the OGB_OPT_SPMV_VARIANT numbers 1..4 chosen for FP64 and
 * FP32 values, and the warps per slice; when the last mixed solve used the
 * half-stored copy (OGB_OPT_SPMV_HALF) fp32_form is 8 + 10 f, f its loop form
 * (OGB_OPT_HALF_FORM). Instrumentation, no reference counterpart. */
OGB_API int ogb_mtrx_spmv_forms(ogb_mtrx *m, int *fp64_form, int *fp32_form, int *warps_per_slice);
/* 1 when the last mixed solve on this matrix preconditioned with the block-Jacobi
 * inverses (OGB_OPT_MIXED_BLOCK_JACOBI), else 0. Instrumentation, no reference
 * counterpart. */
OGB_API int ogb_mtrx_mixed_block_jacobi(ogb_mtrx *m, int *used);
/* SparseMtrx::giveVersion (sparsemtrx.h:82): bumped on every mutation. */
OGB_API int ogb_mtrx_version(ogb_mtrx *m, int64_t *version);

/* ---- linear solver: replaces SparseLinearSystemNM::solve
 *      (src/core/sparselinsystemnm.h:81; IMLSolver::solve imlsolver.C:101-147,
 *      IML++ CG iml/cg.h:22-71, DiagPreconditioner diagpre.C:40-67) --------- */
typedef struct ogb_solve_info {
    int iterations;       /* PCG iterations (sum of inner iterations for MIXED) */
    int outer;            /* iterative-refinement sweeps (MIXED), 0 for FP64 */
    double achieved;      /* final relative residual ||r||/||b|| (FP64 for MIXED) */
    int status;           /* OGB_OK / OGB_E_NOTCONV / OGB_E_BREAKDOWN / OGB_E_ZERODIAG */
} ogb_solve_info;

/* Solve A x = b to ||r||/||b|| <= rtol within maxit iterations; x holds the
 * initial guess on entry (IML CG semantics). Host vectors of neq doubles. */
OGB_API int ogb_pcg_solve(ogb_mtrx *m, const double *b, double *x, double rtol, int maxit,
                  int precision, ogb_solve_info *info);
OGB_API int ogb_pcg_solve_dev(ogb_mtrx *m, const double *b_dev, double *x_dev, double rtol,
                      int maxit, int precision, ogb_solve_info *info);

/* Allocation-free Jacobi-PCG. No counterpart in the reference: it exists for
 * callers that must not allocate device memory while they run (an application
 * that reserves the GPU's memory for its own pool at start-up, or a time-step
 * loop in which cudaMalloc/cudaFree -- cudaFree synchronizes the device -- would
 * stall every stream). The caller passes the CSR matrix (n+1 row pointers,
 * sorted 0-based column indices, values), b and the initial guess x, all in
 * device memory, and the stream to run on (cudaStream_t, 0 = default stream).
 * Same semantics and status codes as ogb_pcg_solve with OGB_PREC_FP64.
 * Limit: n <= 131072 equations (OGB_E_LIMIT beyond). The work vectors live in
 * one file-scope device array of about 5.2 MB that every GPU which loads the
 * library holds until the process exits. All calls share the array: each call
 * clears the parts that must start at zero, and calls that overlap on the GPU
 * race on it. It calls no cudaMalloc, cudaFree or allocating library routine.
 * The call is synchronous -- it reads the solver's scalars from the device
 * after every 16 iterations and returns when the solve has finished -- so it
 * cannot be captured into a CUDA graph. */
OGB_API int ogb_pcg_solve_noalloc(int n, const int64_t *rowptr_dev, const int *colind_dev, const double *val_dev,
                                  const double *b_dev, double *x_dev, double rtol, int maxit, void *stream,
                                  ogb_solve_info *info);

/* ---- direct solver: replaces LDLTFactorization (lstype 0, src/core/ldltfact.C:50-63)
 *      on a Skyline matrix (SparseMtrx::factorized skyline.C:429-491,
 *      backSubstitutionWith skyline.C:248-290) ------------------------------- */
/* Linear solver of every solve on this matrix, numbered as the reference's
 * `lstype` (LinSystSolverType, src/core/linsystsolvertype.h:47-57):
 * OGB_LS_DIRECT (0, ST_Direct) factors the matrix as L D L^T (no pivoting, the
 * upper triangle K(i,j), i <= j, as Skyline::assemble stores it, skyline.C:189-223)
 * once per matrix version and solves by substitution: ogb_pcg_solve*, the Newton
 * and LinearStatic drivers then ignore rtol / maxit / precision and report 0
 * iterations and the FP64 relative residual of the result. OGB_LS_IML (1) and
 * OGB_LS_GPUPCG (9, the default) run the PCG. Batched solves
 * (ogb_batch_*, multi-RHS on model matrices) always run the batched PCG. */
#define OGB_LS_DIRECT 0
#define OGB_LS_IML 1
#define OGB_LS_GPUPCG 9
OGB_API int ogb_mtrx_set_solver(ogb_mtrx *m, int lstype);
/* SparseMtrx::factorized (skyline.C:429-491): factor the current values (the
 * factor is kept until the next mutation). The factor is a dense band of
 * neq x (bw+1) doubles, bw the half bandwidth of the pattern (OGB_E_LIMIT when
 * it does not fit in device memory); OGB_E_ZERODIAG names a zero pivot. */
OGB_API int ogb_ldlt_factorize(ogb_mtrx *m);
/* Half bandwidth of the current factor (OGB_E_STATE before ogb_ldlt_factorize). */
OGB_API int ogb_ldlt_bandwidth(ogb_mtrx *m, int *bandwidth);
/* LDLTFactorization::solve (ldltfact.C:50-63): x = A^-1 b, factoring first when
 * the values changed. Host vectors of neq doubles / device vectors (_dev). */
OGB_API int ogb_ldlt_solve(ogb_mtrx *m, const double *b, double *x);
OGB_API int ogb_ldlt_solve_dev(ogb_mtrx *m, const double *b_dev, double *x_dev);

/* SparseLinearSystemNM::solve(A, B, X) (sparselinsystemnm.h:91, default column
 * loop sparselinsystemnm.C:47-69): nrhs right-hand sides at once. B and X are
 * column-major neq x nrhs (FloatMatrix storage); X holds the initial guesses and
 * receives the solutions. A matrix assembled from a model goes through the
 * batched PCG (four columns per pass, the matrix streamed once for all of them);
 * any other matrix runs the reference's column loop. iterations / achieved /
 * status (optional): nrhs entries. Returns OGB_OK when every column converged,
 * else the first failing column's status. */
OGB_API int ogb_pcg_solve_multi(ogb_mtrx *m, int nrhs, const double *B, double *X, double rtol, int maxit,
                                int precision, int *iterations, double *achieved, int *status);
OGB_API int ogb_pcg_solve_multi_dev(ogb_mtrx *m, int nrhs, const double *B_dev, double *X_dev, double rtol,
                                    int maxit, int precision, int *iterations, double *achieved, int *status);

/* ---- element backend: LSpace / PlaneStress2d / LTRSpace element loops
 *      (NLStructuralElement::computeStiffnessMatrix nlstructuralelement.C:332-446,
 *      ::giveInternalForcesVector :151-240; EngngModel::assemble engngm.C:889-1037,
 *      assembleVectorFromElements :1351-1533) ----------------------------------- */
/* coords: nnodes x ndim; conn: nelem x nnpe (0-based); elem_mat: nelem;
 * mats: nmat x 8; bc_mask: nnodes x ndofpn (1 = prescribed). Host pointers. */
OGB_API int ogb_model_create(ogb_ctx *ctx, int etype, int nnodes, const double *coords, int nelem,
                     const int *conn, const int *elem_mat, int nmat, const double *mats,
                     double thickness, const uint8_t *bc_mask, ogb_model **out);
OGB_API int ogb_model_destroy(ogb_model *md);
OGB_API int ogb_model_neq(ogb_model *md, int *neq, int *npeq);
/* Equation numbers (nnodes x ndofpn, +free / -prescribed), host copy. */
OGB_API int ogb_model_equations(ogb_model *md, int *eq);
/* Build the CSR pattern of this mesh into m and the element-to-CSR scatter map
 * (replaces buildInternalStructure for a mesh whose elements live on the GPU). */
OGB_API int ogb_model_build_matrix(ogb_model *md, ogb_mtrx *m);
/* Tangent stiffness K = sum_e sum_gp B^T D B dV into m (K1 element kernel + K4
 * deterministic gather assembly). Uses the material state of the last stress
 * evaluation (temp values), like TangentAssembler after InternalRhs. */
OGB_API int ogb_model_assemble_stiffness(ogb_model *md, ogb_mtrx *m);
/* The tangent a Newton step of the given precision assembles: OGB_PREC_FP64 as
 * ogb_model_assemble_stiffness; OGB_PREC_MIXED with the element kernel of mixed
 * steps (split-BF16 tensor cores per OGB_OPT_TANGENT_TC, FP32 accuracy). */
OGB_API int ogb_model_assemble_tangent(ogb_model *md, ogb_mtrx *m, int precision);
/* Internal forces f = sum_e sum_gp B^T sigma dV for the total node displacement
 * field u_node (nnodes x ndofpn, prescribed values included); node-indexed
 * output, deterministic. Updates the temp material state. */
OGB_API int ogb_model_internal_forces(ogb_model *md, const double *u_node, double *f_node);
OGB_API int ogb_model_internal_forces_dev(ogb_model *md, const double *u_node_dev, double *f_node_dev);
/* Gauss-point stresses / strains of the last internal-force evaluation
 * (nelem x ngp x nstress), host copy. */
OGB_API int ogb_model_gp_stress(ogb_model *md, double *stress, double *strain);
/* Material state: accept temp values as committed (MaterialStatus::updateYourself). */
OGB_API int ogb_model_commit_state(ogb_model *md);
/* Per-GP state (nelem x ngp x 4): kappa, omega, Le, spare (committed). */
OGB_API int ogb_model_gp_state(ogb_model *md, double *state4);

/* Zero the Newton solution and the material state (a fresh analysis). */
OGB_API int ogb_model_reset_state(ogb_model *md);
/* NonLinearStatic's `initialguess` (engngm.h:207-210, nlinearstatic.C:532-544):
 * 0 = IG_None (default); 1 = IG_Tangent, the step starts from the free-DOF
 * increment K^-1 (-sum_e K_e du_prescribed) that pushes the change of the
 * prescribed values since the last converged step through the tangent of that
 * state (EngngModel::assemblePrescribedExtrapolatedForces, engngm.C:1614-1666). */
OGB_API int ogb_model_set_initial_guess(ogb_model *md, int type);
/* NRSolver's `manrmsteps` (nrsolver.C:120-126 and the re-assembly test at
 * nrsolver.C:285-290): the tangent is always assembled at the start of a step;
 * with manrmsteps = k > 0 (accelerated Newton; k = 1 is full Newton, the
 * default here) it is re-assembled from the current state before the linear
 * solve of every iteration nite > 0 with nite % k == 0; with 0 (modified Newton,
 * the reference's default when the key is absent) the start-of-step tangent
 * serves every iteration of the step. Applies to ogb_nonlinear_step and
 * ogb_batch_nonlinear_step. */
OGB_API int ogb_model_set_nr_mode(ogb_model *md, int manrmsteps);
/* Checkpoint of the analysis state, the device-resident counterpart of the
 * reference's context files (EngngModel::saveStepContext engngm.C:768-777,
 * saveContext / restoreContext engngm.C:1755-1850; each material status's saveContext / restoreContext, e.g.
 * misesmat.C:758-790): the committed Gauss-point state of every element (plastic
 * strain, kappa, damage, Le, crack direction), the Newton solution of the free
 * DOFs, the prescribed values of the last converged step (the IG_Tangent
 * increment starts from them) and the batched Newton solution. A self-describing
 * byte blob: ogb_model_state_bytes gives its size; ogb_model_save_state writes it
 * (call between steps: the temp state is not saved); ogb_model_restore_state
 * loads it into a model of the same mesh and element type (OGB_E_ARG on any
 * mismatch of the header: element type, node, element, Gauss-point, DOF and
 * equation counts). Restoring and continuing gives bit-identical steps. */
OGB_API int ogb_model_state_bytes(ogb_model *md, size_t *bytes);
OGB_API int ogb_model_save_state(ogb_model *md, void *buf, size_t bytes);
OGB_API int ogb_model_restore_state(ogb_model *md, const void *buf, size_t bytes);
/* Bulk read of one block of records of an OOFEM text input deck (host code, no
 * device): `count` records starting at byte `offset`, blank and `#` lines
 * skipped, each `<keyword> <number> ... <field> <n> v1 .. vn ...` (keyword and
 * field matched without regard to case, n <= maxvals). Per record: its number
 * (ids), the n values (vals, maxvals per record), n (nvals), and other[r] = 1
 * when the record carries further fields, which the caller reads with its
 * general parser. *next_offset: byte offset after the block; *lines (optional):
 * lines consumed. Replaces the per-record tokenizer and object instantiation of
 * the dof-manager and element blocks (OOFEMTXTDataReader / OOFEMTXTInputRecord,
 * src/core/oofemtxtdatareader.C, oofemtxtinputrecord.C;
 * Domain::instanciateYourself, src/core/domain.C:485-700). OGB_E_ARG names the
 * first record that does not fit. */
OGB_API int ogb_deck_parse_block(const char *path, int64_t offset, int64_t count, const char *keyword,
                                 const char *field, int maxvals, int64_t *ids, double *vals, int32_t *nvals,
                                 uint8_t *other, int64_t *next_offset, int64_t *lines);
/* Element tangent kernel of the model's last assembly: *tensor_cores = 1 when it
 * was the split-BF16 tensor-core kernel (OGB_OPT_TANGENT_TC), and the device
 * times (ms) of the FP64 and tensor-core kernels measured when the choice was
 * timed (0 before). Instrumentation, no reference counterpart. */
OGB_API int ogb_model_tangent_kernel(ogb_model *md, int *tensor_cores, double *ms_fp64, double *ms_tc);
/* Linear solves of the Newton drivers since the model was created or reset, and
 * their PCG iterations (summed over instances for batched steps). Instrumentation,
 * no reference counterpart. */
OGB_API int ogb_model_solver_stats(ogb_model *md, int64_t *solves, int64_t *iterations);
/* One NonLinearStatic / StaticStructural step with NRSolver
 * (NonLinearStatic::proceedStep nlinearstatic.C:453-565 with controlmode 1,
 * stiffmode 0; StaticStructural::solveYourselfAt staticstructural.C:235-356;
 * NRSolver::solve nrsolver.C:204-402 in the mode set by ogb_model_set_nr_mode,
 * the initial guess set by ogb_model_set_initial_guess; NRSolver::checkConvergence nrsolver.C:593-790 with rtolf and DOF
 * grouping). bc_value / nodal_load: this step's total prescribed values and
 * nodal loads (nnodes x ndofpn). The model keeps the free-DOF solution between
 * steps. The linear systems are solved by PCG to lin_rtol in `precision`. On
 * success the material state is committed (MaterialStatus::updateYourself) and
 * u_node / reactions (optional) receive the converged fields; *iterations is the
 * Newton iteration count of the step. OGB_E_NOTCONV after maxiter iterations
 * (the reference's ConvergenceException), the state then stays uncommitted. */
OGB_API int ogb_nonlinear_step(ogb_model *md, ogb_mtrx *m, const double *bc_value, const double *nodal_load,
                               double rtolf, int maxiter, double lin_rtol, int precision, double *u_node,
                               double *reactions, int *iterations);
OGB_API int ogb_nonlinear_step_dev(ogb_model *md, ogb_mtrx *m, const double *bc_value_dev,
                                   const double *nodal_load_dev, double rtolf, int maxiter, double lin_rtol,
                                   int precision, double *u_node_dev, double *reactions_dev, int *iterations);

/* LinearStatic::solveYourselfAt (linearstatic.C:177-253) in one call: build
 * the pattern (once), assemble K, load = f_ext - f_int(prescribed), PCG, node
 * displacements and reactions (structengngmodel.C:183-201). Host arrays:
 * bc_value/nodal_load/u_node/reactions are nnodes x ndofpn. */
OGB_API int ogb_linear_static(ogb_model *md, ogb_mtrx *m, const double *bc_value,
                      const double *nodal_load, double rtol, int maxit, int precision,
                      double *u_node, double *reactions, ogb_solve_info *info);
/* Same with device-resident inputs/outputs (no host copies). */
OGB_API int ogb_linear_static_dev(ogb_model *md, ogb_mtrx *m, const double *bc_value_dev,
                          const double *nodal_load_dev, double rtol, int maxit,
                          int precision, double *u_node_dev, double *reactions_dev,
                          ogb_solve_info *info);

/* ---- batches: independent meshes and load cases solved together ------------ */
/* Declare the model's mesh to be ninst independent meshes (instances): instance
 * i owns nodes node_start[i] .. node_start[i+1]-1, node_start[0] = 0,
 * node_start[ninst] = nnodes, and every element's nodes lie in one instance
 * (OGB_E_MESH otherwise). Call before the matrix is built; the equation
 * numbering stays that of the concatenated mesh. No reference counterpart: an
 * OOFEM run holds one domain, a batch of runs is a loop of separate runs. */
OGB_API int ogb_model_set_instances(ogb_model *md, int ninst, const int *node_start);
/* LinearStatic for every instance and nrhs load cases (1..4) in one batched
 * Jacobi-PCG: each (instance, load case) pair k = inst * nrhs + c runs its own
 * CG with its own convergence test and stops when it converges. OGB_PREC_FP64:
 * as a separate IMLSolver solve would (iml/cg.h:22-71); OGB_PREC_MIXED: FP32
 * matrix and Krylov vectors, FP64 solution, convergence decided on the FP64
 * residual ||b - K x|| / ||b|| <= rtol (periodic residual replacement).
 * Replaces the loop of
 * SparseLinearSystemNM::solve(A, B, X) (sparselinsystemnm.h:91, the column loop
 * of sparselinsystemnm.C:47-69) and the loop over independent runs.
 * bc_values / loads / u_nodes / reactions: nrhs consecutive nnodes x ndofpn
 * vectors (loads and reactions optional). iterations, achieved (relative
 * residual) and status (OGB_OK / OGB_E_NOTCONV / OGB_E_BREAKDOWN /
 * OGB_E_ZERODIAG): ninst * nrhs entries, optional. Returns OGB_OK when every
 * pair converged, else the first failing pair's status. */
OGB_API int ogb_batch_linear_static(ogb_model *md, ogb_mtrx *m, int nrhs, const double *bc_values,
                                    const double *loads, double rtol, int maxit, int precision,
                                    double *u_nodes, double *reactions, int *iterations, double *achieved,
                                    int *status);
/* Same with device-resident bc_values / loads / u_nodes / reactions. */
OGB_API int ogb_batch_linear_static_dev(ogb_model *md, ogb_mtrx *m, int nrhs, const double *bc_values_dev,
                                        const double *loads_dev, double rtol, int maxit, int precision,
                                        double *u_nodes_dev, double *reactions_dev, int *iterations,
                                        double *achieved, int *status);

/* One NonLinearStatic step of every instance at once (a batch of separate runs,
 * ogb_model_set_instances with each instance's elements contiguous): one
 * internal-force evaluation, one tangent assembly and one batched PCG per Newton
 * iteration for the whole batch, while each instance applies its own NRSolver
 * test (as ogb_nonlinear_step) and stops iterating once it has converged.
 * iterations: ninst entries (Newton iterations of each instance). OGB_OK when
 * every instance converged (state committed); OGB_E_NOTCONV when one reached
 * maxiter (state left uncommitted). No reference counterpart beyond the
 * per-instance NRSolver::solve it repeats. */
OGB_API int ogb_batch_nonlinear_step(ogb_model *md, ogb_mtrx *m, const double *bc_value, const double *nodal_load,
                                     double rtolf, int maxiter, double lin_rtol, int precision, double *u_node,
                                     double *reactions, int *iterations);
OGB_API int ogb_batch_nonlinear_step_dev(ogb_model *md, ogb_mtrx *m, const double *bc_value_dev,
                                         const double *nodal_load_dev, double rtolf, int maxiter,
                                         double lin_rtol, int precision, double *u_node_dev,
                                         double *reactions_dev, int *iterations);

#ifdef __cplusplus
}
#endif
#endif
