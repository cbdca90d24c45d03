"""ctypes binding of liboofem_gb300.so (include/oofem_gb300.h) and a thin
Python mirror of the reference interfaces it replaces:

* :class:`GpuCsrMtrx`   -- ``SparseMtrx`` (src/core/sparsemtrx.h:62-303)
* :class:`GpuPcgSolver` -- ``SparseLinearSystemNM`` / ``IMLSolver``
  (src/core/sparselinsystemnm.h:58-96, src/core/iml/imlsolver.C:101-147)
* :class:`GpuModel`     -- the element loops of ``EngngModel::assemble`` /
  ``assembleVectorFromElements`` for LSpace / PlaneStress2d / LTRSpace

There is no CPU fallback: loading raises if the CUDA library is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboofem_gb300.so")

OGB_OK = 0
ERRORS = {-1: "OGB_E_ARG", -2: "OGB_E_CUDA", -3: "OGB_E_STATE", -4: "OGB_E_PATTERN",
          -5: "OGB_E_NOTCONV", -6: "OGB_E_BREAKDOWN", -7: "OGB_E_ZERODIAG", -8: "OGB_E_MESH",
          -9: "OGB_E_LIMIT"}
PREC_FP64 = 0
PREC_MIXED = 1
OPT_MIXED_VEC32 = 1
OPT_MIXED_DIFF = 2
OPT_MIXED_ORTH = 3
OPT_MIXED_DROP_PPM = 4
OPT_MIXED_P32 = 5
OPT_MIXED_X64 = 6
OPT_SPMV_VARIANT = 7
OPT_SPMV_HALF = 8
OPT_MIXED_BLOCK_JACOBI = 9
OPT_HALF_FORM = 12
OPT_UPDATE_BLOCKS = 13
OPT_TANGENT_TC = 11
OPT_FUSED_UPDATE = 14
OPT_BATCH_FORM = 15
OPT_BATCH_X64 = 16
# linear solver types (the reference's lstype numbers)
LS_DIRECT = 0
LS_IML = 1
LS_GPUPCG = 9
# solver outcomes returned (not raised), like SparseLinearSystemNM::solve's ConvergedReason
SOLVER_STATUS = (0, -5, -6, -7)

# Every entry point of include/oofem_gb300.h: name -> (restype, argtypes)
_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_i64 = C.c_int64
_pi64 = C.POINTER(C.c_int64)
_pi = C.POINTER(C.c_int)
_pd = C.POINTER(C.c_double)


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer", C.c_int), ("achieved", C.c_double),
                ("status", C.c_int)]


SIGNATURES = {
    "ogb_last_error": (C.c_char_p, []),
    "ogb_version": (_i, []),
    "ogb_ctx_create": (_i, [_i, C.POINTER(_vp)]),
    "ogb_ctx_destroy": (_i, [_vp]),
    "ogb_ctx_stream": (_vp, [_vp]),
    "ogb_ctx_synchronize": (_i, [_vp]),
    "ogb_ctx_kernel_launches": (_i64, [_vp]),
    "ogb_ctx_set_option": (_i, [_vp, _i, _i64]),
    "ogb_ctx_profile_enable": (_i, [_vp, _i]),
    "ogb_ctx_profile_read": (_i, [_vp, _pd, _pi64, _pd]),
    "ogb_mtrx_create": (_i, [_vp, C.POINTER(_vp)]),
    "ogb_mtrx_destroy": (_i, [_vp]),
    "ogb_mtrx_build_structure": (_i, [_vp, _i, _i, _vp, _vp]),
    "ogb_mtrx_neq": (_i, [_vp, _pi]),
    "ogb_mtrx_nnz": (_i, [_vp, _pi64]),
    "ogb_mtrx_pattern": (_i, [_vp, _vp, _vp]),
    "ogb_mtrx_values": (_i, [_vp, _vp]),
    "ogb_mtrx_zero": (_i, [_vp]),
    "ogb_mtrx_assemble_begin": (_i, [_vp]),
    "ogb_mtrx_assemble": (_i, [_vp, _i, _vp, _vp]),
    "ogb_mtrx_assemble_end": (_i, [_vp]),
    "ogb_mtrx_times": (_i, [_vp, _vp, _vp]),
    "ogb_mtrx_times_dev": (_i, [_vp, _vp, _vp]),
    "ogb_mtrx_at": (_i, [_vp, _i, _i, _pd]),
    "ogb_mtrx_set_at": (_i, [_vp, _i, _i, _d]),
    "ogb_mtrx_version": (_i, [_vp, _pi64]),
    "ogb_pcg_solve": (_i, [_vp, _vp, _vp, _d, _i, _i, C.POINTER(SolveInfo)]),
    "ogb_pcg_solve_dev": (_i, [_vp, _vp, _vp, _d, _i, _i, C.POINTER(SolveInfo)]),
    "ogb_pcg_solve_noalloc": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _d, _i, _vp, C.POINTER(SolveInfo)]),
    "ogb_model_create": (_i, [_vp, _i, _i, _vp, _i, _vp, _vp, _i, _vp, _d, _vp, C.POINTER(_vp)]),
    "ogb_model_destroy": (_i, [_vp]),
    "ogb_model_neq": (_i, [_vp, _pi, _pi]),
    "ogb_model_equations": (_i, [_vp, _vp]),
    "ogb_model_build_matrix": (_i, [_vp, _vp]),
    "ogb_model_assemble_stiffness": (_i, [_vp, _vp]),
    "ogb_model_assemble_tangent": (_i, [_vp, _vp, _i]),
    "ogb_model_internal_forces": (_i, [_vp, _vp, _vp]),
    "ogb_model_internal_forces_dev": (_i, [_vp, _vp, _vp]),
    "ogb_model_gp_stress": (_i, [_vp, _vp, _vp]),
    "ogb_model_commit_state": (_i, [_vp]),
    "ogb_model_gp_state": (_i, [_vp, _vp]),
    "ogb_model_reset_state": (_i, [_vp]),
    "ogb_model_set_initial_guess": (_i, [_vp, _i]),
    "ogb_model_set_nr_mode": (_i, [_vp, _i]),
    "ogb_mtrx_set_preconditioner": (_i, [_vp, _i]),
    "ogb_mtrx_set_solver": (_i, [_vp, _i]),
    "ogb_mtrx_mixed_block_jacobi": (_i, [_vp, _pi]),
    "ogb_ldlt_factorize": (_i, [_vp]),
    "ogb_ldlt_bandwidth": (_i, [_vp, _pi]),
    "ogb_ldlt_solve": (_i, [_vp, _vp, _vp]),
    "ogb_ldlt_solve_dev": (_i, [_vp, _vp, _vp]),
    "ogb_deck_parse_block": (_i, [C.c_char_p, C.c_int64, C.c_int64, C.c_char_p, C.c_char_p, _i, _vp, _vp, _vp, _vp,
                                  C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ogb_model_state_bytes": (_i, [_vp, C.POINTER(C.c_size_t)]),
    "ogb_model_save_state": (_i, [_vp, _vp, C.c_size_t]),
    "ogb_model_restore_state": (_i, [_vp, _vp, C.c_size_t]),
    "ogb_model_solver_stats": (_i, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ogb_model_tangent_kernel": (_i, [_vp, _pi, _pd, _pd]),
    "ogb_batch_nonlinear_step": (_i, [_vp, _vp, _vp, _vp, _d, _i, _d, _i, _vp, _vp, _vp]),
    "ogb_batch_nonlinear_step_dev": (_i, [_vp, _vp, _vp, _vp, _d, _i, _d, _i, _vp, _vp, _vp]),
    "ogb_nonlinear_step": (_i, [_vp, _vp, _vp, _vp, _d, _i, _d, _i, _vp, _vp, C.POINTER(C.c_int)]),
    "ogb_nonlinear_step_dev": (_i, [_vp, _vp, _vp, _vp, _d, _i, _d, _i, _vp, _vp, C.POINTER(C.c_int)]),
    "ogb_linear_static": (_i, [_vp, _vp, _vp, _vp, _d, _i, _i, _vp, _vp, C.POINTER(SolveInfo)]),
    "ogb_linear_static_dev": (_i, [_vp, _vp, _vp, _vp, _d, _i, _i, _vp, _vp, C.POINTER(SolveInfo)]),
    "ogb_model_set_instances": (_i, [_vp, _i, _vp]),
    "ogb_mtrx_spmv_forms": (_i, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ogb_pcg_solve_multi": (_i, [_vp, _i, _vp, _vp, _d, _i, _i, _vp, _vp, _vp]),
    "ogb_pcg_solve_multi_dev": (_i, [_vp, _i, _vp, _vp, _d, _i, _i, _vp, _vp, _vp]),
    "ogb_batch_linear_static": (_i, [_vp, _vp, _i, _vp, _vp, _d, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "ogb_batch_linear_static_dev": (_i, [_vp, _vp, _i, _vp, _vp, _d, _i, _i, _vp, _vp, _vp, _vp, _vp]),
}

_lib = None


class OgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the CUDA library (fails loudly when it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing; run __graft_entry__.build() (no CPU fallback)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _check(code: int):
    if code != OGB_OK:
        raise OgbError(code, load().ogb_last_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _dptr(t) -> C.c_void_p:
    """Device pointer of a torch tensor."""
    return C.c_void_p(t.data_ptr())


class Context:
    """Device + stream (ogb_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        _check(self.lib.ogb_ctx_create(device, C.byref(h)))
        self.h = h

    @property
    def stream(self) -> int:
        return self.lib.ogb_ctx_stream(self.h)

    def synchronize(self):
        _check(self.lib.ogb_ctx_synchronize(self.h))

    def kernel_launches(self) -> int:
        return self.lib.ogb_ctx_kernel_launches(self.h)

    def set_option(self, option: int, value: int):
        _check(self.lib.ogb_ctx_set_option(self.h, option, value))

    def profile(self, enable: bool):
        _check(self.lib.ogb_ctx_profile_enable(self.h, int(enable)))

    def profile_read(self):
        ms, n, by = C.c_double(), C.c_int64(), C.c_double()
        _check(self.lib.ogb_ctx_profile_read(self.h, C.byref(ms), C.byref(n), C.byref(by)))
        return ms.value, n.value, by.value

    def close(self):
        if self.h:
            self.lib.ogb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuCsrMtrx:
    """SparseMtrx on the GPU: full-pattern CSR (== CompCol colptr/rowind)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        _check(self.lib.ogb_mtrx_create(ctx.h, C.byref(h)))
        self.h = h

    # SparseMtrx::buildInternalStructure from element location arrays
    def build_internal_structure(self, neq: int, locs) -> None:
        if isinstance(locs, np.ndarray) and locs.ndim == 2:
            loc = np.ascontiguousarray(locs, dtype=np.int32).ravel()
            ptr = np.arange(locs.shape[0] + 1, dtype=np.int64) * locs.shape[1]
            ne = locs.shape[0]
        else:
            arrs = [np.asarray(l, dtype=np.int32) for l in locs]
            ptr = np.zeros(len(arrs) + 1, np.int64)
            ptr[1:] = np.cumsum([a.size for a in arrs])
            loc = np.concatenate(arrs) if arrs else np.zeros(0, np.int32)
            ne = len(arrs)
        _check(self.lib.ogb_mtrx_build_structure(self.h, neq, ne, _ptr(ptr), _ptr(loc)))

    @property
    def neq(self) -> int:
        v = C.c_int()
        _check(self.lib.ogb_mtrx_neq(self.h, C.byref(v)))
        return v.value

    @property
    def nnz(self) -> int:
        v = C.c_int64()
        _check(self.lib.ogb_mtrx_nnz(self.h, C.byref(v)))
        return v.value

    def pattern(self):
        n, nz = self.neq, self.nnz
        rp = np.zeros(n + 1, np.int64)
        ci = np.zeros(max(nz, 1), np.int32)
        _check(self.lib.ogb_mtrx_pattern(self.h, _ptr(rp), _ptr(ci)))
        return rp, ci[:nz]

    def values(self) -> np.ndarray:
        v = np.zeros(max(self.nnz, 1))
        _check(self.lib.ogb_mtrx_values(self.h, _ptr(v)))
        return v[:self.nnz]

    def zero(self):
        _check(self.lib.ogb_mtrx_zero(self.h))

    def set_preconditioner(self, lsprecond: int):
        """IML lsprecond: 0 none, 1 diagonal (default), 4 incomplete Cholesky (FP64)."""
        _check(self.lib.ogb_mtrx_set_preconditioner(self.h, int(lsprecond)))

    def set_solver(self, lstype: int):
        """Linear solver of every solve on this matrix, as the reference's lstype:
        0 direct LDL^T (LDLTFactorization on a Skyline matrix), 1 / 9 PCG."""
        _check(self.lib.ogb_mtrx_set_solver(self.h, int(lstype)))

    def factorized(self):
        """SparseMtrx::factorized: factor the current values (L D L^T)."""
        _check(self.lib.ogb_ldlt_factorize(self.h))
        return self

    @property
    def bandwidth(self) -> int:
        v = C.c_int()
        _check(self.lib.ogb_ldlt_bandwidth(self.h, C.byref(v)))
        return v.value

    def ldlt_solve(self, b: np.ndarray) -> np.ndarray:
        """LDLTFactorization::solve: x = A^-1 b (factors first when the values changed)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.neq)
        _check(self.lib.ogb_ldlt_solve(self.h, _ptr(b), _ptr(x)))
        return x

    def last_block_jacobi(self) -> bool:
        """Whether the last mixed solve on this matrix used the block-Jacobi preconditioner."""
        v = C.c_int()
        _check(self.lib.ogb_mtrx_mixed_block_jacobi(self.h, C.byref(v)))
        return bool(v.value)

    def spmv_forms(self):
        """(FP64 form, FP32 form, warps per slice) of the node-block SpMV."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _check(self.lib.ogb_mtrx_spmv_forms(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def assemble_begin(self):
        _check(self.lib.ogb_mtrx_assemble_begin(self.h))

    def assemble(self, loc, mat: np.ndarray) -> int:
        """SparseMtrx::assemble(loc, mat); mat is the element matrix (any
        layout in numpy, passed column-major like FloatMatrix)."""
        loc = np.ascontiguousarray(loc, dtype=np.int32)
        km = np.asfortranarray(mat, dtype=np.float64)
        _check(self.lib.ogb_mtrx_assemble(self.h, loc.size, _ptr(loc),
                                          km.ctypes.data_as(C.c_void_p)))
        return 1

    def assemble_end(self):
        _check(self.lib.ogb_mtrx_assemble_end(self.h))

    def times(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.neq)
        _check(self.lib.ogb_mtrx_times(self.h, _ptr(x), _ptr(y)))
        return y

    def at(self, i: int, j: int) -> float:
        v = C.c_double()
        _check(self.lib.ogb_mtrx_at(self.h, i, j, C.byref(v)))
        return v.value

    def set_at(self, i: int, j: int, value: float):
        _check(self.lib.ogb_mtrx_set_at(self.h, i, j, float(value)))

    @property
    def version(self) -> int:
        v = C.c_int64()
        _check(self.lib.ogb_mtrx_version(self.h, C.byref(v)))
        return v.value

    def close(self):
        if self.h:
            self.lib.ogb_mtrx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuPcgSolver:
    """SparseLinearSystemNM::solve with IML CG + Jacobi semantics
    (lstol / lsiter as in IMLSolver::initializeFrom, imlsolver.C:66-98)."""

    def __init__(self, lstol: float = 1e-5, lsiter: int = 200, precision: int = PREC_FP64, lsprecond: int = 1):
        self.tol = lstol
        self.maxit = lsiter
        self.precision = precision
        self.lsprecond = lsprecond
        self.last = SolveInfo()

    def solve(self, A: GpuCsrMtrx, b: np.ndarray, x: np.ndarray) -> int:
        A.set_preconditioner(self.lsprecond)
        b = np.ascontiguousarray(b, dtype=np.float64)
        assert x.dtype == np.float64 and x.flags.c_contiguous
        info = SolveInfo()
        code = A.lib.ogb_pcg_solve(A.h, _ptr(b), _ptr(x), self.tol, self.maxit, self.precision,
                                   C.byref(info))
        self.last = info
        if code not in SOLVER_STATUS:
            _check(code)
        return code

    def solve_multi(self, A: GpuCsrMtrx, B: np.ndarray, X: np.ndarray) -> int:
        """solve(A, B, X) for a block of right-hand sides: B and X are (nrhs, neq)
        arrays (row c = column c of the reference's FloatMatrix); X holds the
        initial guesses and receives the solutions. Per-column iterations,
        achieved residuals and statuses are kept in self.last_multi."""
        A.set_preconditioner(self.lsprecond)
        B = np.ascontiguousarray(B, dtype=np.float64)
        assert X.dtype == np.float64 and X.flags.c_contiguous and X.shape == B.shape
        nrhs = B.shape[0]
        its = np.zeros(nrhs, np.int32)
        ach = np.zeros(nrhs)
        st = np.zeros(nrhs, np.int32)
        code = A.lib.ogb_pcg_solve_multi(A.h, nrhs, _ptr(B), _ptr(X), self.tol, self.maxit, self.precision,
                                         _ptr(its), _ptr(ach), _ptr(st))
        self.last_multi = (its, ach, st)
        if code not in SOLVER_STATUS:
            _check(code)
        return code


class GpuLdltSolver:
    """LDLTFactorization (src/core/ldltfact.C:50-63), the reference's default
    solver (lstype 0): factor the matrix once per version as L D L^T on the
    device, then solve by substitution. Returns 0 (CR_CONVERGED) or the status
    of a zero pivot."""

    def solve(self, A: GpuCsrMtrx, b: np.ndarray, x: np.ndarray) -> int:
        b = np.ascontiguousarray(b, dtype=np.float64)
        assert x.dtype == np.float64 and x.flags.c_contiguous
        code = A.lib.ogb_ldlt_solve(A.h, _ptr(b), _ptr(x))
        if code not in SOLVER_STATUS:
            _check(code)
        return code


class GpuModel:
    """Element backend for one mesh (one element type)."""

    def __init__(self, ctx: Context, mesh):
        self.ctx = ctx
        self.lib = ctx.lib
        self.mesh = mesh
        self._coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        self._conn = np.ascontiguousarray(mesh.conn, dtype=np.int32)
        self._emat = np.ascontiguousarray(mesh.elem_mat, dtype=np.int32)
        self._mats = np.ascontiguousarray(mesh.material_table(), dtype=np.float64)
        self._bcm = np.ascontiguousarray(mesh.bc_mask, dtype=np.uint8)
        h = C.c_void_p()
        _check(self.lib.ogb_model_create(ctx.h, mesh.elem_type, mesh.nnodes, _ptr(self._coords),
                                         mesh.nelem, _ptr(self._conn), _ptr(self._emat),
                                         self._mats.shape[0], _ptr(self._mats), float(mesh.thickness),
                                         _ptr(self._bcm), C.byref(h)))
        self.h = h

    def neq(self):
        a, b = C.c_int(), C.c_int()
        _check(self.lib.ogb_model_neq(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def equations(self) -> np.ndarray:
        eq = np.zeros((self.mesh.nnodes, self.mesh.ndofpn), np.int32)
        _check(self.lib.ogb_model_equations(self.h, _ptr(eq)))
        return eq

    def build_matrix(self, A: GpuCsrMtrx):
        _check(self.lib.ogb_model_build_matrix(self.h, A.h))

    def assemble_tangent(self, A: GpuCsrMtrx, precision: int = PREC_FP64):
        """The tangent a Newton step of this precision assembles (mixed: tensor-core element kernel)."""
        _check(self.lib.ogb_model_assemble_tangent(self.h, A.h, int(precision)))

    def assemble_stiffness(self, A: GpuCsrMtrx):
        _check(self.lib.ogb_model_assemble_stiffness(self.h, A.h))

    def internal_forces(self, u_node: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u_node, dtype=np.float64)
        f = np.zeros_like(u)
        _check(self.lib.ogb_model_internal_forces(self.h, _ptr(u), _ptr(f)))
        return f

    def gp_stress(self):
        m = self.mesh
        ngp = {1: 8, 2: 4, 3: 1}[m.elem_type]
        ns = 3 if m.elem_type == 2 else 6
        s = np.zeros((m.nelem, ngp, ns))
        e = np.zeros_like(s)
        _check(self.lib.ogb_model_gp_stress(self.h, _ptr(s), _ptr(e)))
        return s, e

    def gp_state(self):
        m = self.mesh
        ngp = {1: 8, 2: 4, 3: 1}[m.elem_type]
        s = np.zeros((m.nelem, ngp, 4))
        _check(self.lib.ogb_model_gp_state(self.h, _ptr(s)))
        return s

    def commit_state(self):
        _check(self.lib.ogb_model_commit_state(self.h))

    def linear_static(self, A: GpuCsrMtrx, bc_value=None, nodal_load=None, rtol=1e-12,
                      maxit=100000, precision=PREC_FP64, want_reactions=True, out=None):
        """out: optional (u, reactions) float64 arrays of the mesh's (nnodes, ndofpn)
        shape to receive the results (e.g. page-locked host buffers)."""
        m = self.mesh
        bcv = np.ascontiguousarray(m.bc_value if bc_value is None else bc_value, dtype=np.float64)
        ld = np.ascontiguousarray(m.nodal_load if nodal_load is None else nodal_load, dtype=np.float64)
        if out is not None:
            u, reac = out
            for a in (u, reac):
                if a is not None and (a.shape != bcv.shape or a.dtype != np.float64 or not a.flags.c_contiguous):
                    raise ValueError("out arrays must be C-contiguous float64 of shape %s" % (bcv.shape,))
            if not want_reactions:
                reac = None
        else:
            u = np.zeros_like(bcv)
            reac = np.zeros_like(bcv) if want_reactions else None
        info = SolveInfo()
        code = self.lib.ogb_linear_static(self.h, A.h, _ptr(bcv), _ptr(ld), rtol, maxit, precision,
                                          _ptr(u), _ptr(reac) if reac is not None else None,
                                          C.byref(info))
        if code not in SOLVER_STATUS:
            _check(code)
        return u, reac, info

    def set_instances(self, node_start):
        """Declare the mesh as independent instances (node ranges); before build_matrix."""
        ns = np.ascontiguousarray(node_start, dtype=np.int32)
        self._ninst = len(ns) - 1
        _check(self.lib.ogb_model_set_instances(self.h, self._ninst, _ptr(ns)))

    def batch_linear_static(self, A: GpuCsrMtrx, bc_values, loads=None, rtol=1e-12, maxit=100000,
                            want_reactions=True, precision=PREC_FP64):
        """LinearStatic of every instance and load case in one batched PCG.

        bc_values / loads: (nrhs, nnodes, ndofpn). Returns (u, reactions, iterations,
        achieved, status) with per-pair arrays of shape (ninst, nrhs)."""
        bcv = np.ascontiguousarray(bc_values, dtype=np.float64)
        nrhs = bcv.shape[0]
        ld = None if loads is None else np.ascontiguousarray(loads, dtype=np.float64)
        ninst = getattr(self, "_ninst", 1)
        u = np.zeros_like(bcv)
        reac = np.zeros_like(bcv) if want_reactions else None
        its = np.zeros((ninst, nrhs), np.int32)
        ach = np.zeros((ninst, nrhs))
        st = np.zeros((ninst, nrhs), np.int32)
        code = self.lib.ogb_batch_linear_static(self.h, A.h, nrhs, _ptr(bcv), _ptr(ld) if ld is not None else None,
                                                rtol, maxit, precision, _ptr(u),
                                                _ptr(reac) if reac is not None else None,
                                                _ptr(its), _ptr(ach), _ptr(st))
        if code not in SOLVER_STATUS:
            _check(code)
        return u, reac, its, ach, st

    def reset_state(self):
        _check(self.lib.ogb_model_reset_state(self.h))

    def solver_stats(self):
        """(linear solves, PCG iterations) of the Newton drivers since creation / reset."""
        a, b = C.c_int64(), C.c_int64()
        _check(self.lib.ogb_model_solver_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_initial_guess(self, kind: int):
        """NonLinearStatic initialguess: 0 IG_None, 1 IG_Tangent."""
        _check(self.lib.ogb_model_set_initial_guess(self.h, int(kind)))

    def save_state(self) -> bytes:
        """Checkpoint of the committed analysis state (GP state, Newton solution,
        last prescribed values) as bytes; restore_state loads it."""
        n = C.c_size_t()
        _check(self.lib.ogb_model_state_bytes(self.h, C.byref(n)))
        buf = (C.c_char * n.value)()
        _check(self.lib.ogb_model_save_state(self.h, buf, n.value))
        return bytes(buf)

    def restore_state(self, blob: bytes):
        buf = C.create_string_buffer(blob, len(blob))
        _check(self.lib.ogb_model_restore_state(self.h, buf, len(blob)))

    # layout of the checkpoint header (StateHeader in csrc/capi.cu): magic, format, etype,
    # nnodes, nelem, ngp, ndofpn, neq, nstate (int32), state_len, nrb_len (int64)
    _STATE_HEADER = struct.Struct("<8s8i2q")

    def committed_state(self) -> np.ndarray:
        """Committed Gauss-point state (nelem, ngp, nstate) as it stands in the
        checkpoint: MisesMat [0..5] plastic strain, [6] kappa; IDM1 [0] kappa,
        [1] damage, [2] crack band length Le (MaterialStatus::saveContext per point)."""
        blob = self.save_state()
        h = self._STATE_HEADER.unpack_from(blob, 0)
        ngp, nstate, state_len = h[5], h[8], h[9]
        st = np.frombuffer(blob, dtype=np.float64, count=state_len, offset=self._STATE_HEADER.size)
        return st.reshape(-1, ngp, nstate).copy() if state_len else np.zeros((0, ngp, nstate))

    def load_committed_state(self, state: np.ndarray):
        """Replace the committed Gauss-point state (same layout as committed_state)
        through the checkpoint path (MaterialStatus::restoreContext per point)."""
        blob = bytearray(self.save_state())
        h = self._STATE_HEADER.unpack_from(blob, 0)
        state_len = h[9]
        st = np.ascontiguousarray(state, dtype=np.float64).ravel()
        if st.size != state_len:
            raise ValueError(f"state has {st.size} values, the model {state_len}")
        off = self._STATE_HEADER.size
        blob[off:off + 8 * state_len] = st.tobytes()
        self.restore_state(bytes(blob))

    def tangent_kernel(self):
        """(tensor cores used by the last tangent assembly, timed FP64 ms, timed tensor-core ms)."""
        k, a, b = C.c_int(), C.c_double(), C.c_double()
        _check(self.lib.ogb_model_tangent_kernel(self.h, C.byref(k), C.byref(a), C.byref(b)))
        return bool(k.value), a.value, b.value

    def set_nr_mode(self, manrmsteps: int):
        """NRSolver manrmsteps: 0 modified Newton, k > 0 re-assembles the tangent
        every k-th iteration (1 = full Newton, the default)."""
        _check(self.lib.ogb_model_set_nr_mode(self.h, int(manrmsteps)))

    def nonlinear_step(self, A: GpuCsrMtrx, bc_value, nodal_load=None, rtolf=1e-8, maxiter=50,
                       lin_rtol=1e-12, precision=PREC_FP64):
        """One NonLinearStatic/NRSolver step; returns (u_node, reactions, newton_iterations)."""
        bcv = np.ascontiguousarray(bc_value, dtype=np.float64)
        ld = None if nodal_load is None else np.ascontiguousarray(nodal_load, dtype=np.float64)
        u = np.zeros_like(bcv)
        reac = np.zeros_like(bcv)
        it = C.c_int(0)
        code = self.lib.ogb_nonlinear_step(self.h, A.h, _ptr(bcv), _ptr(ld) if ld is not None else None,
                                           rtolf, maxiter, lin_rtol, precision, _ptr(u), _ptr(reac),
                                           C.byref(it))
        _check(code)
        return u, reac, it.value

    def batch_nonlinear_step(self, A: GpuCsrMtrx, bc_value, nodal_load=None, rtolf=1e-8, maxiter=50,
                             lin_rtol=1e-12, precision=PREC_FP64):
        """One NonLinearStatic step of every instance; returns (u_node, reactions,
        newton_iterations per instance)."""
        bcv = np.ascontiguousarray(bc_value, dtype=np.float64)
        ld = None if nodal_load is None else np.ascontiguousarray(nodal_load, dtype=np.float64)
        u = np.zeros_like(bcv)
        reac = np.zeros_like(bcv)
        its = np.zeros(getattr(self, "_ninst", 1), np.int32)
        code = self.lib.ogb_batch_nonlinear_step(self.h, A.h, _ptr(bcv), _ptr(ld) if ld is not None else None,
                                                 rtolf, maxiter, lin_rtol, precision, _ptr(u), _ptr(reac),
                                                 _ptr(its))
        _check(code)
        return u, reac, its

    def close(self):
        if self.h:
            self.lib.ogb_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
