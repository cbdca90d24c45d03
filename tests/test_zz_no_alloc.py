"""The allocation-free Jacobi-PCG entry point (ogb_pcg_solve_noalloc).

It serves callers that may not allocate device memory while they run, such as
an application that has reserved the GPU's memory for its own pool, or a
time-step loop where a cudaMalloc/cudaFree (cudaFree synchronizes the device)
would stall its streams. Here the caller's matrix, right-hand side and
solution live in device memory the test allocates up front; the entry point
itself only uses its fixed file-scope work array. Its answer is checked
against the allocating entry point (ogb_pcg_solve) on the same system, on two
calls in a row, with the tolerance of the other PCG parity tests.

Kept in a file of its own, collected last."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _system(oracle):
    g = load_golden("hex_cantilever_20x4x4")
    neq, _, eq = oracle.number_equations(g["bc_mask"])
    loc = oracle.location_arrays(g["conn"], eq)
    rp, ci = oracle.build_pattern(neq, loc)
    val = oracle.assemble_tangent(g, loc, neq, rp, ci)
    b = np.random.default_rng(7).standard_normal(neq)
    return g, neq, loc, rp, ci, val, b


def _vp(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_solve_matches_allocating_solve(native_lib, oracle):
    torch = pytest.importorskip("torch")
    g, neq, loc, rp, ci, val, b = _system(oracle)
    lib = native_lib.load()

    # the existing, allocating entry point on the same CSR system
    ctx = native_lib.Context(0)
    A = native_lib.GpuCsrMtrx(ctx)
    A.build_internal_structure(neq, loc)
    A.assemble_begin()
    D = oracle.isole_d(1, g["mats"][0][1], g["mats"][0][2])
    for e in range(loc.shape[0]):
        A.assemble(loc[e], oracle.elem_stiffness(1, g["coords"][g["conn"][e]], D))
    A.assemble_end()
    assert np.array_equal(A.values(), val)
    x_ref = np.zeros(neq)
    info_ref = native_lib.SolveInfo()
    code = lib.ogb_pcg_solve(A.h, b.ctypes.data_as(C.c_void_p), x_ref.ctypes.data_as(C.c_void_p), RTOL, 100000,
                             native_lib.PREC_FP64, C.byref(info_ref))
    assert code == 0

    # the allocation-free entry point: the caller owns every device buffer
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(rp).to(dev)
    d_ci = torch.from_numpy(ci).to(dev)
    d_val = torch.from_numpy(val).to(dev)
    d_b = torch.from_numpy(b).to(dev)
    for call in range(2):
        d_x = torch.zeros(neq, dtype=torch.float64, device=dev)
        info = native_lib.SolveInfo()
        torch.cuda.synchronize()
        code = lib.ogb_pcg_solve_noalloc(neq, _vp(d_rp), _vp(d_ci), _vp(d_val), _vp(d_b), _vp(d_x), RTOL, 100000,
                                         None, C.byref(info))
        assert code == 0, lib.ogb_last_error()
        x = d_x.cpu().numpy()
        assert info.status == 0 and info.achieved <= RTOL
        assert abs(info.iterations - info_ref.iterations) <= 2
        assert np.abs(x - x_ref).max() / np.abs(x_ref).max() < 1e-9, call


def test_noalloc_rejects_oversized_systems(native_lib):
    lib = native_lib.load()
    info = native_lib.SolveInfo()
    dummy = C.c_void_p(16)
    code = lib.ogb_pcg_solve_noalloc(1 << 20, dummy, dummy, dummy, dummy, dummy, 1e-8, 10, None, C.byref(info))
    assert code == -9
    assert b"maximum" in lib.ogb_last_error()
