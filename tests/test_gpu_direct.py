"""GPU direct solver (lstype 0: the reference's LDLTFactorization on a Skyline
matrix, src/core/ldltfact.C:50-63, skyline.C:248-290, 429-491) against the
reference's own runs, which used that solver (tests/golden/*.npz, written by the
reference executable).

Bars: with the same kind of solver on both sides the solve adds only rounding,
so LinearStatic displacements, reactions, GP stresses and strains agree within
1e-10 relative (to the field's maximum); NonLinearStatic / StaticStructural
Newton runs take exactly the reference's iteration count in every step and
their displacements, reactions, GP stresses, kappa, damage and crack band
lengths agree within 1e-10 relative."""
import numpy as np
import pytest

from conftest import LINEAR_CASES, load_golden
from test_gpu_linear import mesh_from_golden, rel

pytestmark = pytest.mark.gpu

TOL = 1e-10
NONLINEAR_CASES = ["mises_hex_4x2x2", "mises_hex_6x3x3", "mises_hex_10x3x3_ig", "idm1_tet_3"]
SS_CASES = ["ss_mises_hex_6x3x3", "ss_mises_hex_5x2x2_accel", "ss_idm1_tet_3"]


@pytest.fixture(scope="module")
def ctx(native_lib):
    return native_lib.Context(0)


def dense(g):
    cp, ri, v = g["K_colptr"], g["K_rowind"], g["K_val"]
    n = len(cp) - 1
    K = np.zeros((n, n))
    for c in range(n):
        K[ri[cp[c]:cp[c + 1]], c] = v[cp[c]:cp[c + 1]]
    return K


@pytest.mark.parametrize("case", ["hex_cantilever_20x4x4", "tet_cube_3_jit", "quad_rve_8_s3_lc0"])
def test_ldlt_solve_matches_dense_solve(case, ctx, native_lib):
    """x = A^-1 b through the drop-in matrix (location arrays, host element
    matrices) against a dense LU solve of the reference's assembled matrix."""
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    model.assemble_stiffness(A)
    assert rel(A.values(), g["K_val"]) < 1e-12
    K = dense(g)
    b = np.random.default_rng(3).standard_normal(K.shape[0])
    x = np.zeros_like(b)
    assert native_lib.GpuLdltSolver().solve(A, b, x) == 0
    xr = np.linalg.solve(K, b)
    assert rel(x, xr) < 1e-11, rel(x, xr)
    # the factor is kept while the values do not change: same result bit for bit
    bw = A.bandwidth
    x2 = A.ldlt_solve(b)
    assert np.array_equal(x, x2) and A.bandwidth == bw
    # half bandwidth of the pattern: last column of a row minus the row
    rp, ci = A.pattern()
    assert bw == max(int(ci[rp[i + 1] - 1]) - i for i in range(len(rp) - 1))


@pytest.mark.parametrize("case", LINEAR_CASES)
def test_linear_static_direct_matches_reference(case, ctx, native_lib):
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    A.set_solver(native_lib.LS_DIRECT)
    u, reac, info = model.linear_static(A, rtol=1e-30, maxit=1)   # tolerance and maxit do not apply
    assert info.status == 0 and info.iterations == 0 and info.achieved < 1e-10, info.achieved
    assert rel(u, g["s1_u"]) < TOL, rel(u, g["s1_u"])
    assert rel(reac, g["s1_reac"]) < TOL, rel(reac, g["s1_reac"])
    model.internal_forces(u)
    s, e = model.gp_stress()
    assert rel(s, g["s1_stress"]) < TOL
    assert rel(e, g["s1_strain"]) < TOL


def newton_run(g, model, A, native_lib):
    ns = int(g["nsteps"])
    T = float(g["ramp_steps"])
    out = []
    for k in range(1, ns + 1):
        fac = float(g[f"s{k}_time"]) / T
        u, reac, nite = model.nonlinear_step(A, g["bc_value"] * fac, g["nodal_load"] * fac,
                                             rtolf=float(g["rtolf"]), maxiter=int(g["maxiter"]))
        s, _ = model.gp_stress()
        out.append(dict(u=u, reac=reac, nite=nite, stress=s, state=model.gp_state()))
    return out


def check_step(case, k, r, g):
    assert r["nite"] == int(g[f"s{k}_nite"]), (case, k, r["nite"], int(g[f"s{k}_nite"]))
    assert rel(r["u"], g[f"s{k}_u"]) < TOL, (k, rel(r["u"], g[f"s{k}_u"]))
    assert rel(r["reac"], g[f"s{k}_reac"]) < TOL
    assert rel(r["stress"], g[f"s{k}_stress"]) < TOL
    assert rel(r["state"][..., 0], g[f"s{k}_kappa"]) < TOL
    if "idm1" in case:
        assert rel(r["state"][..., 1], g[f"s{k}_omega"]) < TOL
        le = g[f"s{k}_le"]
        dam = le > 0
        if dam.any():
            assert rel(r["state"][..., 2][dam], le[dam]) < TOL


@pytest.mark.parametrize("case", NONLINEAR_CASES)
def test_newton_with_direct_solves_matches_reference(case, ctx, native_lib):
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    model.set_initial_guess(int(g.get("initial_guess", 0)))
    A = native_lib.GpuCsrMtrx(ctx)
    A.set_solver(native_lib.LS_DIRECT)
    for k, r in enumerate(newton_run(g, model, A, native_lib), 1):
        check_step(case, k, r, g)
    solves, iters = model.solver_stats()
    assert solves > 0 and iters == 0


@pytest.mark.parametrize("case", SS_CASES)
def test_static_structural_with_direct_solves_matches_reference(case, ctx, native_lib):
    from oofem_gb300 import engng
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    A.set_solver(native_lib.LS_DIRECT)
    ramp = engng.PiecewiseLinFunction([0.0, float(g["ramp_time"])], [0.0, 1.0])
    mr = int(g["manrmsteps"])
    ss = engng.StaticStructural(model, A, nsteps=int(g["nsteps"]), deltat=float(g["deltat"]), bc_function=ramp,
                                load_function=ramp, rtolf=float(g["rtolf"]), maxiter=int(g["maxiter"]),
                                manrmsteps=0 if mr < 0 else mr)
    for k in range(1, int(g["nsteps"]) + 1):
        res = ss.solve_yourself_at()
        s, _ = model.gp_stress()
        check_step(case, k, dict(u=res.u, reac=res.reactions, nite=res.iterations, stress=s,
                                 state=model.gp_state()), g)


def test_zero_pivot_is_reported(ctx, native_lib):
    """A singular matrix gives the zero-pivot status, not a fault or NaNs."""
    A = native_lib.GpuCsrMtrx(ctx)
    A.build_internal_structure(2, [np.array([1, 2], np.int32)])
    A.assemble_begin()
    A.assemble([1, 2], np.ones((2, 2)))
    A.assemble_end()
    x = np.zeros(2)
    assert native_lib.GpuLdltSolver().solve(A, np.array([1.0, 2.0]), x) == -7
    with pytest.raises(native_lib.OgbError):
        A.factorized()
    # a regular matrix on the same handle factors again after the values change
    A.set_at(2, 2, 3.0)
    assert native_lib.GpuLdltSolver().solve(A, np.array([1.0, 2.0]), x) == 0
    assert np.allclose(np.array([[1, 1], [1, 3]]) @ x, [1.0, 2.0], rtol=0, atol=1e-15)


def test_direct_refactors_after_set_at(ctx, native_lib):
    """Every mutation bumps the version and the next solve refactors
    (NRSolver::applyConstraintsToStiffness scales diagonals through at())."""
    g = load_golden("hex_cantilever_6x3x3_jit")
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    model.assemble_stiffness(A)
    K = dense(g)
    b = np.ones(K.shape[0])
    x1 = A.ldlt_solve(b)
    A.set_at(5, 5, A.at(5, 5) * 1e6)
    K[4, 4] *= 1e6
    x2 = A.ldlt_solve(b)
    assert not np.array_equal(x1, x2)
    assert rel(x2, np.linalg.solve(K, b)) < 1e-11
