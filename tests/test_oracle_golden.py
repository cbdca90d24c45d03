"""The C oracle against golden vectors written by the reference executable
(tests/golden/*.npz via oracle/ref_harness.C) and against the golden values
embedded in the reference's own LTRSpace patch deck (tests/sm/patch300.in)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, LINEAR_CASES, load_golden


def rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


@pytest.mark.parametrize("case", LINEAR_CASES)
def test_numbering_pattern_values(case, oracle):
    g = load_golden(case)
    neq, npeq, eq = oracle.number_equations(g["bc_mask"])
    assert np.array_equal(np.where(eq > 0, eq, 0), g["s1_eq"])
    assert neq == int(g["neq"])
    loc = oracle.location_arrays(g["conn"], eq)
    rp, ci = oracle.build_pattern(neq, loc)
    # CompCol colptr/rowind of the full symmetric pattern == CSR rowptr/colind
    assert np.array_equal(rp, g["K_colptr"])
    assert np.array_equal(ci, g["K_rowind"])
    val = oracle.assemble_tangent(g, loc, neq, rp, ci)
    assert rel(val, g["K_val"]) < 1e-13


@pytest.mark.parametrize("case", LINEAR_CASES)
def test_element_stiffness(case, oracle):
    g = load_golden(case)
    et = int(g["etype"])
    for e in range(1, 5):
        key = f"ke{e}"
        if key not in g:
            continue
        xe = g["coords"][g["conn"][e - 1]]
        m = g["mats"][g["elem_mat"][e - 1]]
        ke = oracle.elem_stiffness(et, xe, oracle.isole_d(et, m[1], m[2]), float(g["thickness"]))
        assert rel(ke, g[key]) < 1e-14


@pytest.mark.parametrize("case", LINEAR_CASES)
def test_linear_static(case, oracle):
    g = load_golden(case)
    r = oracle.linear_static(g, rtol=1e-15, maxit=100000)
    assert r["status"] == 0
    assert rel(r["u"], g["s1_u"]) < 1e-10
    assert rel(r["reac"], g["s1_reac"]) < 1e-10
    assert rel(r["stress"], g["s1_stress"]) < 1e-10
    assert rel(r["strain"], g["s1_strain"]) < 1e-10


def test_patch300_reference_deck(oracle):
    """LTRSpace compression patch test, exact solution from tests/sm/patch300.in."""
    with open(os.path.join(GOLDEN, "patch300.json")) as fh:
        rules = json.load(fh)
    coords = np.array([[0, 0, 0], [3, 0, 0], [0, 3, 0], [0, 0, 6], [3, 0, 6], [0, 3, 6]], float)
    conn = np.array([[1, 2, 3, 4], [4, 5, 2, 3], [4, 6, 5, 3]], np.int32) - 1
    bc = np.zeros((6, 3), np.uint8)
    bc[0:3, :] = 1
    bc[3:6, 0:2] = 1
    load = np.zeros((6, 3))
    load[3:6, 2] = -1.5
    m = dict(etype=3, coords=coords, conn=conn, elem_mat=np.zeros(3, np.int32),
             mats=np.array([[1, 15.0, 0.25, 0, 0, 0, 0, 0]]), bc_mask=bc, bc_value=np.zeros((6, 3)),
             nodal_load=load, thickness=1.0)
    r = oracle.linear_static(m, rtol=1e-14)
    tol = rules["tolerance"]
    for node, dof, v in rules["nodes"]:
        assert abs(r["u"][node - 1, dof - 1] - v) <= tol
    for node, dof, v in rules["reactions"]:
        assert abs(r["reac"][node - 1, dof - 1] - v) <= tol


def test_pcg_matches_reference_iteration_count(oracle):
    """The 20x4x4 cantilever with IML Jacobi-CG at lstol 1e-12: a run of the
    reference executable logged 'nite 111, achieved tol 9.19e-13' (imlsolver.C:131)."""
    g = load_golden("hex_cantilever_20x4x4")
    r = oracle.linear_static(g, rtol=1e-12)
    assert abs(r["iters"] - 111) <= 1
    assert r["achieved"] <= 1e-12
    tip = r["u"][20, 2]
    assert abs(tip - (-1.16468948e-03)) < 5e-11


NONLINEAR_CASES = ["mises_hex_4x2x2", "mises_hex_6x3x3", "mises_hex_10x3x3_ig", "idm1_tet_3"]


@pytest.mark.parametrize("case", NONLINEAR_CASES)
def test_nonlinear_static_newton(case, oracle):
    """NonLinearStatic + NRSolver (full Newton) with MisesMat (J2 radial return)
    and IsotropicDamageMaterial1 (Mazars, exponential cohesive crack, crack
    band) against the reference run step by step: same Newton iteration count,
    same displacements, reactions, GP stresses, kappa and damage."""
    g = load_golden(case)
    ns = int(g["nsteps"])
    times = [float(g[f"s{k}_time"]) for k in range(1, ns + 1)]
    res = oracle.nonlinear_static(g, times, float(g["ramp_steps"]), float(g["rtolf"]), int(g["maxiter"]),
                                  initial_guess=int(g.get("initial_guess", 0)))
    mises = "mises" in case
    for k, r in enumerate(res, 1):
        assert r["nite"] == int(g[f"s{k}_nite"])
        assert rel(r["u"], g[f"s{k}_u"]) < 1e-9
        assert rel(r["reac"], g[f"s{k}_reac"]) < 1e-9
        assert rel(r["stress"], g[f"s{k}_stress"]) < 1e-9
        kap = r["state"][:, 6] if mises else r["state"][:, 0]
        assert rel(kap, g[f"s{k}_kappa"].ravel()) < 1e-9
        if not mises:
            assert rel(r["state"][:, 1], g[f"s{k}_omega"].ravel()) < 1e-9
            le = g[f"s{k}_le"].ravel()
            dam = le > 0
            if dam.any():
                assert rel(r["state"][dam, 2], le[dam]) < 1e-9


SS_CASES = ["ss_mises_hex_6x3x3", "ss_mises_hex_5x2x2_accel"]


@pytest.mark.parametrize("case", SS_CASES)
def test_static_structural(case, oracle):
    """StaticStructural with the reference's defaults (nrsolver, IG_Tangent
    initial guess, modified Newton unless manrmsteps is given; deltat time
    stepping) and MisesMat against the reference run: same Newton iterations per
    step, same displacements, reactions, GP stresses and kappa."""
    g = load_golden(case)
    ns = int(g["nsteps"])
    mr = int(g["manrmsteps"])
    res = oracle.static_structural(g, ns, float(g["ramp_time"]), deltat=float(g["deltat"]),
                                   rtolf=float(g["rtolf"]), maxiter=int(g["maxiter"]),
                                   manrmsteps=0 if mr < 0 else mr)
    for k, r in enumerate(res, 1):
        assert r["nite"] == int(g[f"s{k}_nite"]), (k, r["nite"], int(g[f"s{k}_nite"]))
        assert rel(r["u"], g[f"s{k}_u"]) < 1e-8
        assert rel(r["reac"], g[f"s{k}_reac"]) < 1e-8
        assert rel(r["stress"], g[f"s{k}_stress"]) < 1e-8
        assert rel(r["state"][:, 6], g[f"s{k}_kappa"].ravel()) < 1e-8


@pytest.mark.parametrize("case", ["hex_cantilever_6x3x3_jit_ic", "quad_rve_8_s3_ic", "hex_cantilever_6x3x3_jit_ilu",
                                  "tet_cube_3_jit_ilu", "hex_cantilever_6x3x3_jit_void"])
def test_iml_cg_preconditioners(case, oracle):
    """IML CG with the incomplete-Cholesky (lsprecond 4) and the column ILU
    (lsprecond 2) preconditioners (the reference's factorization loops) and
    without one (lsprecond 0) against the
    reference's runs: the CG iteration count from its log line and the
    displacements."""
    g = load_golden(case)
    r = oracle.linear_static(g, rtol=float(g["lstol"]), precond=int(g["lsprecond"]))
    assert r["status"] == 0
    assert abs(r["iters"] - int(g["cg_nite"][0])) <= 1, (r["iters"], int(g["cg_nite"][0]))
    assert rel(r["u"], g["s1_u"]) < 1e-8
    assert rel(r["reac"], g["s1_reac"]) < 1e-8


def test_static_structural_idm1(oracle):
    """StaticStructural (IG_Tangent, full Newton) with IsotropicDamageMaterial1
    through the softening branch (damage up to 0.93) against the reference run:
    same Newton iterations per step, displacements, reactions, stresses, kappa
    and damage."""
    g = load_golden("ss_idm1_tet_3")
    ns = int(g["nsteps"])
    res = oracle.static_structural(g, ns, float(g["ramp_time"]), deltat=float(g["deltat"]),
                                   rtolf=float(g["rtolf"]), maxiter=int(g["maxiter"]),
                                   manrmsteps=int(g["manrmsteps"]))
    for k, r in enumerate(res, 1):
        assert r["nite"] == int(g[f"s{k}_nite"]), (k, r["nite"], int(g[f"s{k}_nite"]))
        assert rel(r["u"], g[f"s{k}_u"]) < 1e-8
        assert rel(r["reac"], g[f"s{k}_reac"]) < 1e-8
        assert rel(r["stress"], g[f"s{k}_stress"]) < 1e-8
        assert rel(r["state"][:, 0], g[f"s{k}_kappa"].ravel()) < 1e-8
        assert rel(r["state"][:, 1], g[f"s{k}_omega"].ravel()) < 1e-8


MATERIAL_EVAL_CASES = ["mises_hex_4x2x2", "mises_hex_6x3x3", "mises_hex_10x3x3_ig", "ss_mises_hex_6x3x3",
                       "ss_mises_hex_5x2x2_accel", "idm1_tet_3", "ss_idm1_tet_3"]


@pytest.mark.parametrize("case", MATERIAL_EVAL_CASES)
def test_oracle_one_evaluation_from_reference_state(case, oracle):
    """The oracle's material updates, started from the reference's committed state
    of step n (MisesMat: eps_p = eps - D^-1 sigma and kappa; IDM1: kappa, omega, Le)
    at the reference's displacements of step n+1, reproduce the reference's step
    n+1 GP stresses, kappa, damage and reactions within 1e-10 (the GPU test
    tests/test_gpu_material_eval.py runs the same evaluations on the device)."""
    from test_gpu_material_eval import reference_state
    g = load_golden(case)
    mask = g["bc_mask"].astype(bool)
    idm = "idm1" in case
    for n in range(0, int(g["nsteps"])):
        k = n + 1
        st = reference_state(g, n, oracle).reshape(-1, 24)
        f, s, e = oracle.internal_forces(g, g[f"s{k}_u"], st)
        oracle.commit_state(g, st)
        st = st.reshape(g["conn"].shape[0], -1, 24)
        errs = [rel(s, g[f"s{k}_stress"]), rel(e, g[f"s{k}_strain"]), rel(np.where(mask, f, 0), g[f"s{k}_reac"])]
        errs.append(rel(st[..., 0] if idm else st[..., 6], g[f"s{k}_kappa"]))
        if idm:
            errs.append(rel(st[..., 1], g[f"s{k}_omega"]))
            # Le is written into the status by every evaluation with kappa > e0 while the
            # committed damage is zero (idm1.C:1202), so an intermediate Newton iterate can
            # leave one at an undamaged point; where damage is nonzero the converged
            # evaluation set it
            dam = g[f"s{k}_omega"] > 0
            if dam.any():
                errs.append(rel(st[..., 2][dam], g[f"s{k}_le"][dam]))
        assert max(errs) < 1e-10, (case, k, errs)
