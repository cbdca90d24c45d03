"""GPU NonLinearStatic / NRSolver steps with MisesMat and IsotropicDamageMaterial1
against the reference's own Newton runs (tests/golden/{mises,idm1}_*.npz).

Bars: Newton iteration count per step within one of the reference's (the
reference solves each linear system directly, the GPU by PCG to 1e-13, so a
residual sitting right at rtolf may take one more or one fewer iteration);
displacements, reactions, GP stresses, kappa and damage within 1e-7 relative
(to the field's maximum)."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_linear import mesh_from_golden, rel

pytestmark = pytest.mark.gpu

NONLINEAR_CASES = ["mises_hex_4x2x2", "mises_hex_6x3x3", "mises_hex_10x3x3_ig", "idm1_tet_3"]


@pytest.fixture(scope="module")
def ctx(native_lib):
    return native_lib.Context(0)


def run_steps(g, model, A, native_lib, precision=0, lin_rtol=1e-13):
    ns = int(g["nsteps"])
    T = float(g["ramp_steps"])
    out = []
    for k in range(1, ns + 1):
        fac = float(g[f"s{k}_time"]) / T
        u, reac, nite = model.nonlinear_step(A, g["bc_value"] * fac, g["nodal_load"] * fac,
                                             rtolf=float(g["rtolf"]), maxiter=int(g["maxiter"]),
                                             lin_rtol=lin_rtol, precision=precision)
        s, e = model.gp_stress()
        out.append(dict(u=u, reac=reac, nite=nite, stress=s, state=model.gp_state()))
    return out


@pytest.mark.parametrize("case", NONLINEAR_CASES)
def test_newton_steps_match_reference(case, ctx, native_lib):
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    model.set_initial_guess(int(g.get("initial_guess", 0)))
    A = native_lib.GpuCsrMtrx(ctx)
    res = run_steps(g, model, A, native_lib)
    for k, r in enumerate(res, 1):
        assert abs(r["nite"] - int(g[f"s{k}_nite"])) <= 1, (k, r["nite"], int(g[f"s{k}_nite"]))
        assert rel(r["u"], g[f"s{k}_u"]) < 1e-7
        assert rel(r["reac"], g[f"s{k}_reac"]) < 1e-7
        assert rel(r["stress"], g[f"s{k}_stress"]) < 1e-7
        assert rel(r["state"][..., 0], g[f"s{k}_kappa"]) < 1e-7
        if "idm1" in case:
            assert rel(r["state"][..., 1], g[f"s{k}_omega"]) < 1e-7
            le = g[f"s{k}_le"]
            dam = le > 0
            if dam.any():
                assert rel(r["state"][..., 2][dam], le[dam]) < 1e-7


def test_newton_with_mixed_precision_linear_solves(ctx, native_lib):
    """Mixed-precision linear solves inside Newton: the converged states agree
    with the reference to the Newton tolerance."""
    g = load_golden("mises_hex_6x3x3")
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    res = run_steps(g, model, A, native_lib, precision=native_lib.PREC_MIXED, lin_rtol=1e-10)
    for k, r in enumerate(res, 1):
        assert abs(r["nite"] - int(g[f"s{k}_nite"])) <= 1
        assert rel(r["u"], g[f"s{k}_u"]) < 1e-6
        assert rel(r["state"][..., 0], g[f"s{k}_kappa"]) < 1e-5


def test_reset_state_restarts_the_analysis(ctx, native_lib):
    g = load_golden("mises_hex_4x2x2")
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    first = run_steps(g, model, A, native_lib)
    model.reset_state()
    second = run_steps(g, model, A, native_lib)
    assert np.array_equal(first[-1]["u"], second[-1]["u"])
    assert np.array_equal(first[-1]["state"], second[-1]["state"])


def _separate_runs(native_lib, ctx, meshes, facs, ig, **kw):
    out = []
    for m in meshes:
        model = native_lib.GpuModel(ctx, m)
        model.set_initial_guess(ig)
        A = native_lib.GpuCsrMtrx(ctx)
        steps = []
        for f in facs:
            u, reac, nite = model.nonlinear_step(A, m.bc_value * f, None, **kw)
            steps.append((u, reac, nite, model.gp_state()))
        out.append(steps)
    return out


@pytest.mark.parametrize("kind", ["mises", "idm1"])
def test_batched_newton_matches_separate_runs(kind, ctx, native_lib):
    """Batched NonLinearStatic steps (instances of uneven size, each with its own
    NRSolver test) against separate GPU runs of each instance: Newton iteration
    counts per instance within one, displacements, reactions and GP state within
    1e-7."""
    from oofem_gb300 import meshgen as mg
    if kind == "mises":
        ey = 250e6 / 210e9
        meshes = [mg.hex_block_pull(8, 2, 2, h=0.05, jitter=0.2, seed=11, end_disp=3 * ey * 0.4),
                  mg.hex_block_pull(5, 3, 3, h=0.05, jitter=0.2, seed=12, end_disp=2 * ey * 0.25)]
        facs, ig, kw = [0.25, 0.5, 0.75, 1.0], 1, dict(rtolf=1e-8, maxiter=60, lin_rtol=1e-13)
    else:
        # the schedule of the reference's idm1_tet_3 run (6 increments, the first five),
        # on two other meshes; the oracle needs 3/96/17/12/10 and 1/3/45/11/9 iterations
        mat = mg.Material(mg.MAT_IDM1, 30e9, 0.2, e0=1e-4, gf=1000.0)
        meshes = [mg.tet_cube(3, jitter=0.15, seed=21, material=mat, end_disp=3e-4),
                  mg.tet_cube(2, jitter=0.15, seed=22, material=mat, end_disp=2.5e-4)]
        facs, ig, kw = [k / 6 for k in range(1, 6)], 0, dict(rtolf=1e-6, maxiter=400, lin_rtol=1e-13)
    ref = _separate_runs(native_lib, ctx, meshes, facs, ig, **kw)
    big, ns = mg.concat_meshes(meshes)
    model = native_lib.GpuModel(ctx, big)
    model.set_instances(ns)
    model.set_initial_guess(ig)
    A = native_lib.GpuCsrMtrx(ctx)
    e0 = np.cumsum([0] + [m.nelem for m in meshes])
    for k, f in enumerate(facs):
        u, reac, its = model.batch_nonlinear_step(A, big.bc_value * f, None, **kw)
        st = model.gp_state()
        for i in range(len(meshes)):
            ur, rr, nr, sr = ref[i][k]
            sl = slice(ns[i], ns[i + 1])
            assert abs(int(its[i]) - nr) <= 1, (k, i, its, nr)
            assert rel(u[sl], ur) < 1e-7
            assert rel(reac[sl], rr) < 1e-7
            assert rel(st[e0[i]:e0[i + 1]], sr) < 1e-7
