"""StaticStructural on the GPU path (oofem_gb300.engng.StaticStructural over
ogb_nonlinear_step) against the reference's own StaticStructural runs
(tests/golden/ss_*.npz): IG_Tangent initial guess, modified Newton (the
reference's default, 180-240 iterations per plastic step) and accelerated
Newton (manrmsteps 2), deltat time stepping, MisesMat.

Bars as for the NonLinearStatic cases: Newton iterations per step within one
of the reference's (direct solves there, PCG to 1e-13 here); displacements,
reactions, GP stresses and kappa within 1e-7 relative."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_linear import mesh_from_golden, rel

pytestmark = pytest.mark.gpu

SS_CASES = ["ss_mises_hex_6x3x3", "ss_mises_hex_5x2x2_accel"]


@pytest.fixture(scope="module")
def ctx(native_lib):
    return native_lib.Context(0)


@pytest.mark.parametrize("case", SS_CASES)
def test_static_structural_matches_reference(case, ctx, native_lib):
    from oofem_gb300 import engng
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    ramp = engng.PiecewiseLinFunction([0.0, float(g["ramp_time"])], [0.0, 1.0])
    mr = int(g["manrmsteps"])
    ss = engng.StaticStructural(model, A, nsteps=int(g["nsteps"]), deltat=float(g["deltat"]), bc_function=ramp,
                                load_function=ramp, rtolf=float(g["rtolf"]), maxiter=int(g["maxiter"]),
                                manrmsteps=0 if mr < 0 else mr, lstol=1e-13)
    for k in range(1, int(g["nsteps"]) + 1):
        r = ss.solve_yourself_at()
        assert r.number == k and r.time == float(g[f"s{k}_time"])
        assert abs(r.iterations - int(g[f"s{k}_nite"])) <= 1, (k, r.iterations, int(g[f"s{k}_nite"]))
        assert rel(r.u, g[f"s{k}_u"]) < 1e-7
        assert rel(r.reactions, g[f"s{k}_reac"]) < 1e-7
        s, _ = model.gp_stress()
        assert rel(s, g[f"s{k}_stress"]) < 1e-7
        assert rel(model.gp_state()[..., 0], g[f"s{k}_kappa"]) < 1e-7
    with pytest.raises(RuntimeError):
        ss.solve_yourself_at()


def test_modified_newton_reuses_the_start_tangent(ctx, native_lib):
    """Modified Newton solves every iteration of a step with one matrix: the
    element stiffnesses are assembled once per step (plus nothing per
    iteration), where full Newton re-assembles every iteration after the first.
    Both converge to the same state within the Newton tolerance."""
    from oofem_gb300 import engng
    g = load_golden("ss_mises_hex_6x3x3")
    mesh = mesh_from_golden(g)
    ramp = engng.PiecewiseLinFunction([0.0, float(g["ramp_time"])], [0.0, 1.0])
    out = {}
    for mr in (0, 1):
        model = native_lib.GpuModel(ctx, mesh)
        A = native_lib.GpuCsrMtrx(ctx)
        ss = engng.StaticStructural(model, A, nsteps=int(g["nsteps"]), deltat=float(g["deltat"]),
                                    bc_function=ramp, load_function=ramp, rtolf=1e-8, maxiter=400,
                                    manrmsteps=mr, lstol=1e-13)
        res = ss.solve_yourself()
        out[mr] = (res, A.version)
    its0 = sum(r.iterations for r in out[0][0])
    its1 = sum(r.iterations for r in out[1][0])
    assert its1 < its0
    # one assembly per step (modified) against one per step plus one per iteration > 0 (full)
    nsteps = int(g["nsteps"])
    assert out[1][1] - out[0][1] == sum(max(r.iterations - 1, 0) for r in out[1][0])
    assert rel(out[0][0][-1].u, out[1][0][-1].u) < 1e-6
    assert nsteps == len(out[0][0])


def test_context_restart_is_bit_identical(ctx, native_lib):
    """saveStepContext after step 4, restoreStepContext into a fresh model and
    matrix, then steps 5-8: displacements, reactions, GP state and Newton
    iterations identical bit for bit to the uninterrupted run. A context of
    another mesh is refused."""
    from oofem_gb300 import engng
    from oofem_gb300 import meshgen as mg
    g = load_golden("ss_mises_hex_5x2x2_accel")
    mesh = mesh_from_golden(g)
    ramp = engng.PiecewiseLinFunction([0.0, float(g["ramp_time"])], [0.0, 1.0])

    def analysis():
        model = native_lib.GpuModel(ctx, mesh)
        A = native_lib.GpuCsrMtrx(ctx)
        return engng.StaticStructural(model, A, nsteps=int(g["nsteps"]), bc_function=ramp, load_function=ramp,
                                      rtolf=1e-8, maxiter=400, manrmsteps=2, lstol=1e-13)

    full = analysis()
    ref = full.solve_yourself()
    first = analysis()
    for _ in range(4):
        first.solve_yourself_at()
    blob = first.save_context()
    second = analysis()
    second.restore_context(blob)
    rest = second.solve_yourself()
    assert [r.number for r in rest] == [5, 6, 7, 8]
    for a, b in zip(ref[4:], rest):
        assert a.time == b.time and a.iterations == b.iterations
        assert np.array_equal(a.u, b.u) and np.array_equal(a.reactions, b.reactions)
    assert np.array_equal(full.model.gp_state(), second.model.gp_state())
    other = native_lib.GpuModel(ctx, mg.hex_block_pull(4, 2, 2, material=mesh.materials[0], end_disp=1e-4))
    with pytest.raises(native_lib.OgbError) as e:
        other.restore_state(blob[engng._CTX.size:])
    assert e.value.code == -1
