"""Single evaluations of the nonlinear material kernels from the reference's own
state (tests/golden: converged steps of the reference's NonLinearStatic and
StaticStructural runs with MisesMat hexes and IsotropicDamageMaterial1 tets).

For every pair of consecutive steps n -> n+1 of a reference run, the committed
Gauss-point state of step n is loaded into the device model (MisesMat: plastic
strain = strain - D^-1 stress of step n and kappa; IDM1: kappa, damage and crack
band length Le of step n), and one internal-force evaluation runs at the
reference's converged displacements of step n+1. That is one call of
MisesMat::performPlasticityReturn (misesmat.C:181-263) or
IsotropicDamageMaterial::giveRealStressVector (isodamagemodel.C:86-160,
idm1.C:436-470, 808-911) per Gauss point and of
NLStructuralElement::giveInternalForcesVector (nlstructuralelement.C:151-240)
per element, so it must reproduce the reference's step n+1 exactly up to
rounding, independent of any linear solve or Newton path:

* Gauss-point stresses, strains, kappa, damage and (at damaged points) Le within
  1e-10 relative;
* reactions (the internal forces at the prescribed DOFs) within 1e-10 relative.

The tangent of the same state (MisesMat::give3dMaterialStiffnessMatrix
misesmat.C:496-545; the IDM1 secant isodamagemodel.C:63-81), assembled on the
device, agrees with the oracle's tangent of the same state within 1e-12."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_linear import mesh_from_golden, rel

pytestmark = pytest.mark.gpu

TOL = 1e-10
CASES = ["mises_hex_4x2x2", "mises_hex_6x3x3", "mises_hex_10x3x3_ig", "ss_mises_hex_6x3x3",
         "ss_mises_hex_5x2x2_accel", "idm1_tet_3", "ss_idm1_tet_3"]


@pytest.fixture(scope="module")
def ctx(native_lib):
    return native_lib.Context(0)


def reference_state(g, n, oracle, nstate=24):
    """Committed GP state after the reference's step n (n = 0: virgin state)."""
    et = int(g["etype"])
    ne, ngp = g["conn"].shape[0], g["s1_stress"].shape[1]
    st = np.zeros((ne, ngp, nstate))
    if n == 0:
        return st
    kind = int(g["mats"][0][0])
    if kind == 2:   # MisesMat: eps_p = eps - D^-1 sigma, kappa
        for mi, m in enumerate(g["mats"]):
            C = np.linalg.inv(oracle.isole_d(et, m[1], m[2]))
            sel = g["elem_mat"] == mi
            st[sel, :, 0:6] = g[f"s{n}_strain"][sel] - g[f"s{n}_stress"][sel] @ C.T
        st[..., 6] = g[f"s{n}_kappa"]
    else:           # IDM1: kappa, omega, Le
        st[..., 0] = g[f"s{n}_kappa"]
        st[..., 1] = g[f"s{n}_omega"]
        st[..., 2] = g[f"s{n}_le"]
    return st


@pytest.mark.parametrize("case", CASES)
def test_one_evaluation_from_reference_state(case, ctx, native_lib, oracle):
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    neq, _, eq = oracle.number_equations(g["bc_mask"])
    loc = oracle.location_arrays(g["conn"], eq)
    rp, ci = A.pattern()
    mask = g["bc_mask"].astype(bool)
    ns = int(g["nsteps"])
    idm = "idm1" in case
    worst = 0.0
    for n in range(0, ns):
        k = n + 1
        st = reference_state(g, n, oracle)
        model.load_committed_state(st)
        assert np.array_equal(model.committed_state(), st)
        f = model.internal_forces(g[f"s{k}_u"])
        s, e = model.gp_stress()
        reac = np.where(mask, f, 0.0)
        errs = [rel(s, g[f"s{k}_stress"]), rel(e, g[f"s{k}_strain"]), rel(reac, g[f"s{k}_reac"])]
        # tangent of this state (temp values of the evaluation), device vs oracle
        model.assemble_stiffness(A)
        ost = st.reshape(-1, st.shape[-1]).copy()
        oracle.internal_forces(g, g[f"s{k}_u"], ost)
        Kref = oracle.assemble_tangent(g, loc, neq, rp, ci, ost)
        assert rel(A.values(), Kref) < 1e-12, (k, rel(A.values(), Kref))
        model.commit_state()
        gs = model.gp_state()
        errs.append(rel(gs[..., 0], g[f"s{k}_kappa"]))
        if idm:
            errs.append(rel(gs[..., 1], g[f"s{k}_omega"]))
            le = g[f"s{k}_le"]
            # Le where the damage is nonzero: at undamaged points an intermediate Newton
            # iterate of the reference run may have set it (idm1.C:1202 writes it into the
            # status whenever kappa > e0 while the committed damage is zero)
            dam = g[f"s{k}_omega"] > 0
            if dam.any():
                errs.append(rel(gs[..., 2][dam], le[dam]))
        worst = max(worst, max(errs))
        assert max(errs) < TOL, (case, k, errs)
    print(f"{case}: worst relative difference {worst:.2e} over {ns} evaluations")


def test_plastic_evaluation_is_exercised():
    """The MisesMat evaluations above include plastic return mappings with a
    plastic strain already present (kappa grows from a nonzero committed value)."""
    g = load_golden("mises_hex_10x3x3_ig")
    grows = [(g[f"s{k}_kappa"] > g[f"s{k - 1}_kappa"]) & (g[f"s{k - 1}_kappa"] > 0)
             for k in range(2, int(g["nsteps"]) + 1)]
    assert any(x.any() for x in grows)
    gi = load_golden("idm1_tet_3")
    onset = [(gi[f"s{k}_omega"] > 0) & (gi[f"s{k - 1}_omega"] == 0) for k in range(2, int(gi["nsteps"]) + 1)]
    growth = [(gi[f"s{k}_omega"] > gi[f"s{k - 1}_omega"]) & (gi[f"s{k - 1}_omega"] > 0)
              for k in range(2, int(gi["nsteps"]) + 1)]
    assert any(x.any() for x in onset) and any(x.any() for x in growth)
