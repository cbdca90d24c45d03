"""Element stiffness on the tensor cores (split-BF16 tcgen05 products accumulated
in FP32), the opt-in element kernel of mixed-precision Newton tangents
(OGB_OPT_TANGENT_TC).

K_e = sum_gp B^T D B dV (NLStructuralElement::computeStiffnessMatrix,
nlstructuralelement.C:345-376) from the tensor-core kernel agrees with the FP64
CUDA-core kernel to FP32 accuracy (assembled values within 2e-6 relative to the
largest entry) for LSpace, PlaneStress2d and LTRSpace meshes, including per-GP
MisesMat tangents of a plastic state and IDM1 secants of a damaged one, with
exactly symmetric element matrices and several tiles per CTA; mixed
Newton steps with these tangents reach the reference's converged states within
the Newton tolerance (fields within 1e-6, at most one extra Newton iteration
per step)."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_linear import mesh_from_golden, rel

pytestmark = pytest.mark.gpu


def tc_context(native_lib, mode=1):
    c = native_lib.Context(0)
    c.set_option(native_lib.OPT_TANGENT_TC, mode)
    return c


@pytest.mark.parametrize("kind", ["hex", "quad", "tet"])
def test_elastic_tangent_matches_fp64(kind, native_lib):
    from oofem_gb300 import meshgen as mg
    mesh = {"hex": lambda: mg.hex_cantilever(9, 4, 3, jitter=0.2, seed=3),
            "quad": lambda: mg.quad_rve(24, seed=5),
            "tet": lambda: mg.tet_cube_linear(5, jitter=0.1, seed=2)}[kind]()
    c = tc_context(native_lib)
    model = native_lib.GpuModel(c, mesh)
    A = native_lib.GpuCsrMtrx(c)
    model.build_matrix(A)
    model.assemble_tangent(A, native_lib.PREC_FP64)
    assert not model.tangent_kernel()[0]
    k64 = A.values()
    model.assemble_tangent(A, native_lib.PREC_MIXED)
    ktc = A.values()
    if kind == "hex":   # the isotropic hex keeps its FP64 form in every precision
        assert not model.tangent_kernel()[0] and np.array_equal(k64, ktc)
    else:
        assert model.tangent_kernel()[0]
        assert rel(ktc, k64) < 2e-6, rel(ktc, k64)
        assert not np.array_equal(ktc, k64)


@pytest.mark.parametrize("case", ["mises_hex_10x3x3_ig", "idm1_tet_3"])
def test_nonlinear_tangent_matches_fp64(case, native_lib, oracle):
    """Per-GP tangents of the reference's plastic / damaged state at its last step."""
    from test_gpu_material_eval import reference_state
    g = load_golden(case)
    c = tc_context(native_lib)
    model = native_lib.GpuModel(c, mesh_from_golden(g))
    A = native_lib.GpuCsrMtrx(c)
    model.build_matrix(A)
    n = int(g["nsteps"]) - 1
    model.load_committed_state(reference_state(g, n, oracle))
    model.internal_forces(g[f"s{n + 1}_u"])   # temp state of the last step
    model.assemble_tangent(A, native_lib.PREC_FP64)
    k64 = A.values()
    model.assemble_tangent(A, native_lib.PREC_MIXED)
    assert model.tangent_kernel()[0]
    ktc = A.values()
    assert rel(ktc, k64) < 2e-6, rel(ktc, k64)


@pytest.mark.parametrize("case", ["mises_hex_6x3x3", "idm1_tet_3"])
def test_mixed_newton_with_tensor_core_tangents(case, native_lib):
    g = load_golden(case)
    c = tc_context(native_lib)
    model = native_lib.GpuModel(c, mesh_from_golden(g))
    A = native_lib.GpuCsrMtrx(c)
    T = float(g["ramp_steps"])
    for k in range(1, int(g["nsteps"]) + 1):
        fac = float(g[f"s{k}_time"]) / T
        u, reac, nite = model.nonlinear_step(A, g["bc_value"] * fac, g["nodal_load"] * fac, rtolf=float(g["rtolf"]),
                                             maxiter=int(g["maxiter"]), lin_rtol=1e-10,
                                             precision=native_lib.PREC_MIXED)
        assert nite - int(g[f"s{k}_nite"]) in (0, 1), (k, nite, int(g[f"s{k}_nite"]))
        assert rel(u, g[f"s{k}_u"]) < 1e-6
        assert rel(reac, g[f"s{k}_reac"]) < 1e-6
        if nite > 0:
            assert model.tangent_kernel()[0]


def test_timed_choice_records_both_kernels(native_lib):
    g = load_golden("mises_hex_6x3x3")
    c = tc_context(native_lib, mode=2)
    model = native_lib.GpuModel(c, mesh_from_golden(g))
    A = native_lib.GpuCsrMtrx(c)
    model.build_matrix(A)
    model.assemble_tangent(A, native_lib.PREC_MIXED)
    used, t64, ttc = model.tangent_kernel()
    assert t64 > 0 and ttc > 0 and used == (ttc < t64)


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_many_tiles_per_cta(kind, native_lib):
    """Meshes with several tiles per CTA (the kernel loops over tiles with one
    tensor-memory allocation and a flipping mbarrier phase): MisesMat elements in
    their elastic state (per-GP tangents) against the FP64 kernel."""
    from oofem_gb300 import meshgen as mg
    if kind == "hex":
        mesh = mg.hex_block_pull(60, 12, 12, h=0.05, end_disp=1e-3)   # 8,640 hexes: 1,728 tiles
    else:
        mesh = mg.tet_cube_linear(14, jitter=0.1, seed=3)                # 16,464 tets: 1,647 tiles
        mesh.materials = [mg.Material(mg.MAT_MISES, m.E, m.nu, 250e6, 2e9) for m in mesh.materials]
    c = tc_context(native_lib)
    model = native_lib.GpuModel(c, mesh)
    A = native_lib.GpuCsrMtrx(c)
    model.build_matrix(A)
    model.assemble_tangent(A, native_lib.PREC_FP64)
    k64 = A.values()
    model.assemble_tangent(A, native_lib.PREC_MIXED)
    assert model.tangent_kernel()[0]
    ktc = A.values()
    assert np.isfinite(ktc).all()
    assert rel(ktc, k64) < 2e-6, rel(ktc, k64)
    # the element matrices are exactly symmetric (upper triangle mirrored), so is K
    sp = pytest.importorskip("scipy.sparse")
    rp, ci = A.pattern()
    K = sp.csr_matrix((ktc, ci, rp), shape=(len(rp) - 1, len(rp) - 1))
    assert abs(K - K.T).max() == 0.0
