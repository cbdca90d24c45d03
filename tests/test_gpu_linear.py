"""GPU parity of the linear path through the C ABI against the reference's own
golden vectors (tests/golden) and the C oracle.

Bars: CSR pattern and equation numbers bit-exact; assembled values within
1e-12 relative; displacements / reactions / GP stresses within 1e-9 relative
of the reference's direct solve when PCG runs to ||r||/||b|| <= 1e-14 (the
solve tolerance bounds the displacement error, not the kernels); mixed
precision + FP64 refinement to 1e-8 relative residual within 1e-6 of the
reference displacements."""
import numpy as np
import pytest

from conftest import LINEAR_CASES, load_golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


def mesh_from_golden(g):
    from oofem_gb300 import meshgen as mg
    mats = [mg.Material(int(r[0]), r[1], r[2], r[3], r[4], r[5], r[6]) for r in g["mats"]]
    return mg.Mesh(int(g["etype"]), g["coords"], g["conn"].astype(np.int32), g["elem_mat"].astype(np.int32),
                   mats, g["bc_mask"].astype(np.uint8), g["bc_value"], g["nodal_load"],
                   thickness=float(g["thickness"]))


@pytest.fixture(scope="module")
def ctx(native_lib):
    return native_lib.Context(0)


@pytest.mark.parametrize("case", LINEAR_CASES)
def test_model_path_matches_reference(case, ctx, native_lib):
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    eq = model.equations()
    assert np.array_equal(np.where(eq > 0, eq, 0), g["s1_eq"])
    A = native_lib.GpuCsrMtrx(ctx)
    u, reac, info = model.linear_static(A, rtol=1e-14, maxit=100000)
    assert info.status == 0
    rp, ci = A.pattern()
    assert np.array_equal(rp, g["K_colptr"]) and np.array_equal(ci, g["K_rowind"])
    assert rel(A.values(), g["K_val"]) < 1e-12
    assert rel(u, g["s1_u"]) < 1e-9
    assert rel(reac, g["s1_reac"]) < 1e-9
    # GP stresses of the final state: internal forces at u
    model.internal_forces(u)
    s, e = model.gp_stress()
    assert rel(s, g["s1_stress"]) < 1e-9
    assert rel(e, g["s1_strain"]) < 1e-9


@pytest.mark.parametrize("case", LINEAR_CASES)
def test_dropin_sparse_matrix_path(case, ctx, native_lib, oracle):
    """SparseMtrx drop-in: buildInternalStructure from location arrays,
    assemble(loc, Ke) per element from the host, assembleEnd, times, at, solve."""
    g = load_golden(case)
    et = int(g["etype"])
    neq, _, eq = oracle.number_equations(g["bc_mask"])
    loc = oracle.location_arrays(g["conn"], eq)
    A = native_lib.GpuCsrMtrx(ctx)
    A.build_internal_structure(neq, loc)
    rp, ci = A.pattern()
    assert np.array_equal(rp, g["K_colptr"]) and np.array_equal(ci, g["K_rowind"])
    A.assemble_begin()
    for e in range(g["conn"].shape[0]):
        m = g["mats"][g["elem_mat"][e]]
        ke = oracle.elem_stiffness(et, g["coords"][g["conn"][e]], oracle.isole_d(et, m[1], m[2]),
                                   float(g["thickness"]))
        A.assemble(loc[e], ke)
    A.assemble_end()
    val = A.values()
    ref = oracle.assemble_tangent(g, loc, neq, rp, ci)
    assert np.array_equal(val, ref), "staged assembly must add in the reference order"
    assert rel(val, g["K_val"]) < 1e-13
    x = np.random.default_rng(0).standard_normal(neq)
    assert rel(A.times(x), oracle.spmv(rp, ci, ref, x)) < 1e-14
    assert A.at(1, 1) == ref[rp[0] + np.searchsorted(ci[rp[0]:rp[1]], 0)]
    solver = native_lib.GpuPcgSolver(lstol=1e-12, lsiter=100000)
    b = np.random.default_rng(1).standard_normal(neq)
    xg = np.zeros(neq)
    assert solver.solve(A, b, xg) == 0
    xo, st, it, ach = oracle.pcg(rp, ci, ref, b, rtol=1e-12)
    assert abs(solver.last.iterations - it) <= 2
    assert rel(xg, xo) < 1e-9


def test_version_bumps_and_set_at(ctx, native_lib, oracle):
    g = load_golden("hex_cantilever_6x3x3_jit")
    neq, _, eq = oracle.number_equations(g["bc_mask"])
    loc = oracle.location_arrays(g["conn"], eq)
    A = native_lib.GpuCsrMtrx(ctx)
    A.build_internal_structure(neq, loc)
    v0 = A.version
    A.set_at(3, 3, 2.5)
    assert A.at(3, 3) == 2.5 and A.version > v0
    A.zero()
    assert A.at(3, 3) == 0.0
    assert A.at(1, neq) == 0.0   # structural zero reads 0


def test_assembly_is_deterministic(ctx, native_lib):
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(12, 5, 5, jitter=0.2, seed=5)
    vals = []
    for _ in range(2):
        model = native_lib.GpuModel(ctx, mesh)
        A = native_lib.GpuCsrMtrx(ctx)
        model.build_matrix(A)
        model.assemble_stiffness(A)
        vals.append(A.values())
    assert np.array_equal(vals[0], vals[1])


@pytest.mark.parametrize("case", ["hex_cantilever_20x4x4", "tet_cube_3_jit", "quad_rve_8_s3_lc2"])
def test_mixed_precision_refinement(case, ctx, native_lib):
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    u, reac, info = model.linear_static(A, rtol=1e-8, maxit=100000, precision=native_lib.PREC_MIXED)
    assert info.status == 0 and info.achieved <= 1e-8
    assert rel(u, g["s1_u"]) < 1e-5


def test_larger_mesh_pattern_and_residual(ctx, native_lib, oracle):
    """40x8x8 jittered cantilever: pattern bit-exact vs the oracle, values, and
    the FP64 solution's true residual."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(40, 8, 8, jitter=0.2, seed=9)
    md = oracle.mesh_dict(mesh)
    neq, _, eq = oracle.number_equations(mesh.bc_mask)
    loc = oracle.location_arrays(mesh.conn, eq)
    rp, ci = oracle.build_pattern(neq, loc)
    val = oracle.assemble_tangent(md, loc, neq, rp, ci)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    u, reac, info = model.linear_static(A, rtol=1e-10, maxit=100000)
    grp, gci = A.pattern()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
    assert rel(A.values(), val) < 1e-12
    x = u[eq > 0]
    order = np.argsort(eq[eq > 0])
    x = x[order]
    b = mesh.nodal_load[eq > 0][order]
    r = b - oracle.spmv(rp, ci, val, x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-9


def test_failure_status_not_converged(ctx, native_lib):
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(10, 3, 3)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    u, reac, info = model.linear_static(A, rtol=1e-14, maxit=3)
    assert info.status == -5 and info.iterations <= 3 + 16


def test_failure_nan_rhs_is_breakdown(ctx, native_lib, oracle):
    g = load_golden("quad_rve_8_s3_lc0")
    neq, _, eq = oracle.number_equations(g["bc_mask"])
    loc = oracle.location_arrays(g["conn"], eq)
    A = native_lib.GpuCsrMtrx(ctx)
    A.build_internal_structure(neq, loc)
    A.assemble_begin()
    for e in range(g["conn"].shape[0]):
        m = g["mats"][g["elem_mat"][e]]
        A.assemble(loc[e], oracle.elem_stiffness(2, g["coords"][g["conn"][e]], oracle.isole_d(2, m[1], m[2])))
    A.assemble_end()
    b = np.ones(neq)
    b[3] = np.nan
    x = np.zeros(neq)
    code = A.lib.ogb_pcg_solve(A.h, b.ctypes.data_as(__import__("ctypes").c_void_p),
                               x.ctypes.data_as(__import__("ctypes").c_void_p), 1e-10, 1000, 0, None)
    assert code == -6


def test_zero_diagonal_detected(ctx, native_lib):
    A = native_lib.GpuCsrMtrx(ctx)
    A.build_internal_structure(4, np.array([[1, 2], [3, 4]], np.int32))
    A.assemble_begin()
    A.assemble([1, 2], np.array([[2.0, -1.0], [-1.0, 2.0]]))
    A.assemble_end()
    solver = native_lib.GpuPcgSolver(lstol=1e-10, lsiter=100)
    x = np.zeros(4)
    assert solver.solve(A, np.ones(4), x) == -7


def test_negative_tet_volume_rejected(ctx, native_lib):
    from oofem_gb300 import meshgen as mg
    mesh = mg.tet_cube_linear(2)
    mesh.conn[0] = mesh.conn[0][[0, 2, 1, 3]]
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    with pytest.raises(native_lib.OgbError) as ei:
        model.assemble_stiffness(A)
    assert ei.value.code == -8


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-6)])
def test_partially_constrained_nodes(precision, tol, ctx, native_lib, oracle):
    """x=L face with only u_x prescribed: active nodes with prescribed slots
    (identity rows in the node-block solver storage)."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_block_pull(10, 4, 3, jitter=0.2, seed=4, material=mg.Material(1, 210e9, 0.3),
                             end_disp=1e-3)
    ref = oracle.linear_static(oracle.mesh_dict(mesh), rtol=1e-14)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    u, reac, info = model.linear_static(A, rtol=1e-12 if precision == 0 else 1e-10, maxit=100000,
                                        precision=precision)
    assert info.status == 0
    assert rel(u, ref["u"]) < tol
    assert rel(reac, ref["reac"]) < tol


def test_sell_and_csr_operators_agree(ctx, native_lib, oracle):
    """The node-block solver storage and the CSR storage give the same solve."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(16, 4, 4, jitter=0.2, seed=2)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    model.assemble_stiffness(A)
    neq, _ = model.neq()
    eq = model.equations()
    b = np.zeros(neq)
    b[eq[eq > 0] - 1] = mesh.nodal_load[eq > 0]
    s = native_lib.GpuPcgSolver(lstol=1e-12, lsiter=100000)
    x1 = np.zeros(neq)
    assert s.solve(A, b, x1) == 0
    it1 = s.last.iterations
    A.set_at(1, 1, A.at(1, 1))   # any CSR-side mutation makes the solver use the CSR storage
    x2 = np.zeros(neq)
    assert s.solve(A, b, x2) == 0
    assert abs(s.last.iterations - it1) <= 2
    assert rel(x1, x2) < 1e-9


def test_mixed_precision_below_fp32_reach_finishes_in_fp64(ctx, native_lib):
    """A tolerance the FP32 operator cannot reach (1e-13): the mixed solve detects
    that the FP64 residual stopped falling and finishes with the FP64 PCG from its
    current solution; the result converges and matches the FP64 solve."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(24, 5, 5, jitter=0.2, seed=2)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    u64, r64, i64 = model.linear_static(A, rtol=1e-13, precision=native_lib.PREC_FP64)
    um, rm, im = model.linear_static(A, rtol=1e-13, precision=native_lib.PREC_MIXED)
    assert i64.status == 0 and im.status == 0
    assert im.achieved <= 1e-13
    assert rel(um, u64) < 1e-9


def test_spmv_forms_give_identical_results(native_lib):
    """The one-warp SpMV forms (plain loop, prefetching, TMA-staged) compute the
    same products in the same order: mixed and FP64 solves through each of them
    give bit-identical displacements and iteration counts."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(30, 6, 6, jitter=0.2, seed=4)
    out = {}
    for v in (1, 2, 3, 4):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_SPMV_VARIANT, v)
        model = native_lib.GpuModel(c, mesh)
        A = native_lib.GpuCsrMtrx(c)
        um, _, im = model.linear_static(A, rtol=1e-10, precision=native_lib.PREC_MIXED)
        u6, _, i6 = model.linear_static(A, rtol=1e-10, precision=native_lib.PREC_FP64)
        assert im.status == 0 and i6.status == 0
        out[v] = (um, im.iterations, u6, i6.iterations)
    for v in (2, 3, 4):
        assert np.array_equal(out[v][0], out[1][0]) and out[v][1] == out[1][1], v
        assert np.array_equal(out[v][2], out[1][2]) and out[v][3] == out[1][3], v


@pytest.mark.parametrize("kind", ["hex", "quad", "tet"])
def test_half_stored_fp32_operator(kind, native_lib, oracle):
    """Mixed solves through the half-stored FP32 operator (upper blocks stored,
    lower blocks applied as transposes) against the full FP32 copy and the
    oracle: both converge on the FP64 residual, agree with the oracle's solution
    to 1e-7, the half form is bitwise reproducible and reports form 8."""
    from oofem_gb300 import meshgen as mg
    mesh = {"hex": lambda: mg.hex_cantilever(30, 6, 6, jitter=0.2, seed=4),
            "quad": lambda: mg.quad_rve(40, seed=6),
            "tet": lambda: mg.tet_cube_linear(8, jitter=0.1, seed=2)}[kind]()
    ref = oracle.linear_static(oracle.mesh_dict(mesh), rtol=1e-13)
    out = {}
    for half in (0, 2, 2):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_SPMV_HALF, half)
        model = native_lib.GpuModel(c, mesh)
        A = native_lib.GpuCsrMtrx(c)
        u, reac, info = model.linear_static(A, rtol=1e-10, precision=native_lib.PREC_MIXED)
        assert info.status == 0 and info.achieved <= 1e-10
        assert rel(u, ref["u"]) < 1e-7, (half, rel(u, ref["u"]))
        assert rel(reac, ref["reac"]) < 1e-7
        assert (A.spmv_forms()[1] % 10 == 8) == bool(half)
        out.setdefault(half, []).append((u, info.iterations))
    assert np.array_equal(out[2][0][0], out[2][1][0]) and out[2][0][1] == out[2][1][1]
    with pytest.raises(native_lib.OgbError):
        native_lib.Context(0).set_option(native_lib.OPT_SPMV_HALF, 3)


@pytest.mark.parametrize("case", ["hex_cantilever_6x3x3_jit_ic", "quad_rve_8_s3_ic", "hex_cantilever_6x3x3_jit_ilu",
                                  "tet_cube_3_jit_ilu", "hex_cantilever_6x3x3_jit_void"])
def test_iml_preconditioners(case, ctx, native_lib, oracle):
    """lsprecond 4 (incomplete Cholesky) and 2 (column ILU): the reference's
    factorizations, level-scheduled triangular solves on the device; and 0
    (plain CG); against the
    reference's runs: CG iterations within one of its log line, displacements
    within 1e-9; the drop-in solver class gives the same on the assembled
    matrix. IC and ILU are FP64 only; the threshold ILU (3) is refused."""
    g = load_golden(case)
    mesh = mesh_from_golden(g)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    pc = int(g["lsprecond"])
    A.set_preconditioner(pc)
    u, reac, info = model.linear_static(A, rtol=float(g["lstol"]))
    assert info.status == 0
    assert abs(info.iterations - int(g["cg_nite"][0])) <= 1, (info.iterations, int(g["cg_nite"][0]))
    assert rel(u, g["s1_u"]) < 1e-9
    assert rel(reac, g["s1_reac"]) < 1e-9
    ref = oracle.linear_static(g, rtol=float(g["lstol"]), precond=pc)
    solver = native_lib.GpuPcgSolver(lstol=float(g["lstol"]), lsiter=100000, lsprecond=pc)
    x = np.zeros(ref["neq"])
    assert solver.solve(A, ref["b"], x) == 0
    assert abs(solver.last.iterations - ref["iters"]) <= 1
    assert rel(x, ref["x"]) < 1e-9
    if pc in (2, 4):
        with pytest.raises(native_lib.OgbError):
            model.linear_static(A, rtol=1e-8, precision=native_lib.PREC_MIXED)
    with pytest.raises(native_lib.OgbError):
        A.set_preconditioner(3)


@pytest.mark.parametrize("pc", [4, 2])
def test_iml_preconditioners_many_levels(pc, native_lib, oracle):
    """The level-scheduled solves (one cooperative launch per triangular solve,
    grid barrier between levels) on a mesh with ~150 levels per solve: IC and
    ILU CG against the oracle's IML CG with the same preconditioner, iterations
    within one and solutions within 1e-9."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(20, 4, 4, jitter=0.2, seed=7)
    c = native_lib.Context(0)
    model = native_lib.GpuModel(c, mesh)
    A = native_lib.GpuCsrMtrx(c)
    A.set_preconditioner(pc)
    u, reac, info = model.linear_static(A, rtol=1e-10)
    assert info.status == 0
    ref = oracle.linear_static(oracle.mesh_dict(mesh), rtol=1e-10, precond=pc)
    assert abs(info.iterations - ref["iters"]) <= 1, (info.iterations, ref["iters"])
    assert rel(u, ref["u"]) < 1e-9


@pytest.mark.parametrize("kind", ["hex", "quad", "tet"])
def test_block_jacobi_mixed_solve(kind, native_lib, oracle):
    """Mixed solves preconditioned by the FP32 inverses of the node diagonal
    blocks (block Jacobi, the default) against the scalar Jacobi ones and the
    oracle: both converge on the FP64 residual and agree with the oracle's
    solution to 1e-7; the block form is reported, bitwise reproducible, and
    takes no more iterations than the scalar form on these meshes."""
    from oofem_gb300 import meshgen as mg
    mesh = {"hex": lambda: mg.hex_cantilever(30, 6, 6, jitter=0.2, seed=4),
            "quad": lambda: mg.quad_rve(40, seed=6),
            "tet": lambda: mg.tet_cube_linear(8, jitter=0.1, seed=2)}[kind]()
    ref = oracle.linear_static(oracle.mesh_dict(mesh), rtol=1e-13)
    its = {}
    for bj in (0, 1, 1):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_MIXED_BLOCK_JACOBI, bj)
        model = native_lib.GpuModel(c, mesh)
        A = native_lib.GpuCsrMtrx(c)
        u, reac, info = model.linear_static(A, rtol=1e-10, precision=native_lib.PREC_MIXED)
        assert info.status == 0 and info.achieved <= 1e-10
        assert rel(u, ref["u"]) < 1e-7, (bj, rel(u, ref["u"]))
        assert rel(reac, ref["reac"]) < 1e-7
        assert A.last_block_jacobi() == bool(bj)
        its.setdefault(bj, []).append((info.iterations, u))
    assert its[1][0][0] == its[1][1][0] and np.array_equal(its[1][0][1], its[1][1][1])
    assert its[1][0][0] <= its[0][0][0], (its[1][0][0], its[0][0][0])
    # FP64 solves keep the reference's scalar diagonal preconditioner
    c = native_lib.Context(0)
    model = native_lib.GpuModel(c, mesh)
    A = native_lib.GpuCsrMtrx(c)
    model.linear_static(A, rtol=1e-10, precision=native_lib.PREC_FP64)
    assert not A.last_block_jacobi()


def mixed_solve(native_lib, mesh, rtol, **opts):
    c = native_lib.Context(0)
    for k, v in opts.items():
        c.set_option(getattr(native_lib, "OPT_" + k.upper()), v)
    model = native_lib.GpuModel(c, mesh)
    A = native_lib.GpuCsrMtrx(c)
    u, reac, info = model.linear_static(A, rtol=rtol, precision=native_lib.PREC_MIXED)
    assert info.status == 0 and info.achieved <= rtol, (opts, info.status, info.achieved)
    assert A.last_block_jacobi()
    return info.iterations, u, c.kernel_launches()


@pytest.mark.parametrize("kind", ["hex", "quad", "tet"])
def test_fused_update_and_fp32_increment(kind, native_lib, oracle):
    """The block-Jacobi update with the p update in the same cooperative launch
    gives bitwise the iterates of the two-launch form (same sums, same order) in
    one launch fewer per iteration; with the update's dot-product terms summed
    per thread in FP32, or the solution accumulated as an FP32 increment folded
    into the FP64 solution after every batch of iterations, the solve still
    converges on the FP64 residual to the oracle's solution."""
    from oofem_gb300 import meshgen as mg
    mesh = {"hex": lambda: mg.hex_cantilever(30, 6, 6, jitter=0.2, seed=4),
            "quad": lambda: mg.quad_rve(40, seed=6),
            "tet": lambda: mg.tet_cube_linear(8, jitter=0.1, seed=2)}[kind]()
    ref = oracle.linear_static(oracle.mesh_dict(mesh), rtol=1e-13)
    for x64 in (1, 2, 0, 3):
        it0, u0, l0 = mixed_solve(native_lib, mesh, 1e-10, mixed_x64=x64, fused_update=0)
        it1, u1, l1 = mixed_solve(native_lib, mesh, 1e-10, mixed_x64=x64, fused_update=1)
        assert it0 == it1 and np.array_equal(u0, u1), (x64, it0, it1)
        assert l1 < l0
        assert rel(u1, ref["u"]) < 1e-7, (x64, rel(u1, ref["u"]))


def test_fused_update_with_z_in_memory(native_lib):
    """A block range too long for shared memory (one block per SM on 741k active
    nodes: 4,875 nodes of z, 60 KB on 152 SMs) keeps z in memory in the fused
    form: still bitwise the two-launch form."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(150, 60, 80, jitter=0.2, seed=1)
    a = mixed_solve(native_lib, mesh, 1e-6, update_blocks=1, fused_update=0)
    b = mixed_solve(native_lib, mesh, 1e-6, update_blocks=1, fused_update=1)
    assert a[0] == b[0] and np.array_equal(a[1], b[1])



@pytest.mark.parametrize("kind", ["hex", "quad"])
def test_half_stored_forms_are_bitwise_equal(kind, native_lib):
    """The loop forms of the half-stored SpMV (registers bounded for 2 to 5
    resident blocks per SM, values of a group of blocks loaded before or among
    their products) run the same sums in the same order: the mixed solves
    give bitwise equal solutions and iteration counts, and the autotuner reports
    the form it chose."""
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(30, 6, 6, jitter=0.2, seed=4) if kind == "hex" else mg.quad_rve(60, seed=3)
    out = {}
    for f in (1, 2, 3, 4, 5, 6, 0):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_SPMV_HALF, 2)
        c.set_option(native_lib.OPT_HALF_FORM, f)
        model = native_lib.GpuModel(c, mesh)
        A = native_lib.GpuCsrMtrx(c)
        u, reac, info = model.linear_static(A, rtol=1e-10, precision=native_lib.PREC_MIXED)
        assert info.status == 0 and info.achieved <= 1e-10
        form = A.spmv_forms()[1]
        assert form % 10 == 8 and (form // 10 == f if f else 1 <= form // 10 <= 6)
        out[f] = (u, info.iterations)
    for f in (2, 3, 4, 5, 6, 0):
        assert np.array_equal(out[f][0], out[1][0]) and out[f][1] == out[1][1]


def test_option_ranges_are_checked(native_lib):
    """Tuning options outside their documented ranges are refused with OGB_E_ARG
    and leave the context usable."""
    c = native_lib.Context(0)
    for opt, bad in ((native_lib.OPT_HALF_FORM, 7), (native_lib.OPT_MIXED_X64, 4), (native_lib.OPT_BATCH_FORM, 3),
                     (native_lib.OPT_UPDATE_BLOCKS, 9), (native_lib.OPT_SPMV_HALF, 3), (native_lib.OPT_TANGENT_TC, 3)):
        with pytest.raises(native_lib.OgbError) as e:
            c.set_option(opt, bad)
        assert e.value.code == -1, (opt, e.value.code)
    for opt, good in ((native_lib.OPT_HALF_FORM, 6), (native_lib.OPT_MIXED_X64, 3), (native_lib.OPT_BATCH_FORM, 2),
                      (native_lib.OPT_UPDATE_BLOCKS, 8), (native_lib.OPT_FUSED_UPDATE, 0), (native_lib.OPT_BATCH_X64, 1)):
        c.set_option(opt, good)
