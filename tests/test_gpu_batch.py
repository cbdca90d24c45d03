"""Batched solves (independent meshes x load cases in one batched PCG) against
the oracle's separate LinearStatic runs and against the single-mesh GPU path.

Each (instance, load case) pair runs its own CG with its own convergence test,
so its iteration count is that of a separate solve (within one or two
iterations: the batched dot products sum in another order) and its
displacements agree with the oracle's to the solve tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


@pytest.fixture(scope="module")
def ctx(native_lib):
    return native_lib.Context(0)


def _oracle_case(oracle, mesh, bc_value, load, rtol):
    m = oracle.mesh_dict(mesh)
    m["bc_value"] = bc_value
    m["nodal_load"] = load
    return oracle.linear_static(m, rtol=rtol)


def test_rve_batch_three_load_cases(ctx, native_lib, oracle):
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(5, seed=3, side_min=4, side_max=24)
    meshes.append(mg.quad_rve(1, seed=7))            # no free DOF at all
    meshes.insert(2, mg.quad_rve(37, seed=11))       # spans two 1024-row blocks
    big, ns = mg.concat_meshes(meshes)
    model = native_lib.GpuModel(ctx, big)
    model.set_instances(ns)
    A = native_lib.GpuCsrMtrx(ctx)
    nrhs = 3
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(nrhs)])
    rtol = 1e-13
    u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=rtol)
    assert (st == 0).all(), st
    assert (ach <= rtol).all()
    for i, m in enumerate(meshes):
        sl = slice(ns[i], ns[i + 1])
        for lc in range(nrhs):
            ref = _oracle_case(oracle, m, mg.rve_bc_values(m, lc), np.zeros_like(m.bc_value), rtol)
            assert ref["status"] == 0
            assert abs(int(its[i, lc]) - ref["iters"]) <= 2, (i, lc, its[i, lc], ref["iters"])
            assert rel(u[lc, sl], ref["u"]) < 1e-9, (i, lc)
            assert rel(reac[lc, sl], ref["reac"]) < 1e-9, (i, lc)
    assert (its[len(meshes) - 1] == 0).all()       # the all-prescribed RVE converges at once


def test_hex_batch_two_rhs_matches_single_solves(ctx, native_lib):
    """3-D path (3x3 node blocks): two jittered cantilevers of different size,
    two load cases (the nodal load and a scaled, reversed one)."""
    from oofem_gb300 import meshgen as mg
    meshes = [mg.hex_cantilever(10, 3, 3, jitter=0.2, seed=1), mg.hex_cantilever(14, 4, 3, jitter=0.2, seed=2)]
    big, ns = mg.concat_meshes(meshes)
    model = native_lib.GpuModel(ctx, big)
    model.set_instances(ns)
    A = native_lib.GpuCsrMtrx(ctx)
    loads = np.stack([big.nodal_load, -0.5 * big.nodal_load])
    bcv = np.stack([big.bc_value, big.bc_value])
    rtol = 1e-12
    u, reac, its, ach, st = model.batch_linear_static(A, bcv, loads, rtol=rtol)
    assert (st == 0).all()
    for i, m in enumerate(meshes):
        single = native_lib.GpuModel(ctx, m)
        B = native_lib.GpuCsrMtrx(ctx)
        for c, f in enumerate((1.0, -0.5)):
            us, rs, info = single.linear_static(B, nodal_load=f * m.nodal_load, rtol=rtol)
            assert info.status == 0
            assert abs(int(its[i, c]) - info.iterations) <= 2
            sl = slice(ns[i], ns[i + 1])
            assert rel(u[c, sl], us) < 1e-9
            assert rel(reac[c, sl], rs) < 1e-9
    # linearity across the two load cases: u(-0.5 f) = -0.5 u(f) to the solve tolerance
    assert rel(u[1], -0.5 * u[0]) < 1e-9


def test_batch_is_deterministic(ctx, native_lib):
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(4, seed=5, side_min=8, side_max=40)
    big, ns = mg.concat_meshes(meshes)
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    out = []
    for _ in range(2):
        model = native_lib.GpuModel(ctx, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(ctx)
        out.append(model.batch_linear_static(A, bcv, rtol=1e-10)[0])
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("kind", ["quad", "tet"])
def test_batched_spmv_forms_are_bitwise_equal(kind, native_lib):
    """Batched mixed solves with the FP32 SpMV values loaded among the products
    (form 1) or every value of a group loaded first (form 2), and timed (0):
    the same sums in the same order, bitwise equal solutions."""
    from oofem_gb300 import meshgen as mg
    if kind == "quad":
        meshes = mg.rve_batch(4, seed=5, side_min=8, side_max=40)
        big, ns = mg.concat_meshes(meshes)
        bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    else:
        meshes = [mg.tet_cube_linear(6, jitter=0.1, seed=s) for s in (1, 2)]
        big, ns = mg.concat_meshes(meshes)
        bcv = big.bc_value[None]
    out = {}
    for form in (1, 2, 0):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_BATCH_FORM, form)
        model = native_lib.GpuModel(c, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(c)
        out[form] = model.batch_linear_static(A, bcv, rtol=1e-9, precision=native_lib.PREC_MIXED)[0]
    assert np.array_equal(out[1], out[2]) and np.array_equal(out[1], out[0])


def test_batched_block_jacobi(native_lib):
    """Batched mixed solves of two-DOF-per-node meshes precondition with the FP32
    inverses of the 2 x 2 node blocks (the partner row's residual taken from the
    neighbouring lane) unless the option turns it off: both forms converge on the
    FP64 residual to the FP64 batched solution, the block form is reported, and
    its total iteration count is not above the scalar diagonal's (5 % slack)."""
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(6, seed=11, side_min=8, side_max=48)
    big, ns = mg.concat_meshes(meshes)
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    c = native_lib.Context(0)
    model = native_lib.GpuModel(c, big)
    model.set_instances(ns)
    A = native_lib.GpuCsrMtrx(c)
    ref = model.batch_linear_static(A, bcv, rtol=1e-10)[0]
    tot = {}
    for bj in (0, 1):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_MIXED_BLOCK_JACOBI, bj)
        model = native_lib.GpuModel(c, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(c)
        u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=1e-9, precision=native_lib.PREC_MIXED)
        assert (st == 0).all() and (ach <= 1e-9).all()
        assert rel(u, ref) < 1e-6, (bj, rel(u, ref))
        assert A.last_block_jacobi() == bool(bj)
        tot[bj] = int(its.sum())
    print("batched mixed iterations, scalar / block Jacobi:", tot[0], tot[1])
    assert tot[1] <= 1.05 * tot[0], tot


def test_batched_kernel_timing_keeps_the_solve(native_lib):
    """With kernel timing on, a batched mixed solve times one more SpMV launch
    (every pair running), which recomputes q, p.q and alpha of the same search
    directions: the solution is bitwise that of the untimed solve, and the
    sample is reported with its time and algorithmic bytes."""
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(3, seed=7, side_min=8, side_max=32)
    big, ns = mg.concat_meshes(meshes)
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    out = []
    for prof in (False, True):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_BATCH_FORM, 1)
        if prof:
            c.profile(True)
            c.profile_read()
        model = native_lib.GpuModel(c, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(c)
        u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=1e-9, precision=native_lib.PREC_MIXED)
        assert (st == 0).all()
        out.append(u)
        if prof:
            ms, n, by = c.profile_read()
            assert n == 1 and ms > 0 and by > 0, (ms, n, by)
    assert np.array_equal(out[0], out[1])


def test_batched_fp32_increment(native_lib):
    """Batched mixed solves with the solution accumulated as an FP32 increment
    folded into the FP64 solution after every batch of iterations (the default)
    or in FP64 every iteration converge on the FP64 residual to the FP64 batched
    solution."""
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(4, seed=3, side_min=8, side_max=40)
    big, ns = mg.concat_meshes(meshes)
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    c = native_lib.Context(0)
    model = native_lib.GpuModel(c, big)
    model.set_instances(ns)
    A = native_lib.GpuCsrMtrx(c)
    ref = model.batch_linear_static(A, bcv, rtol=1e-10)[0]
    for x64 in (0, 1):
        c = native_lib.Context(0)
        c.set_option(native_lib.OPT_BATCH_X64, x64)
        model = native_lib.GpuModel(c, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(c)
        u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=1e-9, precision=native_lib.PREC_MIXED)
        assert (st == 0).all() and (ach <= 1e-9).all()
        assert rel(u, ref) < 1e-6, (x64, rel(u, ref))


def test_set_instances_rejects_coupled_and_late(ctx, native_lib):
    from oofem_gb300 import meshgen as mg
    m = mg.quad_rve(6, seed=1)
    model = native_lib.GpuModel(ctx, m)
    with pytest.raises(native_lib.OgbError) as e:
        model.set_instances([0, 20, m.nnodes])      # cuts through elements
    assert e.value.code == -8
    with pytest.raises(native_lib.OgbError) as e:
        model.set_instances([0, m.nnodes + 1])
    assert e.value.code == -1
    A = native_lib.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    with pytest.raises(native_lib.OgbError) as e:
        model.set_instances([0, m.nnodes])
    assert e.value.code == -3


def test_rve_batch_mixed_precision(ctx, native_lib, oracle):
    """Mixed precision batch: FP32 matrix and Krylov vectors, FP64 solution,
    convergence decided on the FP64 residual; displacements within 1e-6 of the
    oracle's FP64 solve, every pair's FP64 relative residual <= rtol."""
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(5, seed=4, side_min=6, side_max=30)
    meshes.append(mg.quad_rve(1, seed=2))
    big, ns = mg.concat_meshes(meshes)
    model = native_lib.GpuModel(ctx, big)
    model.set_instances(ns)
    A = native_lib.GpuCsrMtrx(ctx)
    nrhs = 3
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(nrhs)])
    rtol = 1e-10
    u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=rtol, precision=native_lib.PREC_MIXED)
    assert (st == 0).all(), st
    assert (ach <= rtol).all(), ach
    for i, m in enumerate(meshes):
        sl = slice(ns[i], ns[i + 1])
        for lc in range(nrhs):
            ref = _oracle_case(oracle, m, mg.rve_bc_values(m, lc), np.zeros_like(m.bc_value), 1e-13)
            assert rel(u[lc, sl], ref["u"]) < 1e-6, (i, lc, rel(u[lc, sl], ref["u"]))
            assert rel(reac[lc, sl], ref["reac"]) < 1e-6, (i, lc)


def test_hex_batch_mixed_matches_fp64(ctx, native_lib):
    from oofem_gb300 import meshgen as mg
    meshes = [mg.hex_cantilever(12, 3, 3, jitter=0.2, seed=3), mg.hex_cantilever(8, 4, 4, jitter=0.2, seed=4)]
    big, ns = mg.concat_meshes(meshes)
    loads = np.stack([big.nodal_load, 2.0 * big.nodal_load])
    bcv = np.stack([big.bc_value, big.bc_value])
    out = {}
    for prec in (native_lib.PREC_FP64, native_lib.PREC_MIXED):
        model = native_lib.GpuModel(ctx, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(ctx)
        u, reac, its, ach, st = model.batch_linear_static(A, bcv, loads, rtol=1e-10, precision=prec)
        assert (st == 0).all() and (ach <= 1e-10).all()
        out[prec] = u
    assert rel(out[native_lib.PREC_MIXED], out[native_lib.PREC_FP64]) < 1e-6


def test_solve_multi_matches_single_solves(ctx, native_lib, oracle):
    """SparseLinearSystemNM::solve(A, B, X) with five right-hand sides: batched on a
    model-assembled matrix (4 + 1 columns), the column loop on a location-array
    matrix; both against separate single solves."""
    from oofem_gb300 import meshgen as mg
    m = mg.hex_cantilever(8, 3, 3, jitter=0.2, seed=5)
    model = native_lib.GpuModel(ctx, m)
    A = native_lib.GpuCsrMtrx(ctx)
    model.build_matrix(A)
    model.assemble_stiffness(A)
    neq = model.neq()[0]
    rng = np.random.default_rng(0)
    B = rng.standard_normal((5, neq))
    solver = native_lib.GpuPcgSolver(lstol=1e-12, lsiter=100000)
    X = np.zeros_like(B)
    assert solver.solve_multi(A, B, X) == 0
    its, ach, st = solver.last_multi
    assert (st == 0).all() and (ach <= 1e-12).all()
    for c in range(5):
        x = np.zeros(neq)
        assert solver.solve(A, B[c], x) == 0
        assert abs(int(its[c]) - solver.last.iterations) <= 2
        assert rel(X[c], x) < 1e-9
    # location-array matrix (no node-block copy): the column loop
    nq, _, eq = oracle.number_equations(m.bc_mask)
    loc = oracle.location_arrays(m.conn, eq)
    L = native_lib.GpuCsrMtrx(ctx)
    L.build_internal_structure(nq, loc)
    L.assemble_begin()
    for e in range(m.nelem):
        ke = oracle.elem_stiffness(1, m.coords[m.conn[e]], oracle.isole_d(1, m.materials[0].E, m.materials[0].nu))
        L.assemble(loc[e], ke)
    L.assemble_end()
    X2 = np.zeros_like(B)
    assert solver.solve_multi(L, B, X2) == 0
    assert rel(X2, X) < 1e-9
    # mixed precision through the same entry point
    mixed = native_lib.GpuPcgSolver(lstol=1e-10, lsiter=100000, precision=native_lib.PREC_MIXED)
    X3 = np.zeros_like(B)
    assert mixed.solve_multi(A, B, X3) == 0
    assert (mixed.last_multi[1] <= 1e-10).all()
    assert rel(X3, X) < 1e-6


def test_batch_mixed_below_fp32_reach_finishes_in_fp64(ctx, native_lib):
    """Mixed batch at 1e-13: pairs whose FP64 residual stops falling under the
    FP32 operator finish in an FP64 pass from their current solution; every pair
    converges and agrees with the FP64 batch."""
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(3, seed=9, side_min=10, side_max=30)
    big, ns = mg.concat_meshes(meshes)
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    out = {}
    for prec in (native_lib.PREC_FP64, native_lib.PREC_MIXED):
        model = native_lib.GpuModel(ctx, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(ctx)
        u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=1e-13, precision=prec)
        assert (st == 0).all(), (prec, st)
        out[prec] = u
    assert rel(out[native_lib.PREC_MIXED], out[native_lib.PREC_FP64]) < 1e-9


def test_rve_batch_mixed_small_rves_reliable(ctx, native_lib, oracle):
    """Small RVEs (6..30 elements a side) in a mixed batch: every pair's FP64
    replacements keep its CG recurrence consistent, so the iteration counts stay
    near the FP64 batch's and the displacements agree with the oracle to 1e-6
    (a batch that replaced running pairs' residuals under a stale direction
    diverged here and ended on a drifted recursive residual)."""
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(4, seed=8, side_min=6, side_max=30)
    big, ns = mg.concat_meshes(meshes)
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    out = {}
    for prec in (native_lib.PREC_FP64, native_lib.PREC_MIXED):
        model = native_lib.GpuModel(ctx, big)
        model.set_instances(ns)
        A = native_lib.GpuCsrMtrx(ctx)
        u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=1e-10, precision=prec)
        assert (st == 0).all() and (ach <= 1e-10).all()
        out[prec] = (u, its)
    u, its = out[native_lib.PREC_MIXED]
    assert (its <= 1.5 * out[native_lib.PREC_FP64][1] + 16).all(), (its, out[native_lib.PREC_FP64][1])
    for i, m in enumerate(meshes):
        sl = slice(ns[i], ns[i + 1])
        for lc in range(3):
            ref = _oracle_case(oracle, m, mg.rve_bc_values(m, lc), np.zeros_like(m.bc_value), 1e-13)
            assert rel(u[lc, sl], ref["u"]) < 1e-6, (i, lc)
