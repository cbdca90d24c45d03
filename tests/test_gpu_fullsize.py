"""The large linear workload at its full size (290x58x58 LSpace cantilever, 3.03 M
free DOFs), checked through properties that do not need an oracle solve of that
size: the CompCol pattern's size (closed form for a structured grid), global
equilibrium of the reactions with the applied load, linearity of the solution
in the load, agreement of the mixed-precision and FP64 solutions, and bitwise
reproducibility of a solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY, NZ = 290, 58, 58


@pytest.fixture(scope="module")
def full(native_lib):
    from oofem_gb300 import meshgen as mg
    mesh = mg.hex_cantilever(NX, NY, NZ, h=0.05, jitter=0.2, seed=0)
    ctx = native_lib.Context(0)
    model = native_lib.GpuModel(ctx, mesh)
    A = native_lib.GpuCsrMtrx(ctx)
    u64, r64, i64 = model.linear_static(A, rtol=1e-10, maxit=200000, precision=native_lib.PREC_FP64)
    return dict(mesh=mesh, ctx=ctx, model=model, A=A, u64=u64, r64=r64, info64=i64)


def test_pattern_size_closed_form(full):
    # 3 DOFs per node, 3x3 node blocks; x = 0 nodes fixed: a node couples to the
    # 3x3x3 neighbourhood, so nnz = 9 * sum_i cx(i) * sum_j cy(j) * sum_k cz(k)
    nnz = 9 * (3 * NX - 2) * (3 * NY + 1) * (3 * NZ + 1)
    assert full["A"].nnz == nnz
    assert full["model"].neq()[0] == NX * (NY + 1) * (NZ + 1) * 3


def test_equilibrium_of_reactions(full):
    m = full["mesh"]
    assert full["info64"].status == 0
    # internal forces sum to zero over the whole body, so the reactions (internal
    # minus external at prescribed DOFs) sum to minus the applied load
    tot_load = m.nodal_load.sum(axis=0)
    tot_reac = full["r64"].sum(axis=0)
    scale = np.abs(m.nodal_load).sum()
    assert np.abs(tot_reac + tot_load).max() / scale < 1e-7


def test_mixed_matches_fp64_and_is_reproducible(full, native_lib):
    model, A = full["model"], full["A"]
    u1, r1, i1 = model.linear_static(A, rtol=1e-10, maxit=200000, precision=native_lib.PREC_MIXED)
    u2, r2, i2 = model.linear_static(A, rtol=1e-10, maxit=200000, precision=native_lib.PREC_MIXED)
    assert i1.status == 0 and i1.achieved <= 1e-10
    assert np.array_equal(u1, u2) and i1.iterations == i2.iterations
    # displacements and reactions within 1e-8 of the FP64 drop-in's (both solves
    # to ||f - K u|| / ||f|| <= 1e-10 on the FP64 residual)
    scale = np.abs(full["u64"]).max()
    assert np.abs(u1 - full["u64"]).max() / scale < 1e-8
    assert np.abs(r1 - full["r64"]).max() / np.abs(full["r64"]).max() < 1e-8


def test_linearity_in_the_load(full, native_lib):
    """A load scaled by -2 (a power of two: every operation of the solve scales
    exactly, and the deterministic reductions keep their order) gives exactly
    -2 times the displacements, in the same number of iterations."""
    m, model, A = full["mesh"], full["model"], full["A"]
    u2, r2, info = model.linear_static(A, nodal_load=-2.0 * m.nodal_load, rtol=1e-10, maxit=200000,
                                       precision=native_lib.PREC_FP64)
    assert info.status == 0 and info.iterations == full["info64"].iterations
    assert np.array_equal(u2, -2.0 * full["u64"])


def test_rve_batch_full_size_equilibrium(native_lib):
    """The 256-RVE sweep (sides 32..256, three prescribed-strain load cases) in one
    mixed-precision batched solve: every pair converges on its FP64 residual, and
    each RVE's reactions balance (no external load: they sum to zero)."""
    from oofem_gb300 import meshgen as mg
    meshes = mg.rve_batch(256, seed=0)
    big, ns = mg.concat_meshes(meshes)
    ctx = native_lib.Context(0)
    model = native_lib.GpuModel(ctx, big)
    model.set_instances(ns)
    A = native_lib.GpuCsrMtrx(ctx)
    bcv = np.stack([np.concatenate([mg.rve_bc_values(m, lc) for m in meshes]) for lc in range(3)])
    u, reac, its, ach, st = model.batch_linear_static(A, bcv, rtol=1e-8, maxit=100000,
                                                      precision=native_lib.PREC_MIXED)
    assert (st == 0).all() and (ach <= 1e-8).all()
    for i, m in enumerate(meshes):
        sl = slice(ns[i], ns[i + 1])
        # sum_free residual <= sqrt(n_free) ||r|| <= sqrt(n_free) rtol ||b||, and ||b|| is
        # of the order of the reactions: the imbalance is bounded accordingly
        bound = 2.0 * np.sqrt(m.nfree) * 1e-8
        for lc in range(3):
            r = reac[lc, sl]
            assert np.abs(r.sum(axis=0)).max() / np.abs(r).sum() < bound, (i, lc)
