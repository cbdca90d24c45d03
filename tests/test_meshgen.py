import numpy as np

from oofem_gb300 import meshgen as mg


def test_cantilever_sizes():
    m = mg.hex_cantilever(20, 4, 4)
    assert m.nnodes == 525 and m.nelem == 320 and m.nfree == 1500
    m2 = mg.hex_cantilever(200, 40, 40)
    assert m2.nfree == 1008600


def test_hex_orientation_positive_jacobian():
    from oracle import oracle as O
    m = mg.hex_cantilever(5, 3, 2, jitter=0.2, seed=3)
    D = O.isole_d(1, 210e9, 0.3)
    for e in range(m.nelem):
        ke = O.elem_stiffness(1, m.coords[m.conn[e]], D)
        assert np.all(np.diag(ke) > 0)


def test_tets_positive_after_jitter():
    m = mg.tet_cube(6, jitter=0.15, seed=2)
    assert m.nelem == 6 * 6 ** 3
    assert (mg.tet_det_ref(m.coords[m.conn]) > 0).all()


def test_interior_jitter_keeps_boundary_planar():
    m = mg.hex_cantilever(6, 3, 3, jitter=0.2, seed=1)
    x = m.coords
    assert np.allclose(x[np.isclose(x[:, 0], 0.0), 0], 0.0)
    assert np.allclose(np.sort(np.unique(np.round(x[x[:, 1] < 1e-12, 1], 12))), [0.0])


def test_rve_boundary_strain():
    m = mg.quad_rve(16, seed=4, load_case=2)
    bnd = m.bc_mask[:, 0] == 1
    assert np.allclose(m.bc_value[bnd, 0], 5e-4 * m.coords[bnd, 1])
    assert np.allclose(m.bc_value[bnd, 1], 5e-4 * m.coords[bnd, 0])
    assert set(np.unique(m.elem_mat)) <= {0, 1}


def test_concat_meshes_offsets_and_materials():
    from oofem_gb300 import meshgen as mg
    a = mg.quad_rve(3, seed=1)
    b = mg.quad_rve(5, seed=2)
    big, ns = mg.concat_meshes([a, b])
    assert list(ns) == [0, a.nnodes, a.nnodes + b.nnodes]
    assert big.nelem == a.nelem + b.nelem
    assert (big.conn[:a.nelem] == a.conn).all()
    assert (big.conn[a.nelem:] == b.conn + a.nnodes).all()
    # materials concatenated, element indices shifted by the first mesh's table
    assert len(big.materials) == len(a.materials) + len(b.materials)
    assert (big.elem_mat[a.nelem:] == b.elem_mat + len(a.materials)).all()
    assert (big.bc_mask[ns[1]:] == b.bc_mask).all()
    # every element's nodes lie in one instance
    inst = np.searchsorted(ns, big.conn, side="right") - 1
    assert (inst == inst[:, :1]).all()


def test_rve_batch_is_seeded_and_in_range():
    from oofem_gb300 import meshgen as mg
    r1 = mg.rve_batch(6, seed=4, side_min=5, side_max=9)
    r2 = mg.rve_batch(6, seed=4, side_min=5, side_max=9)
    sides = [int(round(np.sqrt(m.nelem))) for m in r1]
    assert all(5 <= n <= 9 for n in sides)
    assert all((x.coords == y.coords).all() and (x.elem_mat == y.elem_mat).all() for x, y in zip(r1, r2))
