"""The input-deck reader (oofem_gb300.deck) on CPU: decks written by the golden
deck writer read back to the same mesh, the committed fixture decks, the
reference's own patch decks (when the reference tree is present) solved by the
oracle against their embedded errorcheck rules, per-condition time functions,
metasteps and the errors for records outside the supported set."""
import os

import numpy as np
import pytest

from oofem_gb300 import deck as dk
from oofem_gb300 import meshgen as mg

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
REF_SM = os.path.join(os.sep, "root", "reference", "tests", "sm")


def _write(tmp_path, mesh, name, analysis="StaticStructural nsteps 1", **kw):
    import sys
    sys.path.insert(0, GOLDEN)
    from decks import write_deck
    p = str(tmp_path / name)
    write_deck(mesh, p, analysis, **kw)
    return p


@pytest.mark.parametrize("kind", ["hex_mises", "quad_two_materials", "tet_idm1"])
def test_round_trip(kind, tmp_path):
    mesh = {"hex_mises": lambda: mg.hex_block_pull(4, 2, 2, jitter=0.2, seed=1, end_disp=1e-3,
                                                   material=mg.Material(mg.MAT_MISES, 210e9, 0.3, sig0=250e6,
                                                                        H=2e9)),
            "quad_two_materials": lambda: mg.quad_rve(6, seed=3, load_case=2),
            "tet_idm1": lambda: mg.tet_cube(2, jitter=0.1, seed=4, end_disp=1e-4,
                                            material=mg.Material(mg.MAT_IDM1, 30e9, 0.2, e0=1e-4, gf=100.0))}[kind]()
    d = dk.read_deck(_write(tmp_path, mesh, kind + ".in"))
    m = d.mesh
    assert m.elem_type == mesh.elem_type and d.analysis_type == "staticstructural"
    np.testing.assert_array_equal(m.coords, mesh.coords)
    np.testing.assert_array_equal(m.conn, mesh.conn)
    np.testing.assert_array_equal(m.bc_mask, mesh.bc_mask)
    np.testing.assert_array_equal(m.bc_value, mesh.bc_value)
    np.testing.assert_array_equal(m.nodal_load, mesh.nodal_load)
    assert m.thickness == mesh.thickness
    np.testing.assert_array_equal(m.material_table()[m.elem_mat], mesh.material_table()[mesh.elem_mat])
    np.testing.assert_array_equal(d.bc_value_at(1.0), mesh.bc_value)
    np.testing.assert_array_equal(d.nodal_load_at(7.0), mesh.nodal_load)


def test_fixture_decks():
    d = dk.read_deck(os.path.join(GOLDEN, "patch300.in"))
    assert d.mesh.elem_type == mg.ELEM_LTRSPACE and d.mesh.nnodes == 6 and d.mesh.nelem == 3
    d = dk.read_deck(os.path.join(GOLDEN, "patch100.in"))
    assert d.mesh.elem_type == mg.ELEM_PLANESTRESS2D and d.mesh.nnodes == 8 and d.mesh.nelem == 5
    d = dk.read_deck(os.path.join(GOLDEN, "ss_mises_hex_5x2x2_accel.in"))
    a = d.analysis
    assert (a.int("nsteps"), a.float("rtolf"), a.int("manrmsteps"), a.int("maxiter")) == (8, 1e-8, 2, 400)
    g = np.load(os.path.join(GOLDEN, "ss_mises_hex_5x2x2_accel.npz"))
    np.testing.assert_array_equal(d.mesh.coords, g["coords"])
    # PiecewiseLinFunction 0 -> 1 over t in [0, 8]
    np.testing.assert_allclose(d.bc_value_at(2.0), g["bc_value"] * 0.25)
    d = dk.read_deck(os.path.join(GOLDEN, "ss_idm1_tet_3.in"))
    g = np.load(os.path.join(GOLDEN, "ss_idm1_tet_3.npz"))
    assert d.mesh.elem_type == mg.ELEM_LTRSPACE and d.analysis.int("manrmsteps") == 1
    np.testing.assert_array_equal(d.mesh.conn, g["conn"])
    assert d.mesh.materials[0].kind == mg.MAT_IDM1 and d.mesh.materials[0].gf == 1000.0


@pytest.mark.skipif(not os.path.isdir(REF_SM), reason="reference tree not present")
@pytest.mark.parametrize("name", ["patch100", "patch101", "patch300"])
def test_reference_patch_decks_with_oracle(name, oracle):
    """The reference's own decks parsed as written and solved by the oracle:
    every #NODE / #REACTION rule of the deck holds within its tolerance."""
    path = os.path.join(REF_SM, name + ".in")
    d = dk.read_deck(path)
    r = oracle.linear_static(oracle.mesh_dict(d.mesh), rtol=1e-14)
    steps = [dk.DeckStep(1, 1.0, r["u"], r["reac"], r["iters"])]
    rules = dk.check_rules(path, d, steps)
    assert len(rules) >= 10 and all(ok for *_, ok in rules), [x for x in rules if not x[3]]


@pytest.mark.skipif(not os.path.isdir(REF_SM), reason="reference tree not present")
@pytest.mark.parametrize("name,msg", [("patch103", "StructTemperatureLoad"), ("patch105", "boundaryLoads"),
                                      ("Mises01", "truss1d"), ("idm11", "rtolv"),
                                      ("brick_nlgeo_1", "nlgeo 1")])
def test_reference_decks_outside_the_path_are_refused(name, msg):
    with pytest.raises(dk.DeckError, match=msg):
        dk.read_deck(os.path.join(REF_SM, name + ".in"))


DECK = """out.out
two conditions on two time functions
NonLinearStatic nsteps 1 nmsteps 1 nmodules 0
nsteps 3 rtolf 1e-6 controlmode 1 manrmsteps 1
domain 2dPlaneStress
OutputManager tstep_all dofman_all element_all
ndofman 4 nelem 1 ncrosssect 1 nmat 1 nbc 3 nic 0 nltf 2 nset 4
Node 1 coords 3 0.0 0.0 0.0
Node 2 coords 3 1.0 0.0 0.0
Node 3 coords 3 1.0 1.0 0.0
Node 4 coords 3 0.0 1.0 0.0 bc 2 0 0
PlaneStress2d 1 nodes 4 1 2 3 4
SimpleCS 1 thick 0.5 material 1 set 1
IsoLE 1 d 1.0 E 100.0 n 0.2 tAlpha 1e-5
BoundaryCondition 1 loadTimeFunction 1 dofs 2 1 2 values 2 0.0 0.0 set 2
BoundaryCondition 2 loadTimeFunction 2 dofs 1 1 values 1 0.01 set 3
NodalLoad 3 loadTimeFunction 1 dofs 2 1 2 Components 2 0.0 -2.0 set 4
ConstantFunction 1 f(t) 1.0
PiecewiseLinFunction 2 nPoints 3 t 3 0.0 1.0 3.0 f(t) 3 0.0 1.0 2.0
Set 1 elementranges {(1 1)}
Set 2 nodes 1 1
Set 3 noderanges {(2 3)}
Set 4 nodes 2 3 4
"""


def test_time_functions_metastep_and_sets(tmp_path):
    p = tmp_path / "two.in"
    p.write_text(DECK)
    d = dk.read_deck(str(p))
    a = d.analysis
    assert d.analysis_type == "nonlinearstatic" and a.int("nsteps") == 3 and a.int("manrmsteps") == 1
    m = d.mesh
    assert m.thickness == 0.5 and m.materials[0].E == 100.0
    np.testing.assert_array_equal(m.bc_mask, [[1, 1], [1, 0], [1, 0], [0, 0]])
    np.testing.assert_allclose(d.bc_value_at(2.0)[:, 0], [0.0, 0.015, 0.015, 0.0])   # 0.01 * f2(2) = 0.01 * 1.5
    np.testing.assert_allclose(d.nodal_load_at(2.0), [[0, 0], [0, 0], [0, -2.0], [0, -2.0]])
    bad = DECK.replace("IsoLE 1 d 1.0 E 100.0 n 0.2 tAlpha 1e-5", "MisesMat 1 d 1.0 E 100.0 n 0.2 sig0 1 htype 1")
    p.write_text(bad)
    with pytest.raises(dk.DeckError, match="MisesMat"):
        dk.read_deck(str(p))
    p.write_text(DECK.replace("loadTimeFunction 2", "loadTimeFunction 5"))
    with pytest.raises(dk.DeckError, match="time function 5"):
        dk.read_deck(str(p))


OLD_STYLE = """old.out
old-style references: node bc / load fields, element mat / crossSect fields
LinearStatic nsteps 1 nmodules 0
domain 3d
OutputManager tstep_all dofman_all element_all
ndofman 5 nelem 2 ncrosssect 1 nmat 1 nbc 3 nic 0 nltf 1
# a comment line inside the node block and a blank line

node 1 coords 3 0.0 0.0 0.0 bc 3 1 1 1
node 2 coords 3 1.0 0.0 0.0 bc 3 1 1 1
node 3 coords 3 0.0 1.0 0.0 bc 3 1 1 1
node 4 coords 3 0.0 0.0 1.0 bc 3 0 2 0 load 1 3
node 5 coords 3 1.0 1.0 1.0
LTRSpace 1 nodes 4 1 2 3 4 crossSect 1 mat 1
ltrspace 2 nodes 4 2 3 4 5 mat 1 crossSect 1
SimpleCS 1
IsoLE 1 d 1.0 E 10.0 n 0.2 tAlpha 0.0
BoundaryCondition 1 loadTimeFunction 1 prescribedvalue 0.0
BoundaryCondition 2 loadTimeFunction 1 prescribedvalue 0.5
NodalLoad 3 loadTimeFunction 1 Components 3 0.0 0.0 -1.0
ConstantFunction 1 f(t) 2.0
"""


def test_old_style_references(tmp_path):
    """Node-record `bc` / `load` references and element-record `mat` /
    `crossSect` fields (records the bulk reader flags and the general parser
    completes), comment and blank lines inside the node block."""
    p = tmp_path / "old.in"
    p.write_text(OLD_STYLE)
    d = dk.read_deck(str(p))
    m = d.mesh
    assert m.elem_type == mg.ELEM_LTRSPACE and m.nnodes == 5 and m.nelem == 2
    np.testing.assert_array_equal(m.bc_mask[:3], 1)
    np.testing.assert_array_equal(m.bc_mask[3], [0, 1, 0])
    assert m.bc_value[3, 1] == 0.5 and d.bc_value_at(0.0)[3, 1] == 1.0      # f(t) = 2
    np.testing.assert_array_equal(d.nodal_load_at(1.0)[3], [0.0, 0.0, -2.0])
    np.testing.assert_array_equal(m.conn, [[0, 1, 2, 3], [1, 2, 3, 4]])
    assert m.materials[m.elem_mat[1]].E == 10.0


def _parse_block(text, tmp_path, count, keyword, field, maxvals):
    import ctypes as C
    from oofem_gb300 import native
    lib = native.load()
    p = tmp_path / "blk.in"
    p.write_bytes(text.encode())
    ids = np.zeros(max(count, 1), np.int64)
    vals = np.zeros((max(count, 1), maxvals))
    nv = np.zeros(max(count, 1), np.int32)
    other = np.zeros(max(count, 1), np.uint8)
    nxt, lines = C.c_int64(), C.c_int64()
    code = lib.ogb_deck_parse_block(str(p).encode(), 0, count, keyword.encode(), field.encode(), maxvals,
                                    ids.ctypes.data, vals.ctypes.data, nv.ctypes.data, other.ctypes.data,
                                    C.byref(nxt), C.byref(lines))
    return code, ids, vals, nv, other, nxt.value, lines.value, lib


def test_bulk_block_reader(tmp_path):
    """ogb_deck_parse_block on its own: comments and blank lines skipped, values,
    counts and the further-fields flag per record, the offset after the block,
    case-insensitive keyword and field; the errors name the record."""
    text = "# c\n\nNODE 7 COORDS 2 1.5 -2e-3\nnode 8 bc 2 1 0 coords 3 1 2 3\nnext record\n"
    code, ids, vals, nv, other, nxt, lines, lib = _parse_block(text, tmp_path, 2, "node", "coords", 3)
    assert code == 0
    assert ids.tolist() == [7, 8] and nv.tolist() == [2, 3] and other.tolist() == [0, 1]
    np.testing.assert_array_equal(vals[0, :2], [1.5, -2e-3])
    np.testing.assert_array_equal(vals[1], [1.0, 2.0, 3.0])
    assert text.encode()[nxt:].startswith(b"next record") and lines == 4
    for bad, msg in [("elem 1 coords 1 0\n", "expected a node record"),
                     ("node 1 nodes 1 0\n", "field coords missing"),
                     ("node 1 coords 4 1 2 3 4\n", "bad coords count"),
                     ("node 1 coords 3 1 2\nnode 2 coords 3 1 2 3\n", "bad coords value"),
                     ("node x coords 1 0\n", "record number missing"),
                     ("node 1 coords 1 0\n", "deck ends inside a block")]:
        count = 2 if "deck ends" in msg or "bad coords value" in msg else 1
        code, *_, lib = _parse_block(bad, tmp_path, count, "node", "coords", 3)
        assert code == -1, bad
        assert msg in lib.ogb_last_error().decode(), (bad, lib.ogb_last_error())


@pytest.mark.parametrize("edit,msg", [("controlmode 1 manrmsteps 1", "linesearch 1"), ("nsteps 3 rtolf", "rtolv")])
def test_analysis_keys_outside_the_runner_are_refused(edit, msg, tmp_path):
    text = DECK.replace("nsteps 3 rtolf 1e-6 controlmode 1 manrmsteps 1",
                        "nsteps 3 rtolf 1e-6 controlmode 1 manrmsteps 1 linesearch 1" if "linesearch" in msg
                        else "nsteps 3 rtolv 1e-6 controlmode 1 manrmsteps 1")
    p = tmp_path / "k.in"
    p.write_text(text)
    with pytest.raises(dk.DeckError, match=msg.split()[0]):
        dk.read_deck(str(p))


def test_material_parameters_outside_the_model_are_refused(tmp_path):
    p = tmp_path / "m.in"
    p.write_text(DECK.replace("IsoLE 1 d 1.0 E 100.0 n 0.2 tAlpha 1e-5", "IsoLE 1 d 1.0 E 100.0 n 0.2 maxOmega 0.9"))
    with pytest.raises(dk.DeckError, match="maxOmega"):
        dk.read_deck(str(p))
