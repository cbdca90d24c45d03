"""Input decks run end to end on the GPU path (oofem_gb300.deck.run_deck): the
reference's PlaneStress2d and LTRSpace patch decks (rewritten fixtures carrying
the reference deck's errorcheck rules) and a StaticStructural MisesMat deck
against the reference's run of the same deck."""
import os

import numpy as np
import pytest

from conftest import load_golden
from test_gpu_linear import rel

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["patch100", "patch101", "patch300"])
@pytest.mark.parametrize("mode", ["direct", "pcg", "mixed"])
def test_patch_decks_meet_their_rules(name, mode, native_lib):
    """The decks ask for the default direct solver: as written they run the
    device LDL^T factorization; PCG to 1e-12 in FP64 and mixed precision meet
    the same rules."""
    from oofem_gb300 import deck as dk
    path = os.path.join(GOLDEN, name + ".in")
    d = dk.read_deck(path)
    steps = dk.run_deck(d, ctx=native_lib.Context(0), lstol=None if mode == "direct" else 1e-12,
                        precision=native_lib.PREC_MIXED if mode == "mixed" else native_lib.PREC_FP64)
    rules = dk.check_rules(path, d, steps)
    assert len(rules) >= 10
    assert all(ok for *_, ok in rules), [r for r in rules if not r[3]]


def test_static_structural_deck_matches_reference(native_lib):
    from oofem_gb300 import deck as dk
    g = load_golden("ss_mises_hex_5x2x2_accel")
    d = dk.read_deck(os.path.join(GOLDEN, "ss_mises_hex_5x2x2_accel.in"))
    steps = dk.run_deck(d, ctx=native_lib.Context(0), lstol=1e-13)
    assert len(steps) == int(g["nsteps"])
    for k, s in enumerate(steps, 1):
        assert s.time == float(g[f"s{k}_time"])
        assert abs(s.iterations - int(g[f"s{k}_nite"])) <= 1
        assert rel(s.u, g[f"s{k}_u"]) < 1e-7
        assert rel(s.reactions, g[f"s{k}_reac"]) < 1e-7


def test_static_structural_deck_direct_matches_reference(native_lib):
    """The same deck as written (lstype 0): the device factorization in every
    Newton iteration takes exactly the reference's iteration counts, fields
    within 1e-10."""
    from oofem_gb300 import deck as dk
    g = load_golden("ss_mises_hex_5x2x2_accel")
    d = dk.read_deck(os.path.join(GOLDEN, "ss_mises_hex_5x2x2_accel.in"))
    steps = dk.run_deck(d, ctx=native_lib.Context(0))
    assert len(steps) == int(g["nsteps"])
    for k, s in enumerate(steps, 1):
        assert s.iterations == int(g[f"s{k}_nite"]), (k, s.iterations, int(g[f"s{k}_nite"]))
        assert rel(s.u, g[f"s{k}_u"]) < 1e-10
        assert rel(s.reactions, g[f"s{k}_reac"]) < 1e-10


@pytest.mark.parametrize("case", ["hex_cantilever_6x3x3_jit_ic", "hex_cantilever_6x3x3_jit_ilu",
                                  "hex_cantilever_6x3x3_jit_void"])
def test_iterative_solver_deck_keeps_its_preconditioner(case, native_lib, tmp_path):
    """A LinearStatic deck for the IML solver (lstype 1 with lsprecond 4 / 2 / 0)
    runs with the same preconditioner: CG iterations within one of the
    reference's run of that deck, displacements within 1e-9."""
    import sys
    from oofem_gb300 import deck as dk
    from test_gpu_linear import mesh_from_golden
    sys.path.insert(0, GOLDEN)
    from decks import write_deck
    g = load_golden(case)
    path = str(tmp_path / (case + ".in"))
    write_deck(mesh_from_golden(g), path, "LinearStatic nsteps 1 lstype 1 smtype 2 lstol 1e-10 lsiter 100000 "
               f"lsprecond {int(g['lsprecond'])}")
    steps = dk.run_deck(dk.read_deck(path), ctx=native_lib.Context(0))
    assert abs(steps[0].iterations - int(g["cg_nite"][0])) <= 1, (steps[0].iterations, int(g["cg_nite"][0]))
    assert rel(steps[0].u, g["s1_u"]) < 1e-9
