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
@pytest.mark.parametrize("mixed", [False, True])
def test_patch_decks_meet_their_rules(name, mixed, native_lib):
    from oofem_gb300 import deck as dk
    path = os.path.join(GOLDEN, name + ".in")
    d = dk.read_deck(path)
    steps = dk.run_deck(d, ctx=native_lib.Context(0), lstol=1e-12,
                        precision=native_lib.PREC_MIXED if mixed else native_lib.PREC_FP64)
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
