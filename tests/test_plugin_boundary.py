"""The OOFEM-side binding (oofem_gb300/plugin/oofem_gb300_plugin.C) compiles
against the reference's headers, links against a reference build, and takes
over the class factory: the reference executable run on an unchanged deck with
`smtype 11 lstype 9` constructs GpuCsrMtrx (without a GPU it then stops at
context creation, which is what this CPU test checks). Skipped unless
OOFEM_REF_SRC and OOFEM_REF_BUILD name a reference source tree and build."""
import os
import subprocess

import pytest

from conftest import ROOT

REF_SRC = os.environ.get("OOFEM_REF_SRC", "")
REF_BUILD = os.environ.get("OOFEM_REF_BUILD", "")

pytestmark = pytest.mark.skipif(
    not (REF_SRC and REF_BUILD and os.path.isdir(os.path.join(REF_SRC, "src"))
         and os.path.exists(os.path.join(REF_BUILD, "liboofem.so"))),
    reason="needs OOFEM_REF_SRC (reference source tree) and OOFEM_REF_BUILD (a reference build)")


def test_plugin_registers_through_the_class_factory(tmp_path, native_lib):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from decks import write_deck
    from oofem_gb300 import meshgen as mg
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "plugin", f"REF_SRC={REF_SRC}",
                        f"REF_BUILD={REF_BUILD}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    deck = str(tmp_path / "gpu.in")
    write_deck(mg.hex_cantilever(4, 2, 2), deck, "LinearStatic nsteps 1 smtype 11 lstype 9 lstol 1e-10 lsiter 1000")
    with open(deck) as fh:
        text = fh.read().replace("nmodules 1", "nmodules 0").replace("refdump tstep_all\n", "")
    with open(deck, "w") as fh:
        fh.write(text)
    env = dict(os.environ)
    env["LD_PRELOAD"] = os.path.join(ROOT, "oracle", "_ref", "liboofem_gb300_plugin.so")
    env["LD_LIBRARY_PATH"] = REF_BUILD + ":" + os.path.join(ROOT, "oofem_gb300")
    r = subprocess.run([os.path.join(REF_BUILD, "oofem"), "-f", deck], capture_output=True, text=True, env=env,
                       cwd=str(tmp_path), timeout=120)
    out = r.stdout + r.stderr
    # the preload worked (no loader error) and the class factory built the plugin's matrix
    assert "cannot be preloaded" not in out and "error while loading shared libraries" not in out, out[-2000:]
    assert "GpuCsrMtrx: constructed by the class factory (smtype 11)" in out, out[-2000:]
    # without a GPU the run then stops at CUDA context creation, with the library's own message
    import torch
    if not torch.cuda.is_available():
        assert r.returncode != 0 and "liboofem_gb300: cudaSetDevice" in out, out[-2000:]
