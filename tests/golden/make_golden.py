"""Generate golden fixtures from the reference executable itself.

Writes seeded synthetic meshes as OOFEM decks (tests/golden/decks.py), runs them
through oracle/_ref/ref_harness (which links the reference's liboofem and dumps
full-precision results), and stores mesh + results as tests/golden/<case>.npz.
It also extracts the golden values embedded in the reference's own patch deck
tests/sm/patch300.in into tests/golden/patch300.json.

Needs a reference build (``make -C oracle ref REF_SRC=... REF_BUILD=...``);
the committed fixtures are what the tests read, so this runs only when the
fixtures are regenerated:

    python tests/golden/make_golden.py [--ref-src DIR] [--work DIR]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oofem_gb300 import meshgen as mg  # noqa: E402
from decks import write_deck  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def parse_dump(path):
    steps = []
    K = None
    kes = {}
    cur = None
    with open(path) as fh:
        lines = fh.read().split("\n")
    i = 0
    while i < len(lines):
        ln = lines[i]
        i += 1
        if not ln:
            continue
        t = ln.split()
        if t[0] == "step":
            cur = {"step": int(t[1]), "time": float(t[2]), "nite": int(t[3]) if len(t) > 3 else 0,
                   "u": [], "gp": [], "reac": []}
            steps.append(cur)
        elif t[0] == "u":
            cur["u"].append((int(t[1]), int(t[2]), int(t[3]), float(t[4])))
        elif t[0] == "gp":
            si = t.index("s")
            ei = t.index("e")
            ki = t.index("k")
            s = [float(v) for v in t[si + 1:ei]]
            e = [float(v) for v in t[ei + 1:ki]]
            cur["gp"].append((int(t[1]), int(t[2]), s, e, float(t[ki + 1]), float(t[ki + 3]),
                              float(t[ki + 5])))
        elif t[0] == "reac":
            cur["reac"].append((int(t[1]), int(t[2]), float(t[3])))
        elif t[0] == "K":
            neq, nnz = int(t[1]), int(t[2])
            colptr = np.array(lines[i].split()[1:], dtype=np.int64)
            rowind = np.array(lines[i + 1].split()[1:], dtype=np.int32)
            val = np.array(lines[i + 2].split()[1:], dtype=np.float64)
            i += 3
            assert colptr.size == neq + 1 and rowind.size == nnz == val.size
            K = (neq, colptr, rowind, val)
        elif t[0] == "ke":
            n = int(t[2])
            kes[int(t[1])] = np.array(t[3:], dtype=np.float64).reshape(n, n)
    return steps, K, kes


def mesh_arrays(mesh: mg.Mesh) -> dict:
    return dict(etype=np.int32(mesh.elem_type), coords=mesh.coords, conn=mesh.conn,
                elem_mat=mesh.elem_mat, mats=mesh.material_table(), bc_mask=mesh.bc_mask,
                bc_value=mesh.bc_value, nodal_load=mesh.nodal_load,
                thickness=np.float64(mesh.thickness))


def step_arrays(mesh: mg.Mesh, step: dict, prefix: str) -> dict:
    nn, nd = mesh.nnodes, mesh.ndofpn
    u = np.zeros((nn, nd))
    eq = np.zeros((nn, nd), np.int32)
    for node, dof, e, v in step["u"]:
        u[node - 1, dof - 1] = v
        eq[node - 1, dof - 1] = e
    ngp = {1: 8, 2: 4, 3: 1}[mesh.elem_type]
    ns = 3 if mesh.elem_type == mg.ELEM_PLANESTRESS2D else 6
    sig = np.zeros((mesh.nelem, ngp, ns))
    eps = np.zeros((mesh.nelem, ngp, ns))
    kap = np.zeros((mesh.nelem, ngp))
    om = np.zeros((mesh.nelem, ngp))
    le = np.zeros((mesh.nelem, ngp))
    for el, g, s, e, k, w, l in step["gp"]:
        sig[el - 1, g - 1] = s
        eps[el - 1, g - 1] = e
        kap[el - 1, g - 1] = k
        om[el - 1, g - 1] = w
        le[el - 1, g - 1] = l
    reac = np.zeros((nn, nd))
    for node, dof, v in step["reac"]:
        reac[node - 1, dof - 1] = v
    return {f"{prefix}u": u, f"{prefix}eq": eq, f"{prefix}stress": sig, f"{prefix}strain": eps,
            f"{prefix}kappa": kap, f"{prefix}omega": om, f"{prefix}le": le,
            f"{prefix}reac": reac, f"{prefix}time": np.float64(step["time"]),
            f"{prefix}nite": np.int32(step["nite"])}


def run_case(name, mesh, work, analysis="LinearStatic nsteps 1", dumpK=True, extra=None, **deck_kw):
    deck = os.path.join(work, name + ".in")
    dump = os.path.join(work, name + ".dump")
    write_deck(mesh, deck, analysis, **deck_kw)
    cmd = [HARNESS, "-f", deck, "-o", dump] + (["-K"] if dumpK else [])
    res = subprocess.run(cmd, cwd=work, capture_output=True, text=True)
    if res.returncode != 0:
        print(res.stdout[-3000:], res.stderr[-3000:])
        raise RuntimeError(f"reference run failed for {name}")
    log = res.stdout
    steps, K, kes = parse_dump(dump)
    out = mesh_arrays(mesh)
    out["nsteps"] = np.int32(len(steps))
    for k, v in (extra or {}).items():
        out[k] = v
    for k, st in enumerate(steps):
        out.update(step_arrays(mesh, st, f"s{k + 1}_"))
    if K is not None:
        neq, colptr, rowind, val = K
        out.update(K_colptr=colptr, K_rowind=rowind, K_val=val, neq=np.int32(neq))
    for e, ke in kes.items():
        out[f"ke{e}"] = ke
    cg = re.findall(r"CG\(\w+\): flag=(\d+), nite (\d+), achieved tol\. (\S+)", log)
    if cg:
        out["cg_nite"] = np.array([int(c[1]) for c in cg], np.int32)
    nr = re.findall(r"Equilibrium reached in\s+(\d+) iterations", log)
    if nr:
        out["nr_iters"] = np.array([int(v) for v in nr], np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: steps={len(steps)} neq={K[0] if K else '-'}")


def patch300(ref_src):
    """Golden values embedded in the reference's LTRSpace patch test deck."""
    path = os.path.join(ref_src, "tests", "sm", "patch300.in")
    rules = {"nodes": [], "reactions": []}
    for ln in open(path):
        m = re.match(r"#NODE tStep 1 number (\d+) dof (\d+) unknown d value (\S+)", ln)
        if m:
            rules["nodes"].append([int(m[1]), int(m[2]), float(m[3])])
        m = re.match(r"#REACTION tStep 1 number (\d+) dof (\d+) value (\S+)", ln)
        if m:
            rules["reactions"].append([int(m[1]), int(m[2]), float(m[3])])
        m = re.match(r"#%BEGIN_CHECK% tolerance (\S+)", ln)
        if m:
            rules["tolerance"] = float(m[1])
    rules["source"] = "tests/sm/patch300.in"
    with open(os.path.join(HERE, "patch300.json"), "w") as fh:
        json.dump(rules, fh, indent=1)


def reference_patch_decks(ref_src):
    """The reference's PlaneStress2d / LTRSpace patch decks (tests/sm/patch100.in, patch101.in,
    patch300.in) read with oofem_gb300.deck, rewritten by decks.write_deck, with the deck's own
    errorcheck rules (#NODE / #REACTION lines and the tolerance) appended as comment lines, so the GPU
    tests can run them through the deck reader without the reference tree."""
    from oofem_gb300 import deck as dk
    for name in ("patch100", "patch101", "patch300"):
        src = os.path.join(ref_src, "tests", "sm", name + ".in")
        d = dk.read_deck(src)
        out = os.path.join(HERE, name + ".in")
        write_deck(d.mesh, out, "StaticStructural nsteps 1")
        rules = [ln.strip() for ln in open(src)
                 if re.match(r"#(NODE|REACTION|%BEGIN_CHECK%)", ln.strip())]
        with open(out, "a") as fh:
            fh.write("# errorcheck rules of tests/sm/%s.in\n" % name)
            fh.write("\n".join(rules) + "\n")
        print(f"{name}: {len(rules)} rule lines")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True, help="reference source tree (its tests/sm decks)")
    ap.add_argument("--work", default=os.path.join(ROOT, "_work", "golden"))
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    os.makedirs(args.work, exist_ok=True)
    patch300(args.ref_src)
    reference_patch_decks(args.ref_src)
    def nonlinear(name, mesh, nsteps, rtolf=1e-8, maxiter=100, initial_guess=0):
        analysis = (f"NonLinearStatic nsteps {nsteps} controlmode 1 rtolf {rtolf!r} maxiter {maxiter} "
                    f"manrmsteps 1 stiffmode 0" + (" initialguess 1" if initial_guess else ""))
        ramp = f"PiecewiseLinFunction 2 nPoints 2 t 2 0.0 {float(nsteps)!r} f(t) 2 0.0 1.0"
        run_case(name, mesh, args.work, analysis=analysis, dumpK=False, bc_ltf=2, load_ltf=2,
                 extra_funcs=(ramp,), extra=dict(rtolf=np.float64(rtolf), ramp_steps=np.int32(nsteps),
                                                 maxiter=np.int32(maxiter),
                                                 initial_guess=np.int32(initial_guess)))

    def static_structural(name, mesh, nsteps, deltat=1.0, rtolf=1e-8, maxiter=400, manrmsteps=None,
                          ramp_time=None):
        # StaticStructural with the reference's defaults: nrsolver, IG_Tangent,
        # modified Newton unless manrmsteps is given
        analysis = (f"StaticStructural nsteps {nsteps} deltat {deltat!r} rtolf {rtolf!r} maxiter {maxiter}"
                    + (f" manrmsteps {manrmsteps}" if manrmsteps is not None else ""))
        tend = nsteps * deltat if ramp_time is None else ramp_time
        ramp = f"PiecewiseLinFunction 2 nPoints 2 t 2 0.0 {float(tend)!r} f(t) 2 0.0 1.0"
        run_case(name, mesh, args.work, analysis=analysis, dumpK=False, bc_ltf=2, load_ltf=2,
                 extra_funcs=(ramp,), extra=dict(rtolf=np.float64(rtolf), ramp_time=np.float64(tend),
                                                 deltat=np.float64(deltat), maxiter=np.int32(maxiter),
                                                 manrmsteps=np.int32(-1 if manrmsteps is None else manrmsteps)))
        # the deck itself, for the deck-reader tests
        with open(os.path.join(args.work, name + ".in")) as src, open(os.path.join(HERE, name + ".in"), "w") as dst:
            dst.write(src.read())

    ey = 250e6 / 210e9
    cases = {
        "hex_cantilever_20x4x4": lambda: run_case(
            "hex_cantilever_20x4x4", mg.hex_cantilever(20, 4, 4), args.work),
        "hex_cantilever_6x3x3_jit": lambda: run_case(
            "hex_cantilever_6x3x3_jit", mg.hex_cantilever(6, 3, 3, jitter=0.2, seed=7), args.work),
        "quad_rve_8_s3": lambda: [run_case(
            f"quad_rve_8_s3_lc{lc}", mg.quad_rve(8, seed=3, load_case=lc), args.work) for lc in range(3)],
        # IML CG with the incomplete-Cholesky and with no preconditioner (lsprecond 4 / 0), CompCol matrix
        "hex_cantilever_6x3x3_jit_ic": lambda: run_case(
            "hex_cantilever_6x3x3_jit_ic", mg.hex_cantilever(6, 3, 3, jitter=0.2, seed=7), args.work,
            analysis="LinearStatic nsteps 1 lstype 1 smtype 2 lstol 1e-10 lsiter 100000 lsprecond 4",
            extra=dict(lsprecond=np.int32(4), lstol=np.float64(1e-10))),
        "quad_rve_8_s3_ic": lambda: run_case(
            "quad_rve_8_s3_ic", mg.quad_rve(8, seed=3, load_case=2), args.work,
            analysis="LinearStatic nsteps 1 lstype 1 smtype 2 lstol 1e-10 lsiter 100000 lsprecond 4",
            extra=dict(lsprecond=np.int32(4), lstol=np.float64(1e-10))),
        "hex_cantilever_6x3x3_jit_ilu": lambda: run_case(
            "hex_cantilever_6x3x3_jit_ilu", mg.hex_cantilever(6, 3, 3, jitter=0.2, seed=7), args.work,
            analysis="LinearStatic nsteps 1 lstype 1 smtype 2 lstol 1e-10 lsiter 100000 lsprecond 2",
            extra=dict(lsprecond=np.int32(2), lstol=np.float64(1e-10))),
        "tet_cube_3_jit_ilu": lambda: run_case(
            "tet_cube_3_jit_ilu", mg.tet_cube_linear(3, jitter=0.15, seed=5), args.work,
            analysis="LinearStatic nsteps 1 lstype 1 smtype 2 lstol 1e-10 lsiter 100000 lsprecond 2",
            extra=dict(lsprecond=np.int32(2), lstol=np.float64(1e-10))),
        "hex_cantilever_6x3x3_jit_void": lambda: run_case(
            "hex_cantilever_6x3x3_jit_void", mg.hex_cantilever(6, 3, 3, jitter=0.2, seed=7), args.work,
            analysis="LinearStatic nsteps 1 lstype 1 smtype 2 lstol 1e-10 lsiter 100000 lsprecond 0",
            extra=dict(lsprecond=np.int32(0), lstol=np.float64(1e-10))),
        "tet_cube_3_jit": lambda: run_case(
            "tet_cube_3_jit", mg.tet_cube_linear(3, jitter=0.15, seed=5), args.work),
        "mises_hex_4x2x2": lambda: nonlinear(
            "mises_hex_4x2x2", mg.hex_block_pull(4, 2, 2, h=0.05, jitter=0.2, seed=3,
                                                 material=mg.Material(mg.MAT_MISES, 210e9, 0.3, sig0=250e6, H=2e9),
                                                 end_disp=3 * ey * 0.2), 6),
        "mises_hex_6x3x3": lambda: nonlinear(
            "mises_hex_6x3x3", mg.hex_block_pull(6, 3, 3, h=0.05, jitter=0.2, seed=8,
                                                 material=mg.Material(mg.MAT_MISES, 210e9, 0.3, sig0=250e6, H=2e9),
                                                 end_disp=4 * ey * 0.3), 8),
        "mises_hex_10x3x3_ig": lambda: nonlinear(
            "mises_hex_10x3x3_ig", mg.hex_block_pull(10, 3, 3, h=0.05, jitter=0.2, seed=9,
                                                     material=mg.Material(mg.MAT_MISES, 210e9, 0.3, sig0=250e6,
                                                                          H=2e9),
                                                     end_disp=3 * ey * 0.5), 10, initial_guess=1),
        "ss_mises_hex_6x3x3": lambda: static_structural(
            "ss_mises_hex_6x3x3", mg.hex_block_pull(6, 3, 3, h=0.05, jitter=0.2, seed=12,
                                                    material=mg.Material(mg.MAT_MISES, 210e9, 0.3, sig0=250e6,
                                                                         H=2e9),
                                                    end_disp=3 * ey * 0.3), 5, deltat=0.5),
        "ss_mises_hex_5x2x2_accel": lambda: static_structural(
            "ss_mises_hex_5x2x2_accel", mg.hex_block_pull(5, 2, 2, h=0.05, jitter=0.2, seed=13,
                                                          material=mg.Material(mg.MAT_MISES, 210e9, 0.3,
                                                                               sig0=250e6, H=2e9),
                                                          end_disp=3 * ey * 0.25), 8, manrmsteps=2),
        "ss_idm1_tet_3": lambda: static_structural(
            "ss_idm1_tet_3", mg.tet_cube(3, jitter=0.15, seed=6,
                                         material=mg.Material(mg.MAT_IDM1, 30e9, 0.2, e0=1e-4, gf=1000.0),
                                         end_disp=3e-4), 5, rtolf=1e-6, maxiter=400, manrmsteps=1, ramp_time=6.0),
        "idm1_tet_3": lambda: nonlinear(
            "idm1_tet_3", mg.tet_cube(3, jitter=0.15, seed=5,
                                      material=mg.Material(mg.MAT_IDM1, 30e9, 0.2, e0=1e-4, gf=1000.0),
                                      end_disp=3e-4), 6, rtolf=1e-6, maxiter=400),
    }
    for name, fn in cases.items():
        if args.only and args.only not in name:
            continue
        fn()


if __name__ == "__main__":
    main()
