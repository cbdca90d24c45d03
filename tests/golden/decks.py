"""Write a :class:`oofem_gb300.meshgen.Mesh` as an OOFEM text input deck.

Used only to produce golden fixtures with the reference executable
(tests/golden/make_golden.py). Record syntax follows the reference's input
manual (doc/oofemInput) and its own decks (tests/sm/*.in).
"""
from __future__ import annotations

import numpy as np

from oofem_gb300 import meshgen as mg


def _f(v) -> str:
    """Shortest round-trip text of a float (numpy scalars included)."""
    return repr(float(v))


def _mat_record(i: int, m: mg.Material) -> str:
    if m.kind == mg.MAT_ISOLE:
        return f"IsoLE {i} d 1.0 E {_f(m.E)} n {_f(m.nu)} talpha 0.0"
    if m.kind == mg.MAT_MISES:
        return f"MisesMat {i} d 1.0 E {_f(m.E)} n {_f(m.nu)} sig0 {_f(m.sig0)} H {_f(m.H)} talpha 0.0"
    if m.kind == mg.MAT_IDM1:
        return (f"idm1 {i} d 1.0 E {_f(m.E)} n {_f(m.nu)} talpha 0.0 e0 {_f(m.e0)} gf {_f(m.gf)} "
                f"equivstraintype 0 damlaw 0")
    raise ValueError(m.kind)


def write_deck(mesh: mg.Mesh, path: str, analysis: str, nsteps: int = 1,
               bc_ltf: int = 1, load_ltf: int = 1, extra_funcs=()) -> None:
    """``analysis`` is the analysis record without nmodules; one ``refdump``
    export module is appended. ``bc_ltf``/``load_ltf`` pick the time function
    of the prescribed values and of the nodal loads; function 1 is constant 1,
    ``extra_funcs`` are further time-function records (numbered from 2)."""
    et = mesh.elem_type
    ndpn = mesh.ndofpn
    nn, ne = mesh.nnodes, mesh.nelem
    lines = [path.rsplit("/", 1)[-1].replace(".in", ".out"), "golden deck",
             f"{analysis} nmodules 1", "refdump tstep_all",
             "domain " + ("2dPlaneStress" if et == mg.ELEM_PLANESTRESS2D else "3d"),
             "OutputManager"]
    # boundary conditions: one record per distinct (dof-mask, values) group
    bc_groups = {}
    for n in range(nn):
        mask = tuple(int(v) for v in mesh.bc_mask[n])
        if not any(mask):
            continue
        dofs = tuple(d + 1 for d in range(ndpn) if mask[d])
        vals = tuple(float(mesh.bc_value[n, d]) for d in range(ndpn) if mask[d])
        bc_groups.setdefault((dofs, vals), []).append(n + 1)
    load_groups = {}
    for n in range(nn):
        f = tuple(float(v) for v in mesh.nodal_load[n])
        if any(v != 0.0 for v in f):
            load_groups.setdefault(f, []).append(n + 1)
    mats = mesh.materials
    ncs = len(mats)
    nbc = len(bc_groups) + len(load_groups)
    nltf = 1 + len(extra_funcs)
    nset = ncs + nbc
    lines.append(f"ndofman {nn} nelem {ne} ncrosssect {ncs} nmat {len(mats)} nbc {nbc} "
                 f"nic 0 nltf {nltf} nset {nset}")
    for n in range(nn):
        c = " ".join(repr(float(v)) for v in mesh.coords[n])
        lines.append(f"node {n + 1} coords {mesh.ndim} {c}")
    name = mg.ELEM_NAMES[et]
    for e in range(ne):
        c = " ".join(str(int(v) + 1) for v in mesh.conn[e])
        lines.append(f"{name} {e + 1} nodes {mesh.nnpe} {c}")
    for i in range(ncs):
        thick = f" thick {_f(mesh.thickness)}" if et == mg.ELEM_PLANESTRESS2D else ""
        lines.append(f"SimpleCS {i + 1}{thick} material {i + 1} set {i + 1}")
    for i, m in enumerate(mats):
        lines.append(_mat_record(i + 1, m))
    setid = ncs
    sets = []
    k = 0
    for (dofs, vals), nodes in bc_groups.items():
        k += 1
        setid += 1
        lines.append(f"BoundaryCondition {k} loadTimeFunction {bc_ltf} dofs {len(dofs)} "
                     + " ".join(map(str, dofs)) + f" values {len(vals)} "
                     + " ".join(repr(v) for v in vals) + f" set {setid}")
        sets.append(f"Set {setid} nodes {len(nodes)} " + " ".join(map(str, nodes)))
    for f, nodes in load_groups.items():
        k += 1
        setid += 1
        lines.append(f"NodalLoad {k} loadTimeFunction {load_ltf} dofs {ndpn} "
                     + " ".join(str(d + 1) for d in range(ndpn)) + f" Components {ndpn} "
                     + " ".join(repr(v) for v in f) + f" set {setid}")
        sets.append(f"Set {setid} nodes {len(nodes)} " + " ".join(map(str, nodes)))
    lines.append("ConstantFunction 1 f(t) 1.0")
    lines.extend(extra_funcs)
    for i in range(ncs):
        els = np.nonzero(mesh.elem_mat == i)[0] + 1
        lines.append(f"Set {i + 1} elements {len(els)} " + " ".join(map(str, els)))
    lines.extend(sets)
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
