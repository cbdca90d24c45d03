"""Reader for OOFEM text input decks, limited to what this library runs, and a
runner that executes a deck on the GPU path.

Accepted (anything else raises DeckError naming the record):
  analysis   LinearStatic, NonLinearStatic (controlmode 1), StaticStructural
             (solvertype nrsolver) with their step, NRSolver and linear-solver keys
  nodes      Node (coords; old-style `bc` / `load` references)
  elements   LSpace, PlaneStress2d, LTRSpace (one type per deck)
  sections   SimpleCS (thick, material, set; or the element's crossSect / mat)
  materials  IsoLE, MisesMat (htype 0, no damage), idm1 (Mazars, exponential
             cohesive law)
  loads      BoundaryCondition (dofs / values / set, or prescribedvalue with node
             `bc` references), NodalLoad (dofs / components / set, or node `load`)
  functions  ConstantFunction, PiecewiseLinFunction
  sets       nodes, noderanges, elements, elementranges, allelements

Record syntax follows the reference's reader (src/core/oofemtxtdatareader.C,
oofemtxtinputrecord.C, src/core/tokenizer.C): one record per line, `#` starts a
comment line, keywords are matched without regard to case, an array field is a
count followed by that many values, a range field is `{(a b) c ...}`. Component
order after the counts record: dof managers, elements, cross sections,
materials, boundary conditions and loads, initial conditions, functions, sets
(Domain::instanciateYourself, src/core/domain.C:485-700).
"""
from __future__ import annotations

import builtins
import dataclasses
import re
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import meshgen as mg
from .engng import ConstantFunction, PiecewiseLinFunction

ELEMENT_TYPES = {"lspace": mg.ELEM_LSPACE, "planestress2d": mg.ELEM_PLANESTRESS2D, "ltrspace": mg.ELEM_LTRSPACE}
NODES_PER_ELEMENT = {mg.ELEM_LSPACE: 8, mg.ELEM_PLANESTRESS2D: 4, mg.ELEM_LTRSPACE: 4}
# lstype values of the reference's direct solvers (linsystsolvertype.h:47-57: ST_Direct, ST_Spooles,
# ST_DSS, ST_MKLPardiso, ST_SuperLU_MT, ST_PardisoProjectOrg): decks asking for one run the device
# LDL^T factorization
DIRECT_LSTYPES = (0, 2, 4, 6, 7, 8)


class DeckError(ValueError):
    pass


_TOKEN = re.compile(r"""\{[^}]*\}|"[^"]*"|'[^']*'|\S+""")


def _tokens(line: str) -> List[str]:
    """Whitespace tokens; `{...}` range groups and quoted strings stay one token."""
    if line.count("{") != line.count("}"):
        raise DeckError(f"unterminated range in: {line[:80]}")
    return [t[1:-1] if t[0] in "\"'" and len(t) > 1 and t[-1] == t[0] else t for t in _TOKEN.findall(line)]


def _ranges(tok: str) -> List[int]:
    """`{(1 4) 7 (9 10)}` -> [1, 2, 3, 4, 7, 9, 10]."""
    body = tok.strip()[1:-1]
    out = []
    for a, b, single in re.findall(r"\(\s*(-?\d+)\s+(-?\d+)\s*\)|(-?\d+)", body):
        if single:
            out.append(int(single))
        else:
            out.extend(range(int(a), int(b) + 1))
    return out


class Record:
    def __init__(self, text: str, lineno: int):
        self.text, self.lineno = text, lineno
        self.tok = _tokens(text)
        if not self.tok:
            raise DeckError(f"line {lineno}: empty record")
        self.keyword = self.tok[0].lower()
        self.number: Optional[int] = None
        if len(self.tok) > 1 and re.fullmatch(r"-?\d+", self.tok[1]):
            self.number = int(self.tok[1])
        self._low = [t.lower() for t in self.tok]

    def _at(self, key: str) -> Optional[int]:
        key = key.lower()
        start = 2 if self.number is not None else 1
        for i in range(start, len(self._low)):
            if self._low[i] == key:
                return i
        return None

    def has(self, key: str) -> bool:
        return self._at(key) is not None

    def _value(self, key: str, k: int = 1) -> str:
        i = self._at(key)
        if i is None or i + k >= len(self.tok):
            raise DeckError(f"line {self.lineno}: field '{key}' missing in: {self.text}")
        return self.tok[i + k]

    def int(self, key: str, default=None) -> int:
        if not self.has(key):
            if default is None:
                raise DeckError(f"line {self.lineno}: field '{key}' missing in: {self.text}")
            return default
        return int(self._value(key))

    def float(self, key: str, default=None) -> float:
        if not self.has(key):
            if default is None:
                raise DeckError(f"line {self.lineno}: field '{key}' missing in: {self.text}")
            return default
        return float(self._value(key))

    def array(self, key: str, kind=builtins.float) -> list:
        i = self._at(key)
        if i is None:
            raise DeckError(f"line {self.lineno}: field '{key}' missing in: {self.text}")
        n = int(self.tok[i + 1])
        vals = self.tok[i + 2:i + 2 + n]
        if len(vals) != n:
            raise DeckError(f"line {self.lineno}: field '{key}' has fewer than {n} values")
        if n > 64:   # long lists (sets): converted in one numpy call
            return np.array(vals, dtype=np.int64 if kind is int else np.float64).tolist()
        return [kind(v) for v in vals]

    def ranges(self, key: str) -> List[int]:
        return _ranges(self._value(key))


def _check_fields(r: Record, fields: Dict[str, str], allowed_values: Dict[str, tuple] = None):
    """Every field of the record must be one of `fields` (name -> "array" for a
    counted list, "scalar" for one value); a field listed in allowed_values must
    hold one of those values. Anything else is a feature outside this reader."""
    allowed_values = allowed_values or {}
    i = 2 if r.number is not None else 1
    while i < len(r.tok):
        key = r._low[i]
        kind = fields.get(key)
        if kind is None:
            raise DeckError(f"line {r.lineno}: field '{r.tok[i]}' of {r.tok[0]} is not supported")
        if kind == "array":
            try:
                n = int(r.tok[i + 1])
            except (IndexError, ValueError):
                raise DeckError(f"line {r.lineno}: bad count of '{r.tok[i]}'") from None
            i += 2 + n
        else:
            if key in allowed_values and (i + 1 >= len(r.tok) or r.tok[i + 1] not in allowed_values[key]):
                raise DeckError(f"line {r.lineno}: {r.tok[i]} {r.tok[i + 1] if i + 1 < len(r.tok) else ''} "
                                f"of {r.tok[0]} is not supported")
            i += 2


@dataclasses.dataclass
class Deck:
    output: str
    description: str
    analysis: Record
    mesh: mg.Mesh
    node_ids: np.ndarray                 # deck number of each node (row of the mesh arrays)
    elem_ids: np.ndarray
    bc_ltf: np.ndarray                   # (nnodes, ndofpn) time function of each prescribed DOF (0: none)
    load_terms: List[Tuple[np.ndarray, int]]   # (nodal load pattern, time function)
    functions: Dict[int, object]

    @property
    def analysis_type(self) -> str:
        return self.analysis.keyword

    def bc_value_at(self, t: float) -> np.ndarray:
        """Prescribed values at time t: value x f_ltf(t) per DOF."""
        out = np.zeros_like(self.mesh.bc_value)
        for f, fn in self.functions.items():
            sel = self.bc_ltf == f
            if sel.any():
                out[sel] = self.mesh.bc_value[sel] * fn.evaluate_at_time(t)
        return out

    def nodal_load_at(self, t: float) -> np.ndarray:
        out = np.zeros_like(self.mesh.nodal_load)
        for pattern, f in self.load_terms:
            out += pattern * self.functions[f].evaluate_at_time(t)
        return out


class _Reader:
    """Record lines of a deck with their line numbers and byte offsets."""

    def __init__(self, path: str):
        self.path = path
        self.fh = open(path, "rb")
        self.lineno = 0

    def close(self):
        self.fh.close()

    def next(self, what: str) -> Tuple[int, str]:
        while True:
            b = self.fh.readline()
            if not b:
                raise DeckError(f"{self.path}: deck ends before the {what}")
            self.lineno += 1
            s = b.decode().strip()
            if s and not s.startswith("#"):
                return self.lineno, s

    def peek_keyword(self) -> str:
        pos, line = self.fh.tell(), self.lineno
        try:
            return self.next("block")[1].split(None, 1)[0].lower()
        finally:
            self.fh.seek(pos)
            self.lineno = line

    def block(self, count: int, keyword: str, field: str, maxvals: int):
        """`count` records `<keyword> <n> ... <field> k v1..vk ...` through the
        library's bulk reader; records with further fields are read in full."""
        from . import native
        import ctypes as C
        lib = native.load()
        ids = np.zeros(count, np.int64)
        vals = np.zeros((count, maxvals))
        nv = np.zeros(count, np.int32)
        other = np.zeros(count, np.uint8)
        start, first_line = self.fh.tell(), self.lineno
        nxt, lines = C.c_int64(), C.c_int64()
        code = lib.ogb_deck_parse_block(self.path.encode(), start, count, keyword.encode(), field.encode(), maxvals,
                                        ids.ctypes.data, vals.ctypes.data, nv.ctypes.data, other.ctypes.data,
                                        C.byref(nxt), C.byref(lines))
        if code != 0:
            raise DeckError(f"{self.path} after line {first_line}: {lib.ogb_last_error().decode()}")
        full: Dict[int, Record] = {}
        if other.any():
            want = set(np.nonzero(other)[0].tolist())
            k = 0
            while k < count:
                ln, text = self.next("block")
                if k in want:
                    full[k] = Record(text, ln)
                k += 1
        self.fh.seek(nxt.value)
        self.lineno = first_line + lines.value
        return ids, vals, nv, full


def read_deck(path: str) -> Deck:
    rd = _Reader(path)
    try:
        return _read(rd, path)
    finally:
        rd.close()


def _read(rd: "_Reader", path: str) -> Deck:
    nxt = rd.next

    output = nxt("output file name")[1]
    description = nxt("description")[1]
    analysis = Record(*reversed(nxt("analysis record")))
    if analysis.keyword not in ("linearstatic", "nonlinearstatic", "staticstructural"):
        raise DeckError(f"analysis '{analysis.tok[0]}' is not supported (LinearStatic, NonLinearStatic, "
                        f"StaticStructural)")
    nms = analysis.int("nmsteps", 0)
    if nms > 1:
        raise DeckError("several metasteps are not supported")
    if nms == 1:
        # one metastep: its record (step count, solver keys) completes the analysis record
        _, ms_text = nxt("metastep record")
        rest = analysis.text.split(None, 1)
        analysis = Record(rest[0] + " " + ms_text + (" " + rest[1] if len(rest) > 1 else ""), analysis.lineno)
    # analysis and solver keys whose semantics this runner does not implement
    for key, ok in (("linesearch", ("0",)), ("rtold", None), ("rtolv", None), ("ddm", None), ("ddv", None),
                    ("stiffmode", ("0",)), ("miniter", ("0",)), ("initialguess", ("0", "1"))):
        if analysis.has(key) and (ok is None or analysis._value(key) not in ok):
            raise DeckError(f"analysis key '{key} {analysis._value(key)}' is not supported")
    for _ in range(analysis.int("nmodules", 0)):
        nxt("export modules")
    dom = Record(*reversed(nxt("domain record")))
    if dom.keyword != "domain":
        raise DeckError(f"line {dom.lineno}: expected the domain record")
    dtype = dom.tok[1].lower() if len(dom.tok) > 1 else "3d"
    om = Record(*reversed(nxt("output manager record")))
    if om.keyword != "outputmanager":
        raise DeckError(f"line {om.lineno}: expected the OutputManager record")
    comp = Record(*reversed(nxt("component counts")))
    counts = dict.fromkeys(("ndofman", "nelem", "ncrosssect", "nmat", "nbc", "nic", "nltf", "nset", "nbarrier"), 0)
    for i in range(len(comp.tok) - 1):   # the record starts with its first count
        if comp._low[i] in counts:
            counts[comp._low[i]] = int(comp.tok[i + 1])
    if counts["nic"]:
        raise DeckError("initial conditions are not supported")

    def block(n, what):
        return [Record(*reversed(nxt(what))) for _ in range(n)]

    nn, ne = counts["ndofman"], counts["nelem"]
    if nn == 0 or ne == 0:
        raise DeckError(f"{path}: no nodes or no elements")
    node_ids, node_vals, node_nv, node_full = rd.block(nn, "node", "coords", 3)
    ekw = rd.peek_keyword()
    if ekw not in ELEMENT_TYPES:
        raise DeckError(f"elements '{ekw}': one of LSpace, PlaneStress2d, LTRSpace per deck is supported")
    elem_ids, elem_vals, elem_nv, elem_full = rd.block(ne, ekw, "nodes", 8)
    sections = block(counts["ncrosssect"], "cross sections")
    mats = block(counts["nmat"], "materials")
    block(counts["nbarrier"], "nonlocal barriers")
    bcs = block(counts["nbc"], "boundary conditions")
    funcs = block(counts["nltf"], "functions")
    sets = block(counts["nset"], "sets")

    # element type and dimensions
    et = ELEMENT_TYPES[ekw]
    ndim = 2 if et == mg.ELEM_PLANESTRESS2D else 3
    nd = mg.DOFS_PER_NODE[et]
    if et == mg.ELEM_PLANESTRESS2D and dtype not in ("2dplanestress", "planestress2d"):
        raise DeckError(f"PlaneStress2d needs domain 2dPlaneStress, not '{dtype}'")

    # nodes
    if (node_nv < ndim).any():
        raise DeckError(f"node {int(node_ids[np.argmax(node_nv < ndim)])}: fewer than {ndim} coordinates")
    coords = np.ascontiguousarray(node_vals[:, :ndim])
    order = np.argsort(node_ids, kind="stable")
    sorted_ids = node_ids[order]
    if (np.diff(sorted_ids) == 0).any():
        raise DeckError("duplicate node numbers")

    dense = bool((node_ids == np.arange(1, nn + 1)).all())   # nodes numbered 1..n in order

    def node_rows(ids) -> np.ndarray:
        ids = np.asarray(ids, np.int64)
        if dense:
            if ids.size and (ids.min() < 1 or ids.max() > nn):
                raise DeckError(f"unknown node {int(ids[(ids < 1) | (ids > nn)][0])}")
            return ids - 1
        pos = np.searchsorted(sorted_ids, ids)
        ok = (pos < len(sorted_ids)) & (sorted_ids[np.minimum(pos, len(sorted_ids) - 1)] == ids)
        if not ok.all():
            raise DeckError(f"unknown node {int(ids[~ok][0])}")
        return order[pos]

    # sets
    set_nodes: Dict[int, List[int]] = {}
    set_elems: Dict[int, List[int]] = {}
    for r in sets:
        if r.keyword != "set":
            raise DeckError(f"line {r.lineno}: expected a Set record")
        ns, es = [], []
        if r.has("nodes"):
            ns += r.array("nodes", int)
        if r.has("noderanges"):
            ns += r.ranges("noderanges")
        if r.has("elements"):
            es += r.array("elements", int)
        if r.has("elementranges"):
            es += r.ranges("elementranges")
        if r.has("allelements"):
            es += elem_ids.tolist()
        set_nodes[r.number] = ns
        set_elems[r.number] = es

    # elements
    nnpe = NODES_PER_ELEMENT[et]
    if (elem_nv != nnpe).any():
        raise DeckError(f"element {int(elem_ids[np.argmax(elem_nv != nnpe)])}: {ekw} needs {nnpe} nodes")
    conn = node_rows(elem_vals[:, :nnpe].astype(np.int64).ravel()).reshape(ne, nnpe).astype(np.int32)
    eorder = np.argsort(elem_ids, kind="stable")
    esorted = elem_ids[eorder]

    edense = bool((elem_ids == np.arange(1, ne + 1)).all())

    def elem_rows(ids) -> np.ndarray:
        ids = np.asarray(ids, np.int64)
        if edense:
            if ids.size and (ids.min() < 1 or ids.max() > ne):
                raise DeckError(f"unknown element {int(ids[(ids < 1) | (ids > ne)][0])}")
            return ids - 1
        pos = np.searchsorted(esorted, ids)
        ok = (pos < len(esorted)) & (esorted[np.minimum(pos, len(esorted) - 1)] == ids)
        if not ok.all():
            raise DeckError(f"unknown element {int(ids[~ok][0])}")
        return eorder[pos]

    # materials
    mat_index: Dict[int, int] = {}
    materials: List[mg.Material] = []
    scalar = lambda *k: {name: "scalar" for name in k}
    mat_fields = {"isole": scalar("d", "e", "n", "talpha"),
                  "misesmat": scalar("d", "e", "n", "talpha", "sig0", "h", "htype", "omega_crit", "a", "yieldtol"),
                  "idm1": scalar("d", "e", "n", "talpha", "e0", "gf", "equivstraintype", "damlaw")}
    for r in mats:
        if r.keyword in mat_fields:   # any other parameter changes the model: refused
            _check_fields(r, mat_fields[r.keyword])
        if r.keyword == "isole":
            # talpha acts only through temperature loads, which are not accepted
            m = mg.Material(mg.MAT_ISOLE, r.float("e"), r.float("n"))
        elif r.keyword == "misesmat":
            if r.int("htype", 0) != 0 or r.float("omega_crit", 0.0) != 0.0 or r.float("a", 0.0) != 0.0:
                raise DeckError(f"line {r.lineno}: MisesMat with hardening type or damage is not supported")
            m = mg.Material(mg.MAT_MISES, r.float("e"), r.float("n"), sig0=r.float("sig0"), H=r.float("h", 0.0))
        elif r.keyword == "idm1":
            if r.int("equivstraintype", 0) != 0 or r.int("damlaw", 0) != 0:
                raise DeckError(f"line {r.lineno}: idm1 supports equivstraintype 0 and damlaw 0 only")
            m = mg.Material(mg.MAT_IDM1, r.float("e"), r.float("n"), e0=r.float("e0"), gf=r.float("gf"))
        else:
            raise DeckError(f"line {r.lineno}: material '{r.tok[0]}' is not supported")
        mat_index[r.number] = len(materials)
        materials.append(m)

    # cross sections -> element materials
    cs_mat: Dict[int, int] = {}
    thick = set()
    elem_cs = np.zeros(ne, np.int64)
    for r in sections:
        if r.keyword != "simplecs":
            raise DeckError(f"line {r.lineno}: cross section '{r.tok[0]}' is not supported")
        if r.has("material"):
            cs_mat[r.number] = r.int("material")
        thick.add(r.float("thick", 1.0))
        if r.has("set") and set_elems.get(r.int("set")):
            elem_cs[elem_rows(set_elems[r.int("set")])] = r.number
    elem_mid = np.array([cs_mat.get(int(c), 0) for c in range(int(elem_cs.max()) + 1)], np.int64)[elem_cs]
    nip_default = {mg.ELEM_LSPACE: ("8",), mg.ELEM_PLANESTRESS2D: ("4",), mg.ELEM_LTRSPACE: ("1",)}[et]
    for r in elem_full.values():   # geometric nonlinearity, other integration rules, loads on elements: refused
        _check_fields(r, {"nodes": "array", "crosssect": "scalar", "mat": "scalar", "nlgeo": "scalar",
                          "nip": "scalar"}, {"nlgeo": ("0",), "nip": nip_default})
    for r in node_full.values():
        _check_fields(r, {"coords": "array", "bc": "array", "load": "array"})
    for k, r in elem_full.items():   # old-style crossSect / mat fields on the element record
        cs = r.int("crosssect", 0) or int(elem_cs[k])
        elem_mid[k] = r.int("mat", 0) or cs_mat.get(cs, 0)
    missing = ~np.isin(elem_mid, list(mat_index))
    if missing.any():
        raise DeckError(f"element {int(elem_ids[np.argmax(missing)])} has no material")
    lut = np.zeros(max(mat_index) + 1, np.int32)
    for mid, i in mat_index.items():
        lut[mid] = i
    elem_mat = lut[elem_mid]
    if len(thick) > 1 and et == mg.ELEM_PLANESTRESS2D:
        raise DeckError("cross sections of different thickness are not supported")

    # boundary conditions and nodal loads
    bc_mask = np.zeros((nn, nd), np.uint8)
    bc_value = np.zeros((nn, nd))
    bc_ltf = np.zeros((nn, nd), np.int64)
    load_terms: List[Tuple[np.ndarray, int]] = []
    bc_by_id = {r.number: r for r in bcs}

    def prescribe(rows, dofs, vals, f):
        for d, v in zip(dofs, vals):
            if not 1 <= d <= nd:
                raise DeckError(f"DOF {d} outside 1..{nd}")
            bc_mask[rows, d - 1] = 1
            bc_value[rows, d - 1] = v
            bc_ltf[rows, d - 1] = f

    for r in bcs:
        f = r.int("loadtimefunction")
        for key in ("isimposedtimefunction", "reference", "loadtype", "csys", "lcs"):
            if r.has(key):
                raise DeckError(f"line {r.lineno}: field '{key}' of {r.tok[0]} is not supported")
        if r.keyword == "boundarycondition":
            if r.has("set"):
                rows = node_rows(set_nodes.get(r.int("set"), []))
                dofs = r.array("dofs", int)
                vals = r.array("values") if r.has("values") else [r.float("prescribedvalue", 0.0)] * len(dofs)
                prescribe(rows, dofs, vals, f)
        elif r.keyword == "nodalload":
            if r.has("set"):
                comps = r.array("components")
                dofs = r.array("dofs", int) if r.has("dofs") else list(range(1, len(comps) + 1))
                pat = np.zeros((nn, nd))
                rows = node_rows(set_nodes.get(r.int("set"), []))
                for d, v in zip(dofs, comps):
                    np.add.at(pat[:, d - 1], rows, v)
                load_terms.append((pat, f))
        else:
            raise DeckError(f"line {r.lineno}: load '{r.tok[0]}' is not supported")
    # old-style references from the node records
    for a, r in node_full.items():
        if r.has("bc"):
            for d, bid in enumerate(r.array("bc", int), 1):
                if bid:
                    b = bc_by_id[bid]
                    prescribe(np.array([a]), [d], [b.float("prescribedvalue", b.float("d", 0.0))],
                              b.int("loadtimefunction"))
        if r.has("load"):
            for lid in r.array("load", int):
                b = bc_by_id[lid]
                comps = b.array("components")
                pat = np.zeros((nn, nd))
                pat[a, :len(comps)] = comps[:nd]
                load_terms.append((pat, b.int("loadtimefunction")))

    # time functions
    functions: Dict[int, object] = {}
    for r in funcs:
        if r.keyword == "constantfunction":
            functions[r.number] = ConstantFunction(r.float("f(t)"))
        elif r.keyword == "piecewiselinfunction":
            functions[r.number] = PiecewiseLinFunction(r.array("t"), r.array("f(t)"))
        else:
            raise DeckError(f"line {r.lineno}: function '{r.tok[0]}' is not supported")
    for f in set(np.unique(bc_ltf[bc_mask == 1]).tolist()) | {f for _, f in load_terms}:
        if f not in functions:
            raise DeckError(f"time function {f} is not defined")

    nodal_load = np.zeros((nn, nd))
    for pat, _ in load_terms:
        nodal_load += pat
    mesh = mg.Mesh(et, coords, conn, elem_mat, materials, bc_mask, bc_value, nodal_load,
                   thickness=thick.pop() if thick else 1.0, name=description)
    return Deck(output, description, analysis, mesh, node_ids, elem_ids, bc_ltf, load_terms, functions)


@dataclasses.dataclass
class DeckStep:
    number: int
    time: float
    u: np.ndarray
    reactions: np.ndarray
    iterations: int       # PCG iterations (LinearStatic) or Newton iterations


def run_deck(deck: Deck, ctx=None, precision: Optional[int] = None, lstol: Optional[float] = None):
    """Run the deck's analysis on the GPU path; a list of DeckStep.

    LinearStatic: step k at time k (LinearStatic::giveNextStep, linearstatic.C:146-156), one PCG solve.
    Decks for an iterative solver (lstype 1 IML, 9 this library) keep its lstol / lsiter / lsprecond
    (IMLSolver defaults 1e-5 / 200 / none; lstype 9 defaults to the diagonal preconditioner); decks for
    the default direct solver (lstype 0) or another direct one run the device LDL^T factorization
    (LDLTFactorization on a Skyline matrix). NonLinearStatic: step k
    at time (k-1) * deltat (nlinearstatic.C:295-325). StaticStructural: oofem_gb300.engng.StaticStructural.
    ``precision`` / ``lstol`` override the linear solver's arithmetic and tolerance."""
    from . import engng, native
    a = deck.analysis
    ctx = ctx or native.Context(0)
    model = native.GpuModel(ctx, deck.mesh)
    K = native.GpuCsrMtrx(ctx)
    prec = native.PREC_FP64 if precision is None else precision
    nsteps = a.int("nsteps", 1)
    out: List[DeckStep] = []
    # lstype 0 (the default) and the other direct solvers factor the matrix; a caller asking for
    # mixed precision or for a PCG tolerance runs such a deck by PCG instead (to `lstol`, else
    # 1e-12); an iterative lstype keeps its lstol / lsiter / lsprecond
    lstype = a.int("lstype", 0)
    if lstype not in DIRECT_LSTYPES + (1, 9):
        raise DeckError(f"lstype {lstype} is not a linear solver of the reference")
    direct = lstype in DIRECT_LSTYPES and lstol is None and prec == native.PREC_FP64
    if direct:
        K.set_solver(native.LS_DIRECT)
    elif lstype in DIRECT_LSTYPES and lstol is None:
        lstol = 1e-12
    elif lstype not in DIRECT_LSTYPES:
        K.set_preconditioner(a.int("lsprecond", 0 if lstype == 1 else 1))
    if deck.analysis_type == "linearstatic":
        tol = lstol if lstol is not None else (0.0 if direct else a.float("lstol", 1e-5))
        maxit = 1 if direct else (1000000 if lstype in DIRECT_LSTYPES else a.int("lsiter", 200))
        for k in range(1, nsteps + 1):
            t = float(k)
            u, reac, info = model.linear_static(K, deck.bc_value_at(t), deck.nodal_load_at(t), rtol=tol,
                                                maxit=maxit, precision=prec)
            if info.status != 0:
                raise native.OgbError(info.status, f"LinearStatic step {k}: linear solver did not converge")
            out.append(DeckStep(k, t, u, reac, info.iterations))
        return out
    tol = lstol if lstol is not None else (0.0 if direct else a.float("lstol", 1e-5))
    if deck.analysis_type == "nonlinearstatic":
        if a.int("controlmode", 1) != 1:
            raise DeckError("NonLinearStatic supports controlmode 1 (direct displacement / load control)")
        model.set_initial_guess(a.int("initialguess", 0))
        model.set_nr_mode(a.int("manrmsteps", 0))
        dt = a.float("deltat", 1.0)
        for k in range(1, nsteps + 1):
            t = (k - 1) * dt
            u, reac, nite = model.nonlinear_step(K, deck.bc_value_at(t), deck.nodal_load_at(t),
                                                 rtolf=a.float("rtolf", 1e-3), maxiter=a.int("maxiter", 100000000),
                                                 lin_rtol=tol, precision=prec)
            out.append(DeckStep(k, t, u, reac, nite))
        return out
    if a.has("solvertype") and a._value("solvertype").lower() != "nrsolver":
        raise DeckError("StaticStructural supports solvertype nrsolver")
    ss = engng.StaticStructural(model, K, nsteps=nsteps, deltat=a.float("deltat", 1.0),
                                prescribed_times=a.array("prescribedtimes") if a.has("prescribedtimes") else None,
                                rtolf=a.float("rtolf", 1e-3), maxiter=a.int("maxiter", 100000000),
                                manrmsteps=a.int("manrmsteps", 0), initial_guess=a.int("initialguess", 1),
                                lstol=tol, precision=prec, bc_at=deck.bc_value_at, load_at=deck.nodal_load_at)
    for r in ss.solve_yourself():
        out.append(DeckStep(r.number, r.time, r.u, r.reactions, r.iterations))
    return out


def check_rules(deck_path: str, deck: Deck, steps: List[DeckStep]):
    """The deck's embedded errorcheck rules (`#NODE tStep s number n dof d unknown d value v`,
    `#REACTION tStep s number n dof d value v`, tolerance from `#%BEGIN_CHECK% tolerance t`;
    ErrorCheckingExportModule, src/core/errorcheckingexportmodule.C): a list of
    (rule text, computed value, expected value, passed)."""
    tol = 1e-6
    rules = []
    nmap = {int(i): k for k, i in enumerate(deck.node_ids)}
    by_step = {s.number: s for s in steps}
    with open(deck_path) as fh:
        for line in fh:
            m = re.match(r"#%BEGIN_CHECK%\s+tolerance\s+(\S+)", line, re.I)
            if m:
                tol = float(m[1])
            m = re.match(r"#NODE\s+tStep\s+(\d+)\s+number\s+(\d+)\s+dof\s+(\d+)\s+unknown\s+d\s+value\s+(\S+)", line, re.I)
            if m and int(m[1]) in by_step:
                got = by_step[int(m[1])].u[nmap[int(m[2])], int(m[3]) - 1]
                rules.append((line.strip(), got, float(m[4]), abs(got - float(m[4])) <= tol))
            m = re.match(r"#REACTION\s+tStep\s+(\d+)\s+number\s+(\d+)\s+dof\s+(\d+)\s+value\s+(\S+)", line, re.I)
            if m and int(m[1]) in by_step:
                got = by_step[int(m[1])].reactions[nmap[int(m[2])], int(m[3]) - 1]
                rules.append((line.strip(), got, float(m[4]), abs(got - float(m[4])) <= tol))
    return rules


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="run an OOFEM input deck on the GPU path")
    ap.add_argument("deck")
    ap.add_argument("--mixed", action="store_true", help="mixed-precision linear solves")
    ap.add_argument("--check", action="store_true", help="verify the deck's embedded #NODE / #REACTION rules")
    args = ap.parse_args(argv)
    from . import native
    deck = read_deck(args.deck)
    steps = run_deck(deck, precision=native.PREC_MIXED if args.mixed else None)
    for s in steps:
        print(json.dumps({"step": s.number, "time": s.time, "iterations": s.iterations,
                          "max_abs_u": float(np.abs(s.u).max())}))
    if args.check:
        rules = check_rules(args.deck, deck, steps)
        bad = [r for r in rules if not r[3]]
        print(json.dumps({"rules": len(rules), "failed": len(bad)}))
        for r in bad:
            print("FAILED", r[0], "got", r[1])
        return 1 if bad else 0
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
