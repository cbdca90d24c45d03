"""Seeded synthetic meshes for the structural hot path.

Every generator returns a :class:`Mesh` whose node and element orderings follow
the reference's conventions, so the same arrays can be written out as an OOFEM
input deck and fed to the reference executable:

* ``lspace`` (8-node hexahedron): element node order follows ``FEI3dHexaLin``
  (``src/core/fei3dhexalin.C:45-63``): nodes 1-4 on the face zeta=+1
  (xi,eta) = (-1,-1), (-1,+1), (+1,+1), (+1,-1); nodes 5-8 the same on zeta=-1.
* ``planestress2d`` (4-node quad): ``FEI2dQuadLin`` order
  (``src/core/fei2dquadlin.C:60-72``): (+1,+1), (-1,+1), (-1,-1), (+1,-1).
* ``ltrspace`` (4-node tetrahedron): ``FEI3dTetLin`` (``src/core/fei3dtetlin.C:45-55``),
  oriented so the reference's determinant (``fei3dtetlin.C:140-146``) is positive.

Nodes of structured grids are numbered x-fastest. Node jitter, where asked for,
moves interior nodes only, so boundary faces stay planar.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

ELEM_LSPACE = 1
ELEM_PLANESTRESS2D = 2
ELEM_LTRSPACE = 3

ELEM_NAMES = {ELEM_LSPACE: "lspace", ELEM_PLANESTRESS2D: "planestress2d",
              ELEM_LTRSPACE: "ltrspace"}
NODES_PER_ELEM = {ELEM_LSPACE: 8, ELEM_PLANESTRESS2D: 4, ELEM_LTRSPACE: 4}
DOFS_PER_NODE = {ELEM_LSPACE: 3, ELEM_PLANESTRESS2D: 2, ELEM_LTRSPACE: 3}

MAT_ISOLE = 1
MAT_MISES = 2
MAT_IDM1 = 3


@dataclasses.dataclass
class Material:
    """Material record. ``kind`` is MAT_ISOLE / MAT_MISES / MAT_IDM1.

    isole:    E, nu                                   (isolinearelasticmaterial.C:65-76)
    misesmat: E, nu, sig0, H  (htype 0, no damage)    (misesmat.C:60-100)
    idm1:     E, nu, e0, gf   (Mazars, exponential cohesive law, damlaw 0)
              (idm1.C:86-348)
    """
    kind: int
    E: float
    nu: float
    sig0: float = 0.0
    H: float = 0.0
    e0: float = 0.0
    gf: float = 0.0

    def as_row(self) -> np.ndarray:
        """Packed 8-double row used by the C-ABI: kind,E,nu,sig0,H,e0,gf,0."""
        return np.array([self.kind, self.E, self.nu, self.sig0, self.H, self.e0,
                         self.gf, 0.0], dtype=np.float64)


@dataclasses.dataclass
class Mesh:
    elem_type: int
    coords: np.ndarray          # (nnodes, ndim) float64
    conn: np.ndarray            # (nelem, nnpe) int32, 0-based node ids
    elem_mat: np.ndarray        # (nelem,) int32, index into materials
    materials: List[Material]
    bc_mask: np.ndarray         # (nnodes, ndofpn) uint8: 1 = prescribed DOF
    bc_value: np.ndarray        # (nnodes, ndofpn) float64, prescribed value at load factor 1
    nodal_load: np.ndarray      # (nnodes, ndofpn) float64, nodal force at load factor 1
    thickness: float = 1.0
    name: str = ""

    @property
    def ndim(self) -> int:
        return self.coords.shape[1]

    @property
    def ndofpn(self) -> int:
        return DOFS_PER_NODE[self.elem_type]

    @property
    def nnodes(self) -> int:
        return self.coords.shape[0]

    @property
    def nelem(self) -> int:
        return self.conn.shape[0]

    @property
    def nnpe(self) -> int:
        return self.conn.shape[1]

    @property
    def nfree(self) -> int:
        return int((self.bc_mask == 0).sum())

    def material_table(self) -> np.ndarray:
        return np.stack([m.as_row() for m in self.materials]).astype(np.float64)


def _grid_index3(nx, ny, nz):
    return lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)


def _jitter(coords: np.ndarray, interior: np.ndarray, amp: float, rng) -> np.ndarray:
    out = coords.copy()
    if amp > 0.0:
        d = rng.uniform(-amp, amp, size=coords.shape)
        out[interior] += d[interior]
    return out


def hex_grid(nx: int, ny: int, nz: int, h: float = 0.05, jitter: float = 0.0,
             seed: int = 0):
    """Structured LSpace grid, nodes x-fastest, hexes ordered x-fastest.

    Returns (coords, conn). ``jitter`` is the amplitude as a fraction of h.
    """
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                          indexing="ij")
    # x-fastest: flatten with k slowest
    ii = i.transpose(2, 1, 0).ravel()
    jj = j.transpose(2, 1, 0).ravel()
    kk = k.transpose(2, 1, 0).ravel()
    coords = np.stack([ii * h, jj * h, kk * h], axis=1).astype(np.float64)
    interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny) & (kk > 0) & (kk < nz)
    rng = np.random.default_rng(seed)
    coords = _jitter(coords, interior, jitter * h, rng)
    nid = _grid_index3(nx, ny, nz)
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ei = ei.transpose(2, 1, 0).ravel()
    ej = ej.transpose(2, 1, 0).ravel()
    ek = ek.transpose(2, 1, 0).ravel()
    conn = np.stack([
        nid(ei, ej, ek + 1), nid(ei, ej + 1, ek + 1), nid(ei + 1, ej + 1, ek + 1), nid(ei + 1, ej, ek + 1),
        nid(ei, ej, ek), nid(ei, ej + 1, ek), nid(ei + 1, ej + 1, ek), nid(ei + 1, ej, ek),
    ], axis=1).astype(np.int32)
    return coords, conn


def hex_cantilever(nx: int, ny: int, nz: int, h: float = 0.05, jitter: float = 0.0,
                   seed: int = 0, E: float = 210e9, nu: float = 0.3,
                   total_force: float = 1e5) -> Mesh:
    """Linear-elastic LSpace cantilever: all DOFs fixed at x=0, a total force
    ``total_force`` in -z split equally over the nodes of the x=L face."""
    coords, conn = hex_grid(nx, ny, nz, h, jitter, seed)
    nn = coords.shape[0]
    ix = np.arange(nn) % (nx + 1)
    bc_mask = np.zeros((nn, 3), np.uint8)
    bc_mask[ix == 0, :] = 1
    load = np.zeros((nn, 3), np.float64)
    tip = ix == nx
    load[tip, 2] = -total_force / float(tip.sum())
    return Mesh(ELEM_LSPACE, coords, conn, np.zeros(conn.shape[0], np.int32),
                [Material(MAT_ISOLE, E, nu)], bc_mask, np.zeros((nn, 3)), load,
                name=f"hex_cantilever_{nx}x{ny}x{nz}_j{jitter}_s{seed}")


def hex_block_pull(nx: int, ny: int, nz: int, h: float = 0.05, jitter: float = 0.0,
                   seed: int = 0, material: Optional[Material] = None,
                   end_disp: float = 1.0) -> Mesh:
    """LSpace block, x=0 face fully fixed, x=L face u_x prescribed to
    ``end_disp`` (at load factor 1); other DOFs of the x=L face free."""
    coords, conn = hex_grid(nx, ny, nz, h, jitter, seed)
    nn = coords.shape[0]
    ix = np.arange(nn) % (nx + 1)
    bc_mask = np.zeros((nn, 3), np.uint8)
    bc_mask[ix == 0, :] = 1
    bc_mask[ix == nx, 0] = 1
    bc_value = np.zeros((nn, 3))
    bc_value[ix == nx, 0] = end_disp
    mat = material or Material(MAT_MISES, 210e9, 0.3, sig0=250e6, H=2e9)
    return Mesh(ELEM_LSPACE, coords, conn, np.zeros(conn.shape[0], np.int32), [mat],
                bc_mask, bc_value, np.zeros((nn, 3)),
                name=f"hex_block_{nx}x{ny}x{nz}_s{seed}")


def quad_grid(n: int, m: int, lx: float = 1.0, ly: float = 1.0):
    hx, hy = lx / n, ly / m
    i, j = np.meshgrid(np.arange(n + 1), np.arange(m + 1), indexing="xy")
    ii, jj = i.ravel(), j.ravel()
    coords = np.stack([ii * hx, jj * hy], axis=1).astype(np.float64)
    nid = lambda a, b: a + (n + 1) * b
    ei, ej = np.meshgrid(np.arange(n), np.arange(m), indexing="xy")
    ei, ej = ei.ravel(), ej.ravel()
    conn = np.stack([nid(ei + 1, ej + 1), nid(ei, ej + 1), nid(ei, ej), nid(ei + 1, ej)],
                    axis=1).astype(np.int32)
    return coords, conn


RVE_STRAINS = (
    ((1e-3, 0.0), (0.0, 0.0)),
    ((0.0, 0.0), (0.0, 1e-3)),
    ((0.0, 5e-4), (5e-4, 0.0)),
)


def quad_rve(n: int, seed: int = 0, vf: float = 0.30, load_case: int = 0,
             E_m: float = 30e9, nu_m: float = 0.2, E_i: float = 300e9,
             nu_i: float = 0.2) -> Mesh:
    """Unit-square PlaneStress2d RVE, n x n quads, thickness 1.

    Circular inclusions with seeded centres and radii are added until their
    (analytic, overlap-ignoring) area fraction reaches ``vf``; an element is an
    inclusion element when its centroid falls inside any circle. All boundary
    nodes carry u = eps . x for the chosen load case (RVE_STRAINS)."""
    coords, conn = quad_grid(n, n)
    rng = np.random.default_rng(seed)
    centres, radii = [], []
    area = 0.0
    while area < vf:
        r = rng.uniform(0.04, 0.12)
        c = rng.uniform(0.0, 1.0, size=2)
        centres.append(c)
        radii.append(r)
        area += math.pi * r * r
    cen = coords[conn].mean(axis=1)
    inc = np.zeros(conn.shape[0], bool)
    for c, r in zip(centres, radii):
        inc |= ((cen - c) ** 2).sum(axis=1) < r * r
    nn = coords.shape[0]
    x, y = coords[:, 0], coords[:, 1]
    bnd = (np.isclose(x, 0.0) | np.isclose(x, 1.0) | np.isclose(y, 0.0) | np.isclose(y, 1.0))
    bc_mask = np.zeros((nn, 2), np.uint8)
    bc_mask[bnd, :] = 1
    eps = np.array(RVE_STRAINS[load_case])
    bc_value = np.zeros((nn, 2))
    bc_value[bnd] = (coords[bnd] @ eps.T)
    mats = [Material(MAT_ISOLE, E_m, nu_m), Material(MAT_ISOLE, E_i, nu_i)]
    return Mesh(ELEM_PLANESTRESS2D, coords, conn, inc.astype(np.int32), mats, bc_mask,
                bc_value, np.zeros((nn, 2)), thickness=1.0,
                name=f"quad_rve_{n}_s{seed}_lc{load_case}")


def rve_bc_values(mesh: Mesh, load_case: int) -> np.ndarray:
    """Boundary displacement field u = eps . x of one RVE load case."""
    eps = np.array(RVE_STRAINS[load_case])
    vals = np.zeros_like(mesh.bc_value)
    bnd = mesh.bc_mask[:, 0] == 1
    vals[bnd] = mesh.coords[bnd] @ eps.T
    return vals


def rve_batch(count: int, seed: int = 0, side_min: int = 32, side_max: int = 256,
              vf: float = 0.30) -> List[Mesh]:
    """``count`` RVEs (quad_rve) with sides n_i ~ U{side_min..side_max} drawn
    from ``seed``; RVE i takes inclusion seed ``seed * 100003 + i``."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_min, side_max + 1, size=count)
    return [quad_rve(int(n), seed=seed * 100003 + i, vf=vf) for i, n in enumerate(sides)]


def concat_meshes(meshes: List[Mesh]):
    """One mesh holding independent meshes back to back (nodes, elements and
    material tables in order); returns (mesh, node_start) with node_start[i] the
    first node of mesh i and node_start[-1] the node count."""
    et = meshes[0].elem_type
    if any(m.elem_type != et or m.thickness != meshes[0].thickness for m in meshes):
        raise ValueError("instances must share element type and thickness")
    node_start = np.zeros(len(meshes) + 1, np.int32)
    node_start[1:] = np.cumsum([m.nnodes for m in meshes])
    mat_off = np.cumsum([0] + [len(m.materials) for m in meshes])
    conn = np.concatenate([m.conn + node_start[i] for i, m in enumerate(meshes)]).astype(np.int32)
    emat = np.concatenate([m.elem_mat + mat_off[i] for i, m in enumerate(meshes)]).astype(np.int32)
    mats = [mat for m in meshes for mat in m.materials]
    big = Mesh(et, np.concatenate([m.coords for m in meshes]), conn, emat, mats,
               np.concatenate([m.bc_mask for m in meshes]), np.concatenate([m.bc_value for m in meshes]),
               np.concatenate([m.nodal_load for m in meshes]), thickness=meshes[0].thickness,
               name=f"batch_{len(meshes)}")
    return big, node_start


def tet_det_ref(x: np.ndarray) -> np.ndarray:
    """detJ of FEI3dTetLin::evaldNdx (fei3dtetlin.C:140-142), x: (..., 4, 3)."""
    x1, x2, x3, x4 = x[..., 0, 0], x[..., 1, 0], x[..., 2, 0], x[..., 3, 0]
    y1, y2, y3, y4 = x[..., 0, 1], x[..., 1, 1], x[..., 2, 1], x[..., 3, 1]
    z1, z2, z3, z4 = x[..., 0, 2], x[..., 1, 2], x[..., 2, 2], x[..., 3, 2]
    return ((x4 - x1) * (y2 - y1) * (z3 - z1) - (x4 - x1) * (y3 - y1) * (z2 - z1) +
            (x3 - x1) * (y4 - y1) * (z2 - z1) - (x2 - x1) * (y4 - y1) * (z3 - z1) +
            (x2 - x1) * (y3 - y1) * (z4 - z1) - (x3 - x1) * (y2 - y1) * (z4 - z1))


_KUHN_PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


def tet_cube(n: int, jitter: float = 0.0, seed: int = 0,
             material: Optional[Material] = None, end_disp: float = 1.0) -> Mesh:
    """Unit cube of n^3 cells, each split into 6 LTRSpace tets (Kuhn split).

    Tets are oriented so the reference's detJ is positive; after jitter any node
    touching an inverted tet is re-drawn (seeded) until every detJ > 0.
    z=0 face fixed; z=1 face u_z prescribed to ``end_disp`` at load factor 1."""
    h = 1.0 / n
    coords, _ = hex_grid(n, n, n, h, 0.0, seed)
    nn = coords.shape[0]
    nid = _grid_index3(n, n, n)
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ci = ci.transpose(2, 1, 0).ravel()
    cj = cj.transpose(2, 1, 0).ravel()
    ck = ck.transpose(2, 1, 0).ravel()
    tets = []
    for p in _KUHN_PERMS:
        v = [np.array([0, 0, 0])]
        for ax in p:
            nv = v[-1].copy()
            nv[ax] = 1
            v.append(nv)
        tets.append(np.stack([nid(ci + a[0], cj + a[1], ck + a[2]) for a in v], axis=1))
    conn = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    det = tet_det_ref(coords[conn])
    flip = det < 0
    conn[flip] = conn[flip][:, [0, 2, 1, 3]]
    ix = np.arange(nn) % (n + 1)
    iy = (np.arange(nn) // (n + 1)) % (n + 1)
    iz = np.arange(nn) // ((n + 1) * (n + 1))
    interior = (ix > 0) & (ix < n) & (iy > 0) & (iy < n) & (iz > 0) & (iz < n)
    rng = np.random.default_rng(seed)
    base = coords.copy()
    if jitter > 0:
        coords = _jitter(base, interior, jitter * h, rng)
        for _ in range(100):
            det = tet_det_ref(coords[conn])
            bad = det <= 0
            if not bad.any():
                break
            redo = np.zeros(nn, bool)
            redo[np.unique(conn[bad])] = True
            redo &= interior
            d = rng.uniform(-jitter * h, jitter * h, size=(int(redo.sum()), 3))
            coords[redo] = base[redo] + d
        else:
            raise RuntimeError("could not draw a valid jittered tet mesh")
    bc_mask = np.zeros((nn, 3), np.uint8)
    bc_mask[iz == 0, :] = 1
    bc_mask[iz == n, 2] = 1
    bc_value = np.zeros((nn, 3))
    bc_value[iz == n, 2] = end_disp
    mat = material or Material(MAT_IDM1, 30e9, 0.2, e0=1e-4, gf=100.0)
    return Mesh(ELEM_LTRSPACE, coords, conn, np.zeros(conn.shape[0], np.int32), [mat],
                bc_mask, bc_value, np.zeros((nn, 3)),
                name=f"tet_cube_{n}_j{jitter}_s{seed}")


def tet_cube_linear(n: int, jitter: float = 0.0, seed: int = 0, E: float = 30e9,
                    nu: float = 0.2, end_disp: float = 1e-4) -> Mesh:
    return tet_cube(n, jitter, seed, Material(MAT_ISOLE, E, nu), end_disp)
