"""ctypes front of the C oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the product path never does. It drives the plain-C restatement
(oracle/oofem_oracle.c) through the same steps as the reference's LinearStatic
(src/sm/EngineeringModels/linearstatic.C:177-253) and NonLinearStatic + NRSolver
(src/core/nrsolver.C:204-402).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboofem_oracle.so")
NSTATE = 24

_lib = None


def build() -> str:
    src = os.path.join(HERE, "oofem_oracle.c")
    if (not os.path.exists(LIB)) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=c99", "-o", LIB, src, "-lm"])
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
    return _lib


def threads() -> int:
    """OpenMP threads of the oracle's element loops (1 when built without OpenMP)."""
    return int(lib().oro_threads())


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def nnpe(et):
    return 8 if et == 1 else 4


def ndofpn(et):
    return 2 if et == 2 else 3


def ngp(et):
    return {1: 8, 2: 4, 3: 1}[et]


def nstress(et):
    return 3 if et == 2 else 6


def number_equations(bc_mask: np.ndarray):
    nn, nd = bc_mask.shape
    eq = np.zeros((nn, nd), np.int32)
    npeq = C.c_int(0)
    m = np.ascontiguousarray(bc_mask, dtype=np.uint8)
    neq = lib().oro_number_equations(nn, nd, _p(m), _p(eq), C.byref(npeq))
    return neq, npeq.value, eq


def location_arrays(conn: np.ndarray, eq: np.ndarray):
    ne, npe = conn.shape
    nd = eq.shape[1]
    loc = np.zeros((ne, npe * nd), np.int32)
    c = np.ascontiguousarray(conn, dtype=np.int32)
    lib().oro_location_arrays(ne, npe, _p(c), nd, _p(eq), _p(loc))
    return loc


def build_pattern(neq: int, loc: np.ndarray):
    ne, nl = loc.shape
    L = lib()
    L.oro_build_pattern.restype = C.c_int64
    rowptr = np.zeros(neq + 1, np.int64)
    nnz = L.oro_build_pattern(neq, ne, nl, _p(loc), _p(rowptr), None)
    colind = np.zeros(max(nnz, 1), np.int32)
    L.oro_build_pattern(neq, ne, nl, _p(loc), _p(rowptr), _p(colind))
    return rowptr, colind[:nnz]


def elem_stiffness(et, xe, D, thickness=1.0, per_gp=False, symmetric=True):
    nl = nnpe(et) * ndofpn(et)
    Ke = np.zeros((nl, nl))
    xe = np.ascontiguousarray(xe, dtype=np.float64)
    D = np.ascontiguousarray(D, dtype=np.float64)
    lib().oro_elem_stiffness(et, _p(xe), _p(D), int(per_gp), C.c_double(thickness),
                             int(symmetric), _p(Ke))
    return Ke


def isole_d(et, E, nu):
    if et == 2:
        D = np.zeros((3, 3))
        lib().oro_isole_dps(C.c_double(E), C.c_double(nu), _p(D))
    else:
        D = np.zeros((6, 6))
        lib().oro_isole_d3d(C.c_double(E), C.c_double(nu), _p(D))
    return D


def assemble_tangent(m: dict, loc, neq, rowptr, colind, state=None):
    et = int(m["etype"])
    coords = np.ascontiguousarray(m["coords"], dtype=np.float64)
    conn = np.ascontiguousarray(m["conn"], dtype=np.int32)
    emat = np.ascontiguousarray(m["elem_mat"], dtype=np.int32)
    mats = np.ascontiguousarray(m["mats"], dtype=np.float64)
    val = np.zeros(colind.size)
    st = None if state is None else _p(state)
    lib().oro_assemble_tangent(et, coords.shape[1], coords.shape[0], _p(coords), conn.shape[0],
                               _p(conn), _p(emat), _p(mats), C.c_double(float(m["thickness"])),
                               st, loc.shape[1], _p(loc), neq, _p(rowptr), _p(colind), _p(val))
    return val


def internal_forces(m: dict, u_node: np.ndarray, state=None, want_enorm=False):
    """Node-indexed internal forces for the total displacement field; updates
    the temp part of ``state`` in place. Returns (f_node, gp_stress, gp_strain)
    and, with want_enorm, the per-DOF-id element force norms as a 4th item."""
    et = int(m["etype"])
    coords = np.ascontiguousarray(m["coords"], dtype=np.float64)
    conn = np.ascontiguousarray(m["conn"], dtype=np.int32)
    emat = np.ascontiguousarray(m["elem_mat"], dtype=np.int32)
    mats = np.ascontiguousarray(m["mats"], dtype=np.float64)
    nn, ne = coords.shape[0], conn.shape[0]
    f = np.zeros((nn, ndofpn(et)))
    sig = np.zeros((ne, ngp(et), nstress(et)))
    eps = np.zeros_like(sig)
    u = np.ascontiguousarray(u_node, dtype=np.float64)
    st = None if state is None else _p(state)
    en = np.zeros(ndofpn(et))
    lib().oro_internal_forces(et, coords.shape[1], nn, _p(coords), ne, _p(conn), _p(emat),
                              _p(mats), C.c_double(float(m["thickness"])), _p(u), st, _p(f),
                              _p(sig), _p(eps), _p(en))
    if want_enorm:
        return f, sig, eps, en
    return f, sig, eps


def commit_state(m: dict, state: np.ndarray):
    et = int(m["etype"])
    mats = np.ascontiguousarray(m["mats"], dtype=np.float64)
    emat = np.asarray(m["elem_mat"])
    g = ngp(et)
    L = lib()
    for e in range(emat.size):
        mp = mats[emat[e]]
        for k in range(g):
            row = state[e * g + k]
            L.oro_commit_state(et, _p(mp), _p(row))


def spmv(rowptr, colind, val, x):
    y = np.zeros(rowptr.size - 1)
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().oro_spmv(rowptr.size - 1, _p(rowptr), _p(colind), _p(val), _p(x), _p(y))
    return y


def pcg(rowptr, colind, val, b, rtol=1e-12, maxit=100000, x0=None):
    n = rowptr.size - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    it = C.c_int(0)
    ach = C.c_double(0)
    st = lib().oro_pcg(n, _p(rowptr), _p(colind), _p(val), _p(b), _p(x), C.c_double(rtol),
                       maxit, C.byref(it), C.byref(ach))
    return x, st, it.value, ach.value


def ic_factor(rowptr, colind, val):
    """CompCol_ICPreconditioner::initialize + ICFactor (src/core/iml/icprecond.C:64-163)
    for a symmetric matrix given as CSR: column k of the lower triangle is row k
    restricted to columns >= k, diagonal first; the factorization loop is the
    reference's, including its row search that only matches at the last entry of
    a column. Returns (pntr, indx, val) of the factor by columns."""
    n = rowptr.size - 1
    pntr = np.zeros(n + 1, np.int64)
    indx, vals = [], []
    for k in range(n):
        cols = colind[rowptr[k]:rowptr[k + 1]]
        sel = cols >= k
        indx.extend(cols[sel].tolist())
        vals.extend(val[rowptr[k]:rowptr[k + 1]][sel].tolist())
        pntr[k + 1] = len(indx)
        if pntr[k] == pntr[k + 1] or indx[pntr[k]] != k:
            raise RuntimeError("IC preconditioner: diagonal not found")
    indx.append(n)   # the successor test of a column's last entry reads the next column's first row
    v = vals
    for k in range(n - 1):
        d = pntr[k]
        z = v[d] = np.sqrt(v[d])
        for i in range(d + 1, pntr[k + 1]):
            v[i] /= z
        for i in range(d + 1, pntr[k + 1]):
            zi = v[i]
            h = indx[i]
            g = i
            for j in range(pntr[h], pntr[h + 1]):
                while g < pntr[k + 1] and indx[g + 1] <= indx[j]:
                    if indx[g] == indx[j]:
                        v[j] -= zi * v[g]
                    g += 1
    if n:
        v[pntr[n - 1]] = np.sqrt(v[pntr[n - 1]])
    return pntr, np.array(indx[:-1], np.int64), np.array(v)


def ic_solve(F, x):
    """CompCol_ICPreconditioner::ICSolve (icprecond.C:166-190): forward and
    backward solves by columns."""
    pntr, indx, val = F
    n = pntr.size - 1
    dest = np.array(x, dtype=np.float64)
    work = np.zeros(n)
    for i in range(n):
        temp = work[i] = (dest[i] + work[i]) / val[pntr[i]]
        for t in range(pntr[i] + 1, pntr[i + 1]):
            work[indx[t]] -= val[t] * temp
    dest[:] = 0.0
    for i in range(n - 1, -1, -1):
        for t in range(pntr[i] + 1, pntr[i + 1]):
            dest[i] -= val[t] * dest[indx[t]]
        dest[i] = (work[i] + dest[i]) / val[pntr[i]]
    return dest


def ilu_factor(rowptr, colind, val):
    """CompCol_ILUPreconditioner::initialize (src/core/iml/iluprecond.C:75-167):
    column i of the symmetric matrix (= row i) split into L (rows > i) and U
    (rows <= i, the diagonal last), then the reference's factorization loop.
    Returns (lp, lr, lv, up, ur, uv) by columns."""
    n = rowptr.size - 1
    lp, up_ = [0], [0]
    lr, lv, ur, uv = [], [], [], []
    for i in range(n):
        for j in range(rowptr[i], rowptr[i + 1]):
            if colind[j] > i:
                lr.append(int(colind[j]))
                lv.append(float(val[j]))
            else:
                ur.append(int(colind[j]))
                uv.append(float(val[j]))
        lp.append(len(lr))
        up_.append(len(ur))
    for i in range(n - 1):
        multiplier = uv[up_[i + 1] - 1]
        for j in range(lp[i], lp[i + 1]):
            lv[j] /= multiplier
        for j in range(up_[i + 1], up_[i + 2] - 1):
            multiplier = uv[j]
            qn, rn = j + 1, lp[i + 1]
            pn = lp[ur[j]]
            while pn < lp[ur[j] + 1] and lr[pn] <= i + 1:
                while qn < up_[i + 2] and ur[qn] < lr[pn]:
                    qn += 1
                if qn < up_[i + 2] and lr[pn] == ur[qn]:
                    uv[qn] -= multiplier * lv[pn]
                pn += 1
            while pn < lp[ur[j] + 1]:
                while rn < lp[i + 2] and lr[rn] < lr[pn]:
                    rn += 1
                if rn < lp[i + 2] and lr[pn] == lr[rn]:
                    lv[rn] -= multiplier * lv[pn]
                pn += 1
    return lp, lr, lv, up_, ur, uv


def ilu_solve(F, x):
    """CompCol_ILUPreconditioner::solve (iluprecond.C:265-289)."""
    lp, lr, lv, up_, ur, uv = F
    n = len(lp) - 1
    work = np.zeros(n)
    for i in range(n):
        work[i] += x[i]
        for t in range(lp[i], lp[i + 1]):
            work[lr[t]] -= lv[t] * work[i]
    y = np.zeros(n)
    for i in range(n - 1, -1, -1):
        y[i] = work[i] / uv[up_[i + 1] - 1]
        for t in range(up_[i], up_[i + 1] - 1):
            work[ur[t]] -= uv[t] * y[i]
    return y


def cg_iml(rowptr, colind, val, b, rtol, maxit, precond: int):
    """IML++ CG (iml/cg.h:22-71) with lsprecond 0 (none), 1 (diagonal), 2 (ILU
    by columns) or 4 (incomplete Cholesky). Pure Python / numpy: small cases only. Returns
    (x, status, iterations, achieved) like pcg."""
    import scipy.sparse as sp
    n = rowptr.size - 1
    A = sp.csr_matrix((val, colind, rowptr), shape=(n, n))
    if precond == 4:
        F = ic_factor(rowptr, colind, val)
        msolve = lambda r: ic_solve(F, r)
    elif precond == 2:
        F = ilu_factor(rowptr, colind, val)
        msolve = lambda r: ilu_solve(F, r)
    elif precond == 1:
        d = A.diagonal()
        msolve = lambda r: r / d
    else:
        msolve = lambda r: r.copy()
    x = np.zeros(n)
    normb = np.linalg.norm(b)
    r = b - A @ x
    if normb == 0.0:
        normb = 1.0
    resid = np.linalg.norm(r) / normb
    if resid <= rtol:
        return x, 0, 0, resid
    rho_1, p = 0.0, None
    for i in range(1, maxit + 1):
        z = msolve(r)
        rho = float(r @ z)
        p = z.copy() if i == 1 else z + (rho / rho_1) * p
        q = A @ p
        alpha = rho / float(p @ q)
        x += alpha * p
        r -= alpha * q
        resid = np.linalg.norm(r) / normb
        if resid <= rtol:
            return x, 0, i, resid
        rho_1 = rho
    return x, 1, maxit, resid


def mesh_dict(mesh) -> dict:
    """Arrays of a meshgen.Mesh in the fixture layout."""
    return dict(etype=mesh.elem_type, coords=mesh.coords, conn=mesh.conn, elem_mat=mesh.elem_mat,
                mats=mesh.material_table(), bc_mask=mesh.bc_mask, bc_value=mesh.bc_value,
                nodal_load=mesh.nodal_load, thickness=mesh.thickness)


def linear_static(m: dict, rtol=1e-12, maxit=100000, load_factor=1.0, bc_factor=1.0, precond: int = 1):
    """LinearStatic::solveYourselfAt (linearstatic.C:177-253): K, load vector
    f_ext - f_int(prescribed u), Jacobi-PCG (or IML CG with lsprecond 0 / 4,
    cg_iml), then reactions (StructuralEngngModel::computeReaction,
    structengngmodel.C:183-201)."""
    et = int(m["etype"])
    bc_mask = np.asarray(m["bc_mask"])
    neq, npeq, eq = number_equations(bc_mask)
    loc = location_arrays(np.asarray(m["conn"]), eq)
    rowptr, colind = build_pattern(neq, loc)
    val = assemble_tangent(m, loc, neq, rowptr, colind)
    u_node = np.where(bc_mask == 1, np.asarray(m["bc_value"]) * bc_factor, 0.0)
    fint, _, _ = internal_forces(m, u_node)
    fext = np.asarray(m["nodal_load"]) * load_factor
    free = eq > 0
    b = np.zeros(neq)
    b[eq[free] - 1] = fext[free] - fint[free]
    if precond == 1:
        x, status, iters, ach = pcg(rowptr, colind, val, b, rtol, maxit)
    else:
        x, status, iters, ach = cg_iml(rowptr, colind, val, b, rtol, maxit, precond)
    u_node[free] = x[eq[free] - 1]
    fint, sig, eps = internal_forces(m, u_node)
    reac = np.where(bc_mask == 1, fint - fext, 0.0)
    return dict(neq=neq, eq=eq, loc=loc, rowptr=rowptr, colind=colind, val=val, b=b, x=x,
                u=u_node, reac=reac, stress=sig, strain=eps, status=status, iters=iters,
                achieved=ach)


def check_convergence(rhs_node, RT_node, eq, enorm, rtolf, nite):
    """NRSolver::checkConvergence with DOF grouping (nrsolver.C:593-790):
    per DOF id, forceErr = sqrt(sum rhs^2 / (sum RT^2 + eNorm)) over free DOFs
    (absolute when the denominator is below 1e-6); converged when every group is
    <= rtolf, and never at iteration 0 with a non-zero error."""
    ok = True
    errs = []
    for d in range(eq.shape[1]):
        free = eq[:, d] > 0
        if not free.any():
            continue
        fe = float((rhs_node[free, d] ** 2).sum())
        den = float((RT_node[free, d] ** 2).sum()) + float(enorm[d])
        err = np.sqrt(fe / den) if den >= 1e-6 else np.sqrt(fe)
        errs.append(err)
        if not np.isfinite(err) or err > rtolf * 1e20:
            raise RuntimeError("NRSolver divergence")
        if err > rtolf:
            ok = False
        if err > 0.0 and nite == 0:
            ok = False
    return ok, errs


def nonlinear_static(m: dict, times, ramp_steps: float, rtolf: float, maxiter: int, initial_guess: int = 0,
                     manrmsteps: int = 1):
    """NonLinearStatic (controlmode 1, tangent stiffness) with NRSolver
    (nrsolver.C:204-402). The tangent is assembled at the start of each step and,
    with manrmsteps k > 0, re-assembled before the solve of every iteration
    nite > 0 with nite % k == 0 (k = 1: full Newton); manrmsteps 0 is modified
    Newton, the start-of-step tangent throughout (nrsolver.C:120-126, 285-290).
    Prescribed values and loads follow
    PiecewiseLinFunction t:[0, ramp_steps] -> f:[0, 1]. initial_guess 1 is
    IG_Tangent (nlinearstatic.C:532-544): before the Newton loop the free DOFs
    take K^-1 (-sum_e K_e du_prescribed), the prescribed increment since the last
    step pushed through the tangent of the last converged state
    (EngngModel::assemblePrescribedExtrapolatedForces, engngm.C:1614-1666). The
    linear systems are solved directly (the reference decks use the default
    Skyline LDL^T). Returns a list of per-step dicts (u, reactions, stresses,
    state, iterations)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    et = int(m["etype"])
    bc_mask = np.asarray(m["bc_mask"])
    neq, npeq, eq = number_equations(bc_mask)
    loc = location_arrays(np.asarray(m["conn"]), eq)
    rowptr, colind = build_pattern(neq, loc)
    ne = np.asarray(m["conn"]).shape[0]
    state = np.zeros((ne * ngp(et), NSTATE))
    free = eq > 0
    X = np.zeros(neq)
    if initial_guess:
        # every DOF numbered (prescribed ones too) for K_e du_p over whole elements
        nall, _, eq_all = number_equations(np.zeros_like(bc_mask))
        loc_all = location_arrays(np.asarray(m["conn"]), eq_all)
        rp_all, ci_all = build_pattern(nall, loc_all)
    u_prev = np.zeros_like(np.asarray(m["bc_value"], dtype=np.float64))
    out = []
    for t in times:
        fac = float(t) / float(ramp_steps)
        u_presc = np.where(bc_mask == 1, np.asarray(m["bc_value"]) * fac, 0.0)
        RT_node = np.where(free, np.asarray(m["nodal_load"]) * fac, 0.0)
        val = assemble_tangent(m, loc, neq, rowptr, colind, state)
        if initial_guess:
            v_all = assemble_tangent(m, loc_all, nall, rp_all, ci_all, state)
            K_all = sp.csr_matrix((v_all, ci_all, rp_all), shape=(nall, nall))
            du = np.where(bc_mask == 1, u_presc - u_prev, 0.0)
            f = (K_all @ du.ravel()).reshape(du.shape)
            b = np.zeros(neq)
            b[eq[free] - 1] = -f[free]
            K = sp.csr_matrix((val, colind, rowptr), shape=(neq, neq))
            X += spla.spsolve(K.tocsc(), b)
        u_prev = u_presc
        nite = 0
        while True:
            u_node = u_presc.copy()
            u_node[free] = X[eq[free] - 1]
            F, sig, eps, en = internal_forces(m, u_node, state, want_enorm=True)
            rhs = np.where(free, RT_node - F, 0.0)
            conv, errs = check_convergence(rhs, RT_node, eq, en, rtolf, nite)
            if conv:
                break
            if nite >= maxiter:
                raise RuntimeError("NRSolver: maximum number of iterations reached")
            if nite > 0 and manrmsteps > 0 and nite % manrmsteps == 0:
                val = assemble_tangent(m, loc, neq, rowptr, colind, state)
            K = sp.csr_matrix((val, colind, rowptr), shape=(neq, neq))
            b = np.zeros(neq)
            b[eq[free] - 1] = rhs[free]
            X += spla.spsolve(K.tocsc(), b)
            nite += 1
        commit_state(m, state)
        reac = np.where(bc_mask == 1, F - np.asarray(m["nodal_load"]) * fac, 0.0)
        out.append(dict(u=u_node, reac=reac, stress=sig, strain=eps, nite=nite, state=state.copy()))
    return out


def static_structural(m: dict, nsteps: int, ramp_time: float, deltat: float = 1.0, prescribed_times=None,
                      rtolf: float = 1e-3, maxiter: int = 100000000, manrmsteps: int = 0,
                      initial_guess: int = 1):
    """StaticStructural (staticstructural.C:235-356): step n at time
    t_{n-1} + deltat (or prescribedtimes[n-1]); IG_Tangent by default, the free DOFs starting from
    the converged solution pushed by K(previous state)^-1 (-sum_e K_e du), du the
    element's total displacement at this step minus that of the last one
    (EngngModel::assembleExtrapolatedForces engngm.C:1536-1610; after
    DofDistributedPrimaryField::advanceSolution only the prescribed DOFs differ);
    NRSolver's defaults: modified Newton (no manrmsteps), rtolf 1e-3, nsmax 1e8
    (nrsolver.C:103-140). Prescribed values and loads follow the ramp
    t:[0, ramp_time] -> [0, 1]."""
    if prescribed_times is not None:
        times = [float(t) for t in prescribed_times]
    else:
        # t_n = t_{n-1} + deltat, accumulated (TimeStepController::giveNextStep)
        times, t = [], 0.0
        for _ in range(nsteps):
            t += deltat
            times.append(t)
    return nonlinear_static(m, times, ramp_time, rtolf, maxiter, initial_guess=initial_guess,
                            manrmsteps=manrmsteps)
