"""Analysis drivers on the GPU path: the reference's StaticStructural engineering
model (src/sm/EngineeringModels/staticstructural.C) stepping a GpuModel, and the
two load-time functions its decks use (ConstantFunction, PiecewiseLinFunction).

Every step runs on the device through ogb_nonlinear_step: tangent assembly,
internal forces with the material update, the NRSolver convergence test and the
PCG solves; the host only evaluates the time functions and scales the
prescribed values and nodal loads of the step.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np

from . import native

IG_NONE = 0
IG_TANGENT = 1

# PiecewiseLinFunction_PRECISION (src/core/piecewiselinfunction.C:44)
_PLF_PRECISION = 1e-12

_CTX = struct.Struct("<8sid")
_CTX_MAGIC = b"OGBSSCTX"


class ConstantFunction:
    """ConstantFunction (src/core/constantfunction.h): f(t) = value."""

    def __init__(self, value: float = 1.0):
        self.value = float(value)

    def evaluate_at_time(self, t: float) -> float:
        return self.value


class PiecewiseLinFunction:
    """PiecewiseLinFunction::evaluateAtTime (src/core/piecewiselinfunction.C:51-82):
    a date within 1e-12 of t gives its value; between dates, linear
    interpolation; after the last date, the last value. Before the first date
    the reference returns that first DATE (not its value) with a warning; this
    is kept so decks evaluate identically."""

    def __init__(self, t, f):
        self.t = [float(v) for v in t]
        self.f = [float(v) for v in f]
        if not self.t or len(self.t) != len(self.f):
            raise ValueError("PiecewiseLinFunction: undefined dates and values")

    def evaluate_at_time(self, time: float) -> float:
        for i, (d, v) in enumerate(zip(self.t, self.f)):
            if abs(d - time) < _PLF_PRECISION:
                return v
            if d > time:
                if i == 0:
                    return d
                xa, xb = self.t[i - 1], d
                ya, yb = self.f[i - 1], v
                return ya + (time - xa) * (yb - ya) / (xb - xa)
        return self.f[-1]


@dataclass
class StepResult:
    number: int
    time: float
    u: np.ndarray            # node displacements (nnodes x ndofpn), prescribed values included
    reactions: np.ndarray    # reactions at prescribed DOFs (zero elsewhere)
    iterations: int          # NRSolver iterations of the step


class StaticStructural:
    """StaticStructural (staticstructural.C) over a GpuModel and its GpuCsrMtrx.

    Keywords follow the analysis record: ``nsteps``, ``deltat`` (default 1) or
    ``prescribed_times`` (prescribedtimes, overriding nsteps), ``initial_guess``
    (initialGuess, default IG_Tangent), and NRSolver's ``rtolf`` (default 1e-3),
    ``maxiter`` (default 1e8) and ``manrmsteps`` (default 0: modified Newton,
    nrsolver.C:103-140). ``lstol`` / ``precision`` configure the PCG of each
    linear solve (the lstol of the solver record). ``bc_function`` /
    ``load_function`` scale the mesh's prescribed values and nodal loads (the
    loadTimeFunction of its boundary conditions and loads); ``bc_at`` / ``load_at``
    (callables of t) replace them when each condition has its own function, as
    read from a deck (oofem_gb300.deck).

    Step times accumulate as in TimeStepController::giveNextStep
    (timestepcontroller.C:74-101): t_n = t_{n-1} + deltat. A step that does not
    converge raises native.OgbError (the reference's ConvergenceException); the
    material state then stays at the last converged step."""

    def __init__(self, model: "native.GpuModel", matrix: "native.GpuCsrMtrx", nsteps: int = 1,
                 deltat: float = 1.0, prescribed_times=None, bc_function=None, load_function=None,
                 rtolf: float = 1e-3, maxiter: int = 100000000, manrmsteps: int = 0,
                 initial_guess: int = IG_TANGENT, lstol: float = 1e-12, precision: int = native.PREC_FP64,
                 bc_at=None, load_at=None):
        if initial_guess not in (IG_NONE, IG_TANGENT):
            raise ValueError(f"Initial guess type: {initial_guess} not supported")
        self.model = model
        self.matrix = matrix
        self.prescribed_times = None if prescribed_times is None else [float(t) for t in prescribed_times]
        self.nsteps = len(self.prescribed_times) if self.prescribed_times else int(nsteps)
        self.deltat = float(deltat)
        self.bc_function = bc_function or ConstantFunction()
        self.load_function = load_function or ConstantFunction()
        m = model.mesh
        # prescribed values and nodal loads at time t: the mesh's patterns times one
        # function each, unless a deck gives them per DOF and load (bc_at / load_at)
        self.bc_at = bc_at or (lambda t: m.bc_value * self.bc_function.evaluate_at_time(t))
        self.load_at = load_at or (lambda t: m.nodal_load * self.load_function.evaluate_at_time(t))
        self.rtolf = float(rtolf)
        self.maxiter = int(maxiter)
        self.manrmsteps = int(manrmsteps)
        self.initial_guess = int(initial_guess)
        self.lstol = float(lstol)
        self.precision = int(precision)
        self.time = 0.0
        self.step = 0
        model.set_initial_guess(self.initial_guess)
        model.set_nr_mode(self.manrmsteps)

    def give_end_of_time_of_interest(self) -> float:
        """StaticStructural::giveEndOfTimeOfInterest (staticstructural.C:192-198)."""
        if self.prescribed_times:
            return self.prescribed_times[-1]
        return self.deltat * self.nsteps

    def _next_time(self) -> float:
        if self.prescribed_times:
            return self.prescribed_times[self.step]
        return self.time + self.deltat

    def solve_yourself_at(self) -> StepResult:
        """StaticStructural::solveYourselfAt (staticstructural.C:235-356) for the next step."""
        if self.step >= self.nsteps:
            raise RuntimeError("StaticStructural: all steps solved")
        t = self._next_time()
        bcv = self.bc_at(t)
        load = self.load_at(t)
        u, reac, nite = self.model.nonlinear_step(self.matrix, bcv, load, rtolf=self.rtolf, maxiter=self.maxiter,
                                                  lin_rtol=self.lstol, precision=self.precision)
        self.step += 1
        self.time = t
        return StepResult(self.step, t, u, reac, nite)

    def save_context(self) -> bytes:
        """EngngModel::saveStepContext / saveContext (engngm.C:768-777, 1755-1812)
        between steps: the
        step number and time, then the model's device state (material statuses,
        Newton solution, last prescribed values)."""
        return _CTX.pack(_CTX_MAGIC, self.step, self.time) + self.model.save_state()

    def restore_context(self, blob: bytes):
        """EngngModel::restoreContext (engngm.C:1814-1850): continue after the
        saved step; the
        following steps are bit-identical to an uninterrupted run."""
        magic, step, time = _CTX.unpack_from(blob)
        if magic != _CTX_MAGIC:
            raise ValueError("not a StaticStructural context")
        if not 0 <= step <= self.nsteps:
            raise ValueError(f"context of step {step} outside this analysis ({self.nsteps} steps)")
        self.model.restore_state(blob[_CTX.size:])
        self.step, self.time = step, time

    def solve_yourself(self):
        """All remaining steps (EngngModel::solveYourself); a list of StepResult."""
        return [self.solve_yourself_at() for _ in range(self.step, self.nsteps)]
