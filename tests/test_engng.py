"""Host logic of the StaticStructural driver (no GPU): the load-time functions
against the reference's PiecewiseLinFunction rules, step times accumulated as
TimeStepController does, and the per-step scaling of prescribed values and
loads handed to the device step (a recording stand-in for GpuModel)."""
import numpy as np
import pytest

from oofem_gb300 import engng


def test_piecewise_lin_function():
    f = engng.PiecewiseLinFunction([0.0, 2.0, 4.0], [0.0, 1.0, 0.5])
    assert f.evaluate_at_time(1.0) == 0.5
    assert f.evaluate_at_time(2.0 + 1e-13) == 1.0          # within the 1e-12 date precision
    assert f.evaluate_at_time(3.0) == 0.75
    assert f.evaluate_at_time(5.0) == 0.5                  # after the last date: last value
    g = engng.PiecewiseLinFunction([1.0, 2.0], [7.0, 8.0])
    assert g.evaluate_at_time(0.5) == 1.0                  # before the first date: the date itself
    assert engng.ConstantFunction(3.0).evaluate_at_time(123.0) == 3.0
    with pytest.raises(ValueError):
        engng.PiecewiseLinFunction([], [])


class _Mesh:
    bc_value = np.array([[1.0, 2.0]])
    nodal_load = np.array([[0.0, -4.0]])


class _Model:
    mesh = _Mesh()

    def __init__(self):
        self.calls = []
        self.ig = self.nr = None

    def set_initial_guess(self, k):
        self.ig = k

    def set_nr_mode(self, k):
        self.nr = k

    def nonlinear_step(self, A, bcv, load, rtolf, maxiter, lin_rtol, precision):
        self.calls.append((bcv.copy(), load.copy(), rtolf, maxiter, lin_rtol, precision))
        return bcv, np.zeros_like(bcv), len(self.calls)


def test_static_structural_steps_and_defaults():
    m = _Model()
    ramp = engng.PiecewiseLinFunction([0.0, 0.3], [0.0, 1.0])
    ss = engng.StaticStructural(m, None, nsteps=3, deltat=0.1, bc_function=ramp)
    assert m.ig == engng.IG_TANGENT and m.nr == 0          # the reference's defaults
    res = ss.solve_yourself()
    # 0.1 + 0.1 + 0.1 accumulated, not 3 * 0.1
    t = 0.0
    for k, r in enumerate(res):
        t += 0.1
        assert r.time == t and r.number == k + 1 and r.iterations == k + 1
        np.testing.assert_array_equal(m.calls[k][0], _Mesh.bc_value * ramp.evaluate_at_time(t))
        np.testing.assert_array_equal(m.calls[k][1], _Mesh.nodal_load)   # constant load function
        assert m.calls[k][2] == 1e-3 and m.calls[k][3] == 100000000
    assert ss.give_end_of_time_of_interest() == pytest.approx(0.3)
    with pytest.raises(RuntimeError):
        ss.solve_yourself_at()


def test_static_structural_prescribed_times():
    m = _Model()
    ss = engng.StaticStructural(m, None, nsteps=99, prescribed_times=[0.5, 2.0], manrmsteps=3,
                                initial_guess=engng.IG_NONE)
    assert ss.nsteps == 2 and m.nr == 3 and m.ig == engng.IG_NONE
    assert [r.time for r in ss.solve_yourself()] == [0.5, 2.0]
    assert ss.give_end_of_time_of_interest() == 2.0
    with pytest.raises(ValueError):
        engng.StaticStructural(_Model(), None, initial_guess=5)


class _StateModel(_Model):
    def __init__(self):
        super().__init__()
        self.restored = None

    def save_state(self):
        return b"DEVICE-STATE"

    def restore_state(self, blob):
        self.restored = blob


def test_context_round_trip_host_side():
    """save_context prefixes the step number and time to the model's state blob;
    restore_context checks the prefix and resumes after the saved step."""
    m = _StateModel()
    ss = engng.StaticStructural(m, None, nsteps=4, deltat=0.25)
    ss.solve_yourself_at()
    ss.solve_yourself_at()
    blob = ss.save_context()
    m2 = _StateModel()
    ss2 = engng.StaticStructural(m2, None, nsteps=4, deltat=0.25)
    ss2.restore_context(blob)
    assert m2.restored == b"DEVICE-STATE" and ss2.step == 2 and ss2.time == 0.5
    assert [r.time for r in ss2.solve_yourself()] == [0.75, 1.0]
    with pytest.raises(ValueError):
        ss2.restore_context(b"X" * len(blob))
    with pytest.raises(ValueError):
        engng.StaticStructural(_StateModel(), None, nsteps=1).restore_context(blob)   # step 2 > nsteps 1
