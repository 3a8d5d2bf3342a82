"""The package's continuation and time-integration drivers against the
reference's own drivers (transiflow/Continuation.py, TimeIntegration.py),
both running over the same CPU backend (the oracle interface), so that every
difference would come from the drivers: same parameter sequence, same
states bit for bit, same interface calls.  Skipped where the reference
package is not importable."""

import contextlib
import io
import sys

import numpy as np
import pytest

from conftest import REFERENCE, has_reference
from oracle.solve import Interface as OracleInterface

pytestmark = pytest.mark.skipif(not has_reference(), reason='reference package not available')


def _reference():
    if REFERENCE not in sys.path:
        sys.path.insert(0, REFERENCE)
    from transiflow.Continuation import Continuation
    from transiflow.TimeIntegration import TimeIntegration
    return Continuation, TimeIntegration


class _Recording:
    """The oracle interface with a log of every call the driver makes."""

    def __init__(self, params, nx, ny):
        self.inner = OracleInterface(params, nx, ny)
        self.calls = []

    def __getattr__(self, name):
        return getattr(self.inner, name)

    def set_parameter(self, name, value):
        self.calls.append(('set', name, value))
        self.inner.set_parameter(name, value)

    def rhs(self, x):
        self.calls.append(('rhs',))
        return self.inner.rhs(x)

    def jacobian(self, x):
        self.calls.append(('jacobian',))
        return self.inner.jacobian(x)

    def solve(self, jac, *args):
        self.calls.append(('solve', len(args)))
        return self.inner.solve(jac, *args)


def _branch(cls, kwargs, target=1200.0, ds=100.0):
    itf = _Recording({}, 10, 10)
    cont = cls(itf, **kwargs)
    pts = []
    with contextlib.redirect_stdout(io.StringIO()):
        x0 = cont.newton(itf.vector())
        out = cont.continuation(x0, 'Reynolds Number', 0, target, ds, return_step=True,
                                callback=lambda i, xx, m: pts.append((m, np.array(xx))))
    return pts, out, itf.calls


@pytest.mark.parametrize('kwargs,ds', [
    ({'newton_tolerance': 1e-8}, 100.0),
    ({'newton_tolerance': 1e-8, 'bordered_solver': True}, 100.0),
    ({'newton_tolerance': 1e-7, 'residual_check': 'dx'}, 100.0),
    # steps too long for a budget of 4 iterations: failed correctors, retries
    # with halved steps and the landing on the target
    ({'newton_tolerance': 1e-8, 'maximum_newton_iterations': 4}, 800.0),
])
def test_continuation_matches_reference_driver(kwargs, ds):
    from transiflow_gb300.continuation import Continuation
    RefContinuation, _ = _reference()
    ref_pts, ref_out, ref_calls = _branch(RefContinuation, kwargs, ds=ds)
    pts, out, calls = _branch(Continuation, kwargs, ds=ds)
    assert [m for m, _ in pts] == [m for m, _ in ref_pts]
    for (_, a), (_, b) in zip(pts, ref_pts):
        assert np.array_equal(a, b)
    assert calls == ref_calls
    assert out[1] == ref_out[1] and out[3] == ref_out[3]
    assert np.array_equal(out[0], ref_out[0]) and np.array_equal(out[2], ref_out[2])


def test_continuation_with_a_given_direction_matches_reference_driver():
    from transiflow_gb300.continuation import Continuation
    RefContinuation, _ = _reference()
    res = []
    for cls in (RefContinuation, Continuation):
        itf = _Recording({}, 8, 8)
        cont = cls(itf, newton_tolerance=1e-8)
        with contextlib.redirect_stdout(io.StringIO()):
            x, mu, dx, dmu = cont.continuation(cont.newton(itf.vector()), 'Reynolds Number', 0, 300, 100,
                                               return_step=True)
            x2, mu2 = cont.continuation(x, 'Reynolds Number', mu, 900, 100, dx=dx.copy(), dmu=dmu)
        res.append((x2, mu2, itf.calls))
    assert res[0][1] == res[1][1]
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][2] == res[1][2]


def test_time_integration_matches_reference_driver():
    from transiflow_gb300.continuation import TimeIntegration
    _, RefTimeIntegration = _reference()
    out = []
    for cls in (RefTimeIntegration, TimeIntegration):
        itf = _Recording({'Reynolds Number': 100}, 8, 8)
        ts = []
        x0 = 0.01 * np.random.default_rng(3).standard_normal(itf.inner.vector().size)
        with contextlib.redirect_stdout(io.StringIO()):
            x, t = cls(itf, theta=0.5).integration(x0, 0.1, 0.3, callback=lambda i, xx, tt: ts.append(tt))
        out.append((x, t, ts, itf.calls))
    assert out[0][1] == out[1][1] and out[0][2] == out[1][2]
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][3] == out[1][3]


def test_checkpoint_files_interchange_with_reference(tmp_path):
    """Parameter and state files written by the package's stand-in base class
    (used when the reference is not importable) are read by the reference's
    BaseInterface, and the other way round."""
    _reference()
    from transiflow.interface.BaseInterface import BaseInterface
    from transiflow_gb300.interface import _Checkpointing

    class Mine(_Checkpointing):
        def __init__(self, p):
            self.parameters = p

        def array_from_vector(self, v):
            return np.asarray(v)

    params = {'Reynolds Number': np.float64(1500.0), 'Count': np.int32(3), 'Shift': 1 + 2j,
              'Profile': np.arange(3.0), 'Problem Type': 'Lid-driven Cavity'}
    x = np.random.default_rng(0).standard_normal(12)
    with contextlib.redirect_stdout(io.StringIO()):
        Mine(dict(params)).save_state(str(tmp_path / 'a'), x)
        ref = BaseInterface({'Reynolds Number': 0.0}, 2, 2, 1, 2, 3)
        y = ref.load_state(str(tmp_path / 'a'))
        ref.save_state(str(tmp_path / 'b'), 2 * y)
        mine = Mine({})
        z = mine.load_state(str(tmp_path / 'b'))
    assert np.array_equal(y, x) and np.array_equal(z, 2 * x)
    assert ref.parameters['Shift'] == 1 + 2j and ref.parameters['Count'] == 3
    assert mine.parameters == {'Reynolds Number': 1500.0, 'Count': 3, 'Shift': 1 + 2j,
                               'Profile': [0.0, 1.0, 2.0], 'Problem Type': 'Lid-driven Cavity'}
