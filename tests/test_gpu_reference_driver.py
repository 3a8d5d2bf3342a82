"""The reference's own drivers (transiflow/Continuation.py,
transiflow/TimeIntegration.py) running unchanged on the CUDA backend through
``transiflow_gb300.Interface``, against the package's own drivers on the same
backend: the same parameter sequence and interface calls, states within 1e-10
relative (the backend's boundary products add with atomics, so two runs
differ at rounding level), and every branch point at ||F|| <= 1e-8.

The reference package comes from an installed copy (``baseline/_ref``, a
``pip install --no-deps`` of the reference); the tests are skipped where
there is none."""

import contextlib
import io
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INSTALLED = os.path.join(ROOT, 'baseline', '_ref')


def _reference():
    if not os.path.isdir(os.path.join(INSTALLED, 'transiflow')):
        pytest.skip('no installed copy of the reference package')
    if INSTALLED not in sys.path:
        sys.path.insert(0, INSTALLED)
    from transiflow.Continuation import Continuation
    from transiflow.TimeIntegration import TimeIntegration
    return Continuation, TimeIntegration


class _Recording:
    """The CUDA interface with a log of the calls a driver makes."""

    def __init__(self, itf):
        self.inner = itf
        self.calls = []

    def __getattr__(self, name):
        return getattr(self.inner, name)

    def set_parameter(self, name, value):
        self.calls.append(('set', name))
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


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize('kwargs', [{'newton_tolerance': 1e-8},
                                    {'newton_tolerance': 1e-8, 'bordered_solver': True}])
def test_reference_continuation_runs_on_the_cuda_backend(kwargs):
    from transiflow_gb300 import Interface
    from transiflow_gb300.continuation import Continuation
    RefContinuation, _ = _reference()
    runs = []
    for cls in (RefContinuation, Continuation):
        itf = _Recording(Interface({'CUDA': {'Tolerance': 1e-10}}, 16, 16))
        cont = cls(itf, **kwargs)
        pts = []
        with contextlib.redirect_stdout(io.StringIO()):
            x0 = cont.newton(itf.vector())
            x, mu = cont.continuation(x0, 'Reynolds Number', 0, 2000, 100,
                                      callback=lambda i, xx, m: pts.append((m, xx.numpy())))
        runs.append((pts, x.numpy(), mu, list(itf.calls), itf.inner))
    (rp, rx, rmu, rcalls, ritf), (pp, px, pmu, pcalls, _) = runs
    assert abs(rmu - 2000) < 1e-3 and abs(pmu - rmu) <= 1e-9 * abs(rmu)
    assert len(rp) == len(pp) >= 10
    for (ma, xa), (mb, xb) in zip(rp, pp):
        assert abs(ma - mb) <= 1e-9 * max(abs(mb), 1.0)
        assert _rel(xa, xb) <= 1e-10
        ritf.set_parameter('Reynolds Number', ma)
        assert ritf.rhs(ritf.vector_from_array(xa)).norm() <= 1e-8
    assert _rel(rx, px) <= 1e-10
    assert rcalls == pcalls


def test_reference_time_integration_runs_on_the_cuda_backend():
    from transiflow_gb300 import Interface
    from transiflow_gb300.continuation import TimeIntegration
    _, RefTimeIntegration = _reference()
    out = []
    x0 = 0.01 * np.random.default_rng(3).standard_normal(8 * 8 * 3)
    for cls in (RefTimeIntegration, TimeIntegration):
        itf = _Recording(Interface({'Reynolds Number': 100, 'CUDA': {'Tolerance': 1e-12}}, 8, 8))
        ts = []
        with contextlib.redirect_stdout(io.StringIO()):
            x, t = cls(itf, theta=0.5).integration(itf.vector_from_array(x0), 0.1, 0.3,
                                                    callback=lambda i, xx, tt: ts.append(tt))
        out.append((x.numpy(), t, ts, itf.calls))
    assert out[0][1] == out[1][1] and out[0][2] == out[1][2]
    assert _rel(out[0][0], out[1][0]) <= 1e-10
    assert out[0][3] == out[1][3]
