"""Newton, pseudo-arclength continuation and time integration on the GPU
backend against the reference branch (tests/golden/branch_ldc2d_16.npz:
2D lid-driven cavity 16x16, Re 0 -> 2000, ds = 100, newton_tolerance 1e-8)."""

import io
import contextlib

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _branch(itf, cont):
    pts = []
    with contextlib.redirect_stdout(io.StringIO()):
        x0 = cont.newton(itf.vector())
        x, mu = cont.continuation(x0, 'Reynolds Number', 0, 2000, 100,
                                  callback=lambda i, xx, m: pts.append((m, xx.numpy())))
    pts.append((mu, x.numpy()))
    return pts


def test_branch_matches_reference_points():
    from transiflow_gb300 import Continuation, Interface
    g = load_golden('branch_ldc2d_16')
    itf = Interface({}, 16, 16)
    pts = _branch(itf, Continuation(itf, newton_tolerance=1e-8))
    mus = np.array([p[0] for p in pts])
    assert len(mus) == len(g['mus'])
    assert np.allclose(mus, g['mus'], rtol=1e-8, atol=1e-8)
    for (mu, x), xr in zip(pts, g['X']):
        assert np.linalg.norm(x - xr) <= 1e-8 * max(np.linalg.norm(xr), 1e-300)
    # every point is a root at its parameter value: ||F|| <= 1e-8
    for mu, x in pts[1:]:
        itf.set_parameter('Reynolds Number', mu)
        assert itf.rhs(itf.vector_from_array(x)).norm() <= 1e-8


def test_reference_driver_code_path_runs_on_device_vectors():
    """The same interface drives the continuation with bordered solves."""
    from transiflow_gb300 import Continuation, Interface
    itf = Interface({}, 12, 12)
    cont = Continuation(itf, newton_tolerance=1e-8, bordered_solver=True)
    with contextlib.redirect_stdout(io.StringIO()):
        x0 = cont.newton(itf.vector())
        x, mu = cont.continuation(x0, 'Reynolds Number', 0, 500, 100)
    assert abs(mu - 500) < 1e-3
    itf.set_parameter('Reynolds Number', mu)
    assert itf.rhs(x).norm() < 1e-7


def test_time_integration_returns_to_steady_state():
    """tests/test_continuation.py:121-165 of the reference, on the GPU."""
    from transiflow_gb300 import Continuation, Interface, TimeIntegration
    nx = 8
    itf = Interface({}, nx, nx, 1, dof=3)
    cont = Continuation(itf, newton_tolerance=1e-8)
    with contextlib.redirect_stdout(io.StringIO()):
        x0 = cont.newton(itf.vector())
        x, mu = cont.continuation(x0, 'Reynolds Number', 0, 500, 100)
        xs = x.numpy()
        m = xs.reshape(1, nx, nx, 3).copy()
        m[0, 1:nx - 1, 1:nx - 1, 0] += 0.1 * np.random.default_rng(0).random((nx - 2, nx - 2))
        x2 = itf.vector_from_array(m.ravel())
        ti = TimeIntegration(itf)
        x3, t = ti.integration(x2, 100, 1000)
    assert np.linalg.norm(xs[0::3] - x3.numpy()[0::3]) < 1e-4
    assert np.linalg.norm(xs[1::3] - x3.numpy()[1::3]) < 1e-4


def test_save_and_load_state_round_trip(tmp_path):
    """save_state / load_state (the reference's checkpoint format: a .npy state
    and a .params JSON file) restore the state and the parameters."""
    import numpy as np
    from transiflow_gb300 import Interface
    itf = Interface({'Reynolds Number': 250}, 8, 6)
    x = itf.vector_from_array(np.random.default_rng(9).standard_normal(itf.n))
    name = str(tmp_path / 'point')
    itf.save_state(name, x)
    other = Interface({'Reynolds Number': 10}, 8, 6)
    y = other.load_state(name)
    assert other.get_parameter('Reynolds Number') == 250
    assert np.array_equal(other.array_from_vector(y), itf.array_from_vector(x))
