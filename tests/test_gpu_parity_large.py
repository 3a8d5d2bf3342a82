"""Branch parity at the benchmark sizes.  Continuation branches may take
different steps than the reference's (different solvers give different
Newton counts, so the step-size control picks other parameter values), so at
a GPU point (x, mu) the GPU backend's Newton root and the oracle's Newton
root at the same mu, both started from the GPU point and tightened to
||F|| < 1e-11, are compared (a branch point itself is only converged to
||F|| <= 1e-8, which at 256^2 leaves it up to ~1e-6 from the exact root):

  * 2D lid-driven cavity 256^2, FP64, Re 0 -> 5000 with ds = 200 (the plain
    2D workload): three points against the oracle's roots;
  * differentially heated cavity 128^2, tanh stretch 1.5, Pr = 1000, Ra
    0 -> 1e6, mixed precision (FP32 factors, FP32 inner products, FP64
    refinement): the error of every point against the FP64 GPU root at its
    Rayleigh number, three points against the oracle's roots;
  * 3D lid-driven cavity 32^3, mixed precision, Re 0 -> 2000: the oracle's
    residual of two GPU points.

Every accepted point must satisfy ||F|| <= 1e-8."""

import contextlib
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _branch(itf, name, start, target, ds, ds_max=1000.0):
    from transiflow_gb300 import Continuation
    cont = Continuation(itf, newton_tolerance=1e-8, quiet=True)
    pts = []
    itf.set_parameter(name, start)
    x0 = cont.newton(itf.vector())
    x, mu = cont.continuation(x0, name, start, target, ds, ds_max=ds_max,
                              callback=lambda i, xx, m: pts.append((m, xx.numpy())))
    pts.append((mu, x.numpy()))
    return pts


def _gpu_root(itf, name, mu, x_guess):
    from transiflow_gb300 import Continuation
    itf.set_parameter(name, mu)
    with contextlib.redirect_stdout(io.StringIO()):
        return Continuation(itf).newton(itf.vector_from_array(x_guess), tol=1e-11).numpy()


def _oracle_root(params, shape, name, mu, x_guess):
    from oracle.solve import Interface as OracleInterface
    from transiflow_gb300.continuation import Continuation
    p = dict(params)
    p[name] = mu
    itf = OracleInterface(p, *shape)
    with contextlib.redirect_stdout(io.StringIO()):
        return Continuation(itf).newton(np.array(x_guess), tol=1e-11)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _fnorm(itf, name, mu, x):
    itf.set_parameter(name, mu)
    return itf.rhs(itf.vector_from_array(x)).norm()


def test_ldc256_fp64_branch_points_are_oracle_roots():
    from transiflow_gb300 import Interface
    itf = Interface({'CUDA': {'Tolerance': 1e-10}}, 256, 256)
    pts = _branch(itf, 'Reynolds Number', 0.0, 5000.0, 200.0)
    assert abs(pts[-1][0] - 5000.0) < 1e-3
    for mu, x in pts[1:]:
        assert _fnorm(itf, 'Reynolds Number', mu, x) <= 1e-8
    for k in (1, len(pts) // 2, len(pts) - 1):
        mu, x = pts[k]
        xg = _gpu_root(itf, 'Reynolds Number', mu, x)
        xr = _oracle_root({}, (256, 256), 'Reynolds Number', mu, x)
        assert _rel(xg, xr) <= 1e-8, (mu, _rel(xg, xr))
        assert _rel(x, xr) <= 1e-4, (mu, _rel(x, xr))


DHC = {'Problem Type': 'Differentially Heated Cavity', 'Prandtl Number': 1000, 'Reynolds Number': 1,
       'Grid Stretching Factor': 1.5}


def test_dhc128_mixed_precision_error_per_point():
    from transiflow_gb300 import Interface
    mixed = Interface(dict(DHC, CUDA={'Factor Precision': 'fp32', 'Inner Precision': 'fp32', 'Tolerance': 1e-10}),
                      128, 128)
    pts = _branch(mixed, 'Rayleigh Number', 0.0, 1e6, 100.0, ds_max=1e8)
    assert abs(pts[-1][0] - 1e6) < 1e-3 * 1e6
    fp64 = Interface(dict(DHC, CUDA={'Factor Precision': 'fp64', 'Tolerance': 1e-12}), 128, 128)
    errors = []
    for mu, x in pts[1:]:
        assert _fnorm(mixed, 'Rayleigh Number', mu, x) <= 1e-8
        x64 = _gpu_root(fp64, 'Rayleigh Number', mu, x)
        xm = _gpu_root(mixed, 'Rayleigh Number', mu, x)
        # the mixed-precision solver's root against the FP64 one, and the
        # branch point (converged to ||F|| <= 1e-8) against the FP64 root
        errors.append((mu, _rel(xm, x64), _rel(x, x64)))
        assert _rel(xm, x64) <= 1e-9, errors[-1]
    print('mixed precision per point (Ra, root error, branch-point error vs the FP64 root):', errors)
    for k in (1, len(pts) // 2, len(pts) - 1):
        mu, x = pts[k]
        xg = _gpu_root(mixed, 'Rayleigh Number', mu, x)
        xr = _oracle_root(DHC, (128, 128), 'Rayleigh Number', mu, x)
        assert _rel(xg, xr) <= 1e-8, (mu, _rel(xg, xr))


def test_ldc3d32_mixed_branch_points_satisfy_oracle_equations():
    from oracle.solve import Interface as OracleInterface
    from transiflow_gb300 import Interface
    itf = Interface({'CUDA': {'Factor Precision': 'fp32', 'Tolerance': 1e-10}}, 32, 32, 32)
    pts = _branch(itf, 'Reynolds Number', 0.0, 2000.0, 100.0)
    assert abs(pts[-1][0] - 2000.0) < 1e-3
    for mu, x in pts[1:]:
        assert _fnorm(itf, 'Reynolds Number', mu, x) <= 1e-8
    for mu, x in (pts[len(pts) // 2], pts[-1]):
        o = OracleInterface({'Reynolds Number': mu}, 32, 32, 32)
        assert np.linalg.norm(o.rhs(x)) <= 1e-8, mu
