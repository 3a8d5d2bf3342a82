"""The other configurations of the workload family at test sizes:
differentially heated cavity on a tanh-stretched grid (plain FP64 factors vs
the mixed FP32-factor mode, both against the CPU oracle), a 3D lid-driven
cavity branch, and the semi-2D case.  Every accepted point must satisfy
||F|| <= 1e-8 and agree with the oracle's Newton root at the same parameter."""

import io
import contextlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _branch(itf, name, start, target, ds, tol=1e-8):
    from transiflow_gb300 import Continuation
    cont = Continuation(itf, newton_tolerance=tol)
    pts = []
    with contextlib.redirect_stdout(io.StringIO()):
        itf.set_parameter(name, start)
        x0 = cont.newton(itf.vector())
        x, mu = cont.continuation(x0, name, start, target, ds,
                                  callback=lambda i, xx, m: pts.append((m, xx.numpy())))
    pts.append((mu, x.numpy()))
    return pts


def _gpu_root(itf, name, mu, x_guess):
    """Newton of the GPU backend at fixed mu, tightened to ||F|| < 1e-11."""
    from transiflow_gb300.continuation import Continuation
    itf.set_parameter(name, mu)
    c = Continuation(itf)
    with contextlib.redirect_stdout(io.StringIO()):
        return c.newton(itf.vector_from_array(x_guess), tol=1e-11).numpy()


def _oracle_root(params, shape, name, mu, x_guess, dim=None, dof=None):
    """Newton of the CPU oracle at fixed mu, started from the GPU point."""
    from oracle.solve import Interface as OracleInterface
    from transiflow_gb300.continuation import Continuation
    p = dict(params)
    p[name] = mu
    itf = OracleInterface(p, *shape, dim=dim, dof=dof)
    c = Continuation(itf)
    with contextlib.redirect_stdout(io.StringIO()):
        return c.newton(np.array(x_guess), tol=1e-11)


DHC = {'Problem Type': 'Differentially Heated Cavity', 'Prandtl Number': 1000, 'Reynolds Number': 1,
       'Grid Stretching Factor': 1.5}


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_dhc_stretched_branch_matches_oracle(precision):
    from transiflow_gb300 import Interface
    p = dict(DHC)
    p['CUDA'] = {'Factor Precision': precision, 'Tolerance': 1e-12}
    itf = Interface(p, 24, 24)
    pts = _branch(itf, 'Rayleigh Number', 0.0, 1e5, 2e4)
    assert abs(pts[-1][0] - 1e5) < 1e-3
    for mu, x in pts[1::10]:
        itf.set_parameter('Rayleigh Number', mu)
        assert itf.rhs(itf.vector_from_array(x)).norm() <= 1e-8
        # the problem is ill-conditioned (Pr = 1000), so ||F|| <= 1e-8 alone fixes x
        # only to ~1e-7; compare the roots both backends converge to from this point
        xg = _gpu_root(itf, 'Rayleigh Number', mu, x)
        xr = _oracle_root(DHC, (24, 24), 'Rayleigh Number', mu, x)
        assert np.linalg.norm(xg - xr) <= 1e-8 * np.linalg.norm(xr)


def test_mixed_and_plain_solvers_reach_the_same_roots():
    """FP32 factors (mixed) and FP64 factors (plain) converge to the same
    roots: Newton from the same points of a plain branch, tightened to
    ||F|| < 1e-11, agree within 1e-8 relative."""
    from transiflow_gb300 import Interface
    itfs = {}
    for precision in ('fp64', 'fp32'):
        p = dict(DHC)
        p['CUDA'] = {'Factor Precision': precision, 'Tolerance': 1e-12}
        itfs[precision] = Interface(p, 20, 20)
    pts = _branch(itfs['fp64'], 'Rayleigh Number', 0.0, 5e4, 1e4)
    for mu, x in pts[1::8]:
        a = _gpu_root(itfs['fp64'], 'Rayleigh Number', mu, x)
        b = _gpu_root(itfs['fp32'], 'Rayleigh Number', mu, x)
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(a)


def test_ldc3d_branch_matches_oracle():
    from transiflow_gb300 import Interface
    itf = Interface({}, 6, 6, 6)
    pts = _branch(itf, 'Reynolds Number', 0.0, 400.0, 100.0)
    assert abs(pts[-1][0] - 400.0) < 1e-3
    for mu, x in pts[1:]:
        itf.set_parameter('Reynolds Number', mu)
        assert itf.rhs(itf.vector_from_array(x)).norm() <= 1e-8
        xg = _gpu_root(itf, 'Reynolds Number', mu, x)
        xr = _oracle_root({}, (6, 6, 6), 'Reynolds Number', mu, x)
        assert np.linalg.norm(xg - xr) <= 1e-8 * np.linalg.norm(xr)


def test_semi2d_branch_matches_2d_branch():
    """tests/test_continuation.py:83-93 of the reference: 3D with nz = 1 agrees
    with the 2D formulation (there within 1e-2; the states here agree to the
    Newton tolerance because both branches run on the same solver)."""
    from transiflow_gb300 import Interface
    x2 = _branch(Interface({}, 8, 8, 1, 2), 'Reynolds Number', 0.0, 500.0, 100.0)[-1][1]
    x3 = _branch(Interface({}, 8, 8, 1, 3), 'Reynolds Number', 0.0, 500.0, 100.0)[-1][1]
    assert np.linalg.norm(x2[0::3] - x3[0::4]) < 1e-2
    assert np.linalg.norm(x2[1::3] - x3[1::4]) < 1e-2
    assert np.linalg.norm(x2[2::3] - x3[3::4]) < 1e-2


def test_preconditioner_reuse_gives_same_solutions():
    from transiflow_gb300 import Interface
    res = {}
    for reuse in (False, True):
        itf = Interface({'CUDA': {'Reuse Factorization': reuse, 'Reuse Policy': 'always', 'Tolerance': 1e-12}},
                        24, 24)
        pts = _branch(itf, 'Reynolds Number', 0.0, 1000.0, 200.0)
        res[reuse] = (pts, dict(itf.solver.stats))
    a, b = res[False][0], res[True][0]
    assert len(a) == len(b)
    for (ma, xa), (mb, xb) in zip(a, b):
        assert abs(ma - mb) <= 1e-8 * max(abs(ma), 1.0)
        assert np.linalg.norm(xa - xb) <= 1e-8 * max(np.linalg.norm(xa), 1e-300)
    assert res[True][1]['factorizations'] < res[False][1]['factorizations']
    assert res[True][1]['reused'] > 0


def test_graph_replay_matches_eager_launches():
    """The factorisation and solve replayed from CUDA graphs give the same
    solutions as eager launches."""
    from transiflow_gb300 import Interface
    rng = np.random.default_rng(9)
    s = 0.3 * rng.standard_normal(32 * 32 * 3)
    bs = [rng.standard_normal(32 * 32 * 3) for _ in range(4)]
    out = {}
    for graphs in (False, True):
        itf = Interface({'Reynolds Number': 800, 'CUDA': {'CUDA Graphs': graphs, 'Reuse Factorization': False}},
                        32, 32)
        ys = []
        for t, b in enumerate(bs):
            J = itf.jacobian(itf.vector_from_array(s + 0.01 * t))
            ys.append(itf.solve(J, itf.vector_from_array(b)).numpy())
        out[graphs] = (ys, itf.solver.stats['graph_kernel_launches'])
    for ya, yb in zip(out[False][0], out[True][0]):
        assert np.linalg.norm(ya - yb) <= 1e-10 * np.linalg.norm(ya)
    assert out[True][1] > 0 and out[False][1] == 0


QG = {'Problem Type': 'Double Gyre', 'Reynolds Number': 16, 'Rossby Parameter': 1000,
      'Wind Stress Parameter': 0}


def test_double_gyre_wind_branch_matches_oracle():
    """The reference's double-gyre continuation (test_continuation.py:400-416):
    wind stress 0 -> 1000 at Re = 16, beta = 1000; every accepted point is a
    root of the oracle's equations too."""
    from transiflow_gb300 import Interface
    itf = Interface(dict(QG), 16, 16)
    pts = _branch(itf, 'Wind Stress Parameter', 0.0, 1000.0, 200.0)
    assert abs(pts[-1][0] - 1000.0) < 1e-3
    assert np.linalg.norm(pts[-1][1]) > 0
    for mu, x in pts[1:]:
        itf.set_parameter('Wind Stress Parameter', mu)
        assert itf.rhs(itf.vector_from_array(x)).norm() <= 1e-8
        xg = _gpu_root(itf, 'Wind Stress Parameter', mu, x)
        xr = _oracle_root(QG, (16, 16), 'Wind Stress Parameter', mu, x)
        assert np.linalg.norm(xg - xr) <= 1e-8 * np.linalg.norm(xr)


AMOC = {'Problem Type': 'AMOC', 'Rayleigh Number': 4e4, 'Prandtl Number': 2.25, 'X-max': 5}


def test_amoc_branches_match_oracle():
    """The reference's AMOC continuation (test_continuation.py:430-466):
    temperature forcing 0 -> 1, then freshwater flux 0 -> 0.2, at 16 x 8;
    every accepted point is a root of the oracle's equations too."""
    from transiflow_gb300 import Interface
    itf = Interface(dict(AMOC), 16, 8)
    pts = _branch(itf, 'Temperature Forcing', 0.0, 1.0, 0.1)
    assert abs(pts[-1][0] - 1.0) < 1e-3
    for mu, x in pts[1::3]:
        itf.set_parameter('Temperature Forcing', mu)
        assert itf.rhs(itf.vector_from_array(x)).norm() <= 1e-8
        xg = _gpu_root(itf, 'Temperature Forcing', mu, x)
        xr = _oracle_root(AMOC, (16, 8), 'Temperature Forcing', mu, x)
        assert np.linalg.norm(xg - xr) <= 1e-8 * np.linalg.norm(xr)
    from transiflow_gb300 import Continuation
    itf.set_parameter('Temperature Forcing', 1.0)
    cont = Continuation(itf, newton_tolerance=1e-8, quiet=True)
    fw = []
    x, mu = cont.continuation(itf.vector_from_array(pts[-1][1]), 'Freshwater Flux', 0.0, 0.2, 0.01,
                              callback=lambda i, xx, m: fw.append((m, xx.numpy())))
    assert abs(mu - 0.2) < 1e-3
    p = dict(AMOC, **{'Temperature Forcing': 1.0})
    for m, xf in fw[1::4] + [(mu, x.numpy())]:
        itf.set_parameter('Freshwater Flux', m)
        xg = _gpu_root(itf, 'Freshwater Flux', m, xf)
        xr = _oracle_root(p, (16, 8), 'Freshwater Flux', m, xf)
        assert np.linalg.norm(xg - xr) <= 1e-8 * np.linalg.norm(xr)
