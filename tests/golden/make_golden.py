"""Generate the golden fixtures in this directory by running the reference.

Usage (needs the reference checkout, which only this container has):
    PYTHONPATH=/root/reference python tests/golden/make_golden.py [fixture names]

Every fixture is computed by the reference itself (BIMAU/transiflow 1.0.1):
``transiflow.Discretization`` for RHS / Jacobian / mass matrix,
``transiflow.interface.SciPy.Interface`` for solves and
``transiflow.Continuation`` for the branch.  The GPU tests compare against
these files, since the reference cannot run on the GPU machine.
"""

import io
import contextlib
import os
import sys

import numpy as np

REF = os.environ.get('TRANSIFLOW_REFERENCE', '/root/reference')
sys.path.insert(0, REF)

from transiflow import Discretization, Continuation          # noqa: E402
from transiflow.interface.SciPy import Interface            # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

# (name, parameters, nx, ny, nz, dim, dof, states)
# states: ('normal', seed, count) -> N(0,1) draws; ('ramp',) -> state[i] = i+1
CASES = [
    ('ldc2d_16_re1000', {'Reynolds Number': 1000}, 16, 16, 1, None, None, ('normal', 0, 8)),
    ('ldc2d_16_re0', {'Reynolds Number': 0}, 16, 16, 1, None, None, ('normal', 0, 2)),
    ('ldc2d_12x10_stretched', {'Reynolds Number': 500, 'Grid Stretching': True}, 12, 10, 1, None, None,
     ('normal', 1, 2)),
    ('ldc3d_4_ramp', {'Reynolds Number': 100}, 4, 4, 4, 3, 4, ('ramp',)),
    ('ldc3d_5x4x3_stretched', {'Reynolds Number': 100, 'Grid Stretching': True}, 5, 4, 3, 3, 4,
     ('normal', 2, 2)),
    ('ldc_semi2d_4', {'Reynolds Number': 100}, 4, 4, 1, 3, 4, ('ramp',)),
    ('dhc2d_8_stretched', {'Problem Type': 'Differentially Heated Cavity', 'Prandtl Number': 1000,
                           'Rayleigh Number': 1e3, 'Reynolds Number': 1, 'Grid Stretching Factor': 1.5},
     8, 8, 1, None, None, ('normal', 3, 2)),
    ('dhc3d_4_ramp', {'Reynolds Number': 1, 'Rayleigh Number': 100, 'Prandtl Number': 100,
                      'Problem Type': 'Differentially Heated Cavity'}, 4, 4, 4, 3, 5, ('ramp',)),
    ('rb3d_4_ramp', {'Reynolds Number': 1, 'Rayleigh Number': 100, 'Prandtl Number': 100,
                     'Problem Type': 'Rayleigh-Benard'}, 4, 4, 4, 3, 5, ('ramp',)),
    ('rb2d_6x5', {'Reynolds Number': 1, 'Rayleigh Number': 1000, 'Prandtl Number': 10,
                  'Problem Type': 'Rayleigh-Benard', 'Biot Number': 0.5, 'Asymmetry Parameter': 0.1},
     6, 5, 1, None, None, ('normal', 4, 2)),
    ('rbp2d_6x5', {'Reynolds Number': 1, 'Rayleigh Number': 1000, 'Prandtl Number': 10,
                   'Problem Type': 'Rayleigh-Benard Perturbation', 'Biot Number': 0.5},
     6, 5, 1, None, None, ('normal', 5, 1)),
    ('qg2d_4_ramp', {'Reynolds Number': 16, 'Rossby Parameter': 1000, 'Wind Stress Parameter': 1000,
                     'Problem Type': 'Double Gyre'}, 4, 4, 1, 2, 4, ('ramp',)),
    ('qg2d_8x6', {'Reynolds Number': 30, 'Rossby Parameter': 500, 'Wind Stress Parameter': 700,
                  'Asymmetry Parameter': 0.3, 'Problem Type': 'Double Gyre'}, 8, 6, 1, None, None,
     ('normal', 6, 2)),
    ('amoc2d_4_ramp', {'Reynolds Number': 16, 'Rayleigh Number': 4e4, 'Prandtl Number': 2.25,
                       'Lewis Number': 1, 'Temperature Forcing': 1, 'Freshwater Flux': 1,
                       'Problem Type': 'AMOC'}, 4, 4, 1, 2, 5, ('ramp',)),
    ('amoc2d_8x4', {'Rayleigh Number': 4e4, 'Prandtl Number': 2.25, 'Lewis Number': 1.2,
                    'Temperature Forcing': 0.7, 'Freshwater Flux': 0.1, 'Asymmetry Parameter': 0.2,
                    'X-max': 5, 'Problem Type': 'AMOC'}, 8, 4, 1, None, None, ('normal', 7, 2)),
]


def _states(spec, n):
    if spec[0] == 'ramp':
        return np.arange(1, n + 1, dtype=np.float64)[None, :]
    _, seed, count = spec
    return np.random.default_rng(seed).standard_normal((count, n))


def discretization_fixture(name, params, nx, ny, nz, dim, dof, spec):
    d = Discretization(dict(params), nx, ny, nz, dim, dof)
    n = nx * ny * nz * d.dof
    X = _states(spec, n)
    out = {'nx': nx, 'ny': ny, 'nz': nz, 'dim': d.dim, 'dof': d.dof, 'states': X,
           'params': np.array(repr(params))}
    rhs, begs, cols, vals = [], [], [], []
    for s in X:
        rhs.append(d.rhs(s))
        A = d.jacobian(s)
        k = A.begA[-1]
        begs.append(np.asarray(A.begA, dtype=np.int64))
        cols.append(np.asarray(A.jcoA[:k], dtype=np.int64))
        vals.append(np.asarray(A.coA[:k]))
    out['rhs'] = np.array(rhs)
    out['begA'] = np.array(begs)
    out['nnz'] = np.array([len(c) for c in cols])
    out['jcoA'] = np.concatenate(cols)
    out['coA'] = np.concatenate(vals)
    M = d.mass_matrix()
    out['mass_begA'] = np.asarray(M.begA, dtype=np.int64)
    out['mass_jcoA'] = np.asarray(M.jcoA[:M.begA[-1]], dtype=np.int64)
    out['mass_coA'] = np.asarray(M.coA[:M.begA[-1]])
    out['x'], out['y'], out['z'] = d.x, d.y, d.z
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **out)


def solve_fixture():
    """Direct and bordered solves of the SciPy backend (SciPy.py:204-258)."""
    itf = Interface({'Reynolds Number': 700}, 12, 12)
    rng = np.random.default_rng(11)
    n = 12 * 12 * 3
    state = rng.standard_normal(n) * 0.3
    b = rng.standard_normal(n)
    V = rng.standard_normal(n)
    W = rng.standard_normal(n)
    J = itf.jacobian(state)
    y = itf.solve(J, b)
    J = itf.jacobian(state)
    y1, y2 = itf.solve(J, b, 0.37, V, W, -1.3)
    np.savez_compressed(os.path.join(HERE, 'solve_ldc2d_12.npz'), state=state, b=b, V=V, W=W, y=y, y1=y1,
                        y2=np.array(y2), rhs2=np.array(0.37), C=np.array(-1.3), re=np.array(700.0))


def branch_fixture():
    """Config-1 branch: 2D LDC 16x16, Newton at Re=0, continuation 0 -> 2000,
    ds = 100, newton_tolerance = 1e-8 (Continuation.py:361-482)."""
    itf = Interface({}, 16, 16)
    cont = Continuation(itf, newton_tolerance=1e-8)
    pts = []
    with contextlib.redirect_stdout(io.StringIO()):
        x0 = cont.newton(itf.vector())
        x, mu = cont.continuation(x0, 'Reynolds Number', 0, 2000, 100,
                                  callback=lambda i, xx, m: pts.append((m, np.array(xx))))
    pts.append((mu, np.array(x)))
    np.savez_compressed(os.path.join(HERE, 'branch_ldc2d_16.npz'), mus=np.array([p[0] for p in pts]),
                        X=np.array([p[1] for p in pts]), x0=np.array(x0))


def main(names=None):
    """Write every fixture, or only the named ones."""
    for case in CASES:
        if names and case[0] not in names:
            continue
        discretization_fixture(*case)
        print('wrote', case[0])
    if not names or 'solve_ldc2d_12' in names:
        solve_fixture()
        print('wrote solve_ldc2d_12')
    if not names or 'branch_ldc2d_16' in names:
        branch_fixture()
        print('wrote branch_ldc2d_16')


if __name__ == '__main__':
    main(sys.argv[1:])
