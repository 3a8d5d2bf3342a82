"""The CPU oracle against the reference: its golden files and fixtures
generated by running it (tests/golden/make_golden.py).  No GPU needed."""

import io
import contextlib
import os

import numpy as np
import pytest

from conftest import DISC_FIXTURES, REFERENCE, golden_csr, golden_params, has_reference, load_golden
from oracle import fvm
from oracle.solve import Interface as OracleInterface


@pytest.mark.parametrize('name', DISC_FIXTURES)
def test_oracle_matches_reference_fixture(name):
    g = load_golden(name)
    d = fvm.Discretization(golden_params(g), int(g['nx']), int(g['ny']), int(g['nz']),
                           int(g['dim']), int(g['dof']))
    for t, s in enumerate(g['states']):
        assert np.array_equal(d.rhs(s), g['rhs'][t])
        A = d.jacobian(s)
        b, j, v = golden_csr(g, t)
        assert np.array_equal(A.begA, b)
        assert np.array_equal(A.jcoA, j)
        assert np.array_equal(A.coA, v)
    M = d.mass_matrix()
    assert np.array_equal(M.begA, g['mass_begA'])
    assert np.array_equal(M.coA, g['mass_coA'])


def _read_matrix(path):
    rows, cols, vals = [], [], []
    with open(path) as f:
        for line in f:
            r, c, v = line.split()
            rows.append(int(r) - 1)
            cols.append(int(c) - 1)
            vals.append(float(v))
    rows = np.array(rows)
    n = rows.max() + 1
    beg = np.zeros(n + 1, dtype=np.int64)
    np.add.at(beg, rows + 1, 1)
    return np.cumsum(beg), np.array(cols), np.array(vals)


# (golden file stem, parameters, dof, what) -- tests/test_fvm.py:547-1137 of the reference
REFERENCE_GOLDENS = [
    ('ldc_lin', {'Reynolds Number': 100}, 4, 'lin'),
    ('bous_lin', {'Reynolds Number': 1, 'Rayleigh Number': 100, 'Prandtl Number': 100}, 5, 'lin'),
    ('ldc_bnd', {'Reynolds Number': 100}, 4, 'bnd'),
    ('bous_bnd', {'Reynolds Number': 1, 'Rayleigh Number': 100, 'Prandtl Number': 100,
                  'Problem Type': 'Rayleigh-Benard'}, 5, 'bnd'),
    ('ldc', {'Reynolds Number': 100}, 4, 'full'),
    ('ldc_stretched', {'Reynolds Number': 100, 'Grid Stretching': True}, 4, 'full'),
    ('bous', {'Reynolds Number': 1, 'Rayleigh Number': 100, 'Prandtl Number': 100,
              'Problem Type': 'Rayleigh-Benard'}, 5, 'full'),
    ('bous_stretched', {'Reynolds Number': 1, 'Rayleigh Number': 100, 'Prandtl Number': 100,
                        'Problem Type': 'Rayleigh-Benard', 'Grid Stretching': True}, 5, 'full'),
    ('dhc', {'Reynolds Number': 1, 'Rayleigh Number': 100, 'Prandtl Number': 100,
             'Problem Type': 'Differentially Heated Cavity'}, 5, 'full'),
]


def _assemble_unfiltered_order(atom, nx, ny, nz, dof):
    """Rows of an atom in the reference test's own assembly order
    (tests/test_fvm.py:431-454): no wrap, config order (z, y, x, d2)."""
    d = fvm.Discretization({}, nx, ny, nz, 3, dof)
    rows, cols, vals = [], [], []
    row = 0
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                for d1 in range(dof):
                    for z in range(3):
                        for y in range(3):
                            for x in range(3):
                                for d2 in range(dof):
                                    a = atom[i, j, k, d1, d2, x, y, z]
                                    if abs(a) > 1e-14:
                                        rows.append(row)
                                        cols.append(row + (x - 1) * dof + (y - 1) * nx * dof
                                                    + (z - 1) * nx * ny * dof + d2 - d1)
                                        vals.append(a)
                    row += 1
    n = nx * ny * nz * dof
    beg = np.zeros(n + 1, dtype=np.int64)
    np.add.at(beg, np.array(rows) + 1, 1)
    return np.cumsum(beg), np.array(cols), np.array(vals)


@pytest.mark.skipif(not has_reference(), reason='reference golden files not available')
@pytest.mark.parametrize('stem,params,dof,what', REFERENCE_GOLDENS)
def test_oracle_matches_reference_golden_files(stem, params, dof, what):
    """The reference's own 4x4x4 golden matrices and vectors (state i+1)."""
    path = os.path.join(REFERENCE, 'tests', 'data', '%s_4x4x4.txt' % stem)
    b_ref, c_ref, v_ref = _read_matrix(path)
    n = 4 * 4 * 4 * dof
    d = fvm.Discretization(dict(params), 4, 4, 4, 3, dof)
    state = np.arange(1, n + 1, dtype=np.float64)
    if what == 'lin':
        b, c, v = _assemble_unfiltered_order(d.linear_part(), 4, 4, 4, dof)
        exact = True
    elif what == 'bnd':
        atom = d.linear_part()
        d.boundaries(atom)
        A = d.assemble_jacobian(atom)
        b, c, v = A.begA, A.jcoA, A.coA
        exact = stem == 'ldc_bnd'
    else:
        A = d.jacobian(state)
        b, c, v = A.begA, A.jcoA, A.coA
        exact = False
    assert np.array_equal(b[:len(b_ref)], b_ref)
    assert np.array_equal(c[:len(c_ref)], c_ref)
    if exact:
        assert np.array_equal(v[:len(v_ref)], v_ref)
    else:
        assert np.allclose(v[:len(v_ref)], v_ref, rtol=1e-6, atol=0)
    if what == 'full':
        rhs_ref = np.loadtxt(os.path.join(REFERENCE, 'tests', 'data', '%s_rhs_4x4x4.txt' % stem))
        assert np.allclose(d.rhs(state), rhs_ref, rtol=1e-6, atol=1e-12)


@pytest.mark.skipif(not has_reference(), reason='reference golden files not available')
def test_oracle_matches_reference_double_gyre_golden_file():
    """The reference's own quasi-geostrophic (Double Gyre) 4x4x1 golden
    matrix and right-hand side (test_fvm.py:1177-1215, state i+1)."""
    params = {'Reynolds Number': 16, 'Rossby Parameter': 1000, 'Wind Stress Parameter': 1000,
              'Problem Type': 'Double Gyre'}
    b_ref, c_ref, v_ref = _read_matrix(os.path.join(REFERENCE, 'tests', 'data', 'qg_4x4x1.txt'))
    d = fvm.Discretization(dict(params), 4, 4, 1, 2, 4)
    state = np.arange(1, 4 * 4 * 4 + 1, dtype=np.float64)
    A = d.jacobian(state)
    assert np.array_equal(A.begA[:len(b_ref)], b_ref)
    assert np.array_equal(A.jcoA[:len(c_ref)], c_ref)
    assert np.allclose(A.coA[:len(v_ref)], v_ref, rtol=1e-6, atol=0)
    rhs_ref = np.loadtxt(os.path.join(REFERENCE, 'tests', 'data', 'qg_rhs_4x4x1.txt'))
    assert np.allclose(d.rhs(state), rhs_ref, rtol=1e-6, atol=1e-12)


@pytest.mark.skipif(not has_reference(), reason='reference golden files not available')
def test_oracle_matches_reference_amoc_golden_file():
    """The reference's own AMOC 4x4x1 golden matrix and right-hand side
    (test_fvm.py:1217-1255, state i+1)."""
    params = {'Reynolds Number': 16, 'Rayleigh Number': 4e4, 'Prandtl Number': 2.25, 'Lewis Number': 1,
              'Temperature Forcing': 1, 'Freshwater Flux': 1, 'Problem Type': 'AMOC'}
    b_ref, c_ref, v_ref = _read_matrix(os.path.join(REFERENCE, 'tests', 'data', 'amoc_4x4x1.txt'))
    d = fvm.Discretization(dict(params), 4, 4, 1, 2, 5)
    state = np.arange(1, 4 * 4 * 5 + 1, dtype=np.float64)
    A = d.jacobian(state)
    assert np.array_equal(A.begA[:len(b_ref)], b_ref)
    assert np.array_equal(A.jcoA[:len(c_ref)], c_ref)
    assert np.allclose(A.coA[:len(v_ref)], v_ref, rtol=1e-6, atol=0)
    rhs_ref = np.loadtxt(os.path.join(REFERENCE, 'tests', 'data', 'amoc_rhs_4x4x1.txt'))
    assert np.allclose(d.rhs(state), rhs_ref, rtol=1e-6, atol=1e-12)


def test_oracle_solve_matches_fixture():
    g = load_golden('solve_ldc2d_12')
    itf = OracleInterface({'Reynolds Number': float(g['re'])}, 12, 12)
    J = itf.jacobian(g['state'])
    assert np.array_equal(itf.solve(J, g['b']), g['y'])
    J = itf.jacobian(g['state'])
    y1, y2 = itf.solve(J, g['b'], float(g['rhs2']), g['V'], g['W'], float(g['C']))
    assert np.array_equal(y1, g['y1'])
    assert y2 == float(g['y2'])


def test_jacobian_fd_consistency():
    """tests/test_jacobian.py:139-230 of the reference on a 13x7x5 grid."""
    rng = np.random.default_rng(7)
    nx, ny, nz, dof = 13, 7, 5, 5
    d = fvm.Discretization({'Reynolds Number': 100, 'Rayleigh Number': 1e3, 'Prandtl Number': 10,
                            'Problem Type': 'Differentially Heated Cavity'}, nx, ny, nz, 3, dof)

    def rand_state():
        m = rng.random((nx, ny, nz, dof))
        m[nx - 1, :, :, 0] = 0
        m[:, ny - 1, :, 1] = 0
        m[:, :, nz - 1, 2] = 0
        return fvm.state_vec(m)

    s, p = rand_state(), rand_state()
    A = d.jacobian(s).to_scipy()
    f0 = d.rhs(s)
    for i in range(3, 9):
        eps = 10.0 ** -i
        assert np.linalg.norm((d.rhs(s + eps * p) - f0) / eps - A @ p) < max(eps, 10.0 ** (-14 + i)) * 10


def test_continuation_driver_matches_reference_branch():
    """transiflow_gb300.Continuation over the oracle reproduces the branch the
    reference Continuation computed over the reference SciPy backend."""
    from transiflow_gb300.continuation import Continuation
    g = load_golden('branch_ldc2d_16')
    itf = OracleInterface({}, 16, 16)
    cont = Continuation(itf, newton_tolerance=1e-8)
    pts = []
    with contextlib.redirect_stdout(io.StringIO()):
        x0 = cont.newton(itf.vector())
        x, mu = cont.continuation(x0, 'Reynolds Number', 0, 2000, 100,
                                  callback=lambda i, xx, m: pts.append((m, np.array(xx))))
    pts.append((mu, np.array(x)))
    assert np.array_equal(np.array([p[0] for p in pts]), g['mus'])
    assert np.array_equal(np.array([p[1] for p in pts]), g['X'])
