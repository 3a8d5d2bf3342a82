"""Generalised eigenvalues J v = lambda M v near a target (Interface.eigs)
against ARPACK shift-and-invert on the oracle's gauged pencil, the way the
reference's own tests compute reference eigenvalues (jada_fixtures.py:72-87)."""

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from conftest import load_golden
from oracle.solve import Interface as OracleInterface, bordered_matrix


def _oracle_eigs(params, nx, x, sigma, k):
    o = OracleInterface(dict(params), nx, nx)
    J = sp.csc_matrix(o.jacobian(x))
    A = bordered_matrix(J, o.pressure_row, fix_pressure_row=True)
    d = np.asarray(o.mass_matrix().diagonal()).copy()
    d[o.pressure_row] = 0.0
    M = sp.diags(d).tocsc()
    lam = sla.eigs(A, k=k, M=M, sigma=sigma, tol=1e-12, v0=np.ones(A.shape[0]))[0]
    return lam


@pytest.mark.gpu
@pytest.mark.parametrize('point', [6, 17])
def test_eigs_match_arpack_on_the_oracle_pencil(built_lib, point):
    from transiflow_gb300 import Interface
    g = load_golden('branch_ldc2d_16')
    re, x = float(g['mus'][point]), g['X'][point]
    params = {'Reynolds Number': re,
              'Eigenvalue Solver': {'Number of Eigenvalues': 4, 'Target': 0.0, 'Tolerance': 1e-12}}
    itf = Interface(dict(params), 16, 16)
    lam, V = itf.eigs(itf.vector_from_array(x), return_eigenvectors=True)
    ref = _oracle_eigs({'Reynolds Number': re}, 16, x, 0.0, 4)
    assert len(lam) == 4
    # the same eigenvalues nearest the target (a complex pair may be
    # represented by either member)
    cand = np.concatenate([ref, np.conj(ref)])
    for l in lam:
        assert np.min(np.abs(cand - l)) <= 1e-8 * max(1.0, abs(l))
    # ordered like the reference: largest real part first
    assert all(lam[i].real >= lam[i + 1].real - 1e-12 for i in range(len(lam) - 1))
    # eigenpairs of the GPU operators
    J = itf.jacobian(itf.vector_from_array(x)).to_scipy()
    M = itf.mass_matrix().to_scipy()
    for i in range(len(lam)):
        v = V[:, i]
        r = J @ v - lam[i] * (M @ v)
        assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(J @ v)
