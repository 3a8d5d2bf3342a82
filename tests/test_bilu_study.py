"""Why the GPU solver factors the Jacobian exactly instead of using block
ILU(0): right-preconditioned GMRES with block ILU(0) (dof x dof cell blocks,
natural order; oracle/bilu.py) makes no progress on the gauged saddle-point
Jacobians of the lid-driven cavity, in Stokes flow and with convection,
while the exact factorisation of the same matrix solves it in one
iteration.  The residuals are the true ones, ||b - A x|| / ||b||."""

import numpy as np
import pytest
from scipy.sparse.linalg import splu

from oracle import bilu
from oracle.solve import Interface


@pytest.mark.parametrize('re,state', [(0.0, 'zero'), (5000.0, 'random')])
def test_block_ilu0_gmres_stalls_where_the_exact_factorisation_solves(re, state):
    n = 32
    itf = Interface({'Reynolds Number': re}, n, n)
    rng = np.random.default_rng(1)
    x = np.zeros(itf.dof * n * n) if state == 'zero' else rng.standard_normal(itf.dof * n * n)
    A = bilu.gauged(itf, x)
    L, U = bilu.block_ilu0(A, itf.dof)
    # ILU(0): the product matches A on A's block pattern
    assert abs((L @ U - A).multiply(A != 0)).max() <= 1e-10 * abs(A).max()
    b = rng.standard_normal(A.shape[0])
    b[itf.pressure_row] = 0.0
    its, res = bilu.gmres_iterations(A, b, bilu.bilu_preconditioner(A, itf.dof), restart=50, maxit=300)
    assert its is None or res > 1e-2
    assert res > 1e-2
    lu = splu(A.tocsc())
    its, res = bilu.gmres_iterations(A, b, lu.solve, restart=50, maxit=50)
    assert its is not None and its <= 2 and res <= 1e-10
