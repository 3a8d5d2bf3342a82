"""Restatement of the SciPy backend's direct solve (TEST INFRASTRUCTURE ONLY).

Follows transiflow/interface/SciPy.py of BIMAU/transiflow 1.0.1:
  compute_bordered_matrix  SciPy.py:51-129
  _compute_factorization   SciPy.py:131-162 (LU cached on the matrix object)
  direct_solve             SciPy.py:204-258
The factorisation is SciPy's SuperLU (``scipy.sparse.linalg.splu``, default
COLAMD ordering) called on the same CSC arrays the reference builds.
"""

import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import splu

from . import fvm


def _as_columns(V):
    V = np.asarray(V, dtype=np.float64)
    return V[:, None] if V.ndim == 1 else V


def bordered_matrix(jac, pressure_row, V=None, W=None, C=None, fix_pressure_row=True,
                    border_scaling=1e-3):
    """Gauged and optionally bordered CSC matrix ``[A, sV; sW^T, s^2 C]``.

    The reference walks the CSC arrays column by column: the gauge column is
    replaced by a single -1 on the diagonal and every entry in the gauge row is
    dropped; border entries follow each column's own entries (SciPy.py:93-126).
    """
    jac = jac.tocsc()
    n = jac.shape[0]
    b = 0
    if V is not None:
        Vc = _as_columns(V)
        b = Vc.shape[1]
        Wc = Vc if W is None else _as_columns(W)
        if C is None:
            Cm = np.zeros((b, b))
        elif np.ndim(C) == 0:
            Cm = np.full((b, b), float(C))
        else:
            Cm = np.asarray(C, dtype=np.float64).reshape(b, b)
    col = np.repeat(np.arange(n), np.diff(jac.indptr))
    row = jac.indices.astype(np.int64)
    val = jac.data.astype(np.float64)
    seq = np.arange(len(val), dtype=np.int64)
    if fix_pressure_row:
        keep = (row != pressure_row) & (col != pressure_row)
        col, row, val, seq = col[keep], row[keep], val[keep], seq[keep]
        col = np.append(col, pressure_row)
        row = np.append(row, pressure_row)
        val = np.append(val, -1.0)
        seq = np.append(seq, -1)
    big = len(jac.data) + 1
    # the gauge column carries no border entry (the `continue` at SciPy.py:100)
    bcols = np.arange(n)
    if fix_pressure_row:
        bcols = bcols[bcols != pressure_row]
    for j in range(b):
        col = np.concatenate([col, bcols])
        row = np.concatenate([row, np.full(len(bcols), n + j)])
        val = np.concatenate([val, border_scaling * Wc[bcols, j]])
        seq = np.concatenate([seq, np.full(len(bcols), big + j)])
    order = np.lexsort((seq, col))
    col, row, val = col[order], row[order], val[order]
    ptr = np.zeros(n + b + 1, dtype=np.int64)
    np.add.at(ptr, col + 1, 1)
    ptr = np.cumsum(ptr)
    rows = [row]
    vals = [val]
    for i in range(b):
        rows.append(np.arange(n))
        vals.append(border_scaling * Vc[:, i])
        rows.append(n + np.arange(b))
        vals.append(border_scaling * border_scaling * Cm[:, i])
        ptr[n + 1 + i] = ptr[n + i] + n + b
    data = np.concatenate(vals)
    indices = np.concatenate(rows)
    return sp.csc_matrix((data, indices, ptr), shape=(n + b, n + b))


class Interface:
    """The SciPy backend's contract over the oracle discretisation:
    vector, rhs, jacobian, mass_matrix, solve, set/get_parameter."""

    def __init__(self, parameters, nx, ny, nz=1, dim=None, dof=None, x=None, y=None, z=None):
        self.parameters = parameters
        self.discretization = fvm.Discretization(parameters, nx, ny, nz, dim, dof, x, y, z)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dim = self.discretization.dim
        self.dof = self.discretization.dof
        self.pressure_row = self.dim
        self.border_scaling = 1e-3

    def vector(self):
        return np.zeros(self.nx * self.ny * self.nz * self.dof)

    def set_parameter(self, name, value):
        self.discretization.set_parameter(name, value)

    def get_parameter(self, name):
        return self.discretization.get_parameter(name)

    def rhs(self, state):
        return self.discretization.rhs(state)

    def jacobian(self, state):
        return self.discretization.jacobian(state).to_scipy().tocsc()

    def mass_matrix(self):
        return self.discretization.mass_matrix().to_scipy().tocsc()

    def _factorize(self, jac, V, W, C):
        lu = getattr(jac, 'lu', None)
        bordered = getattr(jac, 'bordered_lu', False)
        if lu is not None and (V is not None) == bordered:
            return
        fix = self.dof > self.dim and self.pressure_row is not None
        A = bordered_matrix(jac, self.pressure_row, V, W, C, fix, self.border_scaling)
        jac.lu = splu(A)
        jac.bordered_lu = V is not None

    def solve(self, jac, rhs, rhs2=None, V=None, W=None, C=None):
        x = np.array(rhs, dtype=np.float64, copy=True)
        if self.dof > self.dim:
            x[self.pressure_row] = 0
        if rhs2 is not None:
            x = np.append(rhs, rhs2 * self.border_scaling)
        self._factorize(jac, V, W, C)
        y = jac.lu.solve(x)
        if jac.bordered_lu:
            b = rhs2.shape[0] if hasattr(rhs2, 'shape') and len(rhs2.shape) > 0 else 1
            y1 = y[:-b]
            y2 = y[-b:] * self.border_scaling
            if np.isscalar(rhs2):
                y2 = y2.item()
            return y1, y2
        return y
