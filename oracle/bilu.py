"""Block ILU(0)-preconditioned GMRES on the oracle's gauged Jacobians
(TEST INFRASTRUCTURE ONLY).

This is the study behind the GPU solver's choice of an exact multifrontal
factorisation over block ILU(0) as the preconditioner of its Krylov solves
(tests/test_bilu_study.py runs it).  Block ILU(0): dof x dof cell blocks in
the natural cell order (x fastest), no fill outside the block pattern of the
matrix, the diagonal blocks inverted exactly -- the block variant of ILU(0)
in Saad, Iterative Methods for Sparse Linear Systems, 2nd ed., 10.3 and 10.7.
The gauge follows the reference's direct solve (transiflow/interface/
SciPy.py:93-103, restated in oracle/solve.py: bordered_matrix).
"""

import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import LinearOperator, gmres, spsolve_triangular

from .solve import bordered_matrix


def gauged(itf, state):
    """The oracle interface's Jacobian at ``state`` with the pressure gauge
    of the reference's direct solve, as CSR."""
    J = itf.jacobian(state)
    fix = itf.dof > itf.dim
    return sp.csr_matrix(bordered_matrix(J, itf.pressure_row, fix_pressure_row=fix))


def block_ilu0(A, b):
    """Block ILU(0) of CSR ``A`` with b x b blocks: returns (L, U), L unit
    block-lower and U block-upper triangular CSR matrices on the block
    pattern of A, with A ~ L U."""
    B = sp.bsr_matrix(A, blocksize=(b, b))
    B.sort_indices()
    indptr, indices = B.indptr, B.indices
    data = B.data.astype(np.float64).copy()
    nb = A.shape[0] // b
    diag = np.empty(nb, dtype=np.int64)
    inv_diag = np.empty((nb, b, b))
    for i in range(nb):
        lo, hi = indptr[i], indptr[i + 1]
        pos = {int(c): p for p, c in zip(range(lo, hi), indices[lo:hi])}
        for p in range(lo, hi):
            k = int(indices[p])
            if k >= i:
                break
            data[p] = data[p] @ inv_diag[k]
            for q in range(diag[k] + 1, indptr[k + 1]):
                j = int(indices[q])
                t = pos.get(j)
                if t is not None:
                    data[t] -= data[p] @ data[q]
        diag[i] = pos[i]
        try:
            inv_diag[i] = np.linalg.inv(data[diag[i]])
        except np.linalg.LinAlgError:
            inv_diag[i] = np.linalg.pinv(data[diag[i]])
    # the strictly lower blocks form L (unit diagonal added); the diagonal
    # blocks, whole, and the upper blocks form U
    Fc = sp.bsr_matrix((data, indices, indptr), shape=A.shape).tocoo()
    lower_block = (Fc.row // b) > (Fc.col // b)
    L = sp.csr_matrix((Fc.data[lower_block], (Fc.row[lower_block], Fc.col[lower_block])), shape=A.shape)
    L = (L + sp.identity(A.shape[0], format='csr')).tocsr()
    U = sp.csr_matrix((Fc.data[~lower_block], (Fc.row[~lower_block], Fc.col[~lower_block])), shape=A.shape)
    return L.tocsr(), U.tocsr()


def gmres_iterations(A, rhs, precond, restart, maxit, rtol=1e-8):
    """Right-preconditioned GMRES(restart): SciPy's GMRES on A M^-1 u = rhs,
    x = M^-1 u, so the residual it monitors is the true one, rhs - A x.
    Returns the iterations until ||rhs - A x|| <= rtol ||rhs|| (None if that
    does not happen within maxit iterations) and the relative residual
    reached."""
    hist = []
    n = A.shape[0]
    AM = LinearOperator((n, n), matvec=lambda u: A @ precond(u))
    u, _ = gmres(AM, rhs, rtol=rtol, atol=0.0, restart=restart, maxiter=max(1, maxit // restart),
                 callback=lambda r: hist.append(float(r)), callback_type='pr_norm')
    its = next((k + 1 for k, r in enumerate(hist) if r <= rtol), None)
    x = precond(u)
    return its, float(np.linalg.norm(rhs - A @ x) / np.linalg.norm(rhs))


def bilu_preconditioner(A, b):
    L, U = block_ilu0(A, b)

    def apply(v):
        y = spsolve_triangular(L, v, lower=True, unit_diagonal=True)
        return spsolve_triangular(U, y, lower=False)
    return apply
