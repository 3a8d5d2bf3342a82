"""Device matrices returned by the CUDA interface.

``StencilMatrix`` is the Jacobian in the fixed-width stencil CSR (pattern
shared by every Jacobian of one interface, values per matrix).
``DiagonalMatrix`` is the mass matrix.  Together they provide what the
drivers use: ``A @ x`` (TimeIntegration.py:47), ``J - M / (theta dt)``
(TimeIntegration.py:58), plus export to the reference's compressed CSR for
parity checks (CrsMatrix.compress, CrsMatrix.py:52-71).

Like the reference's Jacobian objects (SciPy.py:131-162), a StencilMatrix
carries the factorisation of its gauged values once ``solve`` computed it, so
the two solves of one Newton-corrector iteration share it.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .vector import DeviceVector, _stream


class Pattern:
    """Row pointers and columns of the stencil CSR of one grid (device)."""

    def __init__(self, rowptr, cols, n, width, row_offset, slot):
        self.rowptr = rowptr
        self.cols = cols
        self.n = n
        self.width = width
        self.row_offset = row_offset
        self.slot = slot

    @property
    def nnz(self):
        return int(self.cols.numel())


class StencilMatrix:
    def __init__(self, pattern, values, gauge=None):
        self.pattern = pattern
        self.values = values
        self.gauge = gauge
        self.lu = None          # cached factorisation (solver.Factorization)
        self.bordered_lu = False

    @property
    def shape(self):
        return (self.pattern.n, self.pattern.n)

    @property
    def dtype(self):
        return np.dtype(np.float64)

    @property
    def nnz(self):
        return self.pattern.nnz

    def matvec(self, x, out=None, values=None):
        lib = _lib.load()
        if not isinstance(x, DeviceVector):
            x = DeviceVector.from_array(np.asarray(x))
        y = out if out is not None else DeviceVector(torch.empty_like(x.data))
        v = self.values if values is None else values
        _lib.check(lib.tf_spmv_f64(self.pattern.n, self.pattern.rowptr.data_ptr(), self.pattern.cols.data_ptr(),
                                   v.data_ptr(), x.data.data_ptr(), y.data.data_ptr(), 1.0, 0.0, _stream()),
                   'tf_spmv_f64')
        return y

    def __matmul__(self, x):
        if isinstance(x, DeviceVector):
            return self.matvec(x)
        return self.matvec(DeviceVector.from_array(np.asarray(x))).numpy()

    def _with_values(self, values):
        return StencilMatrix(self.pattern, values)

    def copy(self):
        return self._with_values(self.values.clone())

    def __sub__(self, other):
        if isinstance(other, DiagonalMatrix):
            return self._add_diag(-1.0, other)
        return NotImplemented

    def __add__(self, other):
        if isinstance(other, DiagonalMatrix):
            return self._add_diag(1.0, other)
        return NotImplemented

    def _add_diag(self, a, D):
        out = self.values.clone()
        lib = _lib.load()
        _lib.check(lib.tf_add_diagonal(self.pattern.n, self.pattern.rowptr.data_ptr(),
                                       self.pattern.cols.data_ptr(), out.data_ptr(), a,
                                       D.diag.data_ptr(), _stream()), 'tf_add_diagonal')
        return self._with_values(out)

    def __mul__(self, s):
        out = torch.empty_like(self.values)
        lib = _lib.load()
        _lib.check(lib.tf_vec_axpby(out.numel(), float(s), self.values.data_ptr(), 0.0, None,
                                    out.data_ptr(), _stream()), 'tf_vec_axpby')
        return self._with_values(out)

    __rmul__ = __mul__

    def __truediv__(self, s):
        return self * (1 / s)

    def __neg__(self):
        return self * -1.0

    # -- export --------------------------------------------------------------
    def compact(self):
        """Reference-format CSR (begA, jcoA, coA) as NumPy arrays."""
        lib = _lib.load()
        n = self.pattern.n
        dev = self.values.device
        rowptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
        wbytes = lib.tf_csr_compact_workspace_bytes(n)
        work = torch.empty((wbytes + 7) // 8, dtype=torch.float64, device=dev)
        nnz = ctypes.c_int64(0)
        _lib.check(lib.tf_csr_compact(n, self.pattern.rowptr.data_ptr(), self.pattern.cols.data_ptr(),
                                      self.values.data_ptr(), rowptr.data_ptr(), None, None, ctypes.byref(nnz),
                                      work.data_ptr(), wbytes, _stream()), 'tf_csr_compact')
        cols = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)
        vals = torch.empty(max(nnz.value, 1), dtype=torch.float64, device=dev)
        _lib.check(lib.tf_csr_compact(n, self.pattern.rowptr.data_ptr(), self.pattern.cols.data_ptr(),
                                      self.values.data_ptr(), rowptr.data_ptr(), cols.data_ptr(),
                                      vals.data_ptr(), None, work.data_ptr(), wbytes, _stream()),
                   'tf_csr_compact')
        k = nnz.value
        return (rowptr.cpu().numpy().astype(np.int64), cols[:k].cpu().numpy().astype(np.int64),
                vals[:k].cpu().numpy())

    def to_scipy(self):
        import scipy.sparse as sp
        b, j, v = self.compact()
        return sp.csr_matrix((v, j, b), shape=self.shape)

    def toarray(self):
        return self.to_scipy().toarray()


class DiagonalMatrix:
    """Diagonal matrix on the device (the mass matrix, Discretization.py:417-548)."""

    def __init__(self, diag):
        self.diag = diag

    @property
    def shape(self):
        n = self.diag.numel()
        return (n, n)

    def __matmul__(self, x):
        host = not isinstance(x, DeviceVector)
        xv = DeviceVector.from_array(np.asarray(x)) if host else x
        y = DeviceVector(torch.zeros_like(xv.data))
        lib = _lib.load()
        _lib.check(lib.tf_diag_axpy(y.size, 1.0, self.diag.data_ptr(), xv.data.data_ptr(), y.data.data_ptr(),
                                    _stream()), 'tf_diag_axpy')
        return y.numpy() if host else y

    def __mul__(self, s):
        out = torch.empty_like(self.diag)
        lib = _lib.load()
        _lib.check(lib.tf_vec_axpby(out.numel(), float(s), self.diag.data_ptr(), 0.0, None, out.data_ptr(),
                                    _stream()), 'tf_vec_axpby')
        return DiagonalMatrix(out)

    __rmul__ = __mul__

    def __truediv__(self, s):
        return self * (1 / s)

    def diagonal(self):
        return self.diag.cpu().numpy()

    def to_scipy(self):
        import scipy.sparse as sp
        d = self.diagonal()
        return sp.diags(d).tocsr()
