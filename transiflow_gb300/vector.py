"""DeviceVector: an FP64 state vector resident on the GPU.

Continuation and TimeIntegration treat vectors as NumPy-like objects: they
read ``x.size`` (Continuation.py:429), add, subtract and scale them, update
them in place (``x += dx``, ``dx /= ds``; Continuation.py:169, 285-286,
347-348), take ``x.dot(y)`` (Continuation.py:142, 162) and compute norms
through ``x.T.conj() @ x`` (utils.py:5-21).  A bare ``torch.Tensor`` fails
at ``x.size`` (a method there), so this thin wrapper provides that contract.
All arithmetic runs in libtfcuda kernels; ``dot`` returns a Python float,
which is the host synchronisation point of the drivers.
"""

import ctypes

import numpy as np
import torch

from . import _lib


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class DeviceVector:
    __array_priority__ = 1000   # make numpy defer to our operators

    def __init__(self, data):
        if not (isinstance(data, torch.Tensor) and data.is_cuda and data.dtype == torch.float64
                and data.dim() == 1 and data.is_contiguous()):
            raise TypeError('DeviceVector needs a contiguous 1-D float64 CUDA tensor')
        self.data = data

    # -- construction ------------------------------------------------------
    @classmethod
    def zeros(cls, n, device=None):
        return cls(torch.zeros(n, dtype=torch.float64, device=device or 'cuda'))

    @classmethod
    def from_array(cls, a, device=None):
        t = torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64))
        return cls(t.to(device or 'cuda', non_blocking=False))

    def _like(self):
        return DeviceVector(torch.empty_like(self.data))

    # -- shape -----------------------------------------------------------------
    @property
    def size(self):
        return self.data.numel()

    @property
    def shape(self):
        return (self.data.numel(),)

    @property
    def dtype(self):
        return np.dtype(np.float64)

    def __len__(self):
        return self.data.numel()

    @property
    def T(self):
        return self

    def conj(self):
        return self

    # -- kernels ---------------------------------------------------------------
    def _axpby(self, a, x, b, y, out):
        lib = _lib.load()
        _lib.check(lib.tf_vec_axpby(self.size, float(a), None if x is None else x.data.data_ptr(),
                                    float(b), None if y is None else y.data.data_ptr(),
                                    out.data.data_ptr(), _stream()), 'tf_vec_axpby')
        return out

    def dot(self, other):
        other = _as_vec(other)
        return _dot(self, other)

    def __matmul__(self, other):
        return self.dot(other)

    def norm(self):
        return float(np.sqrt(abs(self.dot(self))))

    # -- arithmetic -----------------------------------------------------------
    def __add__(self, other):
        if isinstance(other, DeviceVector):
            return self._axpby(1.0, self, 1.0, other, self._like())
        return NotImplemented

    __radd__ = __add__

    def __sub__(self, other):
        if isinstance(other, DeviceVector):
            return self._axpby(1.0, self, -1.0, other, self._like())
        return NotImplemented

    def __rsub__(self, other):
        if isinstance(other, DeviceVector):
            return self._axpby(1.0, other, -1.0, self, self._like())
        return NotImplemented

    def __mul__(self, s):
        if np.ndim(s) == 0 and not isinstance(s, DeviceVector):
            return self._axpby(float(s), self, 0.0, None, self._like())
        return NotImplemented

    __rmul__ = __mul__

    def __truediv__(self, s):
        if np.ndim(s) == 0 and not isinstance(s, DeviceVector):
            return self._div(float(s), self._like())
        return NotImplemented

    def _div(self, s, out):
        lib = _lib.load()
        _lib.check(lib.tf_vec_div(self.size, self.data.data_ptr(), s, out.data.data_ptr(), _stream()),
                   'tf_vec_div')
        return out

    def __neg__(self):
        return self._axpby(-1.0, self, 0.0, None, self._like())

    def __iadd__(self, other):
        if isinstance(other, DeviceVector):
            return self._axpby(1.0, self, 1.0, other, self)
        return NotImplemented

    def __isub__(self, other):
        if isinstance(other, DeviceVector):
            return self._axpby(1.0, self, -1.0, other, self)
        return NotImplemented

    def __imul__(self, s):
        return self._axpby(float(s), self, 0.0, None, self)

    def __itruediv__(self, s):
        return self._div(float(s), self)

    # -- host interop -----------------------------------------------------------
    def copy(self):
        return DeviceVector(self.data.clone())

    def numpy(self):
        return self.data.cpu().numpy()

    def __array__(self, dtype=None, copy=None):
        a = self.numpy()
        return a.astype(dtype) if dtype is not None else a

    def __getitem__(self, idx):
        r = self.data[idx]
        return float(r) if r.dim() == 0 else r.cpu().numpy()

    def __setitem__(self, idx, value):
        if isinstance(value, DeviceVector):
            value = value.data
        elif not np.isscalar(value):
            value = torch.as_tensor(np.asarray(value, dtype=np.float64), device=self.data.device)
        self.data[idx] = value

    def __repr__(self):
        return 'DeviceVector(n=%d)' % self.size


def _as_vec(x):
    if isinstance(x, DeviceVector):
        return x
    return DeviceVector.from_array(np.asarray(x))


_work = {}


def _dot(a, b):
    lib = _lib.load()
    n = a.size
    # one workspace per stream: threads driving instances on their own
    # streams must not share partial sums
    key = (a.data.device, torch.cuda.current_stream().cuda_stream)
    need = lib.tf_vec_mdot_workspace_bytes(n, 1)
    buf = _work.get(key)
    if buf is None or buf.numel() * 8 < need + 8:
        buf = torch.empty((need + 16) // 8 + 1, dtype=torch.float64, device=a.data.device)
        _work[key] = buf
    out = buf[:1]
    work = buf[1:]
    _lib.check(lib.tf_vec_mdot(n, 1, a.data.data_ptr(), n, b.data.data_ptr(), out.data_ptr(),
                               work.data_ptr(), work.numel() * 8, _stream()), 'tf_vec_mdot')
    return float(out.item())
