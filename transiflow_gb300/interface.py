"""The ``CUDA`` backend behind TransiFlow's interface contract.

``Interface`` has the constructor signature of
``transiflow.interface.BaseInterface`` (BaseInterface.py:45-46) and
provides the methods the drivers call -- ``vector``, ``rhs``, ``jacobian``,
``mass_matrix``, ``solve`` (SciPy.py:37-49, 311-315), ``set_parameter`` /
``get_parameter`` (BaseInterface.py:94-116), ``save_state`` /
``load_state`` (BaseInterface.py:118-215; inherited from the reference's
``BaseInterface`` when that package is importable) and ``vector_from_array`` /
``array_from_vector`` -- so ``Continuation`` and ``TimeIntegration`` run on
it unchanged.  States live on the GPU as :class:`DeviceVector`; the
discretisation, the Jacobian and the solves run in libtfcuda kernels.
``eigs`` computes the eigenvalues nearest a real target by shift-and-invert
Arnoldi with the GPU solver.

Backend options go in the ``'CUDA'`` sub-dictionary of the parameters:
  'Factor Precision'  'fp64' (default) or 'fp32' for the preconditioner LU
  'Tolerance'         GMRES relative residual (default 1e-12)
  'Restart'           GMRES restart length (default 50)
  'Maximum Iterations'  GMRES iteration cap (default 500)
  'Reuse Factorization'  precondition a new Jacobian with the latest
                      factorisation and refactor only if GMRES needs more than
                      'Reuse Iterations' (default 20) iterations (default True)
  'Reuse Policy'      'cost' (default): try a reuse only while the Jacobian
                      values differ from the factored ones by at most
                      'Reuse Drift' (relative 2-norm, default 0.05; halved
                      after a failed attempt, grown after a success) and with
                      at most as many GMRES iterations as cost one
                      factorisation (both measured); 'always'
  'Inverse Apply'     invert the factored own blocks once per factorisation
                      and apply them by parallel triangular products instead
                      of substitution (default True)
  'Dataflow Apply'    with 'Inverse Apply': run both sweeps of an application
                      in one persistent launch in which each front waits only
                      for the fronts it depends on (default False; plans whose
                      widest front does not fit that launch's shared memory
                      keep one launch per tree height)
  'Dataflow Fuse Tiles', 'Dataflow Chunk Tiles'
                      fronts with at most this many 32x32 factor tiles per
                      sweep run as one task (default 48); target tiles per task
                      of the other fronts (default 24)
  'Tensor Cores'      FP32 factors: tree heights whose widest front has at
                      least 'Tensor Core Min Front' (default 1024) rows are
                      factored in blocks of 256 columns whose trailing updates
                      run on the tensor cores (tcgen05, FP32 sums) (default
                      True); 'Tensor Core Precision' 'tf32x3' (default:
                      operands split into TF32 high parts and remainders,
                      three products, close to FP32) or 'tf32' (one product)
  'Factor Storage'    FP32 factors: 'fp32' (default) or 'bf16' -- after each
                      factorisation the entries the preconditioner reads are
                      rounded to a BF16 copy, and every application reads
                      that copy (half the bytes) with FP32 products and sums
  'Equilibrate'       FP32 factors: factor the operator scaled by powers of two
                      per row and column (1 / the largest entry), so that the
                      FP32 rounding does not wipe out badly scaled equations
                      (default True; FP64 factors are never scaled)
  'Inner Precision'   'fp64' (default) or 'fp32': the Arnoldi products of
                      FGMRES use an FP32 copy of the gauged Jacobian (SpMV in
                      FP32 values, FP64 vectors); every restart cycle stops
                      after gaining six digits and the next starts from the
                      FP64 residual (iterative refinement), so the solve still
                      meets 'Tolerance' in FP64
  'Bordered Solve'    'krylov' (default): a bordered system [J, V; W^T, C]
                      is solved by one FGMRES on the bordered matrix,
                      preconditioned by the Jacobian's factorisation (block
                      preconditioner, one application per iteration);
                      'elimination': block elimination with two solves of
                      the Jacobian
  'Tune Application'  FP32 / BF16 factors: time the application's launch
                      shapes (warps per SM a height aims for) on the first
                      factorisation and keep the fastest, cached per GPU,
                      grid and precision in TRANSIFLOW_GB300_TUNE_CACHE or
                      ~/.cache/transiflow_gb300/tune.json (default True)
  'Leaf Cells'        grid cells of a box at which nested dissection stops
                      splitting (default 48)
  'CUDA Graphs'       replay the factorisation and solve launch sequences from
                      captured CUDA graphs (default True)
  'Fuse Jacobian'     compute the Jacobian together with the RHS and reuse it
                      when jacobian() is called at the same state and
                      parameters (default False)
With the reference's ``'Use Iterative Solver': True``, the GMRES restart,
iteration cap and tolerance come from its ``'Iterative Solver'`` dictionary
('Restart' 100, 'Maximum Iterations' 1000, 'Convergence Tolerance' 1e-6 by
default, as in SciPy.py:281-287); the preconditioner stays the LU above.
"""

import ctypes
import json

import numpy as np
import torch

from . import _lib, grid
from .matrix import DiagonalMatrix, Pattern, StencilMatrix
from .solver import Solver
from .vector import DeviceVector, _stream


def _jsonable(obj):
    """``default`` hook of json.dump for the parameter files: NumPy scalars
    and arrays become plain numbers and lists, complex numbers the tagged
    object ``{"__complex__": true, "real": .., "imag": ..}``."""
    if isinstance(obj, (complex, np.complexfloating)):
        return {'__complex__': True, 'real': obj.real, 'imag': obj.imag}
    if isinstance(obj, np.ndarray):
        return obj.tolist()
    if isinstance(obj, np.generic):
        return obj.item()
    raise TypeError('%s is not JSON serialisable' % type(obj).__name__)


def _unjson(obj):
    return complex(obj['real'], obj['imag']) if obj.get('__complex__') else obj


class _Checkpointing:
    """Parameter access and state checkpoints when the reference package is
    not importable (with it, ``transiflow.interface.BaseInterface`` provides
    them).  The files are the reference's: ``<name>.params`` holds the
    parameter dictionary as JSON (complex values tagged), ``<name>.npy`` the
    state (BaseInterface.py:118-215)."""

    def set_parameter(self, name, value):
        self.parameters[name] = value

    def get_parameter(self, name, default=0):
        return self.parameters[name] if name in self.parameters else default

    def save_json(self, name, obj):
        with open(name, 'w') as f:
            json.dump(obj, f, default=_jsonable)

    def load_json(self, name):
        with open(name) as f:
            return json.load(f, object_hook=_unjson)

    def save_parameters(self, name):
        path = name + '.params'
        self.save_json(path, self.parameters)
        print('Wrote parameters to', path, flush=True)

    def load_parameters(self, name):
        path = name + '.params'
        before = dict(self.parameters)
        self.parameters.update(self.load_json(path))
        print('Read parameters from', path, flush=True)
        for key in self.parameters:
            if self.parameters[key] != before.get(key):
                print("Updated '%s' from %s to %s" % (key, before.get(key), self.parameters[key]), flush=True)

    def save_state(self, name, x):
        self.save_parameters(name)
        path = name if name.endswith('.npy') else name + '.npy'
        np.save(path, self.array_from_vector(x))
        print('Wrote state to', path, flush=True)

    def load_state(self, name):
        self.load_parameters(name)
        path = name if name.endswith('.npy') else name + '.npy'
        x = np.load(path)
        print('Read state from', path, flush=True)
        return x


try:
    # the reference's interface base class, when its package is importable
    from transiflow.interface.BaseInterface import BaseInterface as _ContractBase
except ImportError:
    _ContractBase = None

_Base = _ContractBase if _ContractBase is not None else _Checkpointing


class Interface(_Base):
    """The CUDA backend.  Subclasses ``transiflow.interface.BaseInterface``
    when the reference package is importable (parameter access and
    checkpoints then come from there), a stand-in with the same file format
    otherwise."""

    def __init__(self, parameters, nx, ny, nz=1, dim=None, dof=None, x=None, y=None, z=None,
                 boundary_conditions=None, device=None):
        if not torch.cuda.is_available():
            raise _lib.CudaBackendError('the CUDA backend needs a GPU')
        if _ContractBase is not None:
            _ContractBase.__init__(self, parameters, nx, ny, nz, dim, dof, x, y, z, boundary_conditions)
        self.lib = _lib.load()
        self.device = torch.device(device or 'cuda')
        self.parameters = parameters
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dim = dim if dim is not None else (3 if nz > 1 else 2)
        self.dof = dof if dof is not None else grid.default_dof(parameters, self.dim)
        self.boundary_conditions = boundary_conditions
        p = parameters
        self.x = np.asarray(x) if x is not None else grid.coordinate_vector(p, p.get('X-min', 0.0), p.get('X-max', 1.0), nx)
        self.y = np.asarray(y) if y is not None else grid.coordinate_vector(p, p.get('Y-min', 0.0), p.get('Y-max', 1.0), ny)
        self.z = np.asarray(z) if z is not None else grid.coordinate_vector(p, p.get('Z-min', 0.0), p.get('Z-max', 1.0), nz)
        self.n = nx * ny * nz * self.dof
        self.pressure_row = self.dim
        self.border_scaling = 1e-3
        table = grid.metric_table((self.x, self.y, self.z), (nx, ny, nz))
        self._metric = torch.as_tensor(table.ravel()).to(self.device)
        self._stride = table.shape[2]
        self._aux = torch.as_tensor(grid.aux_table(self.y, ny).ravel()).to(self.device)
        self._prof = None
        # validate the problem type and boundary program now
        self._problem()
        # pattern of the stencil CSR
        row_offset = np.zeros(self.dof + 1, dtype=np.int32)
        slot = np.zeros(self.dof * self.dof * 27, dtype=np.int32)
        _lib.check(self.lib.tf_stencil_layout(self.dim, self.dof, row_offset.ctypes.data, slot.ctypes.data),
                   'tf_stencil_layout')
        width = int(row_offset[-1])
        ncell = nx * ny * nz
        rowptr = torch.empty(self.n + 1, dtype=torch.int32, device=self.device)
        cols = torch.empty(ncell * width, dtype=torch.int32, device=self.device)
        prob = self._problem()
        _lib.check(self.lib.tf_stencil_pattern(ctypes.byref(prob), rowptr.data_ptr(), cols.data_ptr(), _stream()),
                   'tf_stencil_pattern')
        self.pattern = Pattern(rowptr, cols, self.n, width, row_offset, slot.reshape(self.dof, self.dof, 27))
        opts = parameters.get('CUDA', {})
        restart, tol, maxit = opts.get('Restart', 50), opts.get('Tolerance', 1e-12), opts.get('Maximum Iterations', 500)
        if parameters.get('Use Iterative Solver', False):
            # the reference's GMRES settings (SciPy.py:281-287) take precedence
            it = parameters.get('Iterative Solver', {})
            restart = it.get('Restart', 100)
            maxit = it.get('Maximum Iterations', 1000)
            tol = it.get('Convergence Tolerance', 1e-6)
        self.solver = Solver(self, restart=restart, tol=tol, maxit=maxit,
                             precision=opts.get('Factor Precision', 'fp64'),
                             reuse=opts.get('Reuse Factorization', True),
                             reuse_maxit=opts.get('Reuse Iterations', 20),
                             graphs=opts.get('CUDA Graphs', True),
                             reuse_policy=opts.get('Reuse Policy', 'cost'),
                             reuse_drift=opts.get('Reuse Drift', 0.05),
                             inverse=opts.get('Inverse Apply', True),
                             flow=opts.get('Dataflow Apply', False),
                             flow_fuse_tiles=int(opts.get('Dataflow Fuse Tiles', 48)),
                             flow_chunk_tiles=int(opts.get('Dataflow Chunk Tiles', 24)),
                             leaf_cells=int(opts.get('Leaf Cells', 48)),
                             tc_min_front=(int(opts.get('Tensor Core Min Front', 1024))
                                           if opts.get('Tensor Cores', True) else 0),
                             tc_terms=1 if opts.get('Tensor Core Precision', 'tf32x3') == 'tf32' else 3,
                             storage=opts.get('Factor Storage', 'fp32'),
                             inner=opts.get('Inner Precision', 'fp64'),
                             equilibrate=opts.get('Equilibrate', True),
                             bordered=opts.get('Bordered Solve', 'krylov'),
                             tune=opts.get('Tune Application', True))
        self.fuse = opts.get('Fuse Jacobian', False)
        self._cached_jac = None
        self.calls = {'rhs': 0, 'jacobian': 0, 'solve': 0, 'fused_jacobians': 0}

    def _problem(self):
        return grid.make_problem(self.parameters, self.nx, self.ny, self.nz, self.dim, self.dof,
                                 self.x, self.y, self.z, self._metric.data_ptr(), self._stride,
                                 self.boundary_conditions, self._aux.data_ptr(), self._upload_profiles)

    def _upload_profiles(self, table):
        """Device copy of the boundary forcing profiles (they depend on the
        parameters, so every assembly refreshes them; the copy is ordered on
        the current stream before the kernels that read it)."""
        t = torch.as_tensor(np.ascontiguousarray(table.ravel()))
        if self._prof is None or self._prof.numel() != t.numel():
            self._prof = torch.empty(t.numel(), dtype=torch.float64, device=self.device)
        self._prof.copy_(t)
        return self._prof.data_ptr()

    # -- vectors -----------------------------------------------------------------
    def vector(self):
        return DeviceVector.zeros(self.n, self.device)

    def vector_from_array(self, array):
        return DeviceVector.from_array(np.asarray(array), self.device)

    def array_from_vector(self, vector):
        return vector.numpy() if isinstance(vector, DeviceVector) else np.asarray(vector)

    def _as_device(self, state):
        if isinstance(state, DeviceVector):
            return state
        return DeviceVector.from_array(np.asarray(state), self.device)

    # -- discretisation ------------------------------------------------------
    def _key(self, state):
        return (state.data.data_ptr(), state.data._version,
                json.dumps(self.parameters, sort_keys=True, default=lambda o: repr(o)))

    def rhs(self, state):
        """F(state), Discretization.rhs (Discretization.py:367-390)."""
        self.calls['rhs'] += 1
        x = self._as_device(state)
        out = torch.empty(self.n, dtype=torch.float64, device=self.device)
        prob = self._problem()
        jv = None
        if self.fuse:
            jv = torch.empty(self.pattern.nnz, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.tf_assemble(ctypes.byref(prob), x.data.data_ptr(), out.data_ptr(),
                                        None if jv is None else jv.data_ptr(), _stream()), 'tf_assemble')
        if jv is not None:
            self._cached_jac = (self._key(x), jv)
        result = DeviceVector(out)
        return result if isinstance(state, DeviceVector) else result.numpy()

    def jacobian(self, state):
        """J(state) in the stencil CSR, Discretization.jacobian (Discretization.py:392-415)."""
        self.calls['jacobian'] += 1
        x = self._as_device(state)
        if self._cached_jac is not None and self._cached_jac[0] == self._key(x):
            self.calls['fused_jacobians'] += 1
            jv = self._cached_jac[1]
            self._cached_jac = None
            return StencilMatrix(self.pattern, jv)
        jv = torch.empty(self.pattern.nnz, dtype=torch.float64, device=self.device)
        prob = self._problem()
        _lib.check(self.lib.tf_assemble(ctypes.byref(prob), x.data.data_ptr(), None, jv.data_ptr(), _stream()),
                   'tf_assemble')
        return StencilMatrix(self.pattern, jv)

    def mass_matrix(self):
        """Diagonal mass matrix, Discretization.mass_matrix (Discretization.py:417-548)."""
        d = torch.empty(self.n, dtype=torch.float64, device=self.device)
        prob = self._problem()
        _lib.check(self.lib.tf_mass_diag(ctypes.byref(prob), d.data_ptr(), _stream()), 'tf_mass_diag')
        return DiagonalMatrix(d)

    # -- solves -----------------------------------------------------------------
    def solve(self, jac, rhs, rhs2=None, V=None, W=None, C=None):
        """Solve J y = rhs (or the bordered system), SciPy.Interface.solve (SciPy.py:311-315)."""
        self.calls['solve'] += 1
        host = not isinstance(rhs, DeviceVector)
        out = self.solver.solve(jac, rhs, rhs2, V, W, C)
        if rhs2 is None:
            return out.numpy() if host else out
        y, y2 = out
        return (y.numpy() if host else y), y2

    def eigs(self, state, return_eigenvectors=False, enable_recycling=False):
        """Generalised eigenvalues of J(u, p) v = lambda M v closest to the
        target (the contract of BaseInterface.eigs, BaseInterface.py:355-386),
        by shift-and-invert Arnoldi: ARPACK through scipy.sparse.linalg.eigs,
        as the reference's tests compute them (tests/jada_fixtures.py:72-87),
        on the operator (J - sigma M)^-1 M, whose every application is one
        solve with the GPU factorisation of the gauged J - sigma M.
        'Eigenvalue Solver' options: 'Number of Eigenvalues' (5), 'Target'
        (0, real), 'Tolerance' (1e-7).  The eigenvalues are ordered as the
        reference orders them: largest real part first, real parts >= 100
        last.  enable_recycling is accepted and ignored."""
        import scipy.sparse.linalg as sla
        opts = self.parameters.get('Eigenvalue Solver', {})
        num = int(opts.get('Number of Eigenvalues', 5))
        target = complex(opts.get('Target', 0.0))
        if target.imag != 0:
            raise NotImplementedError('complex eigenvalue targets')
        sigma = target.real
        tol = float(opts.get('Tolerance', 1e-7))
        x = state if isinstance(state, DeviceVector) else self.vector_from_array(state)
        J = self.jacobian(x)
        M = self.mass_matrix()
        A = J - M * sigma if sigma != 0 else J

        def op(v):
            b = M @ DeviceVector.from_array(np.ascontiguousarray(np.real(v), dtype=np.float64), self.device)
            return self.solve(A, b).numpy()

        n = self.n
        OP = sla.LinearOperator((n, n), matvec=op, dtype=np.float64)
        v0 = np.random.default_rng(0).standard_normal(n)
        k = min(num, n - 2)
        if return_eigenvectors:
            mu, V = sla.eigs(OP, k=k, which='LM', tol=tol, v0=v0)
        else:
            mu = sla.eigs(OP, k=k, which='LM', tol=tol, v0=v0, return_eigenvectors=False)
        lam = sigma + 1 / mu
        order = sorted(range(len(lam)), key=lambda i: -lam[i].real if lam[i].real < 100 else 100)
        if return_eigenvectors:
            return lam[order][:num], V[:, order][:, :num]
        return lam[order][:num]

    def load_state(self, name):
        """The checkpointed state as a device vector (the base class reads it
        into host memory)."""
        return self.vector_from_array(super().load_state(name))


def create(parameters, nx, ny, nz=1, dim=None, dof=None, boundary_conditions=None, backend='CUDA'):
    """transiflow.interface.create with a 'CUDA' backend (create.py:4-68).

    Other backend names are delegated to the reference package when it is
    importable."""
    if backend.lower() == 'cuda':
        return Interface(parameters, nx, ny, nz, dim, dof, boundary_conditions=boundary_conditions)
    from transiflow.interface import create as ref_create   # the reference's own backends
    return ref_create(parameters, nx, ny, nz, dim, dof, boundary_conditions=boundary_conditions, backend=backend)
