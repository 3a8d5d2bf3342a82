"""Linear solves for the CUDA backend.

The reference solves every Newton system with SuperLU on the gauged (and
optionally bordered) Jacobian (transiflow/interface/SciPy.py:131-258).  Here
the same gauged system is solved by flexible GMRES in FP64 whose
preconditioner is a nested-dissection multifrontal LU of the gauged Jacobian
computed on the GPU (``tf_nd_*``): in FP64 it is an exact factorisation and
GMRES converges in one or two iterations; in FP32 ('Factor Precision':
'fp32') it is the mixed-precision variant, with the residual, the Krylov
basis and the update kept in FP64.

Pressure gauge and bordering follow the reference: the right-hand side's
gauge entry is zeroed (SciPy.py:211-216), and a bordered system
``[A, sV; sW^T, s^2 C]`` (SciPy.py:51-129) is solved by block elimination
with two solves of the gauged Jacobian.
"""

import math

import numpy as np
import torch

from . import _lib
from .ndplan import build_plan
from .vector import DeviceVector, _stream


class NdPlanDevice:
    """The elimination plan of one grid, uploaded once."""

    def __init__(self, pattern, nx, ny, nz, dof, pressure_var, leaf_cells=48):
        rowptr = pattern.rowptr.cpu().numpy()
        cols = pattern.cols.cpu().numpy()
        p = build_plan(nx, ny, nz, dof, rowptr, cols, leaf_cells=leaf_cells, pressure_var=pressure_var)
        self.host = p
        dev = pattern.rowptr.device

        def up(a, dt):
            return torch.as_tensor(np.ascontiguousarray(a, dtype=dt)).to(dev)

        self.n_own = up(p.n_own, np.int32)
        self.f = up(p.f, np.int32)
        self.parent = up(p.parent, np.int32)
        self.front_off = up(p.front_off, np.int64)
        self.idx_off = up(p.idx_off, np.int64)
        self.idx = up(p.idx, np.int32)
        self.ea_off = up(p.ea_map_off, np.int64)
        self.ea_map = up(p.ea_map if len(p.ea_map) else np.zeros(1), np.int32)
        self.scat_pos = up(p.scat_pos, np.int64)
        self.scat_src = up(p.scat_src, np.int32)
        piv_off = np.zeros(p.nnodes + 1, dtype=np.int64)
        piv_off[1:] = np.cumsum(p.n_own)
        self.piv_off = up(piv_off, np.int64)
        rank = np.zeros(p.nnodes, dtype=np.int32)
        seen = {}
        for t in range(p.nnodes):
            par = int(p.parent[t])
            if par >= 0:
                rank[t] = seen.get(par, 0)
                seen[par] = rank[t] + 1
        assert rank.max(initial=0) <= 1
        self.rank = up(rank, np.int32)
        levels = p.levels
        self.level_ptr = np.zeros(len(levels) + 1, dtype=np.int32)
        for h, lv in enumerate(levels):
            assert np.all(np.diff(lv) == 1) and (h == 0 or lv[0] == self.level_ptr[h])
            self.level_ptr[h + 1] = lv[-1] + 1 if len(lv) else self.level_ptr[h]
        self.max_own = np.array([p.n_own[lv].max() for lv in levels], dtype=np.int32)
        self.max_f = np.array([p.f[lv].max() for lv in levels], dtype=np.int32)
        self.front_elems = int(p.front_off[-1])
        s = _lib.NdPlan()
        s.n = p.n
        s.nnodes = p.nnodes
        s.nlevels = len(levels)
        s.level_ptr = self.level_ptr.ctypes.data
        s.max_own = self.max_own.ctypes.data
        s.max_f = self.max_f.ctypes.data
        s.d_n_own = self.n_own.data_ptr()
        s.d_f = self.f.data_ptr()
        s.d_parent = self.parent.data_ptr()
        s.d_front_off = self.front_off.data_ptr()
        s.d_idx_off = self.idx_off.data_ptr()
        s.d_idx = self.idx.data_ptr()
        s.d_ea_off = self.ea_off.data_ptr()
        s.d_ea_map = self.ea_map.data_ptr()
        s.nscat = len(p.scat_pos)
        s.d_scat_pos = self.scat_pos.data_ptr()
        s.d_scat_src = self.scat_src.data_ptr()
        s.scat_level_ptr = None
        s.d_piv_off = self.piv_off.data_ptr()
        s.d_rank = self.rank.data_ptr()
        s.front_elems = self.front_elems
        self.struct = s
        self.flops = p.flops


class Factorization:
    """Gauged values and their multifrontal LU, owned by one StencilMatrix."""

    def __init__(self, solver, jac, precision):
        self.solver = solver
        self.precision = precision
        self.n = jac.pattern.n
        lib = _lib.load()
        pat = jac.pattern
        self.gauged = torch.empty_like(jac.values)
        _lib.check(lib.tf_gauge_values(self.n, pat.rowptr.data_ptr(), pat.cols.data_ptr(), jac.values.data_ptr(),
                                       solver.gauge, self.gauged.data_ptr(), _stream()), 'tf_gauge_values')
        self.fronts, self.piv = solver._front_buffers(precision, self)
        info = solver.info
        info.zero_()
        fn = lib.tf_nd_factor_f64 if precision == 'fp64' else lib.tf_nd_factor_f32
        _lib.check(fn(_struct_ptr(solver.plan.struct), self.gauged.data_ptr(), self.fronts.data_ptr(),
                      self.piv.data_ptr(), info.data_ptr(), _stream()), 'tf_nd_factor')
        self.zero_pivots = None
        self.jac = jac

    def valid(self):
        return self.solver._owner.get(self.precision) is self

    def apply(self, x):
        """In place: x <- M^-1 x."""
        lib = _lib.load()
        fn = lib.tf_nd_solve_f64 if self.precision == 'fp64' else lib.tf_nd_solve_f32
        _lib.check(fn(_struct_ptr(self.solver.plan.struct), self.fronts.data_ptr(), self.piv.data_ptr(),
                      x.data_ptr(), _stream()), 'tf_nd_solve')

    def matvec(self, x, out):
        lib = _lib.load()
        pat = self.jac.pattern
        _lib.check(lib.tf_spmv_f64(self.n, pat.rowptr.data_ptr(), pat.cols.data_ptr(), self.gauged.data_ptr(),
                                   x.data_ptr(), out.data_ptr(), 1.0, 0.0, _stream()), 'tf_spmv_f64')


def _struct_ptr(s):
    import ctypes
    return ctypes.cast(ctypes.pointer(s), ctypes.c_void_p)


class Solver:
    """Per-interface solver state: the plan, factor buffers, Krylov workspace."""

    def __init__(self, interface, restart=50, tol=1e-12, maxit=500, precision='fp64'):
        self.itf = interface
        self.gauge = interface.pressure_row if interface.dof > interface.dim else -1
        self.restart = restart
        self.tol = tol
        self.maxit = maxit
        self.precision = precision
        self.plan = None
        self._fronts = {}
        self._owner = {}
        self.info = None
        self._V = None
        self._Z = None
        self._mdot_work = None
        self.stats = {'factorizations': 0, 'solves': 0, 'gmres_iterations': 0, 'last_relres': None}

    def _ensure_plan(self, pattern):
        if self.plan is None:
            itf = self.itf
            self.plan = NdPlanDevice(pattern, itf.nx, itf.ny, itf.nz, itf.dof,
                                     itf.dim if itf.dof > itf.dim else None)
            self.info = torch.zeros(1, dtype=torch.int32, device=pattern.rowptr.device)

    def _front_buffers(self, precision, owner):
        dt = torch.float64 if precision == 'fp64' else torch.float32
        bufs = self._fronts.get(precision)
        if bufs is None:
            dev = self.itf.device
            bufs = (torch.empty(self.plan.front_elems, dtype=dt, device=dev),
                    torch.empty(self.plan.host.n, dtype=torch.int32, device=dev))
            self._fronts[precision] = bufs
        self._owner[precision] = owner
        return bufs

    def factorization(self, jac):
        self._ensure_plan(jac.pattern)
        fac = jac.lu
        if fac is None or not isinstance(fac, Factorization) or not fac.valid() or fac.precision != self.precision:
            fac = Factorization(self, jac, self.precision)
            jac.lu = fac
            self.stats['factorizations'] += 1
        return fac

    # -- Krylov ---------------------------------------------------------------
    def _workspace(self, n, dev):
        m = self.restart
        if self._V is None or self._V.shape[1] != n:
            self._V = torch.empty((m + 1, n), dtype=torch.float64, device=dev)
            self._Z = torch.empty((m, n), dtype=torch.float64, device=dev)
            lib = _lib.load()
            wb = lib.tf_vec_mdot_workspace_bytes(n, m + 1)
            self._mdot_work = torch.empty((wb + 7) // 8 + m + 2, dtype=torch.float64, device=dev)
        return self._V, self._Z

    def _mdot(self, V, k, w):
        lib = _lib.load()
        n = w.numel()
        out = self._mdot_work[:k]
        work = self._mdot_work[self.restart + 2:]
        _lib.check(lib.tf_vec_mdot(n, k, V.data_ptr(), V.stride(0), w.data_ptr(), out.data_ptr(),
                                   work.data_ptr(), work.numel() * 8, _stream()), 'tf_vec_mdot')
        return out

    def _mgs(self, V, k, h, w):
        lib = _lib.load()
        _lib.check(lib.tf_vec_mgs_update(w.numel(), k, V.data_ptr(), V.stride(0), h.data_ptr(), w.data_ptr(),
                                         _stream()), 'tf_vec_mgs_update')

    def _axpby(self, a, x, b, y, z):
        lib = _lib.load()
        _lib.check(lib.tf_vec_axpby(z.numel(), float(a), None if x is None else x.data_ptr(), float(b),
                                    None if y is None else y.data_ptr(), z.data_ptr(), _stream()), 'tf_vec_axpby')

    def _norm(self, w, V=None):
        out = self._mdot(w.view(1, -1), 1, w)
        return math.sqrt(max(float(out.item()), 0.0))

    def fgmres(self, fac, b):
        """Solve A_g x = b (b: float64 CUDA tensor); returns (x, iterations, relres)."""
        n = b.numel()
        V, Z = self._workspace(n, b.device)
        m = self.restart
        x = torch.zeros_like(b)
        r = b.clone()
        bn = self._norm(b)
        if bn == 0.0:
            return x, 0, 0.0
        its = 0
        relres = 1.0
        tmp = torch.empty_like(b)
        while its < self.maxit:
            beta = self._norm(r)
            relres = beta / bn
            if relres <= self.tol:
                break
            self._axpby(1.0 / beta, r, 0.0, None, V[0])
            g = np.zeros(m + 1)
            g[0] = beta
            H = np.zeros((m + 1, m))
            cs = np.zeros(m)
            sn = np.zeros(m)
            k = 0
            for j in range(m):
                Z[j].copy_(V[j])
                fac.apply(Z[j])
                fac.matvec(Z[j], V[j + 1])
                w = V[j + 1]
                h = self._mdot(V, j + 1, w).clone()
                self._mgs(V, j + 1, h, w)
                h2 = self._mdot(V, j + 1, w)
                self._mgs(V, j + 1, h2, w)
                hh = (h + h2).cpu().numpy()
                hn = self._norm(w)
                H[:j + 1, j] = hh
                H[j + 1, j] = hn
                if hn > 0:
                    self._axpby(1.0 / hn, w, 0.0, None, w)
                for i in range(j):
                    t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                    H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                    H[i, j] = t
                d = math.hypot(H[j, j], H[j + 1, j])
                cs[j] = H[j, j] / d if d else 1.0
                sn[j] = H[j + 1, j] / d if d else 0.0
                H[j, j] = d
                H[j + 1, j] = 0.0
                g[j + 1] = -sn[j] * g[j]
                g[j] = cs[j] * g[j]
                its += 1
                k = j + 1
                if abs(g[j + 1]) <= self.tol * bn or its >= self.maxit or hn == 0:
                    break
            y = np.linalg.solve(np.triu(H[:k, :k]), g[:k]) if k else np.zeros(0)
            yd = torch.as_tensor(y, dtype=torch.float64).to(b.device)
            # x += Z[:k]^T y
            self._mgs(Z, k, -yd, x) if k else None
            # true residual
            fac.matvec(x, tmp)
            self._axpby(1.0, b, -1.0, tmp, r)
        self.stats['gmres_iterations'] += its
        self.stats['last_relres'] = relres
        return x, its, relres

    # -- the reference's solve contract ---------------------------------------
    def solve(self, jac, rhs, rhs2=None, V=None, W=None, C=None):
        itf = self.itf
        fac = self.factorization(jac)
        self.stats['solves'] += 1
        b = _to_tensor(rhs, itf.device).clone()
        if rhs2 is None:
            if self.gauge >= 0:
                b[self.gauge] = 0.0
            x, its, rr = self.fgmres(fac, b)
            if not math.isfinite(rr) or rr > max(self.tol, 1e-6):
                raise RuntimeError('GMRES did not converge: relative residual %.3e after %d iterations' % (rr, its))
            return DeviceVector(x)
        return self._bordered(fac, b, rhs2, V, W, C)

    def _bordered(self, fac, b, rhs2, V, W, C):
        """Block elimination of [A_g, sV; sW'^T, s^2 C][y; t] = [b; s rhs2], where
        W' is W without its gauge entry (SciPy.py:93-126) and b keeps its gauge
        entry (SciPy.py:226-227)."""
        itf = self.itf
        s = itf.border_scaling
        if np.ndim(rhs2) != 0:
            raise NotImplementedError('bordered solves with more than one border vector')
        Vt = _to_tensor(V, itf.device)
        Wt = _to_tensor(W if W is not None else V, itf.device).clone()
        if self.gauge >= 0:
            Wt[self.gauge] = 0.0
        Cv = 0.0 if C is None else float(C)
        y0, i0, r0 = self.fgmres(fac, b.clone())
        y1, i1, r1 = self.fgmres(fac, (s * Vt).contiguous())
        if max(r0, r1) > max(self.tol, 1e-6):
            raise RuntimeError('GMRES did not converge in a bordered solve')
        wy0 = float(_dot_t(Wt, y0))
        wy1 = float(_dot_t(Wt, y1))
        # s W'^T y + s^2 C t = s rhs2, with y = y0 - t y1
        t = (s * float(rhs2) - s * wy0) / (s * s * Cv - s * wy1)
        self._axpby(1.0, y0, -t, y1, y0)
        return DeviceVector(y0), t * s


def _to_tensor(v, device):
    if isinstance(v, DeviceVector):
        return v.data
    if isinstance(v, torch.Tensor):
        return v.to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64)).to(device)


def _dot_t(a, b):
    from .vector import _dot
    return _dot(DeviceVector(a), DeviceVector(b))
