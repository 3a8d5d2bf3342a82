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
``B = [A, sV; sW^T, s^2 C]`` (SciPy.py:51-129) is solved as one system: FGMRES
on B with the block preconditioner built from the factorisation M of the
gauged Jacobian (one application of M per iteration, and one for M sV per
solve), where the reference factors B itself.  Block elimination with two
solves of the gauged Jacobian remains available ('Bordered Solve':
'elimination').
"""

import ctypes
import json
import math
import os
import threading

import numpy as np
import torch

from . import _lib
from .ndplan import build_plan
from .vector import DeviceVector, _stream


# Elimination plans depend only on the grid shape and the variables, so
# interfaces of the same shape share one (keyed by shape and device).
_PLANS = {}
_PLANS_LOCK = threading.Lock()
_CAPTURE_LOCK = threading.Lock()


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


class GaugedOperator:
    """The gauged copy of one Jacobian's values: the operator GMRES solves with."""

    def __init__(self, solver, jac):
        self.n = jac.pattern.n
        self.jac = jac
        lib = _lib.load()
        pat = jac.pattern
        self.values = torch.empty_like(jac.values)
        _lib.check(lib.tf_gauge_values(self.n, pat.rowptr.data_ptr(), pat.cols.data_ptr(), jac.values.data_ptr(),
                                       solver.gauge, self.values.data_ptr(), _stream()), 'tf_gauge_values')

    def matvec(self, x, out):
        lib = _lib.load()
        pat = self.jac.pattern
        _lib.check(lib.tf_spmv_f64(self.n, pat.rowptr.data_ptr(), pat.cols.data_ptr(), self.values.data_ptr(),
                                   x.data_ptr(), out.data_ptr(), 1.0, 0.0, _stream()), 'tf_spmv_f64')


class _Graphed:
    """A libtfcuda launch sequence captured once in a CUDA graph and replayed.

    The sequence reads and writes fixed buffers only, so every replay redoes
    the same work on the buffers' current contents.  The first call runs the
    sequence eagerly (it also initialises per-kernel attributes outside any
    capture), the second captures it, later calls replay it."""

    def __init__(self, fn, counter):
        self.fn = fn
        self.graph = None
        self.calls = 0
        self.kernels = 0
        self.counter = counter
        self.failed = False

    def __call__(self):
        self.calls += 1
        if self.graph is not None:
            self.graph.replay()
            self.counter['graph_kernel_launches'] += self.kernels
            return
        if self.calls == 1 or self.failed:
            self.fn()
            return
        lib = _lib.load()
        # Captured with capture_begin/capture_end on a non-default stream of
        # this thread (torch.cuda.graph would synchronise the whole device,
        # which fails while another thread's stream is capturing), one
        # capture at a time.
        cur = torch.cuda.current_stream()
        side = cur if cur != torch.cuda.default_stream() else _lib.new_stream(cur.device)
        g = torch.cuda.CUDAGraph()
        with _CAPTURE_LOCK:
            side.wait_stream(cur)
            before = lib.tf_launch_count()
            try:
                with torch.cuda.stream(side):
                    g.capture_begin(capture_error_mode='thread_local')
                    try:
                        self.fn()
                    finally:
                        g.capture_end()
            except RuntimeError:
                self.failed = True
                cur.wait_stream(side)
                self.fn()
                return
            cur.wait_stream(side)
        self.kernels = lib.tf_launch_count() - before
        self.graph = g
        g.replay()
        self.counter['graph_kernel_launches'] += self.kernels


class Factorization:
    """Multifrontal LU of a gauged operator in the solver's front buffers.

    Only the most recent factorisation of a precision is valid: the fronts are
    one buffer per solver.  It is applied as a preconditioner."""

    def __init__(self, solver, op, precision):
        self.solver = solver
        self.precision = precision
        self.op = op
        self.fronts, self.piv = solver._front_buffers(precision, self)
        eng = solver._engine(precision)
        solver._copy(op.values, eng.staging)
        eng.factor()
        if solver.tune and not eng.tuned:
            eng.tune(solver._tune_key(precision), _TUNE_CACHE)

    def valid(self):
        return self.solver._owner.get(self.precision) is self

    def apply(self, x):
        """In place: x <- M^-1 x."""
        eng = self.solver._engine(self.precision)
        self.solver._copy(x, eng.vec)
        eng.solve()
        self.solver._copy(eng.vec, x)


# -- run-time tuning of the application's launch shape -----------------------
# Warps per SM a height's FP32 / BF16 application launch aims for before its
# warps take fewer column tiles (the plan's apply_waves).
APPLY_WAVES = (16, 32, 64, 128)


def pick_fastest(candidates, time_fn, repeats=3):
    """The candidate with the least median of ``repeats`` timings
    (``time_fn(c)`` returns seconds); ties go to the earlier candidate."""
    best, best_t = None, None
    for c in candidates:
        ts = sorted(time_fn(c) for _ in range(repeats))
        t = ts[len(ts) // 2]
        if best_t is None or t < best_t:
            best, best_t = c, t
    return best


class TuneCache:
    """Tuned values per key, in memory and in a JSON file (read once,
    rewritten after each new entry).  A file that cannot be read or written
    only costs a re-tuning; the path is TRANSIFLOW_GB300_TUNE_CACHE, else
    ~/.cache/transiflow_gb300/tune.json."""

    def __init__(self, path=None):
        self.path = path or os.environ.get('TRANSIFLOW_GB300_TUNE_CACHE') or os.path.join(
            os.path.expanduser('~'), '.cache', 'transiflow_gb300', 'tune.json')
        self.lock = threading.Lock()
        self.data = None

    def _load(self):
        if self.data is None:
            try:
                with open(self.path) as f:
                    d = json.load(f)
                self.data = d if isinstance(d, dict) else {}
            except (OSError, ValueError):
                self.data = {}

    def get(self, key):
        with self.lock:
            self._load()
            return self.data.get(key)

    def put(self, key, value):
        with self.lock:
            self._load()
            self.data[key] = value
            try:
                os.makedirs(os.path.dirname(self.path) or '.', exist_ok=True)
                tmp = self.path + '.%d.tmp' % os.getpid()
                with open(tmp, 'w') as f:
                    json.dump(self.data, f, indent=1, sort_keys=True)
                os.replace(tmp, self.path)
            except OSError:
                pass


_TUNE_CACHE = TuneCache()


class _Engine:
    """Fixed buffers of one factor precision and the (graphed) launch
    sequences that factor and apply the LU."""

    def __init__(self, solver, precision, graphs):
        lib = _lib.load()
        plan = solver.plan
        self.staging = torch.empty(solver.itf.pattern.nnz, dtype=torch.float64, device=solver.itf.device)
        self.vec = torch.empty(plan.host.n, dtype=torch.float64, device=solver.itf.device)
        fronts, piv = solver._fronts_raw(precision)
        info = solver.info
        f64 = precision == 'fp64'
        fac_fn = lib.tf_nd_factor_f64 if f64 else lib.tf_nd_factor_f32
        # this engine's copy of the plan descriptor (plans are shared between
        # interfaces of the same grid; the factorisation options are not)
        self.struct = _lib.NdPlan.from_buffer_copy(plan.struct)
        self.struct.tc_min_front = solver.tc_min_front if not f64 else 0
        self.struct.tc_terms = solver.tc_terms
        sp = _struct_ptr(self.struct)
        dev = solver.itf.device
        # FP32 factors of an equilibrated copy of the operator: powers-of-two
        # row and column scales keep the FP32 factorisation of badly scaled
        # Jacobians (Pr = 1000 convection) useful; the staging buffer keeps
        # the unscaled values (the reuse policy measures drift on them)
        self.equil = (not f64) and solver.equilibrate
        n = plan.host.n
        if self.equil:
            self.scaled = torch.empty_like(self.staging)
            self.rscale = torch.empty(n, dtype=torch.float64, device=dev)
            self.cscale = torch.empty(n, dtype=torch.float64, device=dev)
        src = self.scaled if self.equil else self.staging
        # FP32 factors may be applied from a BF16 copy (half the bytes)
        self.bf16 = None
        if not f64 and solver.storage == 'bf16':
            if not solver.inverse or solver.flow:
                raise ValueError("BF16 factor storage needs 'Inverse Apply' with the per-height application")
            self.bf16 = torch.empty(plan.front_elems, dtype=torch.bfloat16, device=dev)
        if solver.inverse:
            # invert the own blocks once per factorisation; apply with
            # parallel triangular products instead of substitution chains
            inv_fn = lib.tf_nd_invert_f64 if f64 else lib.tf_nd_invert_f32
            sol_fn = lib.tf_nd_solve_inv_f64 if f64 else lib.tf_nd_solve_inv_f32
            wbytes = lib.tf_nd_invert_workspace_bytes(sp, 8 if f64 else 4)
            self.work = torch.empty(max(1, (wbytes + 7) // 8), dtype=torch.float64, device=dev)
            self.flow = None
            if solver.flow:
                # both sweeps in one persistent launch (dataflow over the
                # elimination tree); plans whose widest front does not fit
                # the launch's shared memory keep the per-height launches
                fuse, chunk = solver.flow_fuse_tiles, solver.flow_chunk_tiles
                fbytes = lib.tf_nd_flow_workspace_bytes(sp, fuse, chunk)
                if fbytes:
                    flow = torch.empty((fbytes + 7) // 8, dtype=torch.float64, device=dev)
                    code = lib.tf_nd_flow_prepare(sp, flow.data_ptr(), fbytes, 8 if f64 else 4, fuse, chunk)
                    if code == 0:
                        self.flow = flow
                    elif code != 4:     # TF_ERR_SIZE: fall back to the per-height launches
                        _lib.check(code, 'tf_nd_flow_prepare')
            if self.flow is not None:
                flow_fn = lib.tf_nd_solve_flow_f64 if f64 else lib.tf_nd_solve_flow_f32

                def solve():
                    _lib.check(flow_fn(sp, fronts.data_ptr(), piv.data_ptr(), self.vec.data_ptr(),
                                       self.flow.data_ptr(), _stream()), 'tf_nd_solve_flow')
            else:
                sbytes = lib.tf_nd_solve_inv_workspace_bytes(sp)
                self.scratch = torch.empty(max(1, sbytes // 8), dtype=torch.float64, device=dev)
                if self.bf16 is not None:
                    # the FP32 factors' BF16 copy, applied in FP32

                    def solve():
                        _lib.check(lib.tf_nd_solve_inv_bf16(sp, self.bf16.data_ptr(), piv.data_ptr(),
                                                            self.vec.data_ptr(), self.scratch.data_ptr(), _stream()),
                                   'tf_nd_solve_inv_bf16')
                else:

                    def solve():
                        _lib.check(sol_fn(sp, fronts.data_ptr(), piv.data_ptr(), self.vec.data_ptr(),
                                          self.scratch.data_ptr(), _stream()), 'tf_nd_solve_inv')

            # the inversion of each height overlaps the factorisation of the
            # heights above it on a second stream
            self.aux = _lib.new_stream(dev)
            facinv_fn = lib.tf_nd_factor_inv_f64 if f64 else lib.tf_nd_factor_inv_f32

            def factor():
                _lib.check(facinv_fn(sp, src.data_ptr(), fronts.data_ptr(), piv.data_ptr(),
                                     info.data_ptr(), self.work.data_ptr(), wbytes, _stream(),
                                     ctypes.c_void_p(self.aux.cuda_stream)), 'tf_nd_factor_inv')
                if self.bf16 is not None:
                    _lib.check(lib.tf_nd_factors_to_bf16(sp, fronts.data_ptr(), self.bf16.data_ptr(), _stream()),
                               'tf_nd_factors_to_bf16')
        else:
            self.flow = None
            sol_fn = lib.tf_nd_solve_f64 if f64 else lib.tf_nd_solve_f32

            def factor():
                _lib.check(fac_fn(sp, src.data_ptr(), fronts.data_ptr(), piv.data_ptr(),
                                  info.data_ptr(), _stream()), 'tf_nd_factor')

            def solve():
                _lib.check(sol_fn(sp, fronts.data_ptr(), piv.data_ptr(), self.vec.data_ptr(), _stream()),
                           'tf_nd_solve')

        if self.equil:
            pat = solver.itf.pattern
            factor_scaled, solve_scaled = factor, solve

            def factor():
                _lib.check(lib.tf_equilibrate(n, pat.rowptr.data_ptr(), pat.cols.data_ptr(), self.staging.data_ptr(),
                                              self.rscale.data_ptr(), self.cscale.data_ptr(), self.scaled.data_ptr(),
                                              _stream()), 'tf_equilibrate')
                factor_scaled()

            def solve():
                # M^-1 b = D_c (LU of D_r A D_c)^-1 (D_r b)
                _lib.check(lib.tf_vec_mul(n, self.rscale.data_ptr(), self.vec.data_ptr(), self.vec.data_ptr(),
                                          _stream()), 'tf_vec_mul')
                solve_scaled()
                _lib.check(lib.tf_vec_mul(n, self.cscale.data_ptr(), self.vec.data_ptr(), self.vec.data_ptr(),
                                          _stream()), 'tf_vec_mul')

        self.solve_raw = solve
        self.lib = lib
        # FP32 / BF16 per-height applications have a launch shape to tune
        self.tuned = f64 or not solver.inverse or self.flow is not None
        if graphs:
            self.factor = _Graphed(factor, solver.stats)
            self.solve = _Graphed(solve, solver.stats)
        else:
            self.factor, self.solve = factor, solve


    def tune(self, key, cache):
        """Time the FP32 / BF16 application (on the factors just computed)
        for each APPLY_WAVES target, keep the fastest in this engine's plan
        descriptor and in the cache.  Runs before any CUDA graph holds an
        application, so every later capture uses the tuned launches."""
        self.tuned = True
        best = cache.get(key)
        if best not in APPLY_WAVES:
            lib = self.lib
            _lib.check(lib.tf_vec_fill(self.vec.numel(), 1.0, self.vec.data_ptr(), _stream()), 'tf_vec_fill')

            def timed(w):
                self.struct.apply_waves = w
                self.solve_raw()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                self.solve_raw()
                e1.record()
                e1.synchronize()
                return e0.elapsed_time(e1) / 1000.0
            best = pick_fastest(APPLY_WAVES, timed)
            cache.put(key, best)
        self.struct.apply_waves = best

    def check(self):
        """Raises when a bounded wait of the dataflow application gave up
        since the last check (synchronising)."""
        if self.flow is not None:
            _lib.check(self.lib.tf_nd_flow_status(self.flow.data_ptr()), 'tf_nd_solve_flow')


def _struct_ptr(s):
    import ctypes
    return ctypes.cast(ctypes.pointer(s), ctypes.c_void_p)


class Solver:
    """Per-interface solver state: the plan, factor buffers, Krylov workspace."""

    def __init__(self, interface, restart=50, tol=1e-12, maxit=500, precision='fp64', reuse=True,
                 reuse_maxit=20, graphs=True, reuse_policy='cost', reuse_drift=0.05, inverse=True, flow=False,
                 flow_fuse_tiles=48, flow_chunk_tiles=24, leaf_cells=48, tc_min_front=1024,
                 tc_terms=3, storage='fp32', inner='fp64', equilibrate=True, bordered='krylov', tune=True):
        self.itf = interface
        # FP32 / BF16 factors: time the application's launch shapes once per
        # GPU, grid and precision (cached) and keep the fastest
        self.tune = bool(tune)
        # bordered systems: one FGMRES on the bordered matrix, or block
        # elimination with two solves of the gauged Jacobian
        if bordered not in ('krylov', 'elimination'):
            raise ValueError("'Bordered Solve' must be 'krylov' or 'elimination'")
        self.bordered = bordered
        self._bws = None
        # FP32 factorisations: heights whose widest front has at least this
        # many rows use blocked rank-256 tensor-core updates (0: never)
        self.tc_min_front = int(tc_min_front)
        # 1: plain TF32 products; 3: split operands, close to FP32 accuracy
        self.tc_terms = int(tc_terms)
        # FP32 factors: applied from the FP32 fronts or from a BF16 copy
        if storage not in ('fp32', 'bf16'):
            raise ValueError("'Factor Storage' must be 'fp32' or 'bf16'")
        self.storage = storage
        # precision of the Arnoldi operator products: the FP64 Jacobian, or an
        # FP32 copy inside cycles whose FP64 residuals refine the solution
        if inner not in ('fp64', 'fp32'):
            raise ValueError("'Inner Precision' must be 'fp64' or 'fp32'")
        self.inner = inner
        self._opbuf32 = None
        # FP32 factors: factor the row- and column-equilibrated operator
        self.equilibrate = bool(equilibrate)
        # grid cells at which nested dissection stops splitting a box
        self.leaf_cells = leaf_cells
        self.inverse = inverse
        # dataflow application (one launch for both sweeps) of the inverted factors
        self.flow = flow and inverse
        self.flow_fuse_tiles = flow_fuse_tiles
        self.flow_chunk_tiles = flow_chunk_tiles
        self.graphs = graphs
        self._engines = {}
        self.reuse = reuse
        self.reuse_maxit = reuse_maxit
        self._prec = None
        # running cost estimates (seconds): one factorisation, one GMRES iteration
        self._cost_factor = None
        self._cost_iter = None
        self._pending = []
        self.reuse_policy = reuse_policy
        # relative change of the Jacobian values up to which a reuse is tried;
        # adapted: halved after a failed attempt, grown after a success
        self._drift_tol = reuse_drift
        self._drift_work = None
        self._steps = {}
        self._opbuf = None
        self._opbuf_src = None
        # solves per operator and GMRES iterations with a fresh factorisation
        self._solves_per_op = 1.0
        self._its_fresh = 1.0
        self._last_op = None
        self._last_op_solves = 0
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
        self.stats = {'factorizations': 0, 'solves': 0, 'gmres_iterations': 0, 'last_relres': None,
                      'reused': 0, 'refactored_after_reuse': 0, 'graph_kernel_launches': 0}

    def _ensure_plan(self, pattern):
        if self.plan is None:
            itf = self.itf
            pvar = itf.dim if itf.dof > itf.dim else None
            key = (itf.nx, itf.ny, itf.nz, itf.dim, itf.dof, pvar, self.leaf_cells, str(pattern.rowptr.device))
            with _PLANS_LOCK:
                plan = _PLANS.get(key)
                if plan is None:
                    plan = NdPlanDevice(pattern, itf.nx, itf.ny, itf.nz, itf.dof, pvar, leaf_cells=self.leaf_cells)
                    # the uploads ran on this thread's stream: finish them
                    # before another thread's stream can read the plan
                    torch.cuda.current_stream().synchronize()
                    _PLANS[key] = plan
            self.plan = plan
            self.info = torch.zeros(1, dtype=torch.int32, device=pattern.rowptr.device)

    def _fronts_raw(self, precision):
        dt = torch.float64 if precision == 'fp64' else torch.float32
        bufs = self._fronts.get(precision)
        if bufs is None:
            dev = self.itf.device
            bufs = (torch.empty(self.plan.front_elems, dtype=dt, device=dev),
                    torch.empty(self.plan.host.n, dtype=torch.int32, device=dev))
            self._fronts[precision] = bufs
        return bufs

    def _front_buffers(self, precision, owner):
        bufs = self._fronts_raw(precision)
        self._owner[precision] = owner
        return bufs

    def _engine(self, precision):
        eng = self._engines.get(precision)
        if eng is None:
            eng = _Engine(self, precision, self.graphs)
            self._engines[precision] = eng
        return eng

    def _tune_key(self, precision):
        itf = self.itf
        return '%s|%dx%dx%d|dof%d|%s|%s|apply_waves' % (torch.cuda.get_device_name(itf.device), itf.nx, itf.ny,
                                                        itf.nz, itf.dof, precision, self.storage)

    def operator(self, jac):
        self._ensure_plan(jac.pattern)
        op = getattr(jac, '_gauged', None)
        if op is None:
            op = GaugedOperator(self, jac)
            jac._gauged = op
        return op

    def factorize(self, op):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fac = Factorization(self, op, self.precision)
        e1.record()
        self._pending.append((e0, e1))
        self.stats['factorizations'] += 1
        self._prec = fac
        op.jac.lu = fac
        return fac

    def factorization(self, jac):
        """The factorisation of jac itself (computed if needed)."""
        op = self.operator(jac)
        fac = jac.lu
        if not isinstance(fac, Factorization) or not fac.valid() or fac.precision != self.precision:
            fac = self.factorize(op)
        return fac

    # -- Krylov ---------------------------------------------------------------
    def _workspace(self, n, dev):
        m = self.restart
        if self._V is None or self._V.shape[1] != n:
            self._steps = {}
            self._V = torch.empty((m + 1, n), dtype=torch.float64, device=dev)
            self._Z = torch.empty((m, n), dtype=torch.float64, device=dev)
            lib = _lib.load()
            wb = lib.tf_vec_mdot_workspace_bytes(n, m + 1)
            self._mdot_work = torch.empty((wb + 7) // 8 + m + 2, dtype=torch.float64, device=dev)
            self._hbuf = torch.empty(2 * (m + 1) + 1, dtype=torch.float64, device=dev)
        return self._V, self._Z

    def _mdot_into(self, V, k, w, out):
        lib = _lib.load()
        n = w.numel()
        work = self._mdot_work[self.restart + 2:]
        _lib.check(lib.tf_vec_mdot(n, k, V.data_ptr(), V.stride(0), w.data_ptr(), out.data_ptr(),
                                   work.data_ptr(), work.numel() * 8, _stream()), 'tf_vec_mdot')

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

    def _copy(self, src, dst):
        self._axpby(1.0, src, 0.0, None, dst)

    def _zero(self, z):
        lib = _lib.load()
        _lib.check(lib.tf_vec_fill(z.numel(), 0.0, z.data_ptr(), _stream()), 'tf_vec_fill')

    def _axpby(self, a, x, b, y, z):
        lib = _lib.load()
        _lib.check(lib.tf_vec_axpby(z.numel(), float(a), None if x is None else x.data_ptr(), float(b),
                                    None if y is None else y.data_ptr(), z.data_ptr(), _stream()), 'tf_vec_axpby')

    def _norm(self, w, V=None):
        out = self._mdot(w.view(1, -1), 1, w)
        return math.sqrt(max(float(out.item()), 0.0))

    def _arnoldi_step(self, op, fac, j):
        """One flexible Arnoldi step on fixed buffers: Z[j] = M^-1 V[j],
        w = A Z[j] into V[j+1], classical Gram-Schmidt twice against V[0..j]
        (coefficients into the host-read buffer), ||w||^2 last, w scaled to
        unit norm.  The operator's values sit in a fixed buffer too, so every
        (precision, j) step is one CUDA graph, captured on its second use and
        replayed afterwards."""
        if self._opbuf is None or self._opbuf.numel() != op.values.numel():
            self._opbuf = torch.empty_like(op.values)
            self._opbuf_src = None
        if self._opbuf_src is not op:
            self._copy(op.values, self._opbuf)
            if self.inner == 'fp32':
                if self._opbuf32 is None or self._opbuf32.numel() != op.values.numel():
                    self._opbuf32 = torch.empty(op.values.numel(), dtype=torch.float32, device=op.values.device)
                _lib.check(_lib.load().tf_vec_to_f32(op.values.numel(), op.values.data_ptr(),
                                                     self._opbuf32.data_ptr(), _stream()), 'tf_vec_to_f32')
            self._opbuf_src = op
        key = (fac.precision, j)
        step = self._steps.get(key)
        if step is None:
            eng = self._engine(fac.precision)
            V, Z = self._V, self._Z
            hbuf = self._hbuf[:2 * (j + 1) + 1]
            h, h2, ww = hbuf[:j + 1], hbuf[j + 1:2 * (j + 1)], hbuf[2 * (j + 1):]
            w = V[j + 1]
            lib = _lib.load()
            pat = op.jac.pattern
            opbuf = self._opbuf
            # inner products with the FP32 copy of the operator ('Inner
            # Precision' fp32) or the FP64 operator itself
            spmv = lib.tf_spmv_f32 if self.inner == 'fp32' else lib.tf_spmv_f64
            opvals = self._opbuf32 if self.inner == 'fp32' else opbuf

            def fn():
                self._copy(V[j], eng.vec)
                eng.solve_raw()
                self._copy(eng.vec, Z[j])
                _lib.check(spmv(op.n, pat.rowptr.data_ptr(), pat.cols.data_ptr(), opvals.data_ptr(),
                                Z[j].data_ptr(), w.data_ptr(), 1.0, 0.0, _stream()), 'tf_spmv')
                self._mdot_into(V, j + 1, w, h)
                self._mgs(V, j + 1, h, w)
                self._mdot_into(V, j + 1, w, h2)
                self._mgs(V, j + 1, h2, w)
                self._mdot_into(w.view(1, -1), 1, w, ww)
                # a zero norm (breakdown) makes w non-finite; the caller stops there
                _lib.check(lib.tf_vec_scale_rsqrt(w.numel(), ww.data_ptr(), w.data_ptr(), _stream()),
                           'tf_vec_scale_rsqrt')

            step = _Graphed(fn, self.stats) if self.graphs else fn
            self._steps[key] = step
        step()

    def fgmres(self, op, fac, b, maxit=None):
        """Solve A_g x = b (b: float64 CUDA tensor) with preconditioner fac;
        returns (x, iterations, relres)."""
        maxit = self.maxit if maxit is None else maxit
        import time
        n = b.numel()
        V, Z = self._workspace(n, b.device)
        m = self.restart
        x = torch.empty_like(b)
        self._zero(x)
        r = torch.empty_like(b)
        self._copy(b, r)
        bn = self._norm(b)
        # the norm synchronises: work queued before this solve (a
        # factorisation) is not charged to the iterations
        t_start = time.perf_counter()
        if bn == 0.0:
            return x, 0, 0.0
        its = 0
        relres = 1.0
        tmp = torch.empty_like(b)
        inner_gain = 1e-6 if self.inner == 'fp32' else 0.0
        while its < maxit:
            beta = self._norm(r)
            relres = beta / bn
            if relres <= self.tol:
                break
            self._axpby(1.0 / beta, r, 0.0, None, V[0])
            # the Hessenberg columns and Givens rotations are a few dozen
            # scalars per step: plain Python floats (no NumPy call overhead)
            g = [0.0] * (m + 1)
            g[0] = beta
            cols = []
            cs = [0.0] * m
            sn = [0.0] * m
            k = 0
            for j in range(m):
                self._arnoldi_step(op, fac, j)
                # the CGS2 coefficients and the new vector's norm, one sync
                hb = self._hbuf[:2 * (j + 1) + 1].tolist()
                col = [hb[i] + hb[j + 1 + i] for i in range(j + 1)]
                hn = math.sqrt(max(hb[-1], 0.0))
                col.append(hn)
                for i in range(j):
                    t = cs[i] * col[i] + sn[i] * col[i + 1]
                    col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1]
                    col[i] = t
                d = math.hypot(col[j], col[j + 1])
                cs[j] = col[j] / d if d else 1.0
                sn[j] = col[j + 1] / d if d else 0.0
                col[j] = d
                col[j + 1] = 0.0
                cols.append(col)
                g[j + 1] = -sn[j] * g[j]
                g[j] = cs[j] * g[j]
                its += 1
                k = j + 1
                # with FP32 inner products a cycle can only gain about six
                # digits on its own starting residual; the FP64 residual below
                # then starts the next cycle (iterative refinement)
                if abs(g[j + 1]) <= max(self.tol * bn, inner_gain * beta) or its >= maxit or hn == 0:
                    break
            if k:
                R = np.zeros((k, k))
                for jj in range(k):
                    R[:jj + 1, jj] = cols[jj][:jj + 1]
                y = np.linalg.solve(R, np.asarray(g[:k]))
            else:
                y = np.zeros(0)
            yd = torch.as_tensor(-y, dtype=torch.float64).to(b.device)
            # x += Z[:k]^T y
            self._mgs(Z, k, yd, x) if k else None
            # true residual
            op.matvec(x, tmp)
            self._axpby(1.0, b, -1.0, tmp, r)
        self.stats['gmres_iterations'] += its
        self.stats['last_relres'] = relres
        if its and isinstance(fac, Factorization):
            self._engine(fac.precision).check()
        if its:
            self._cost_iter = self._ema(self._cost_iter, (time.perf_counter() - t_start) / its)
        return x, its, relres

    # -- the reference's solve contract ---------------------------------------
    @staticmethod
    def _ema(old, new):
        return new if old is None else 0.7 * old + 0.3 * new

    def _reuse_limit(self):
        """GMRES iterations a reused factorisation may take before a fresh
        factorisation would have been cheaper (at most reuse_maxit)."""
        done = [(a, b) for a, b in self._pending if b.query()]
        for a, b in done:
            self._cost_factor = self._ema(self._cost_factor, a.elapsed_time(b) / 1000.0)
        self._pending = [(a, b) for a, b in self._pending if (a, b) not in done]
        if self.reuse_policy == 'always':
            return self.reuse_maxit
        if self._cost_factor is None or self._cost_iter is None:
            return self.reuse_maxit
        # a Jacobian serves about m solves (two per continuation corrector
        # step); reusing costs m times the iterations, refactoring costs one
        # factorisation plus m times the iterations of a fresh factorisation
        m = self._solves_per_op
        its_f = self._its_fresh
        return int(min(self.reuse_maxit, (self._cost_factor / self._cost_iter + m * its_f) / m))

    def _count_solve(self, op):
        if op is not self._last_op:
            if self._last_op is not None:
                self._solves_per_op = 0.8 * self._solves_per_op + 0.2 * self._last_op_solves
            self._last_op, self._last_op_solves = op, 0
        self._last_op_solves += 1

    def _solve_gauged(self, op, b):
        """x with A_g x = b to the tolerance, reusing the latest factorisation
        as preconditioner while that is cheaper than refactoring."""
        self._count_solve(op)
        own = op.jac.lu
        if isinstance(own, Factorization) and own.valid() and own.precision == self.precision:
            x, its, rr = self.fgmres(op, own, b)
            self._its_fresh = 0.8 * self._its_fresh + 0.2 * its
            return x, its, rr
        prec = self._prec
        limit = self._reuse_limit() if self.reuse else 0
        seen = getattr(op, '_reuse_its', None)
        if seen is not None and self.reuse_policy != 'always' and self._cost_factor and self._cost_iter:
            # a reuse on this operator already took `seen` iterations: refactor
            # now if that is dearer than a factorisation
            limit = 0 if seen * self._cost_iter > self._cost_factor + self._its_fresh * self._cost_iter else limit
        if limit >= 2 and prec is not None and prec.valid() and prec.precision == self.precision:
            if self.reuse_policy == 'always' or seen is not None or self._drift(op) <= self._drift_tol:
                x, its, rr = self.fgmres(op, prec, b, maxit=limit)
                if math.isfinite(rr) and rr <= self.tol:
                    self.stats['reused'] += 1
                    op._reuse_its = its
                    self._drift_tol = min(0.5, 1.25 * self._drift_tol)
                    return x, its, rr
                self.stats['refactored_after_reuse'] += 1
                self._drift_tol *= 0.5
        x, its, rr = self.fgmres(op, self.factorize(op), b)
        self._its_fresh = 0.8 * self._its_fresh + 0.2 * its
        return x, its, rr

    def _drift(self, op):
        """||A_new - A_f|| / ||A_f|| over the stencil values, A_f being the
        operator of the latest factorisation (its values are still in the
        engine's staging buffer)."""
        lib = _lib.load()
        eng = self._engine(self.precision)
        m = op.values.numel()
        if self._drift_work is None or self._drift_work[0].numel() != m:
            wb = lib.tf_vec_mdot_workspace_bytes(m, 1)
            self._drift_work = (torch.empty(m, dtype=torch.float64, device=op.values.device),
                                torch.empty((wb + 7) // 8, dtype=torch.float64, device=op.values.device),
                                torch.empty(2, dtype=torch.float64, device=op.values.device))
        d, work, out = self._drift_work
        self._axpby(1.0, op.values, -1.0, eng.staging, d)
        for v, o in ((d, out[0:1]), (eng.staging, out[1:2])):
            _lib.check(lib.tf_vec_mdot(m, 1, v.data_ptr(), m, v.data_ptr(), o.data_ptr(), work.data_ptr(),
                                       work.numel() * 8, _stream()), 'tf_vec_mdot')
        dn, fn = out.cpu().numpy()
        return math.sqrt(max(dn, 0.0) / fn) if fn > 0 else math.inf

    def solve(self, jac, rhs, rhs2=None, V=None, W=None, C=None):
        itf = self.itf
        op = self.operator(jac)
        self.stats['solves'] += 1
        src = _to_tensor(rhs, itf.device)
        b = torch.empty_like(src)
        self._copy(src, b)
        if rhs2 is None:
            if self.gauge >= 0:
                lib = _lib.load()
                _lib.check(lib.tf_vec_fill(1, 0.0, b.data_ptr() + 8 * self.gauge, _stream()), 'tf_vec_fill')
            x, its, rr = self._solve_gauged(op, b)
            if not math.isfinite(rr) or rr > max(self.tol, 1e-6):
                raise RuntimeError('GMRES did not converge: relative residual %.3e after %d iterations' % (rr, its))
            return DeviceVector(x)
        return self._bordered(op, b, rhs2, V, W, C)

    def _bordered(self, op, b, rhs2, V, W, C):
        """[A_g, sV; sW'^T, s^2 C][y; t] = [b; s rhs2], where W' is W without
        its gauge entry (SciPy.py:93-126) and b keeps its gauge entry
        (SciPy.py:226-227)."""
        itf = self.itf
        s = itf.border_scaling
        if np.ndim(rhs2) != 0:
            raise NotImplementedError('bordered solves with more than one border vector')
        Vt = _to_tensor(V, itf.device)
        Wt = _to_tensor(W if W is not None else V, itf.device).clone()
        if self.gauge >= 0:
            Wt[self.gauge] = 0.0
        Cv = 0.0 if C is None else float(C)
        if self.bordered == 'krylov':
            return self._bordered_krylov(op, b, s * float(rhs2), (s * Vt).contiguous(), (s * Wt).contiguous(),
                                         s * s * Cv, s)
        y0, i0, r0 = self._solve_gauged(op, b.clone())
        y1, i1, r1 = self._solve_gauged(op, (s * Vt).contiguous())
        if max(r0, r1) > max(self.tol, 1e-6):
            raise RuntimeError('GMRES did not converge in a bordered solve')
        wy0 = float(_dot_t(Wt, y0))
        wy1 = float(_dot_t(Wt, y1))
        # s W'^T y + s^2 C t = s rhs2, with y = y0 - t y1
        t = (s * float(rhs2) - s * wy0) / (s * s * Cv - s * wy1)
        self._axpby(1.0, y0, -t, y1, y0)
        return DeviceVector(y0), t * s

    # -- the bordered system as one Krylov solve ------------------------------
    def _bordered_workspace(self, n, dev):
        m = self.restart
        if self._bws is None or self._bws['V'].shape[1] != n + 1:
            lib = _lib.load()
            wb = lib.tf_vec_mdot_workspace_bytes(n + 1, m + 1)
            self._bws = {'V': torch.empty((m + 1, n + 1), dtype=torch.float64, device=dev),
                         'Z': torch.empty((m, n + 1), dtype=torch.float64, device=dev),
                         'h': torch.empty(m + 2, dtype=torch.float64, device=dev),
                         'work': torch.empty((wb + 7) // 8, dtype=torch.float64, device=dev),
                         'q': torch.empty(n, dtype=torch.float64, device=dev),
                         'r': torch.empty(n + 1, dtype=torch.float64, device=dev),
                         'x': torch.empty(n + 1, dtype=torch.float64, device=dev)}
        return self._bws

    def _bdot(self, V, k, w, out):
        """out[:k] = V[:k] . w over w's length (device)."""
        lib = _lib.load()
        ws = self._bws['work']
        _lib.check(lib.tf_vec_mdot(w.numel(), k, V.data_ptr(), V.stride(0), w.data_ptr(), out.data_ptr(),
                                   ws.data_ptr(), ws.numel() * 8, _stream()), 'tf_vec_mdot')

    def _bordered_fgmres(self, op, fac, u, w, c, b, beta, maxit):
        """Flexible GMRES on B = [A_g, u; w^T, c] with the block
        preconditioner P^-1 [r; rho] = [z - tau q; tau], z = M r, q = M u,
        tau = (rho - w.z) / (c - w.q): exact when M = A_g^-1, so the
        iterations are those of one solve with A_g.  Returns (x (n+1),
        iterations, relative residual)."""
        n = op.n
        ws = self._bordered_workspace(n, b.device)
        V, Z, h, q, r, x = ws['V'], ws['Z'], ws['h'], ws['q'], ws['r'], ws['x']
        m = self.restart
        eng = self._engine(fac.precision)
        lib = _lib.load()

        def prec(src, dst):
            self._copy(src, eng.vec)
            eng.solve()
            self._copy(eng.vec, dst)

        def fill(t, i, v):
            _lib.check(lib.tf_vec_fill(1, float(v), t.data_ptr() + 8 * i, _stream()), 'tf_vec_fill')

        def scalar(t, i):
            return float(t[i].item())

        prec(u, q)
        self._bdot(w.view(1, -1), 1, q, h)
        delta = c - scalar(h, 0)
        if delta == 0.0 or not math.isfinite(delta):
            raise RuntimeError('singular bordered preconditioner')
        # right-hand side [b; beta]
        self._copy(b, r[:n])
        fill(r, n, beta)
        self._bdot(r.view(1, -1), 1, r, h)
        bn = math.sqrt(max(scalar(h, 0), 0.0))
        self._zero(x)
        if bn == 0.0:
            return x, 0, 0.0
        its, relres = 0, 1.0
        tmp = torch.empty(n, dtype=torch.float64, device=b.device)
        while its < maxit:
            self._bdot(r.view(1, -1), 1, r, h)
            rn = math.sqrt(max(scalar(h, 0), 0.0))
            relres = rn / bn
            if relres <= self.tol:
                break
            self._axpby(1.0 / rn, r, 0.0, None, V[0])
            g = [0.0] * (m + 1)
            g[0] = rn
            cols, cs, sn = [], [0.0] * m, [0.0] * m
            k = 0
            for j in range(m):
                vj, zj, wv = V[j], Z[j], V[j + 1]
                rho = scalar(vj, n)
                prec(vj[:n], zj[:n])
                self._bdot(w.view(1, -1), 1, zj[:n], h)
                tau = (rho - scalar(h, 0)) / delta
                self._axpby(1.0, zj[:n], -tau, q, zj[:n])
                fill(zj, n, tau)
                # B z: A_g z_top + tau u; the last row of B P^-1 returns rho
                op.matvec(zj[:n], wv[:n])
                self._axpby(1.0, wv[:n], tau, u, wv[:n])
                fill(wv, n, rho)
                # classical Gram-Schmidt, twice
                col = [0.0] * (j + 2)
                for _ in range(2):
                    self._bdot(V, j + 1, wv, h)
                    hj = h[:j + 1]
                    self._mgs(V, j + 1, hj, wv)
                    for i, v in enumerate(hj.tolist()):
                        col[i] += v
                self._bdot(wv.view(1, -1), 1, wv, h)
                hn = math.sqrt(max(scalar(h, 0), 0.0))
                col[j + 1] = hn
                if hn > 0:
                    self._axpby(1.0 / hn, wv, 0.0, None, wv)
                for i in range(j):
                    t = cs[i] * col[i] + sn[i] * col[i + 1]
                    col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1]
                    col[i] = t
                d = math.hypot(col[j], col[j + 1])
                cs[j] = col[j] / d if d else 1.0
                sn[j] = col[j + 1] / d if d else 0.0
                col[j], col[j + 1] = d, 0.0
                cols.append(col)
                g[j + 1] = -sn[j] * g[j]
                g[j] = cs[j] * g[j]
                its += 1
                k = j + 1
                if abs(g[j + 1]) <= self.tol * bn or its >= maxit or hn == 0:
                    break
            R = np.zeros((k, k))
            for jj in range(k):
                R[:jj + 1, jj] = cols[jj][:jj + 1]
            y = np.linalg.solve(R, np.asarray(g[:k]))
            yd = torch.as_tensor(-y, dtype=torch.float64).to(b.device)
            self._mgs(Z, k, yd, x)
            # true residual [b - A_g x_top - x_n u; beta - w.x_top - c x_n]
            xn = scalar(x, n)
            op.matvec(x[:n], tmp)
            self._axpby(1.0, b, -1.0, tmp, r[:n])
            self._axpby(1.0, r[:n], -xn, u, r[:n])
            self._bdot(w.view(1, -1), 1, x[:n], h)
            fill(r, n, beta - scalar(h, 0) - c * xn)
        self.stats['gmres_iterations'] += its
        self.stats['last_relres'] = relres
        if its:
            self._engine(fac.precision).check()
        return x, its, relres

    def _bordered_krylov(self, op, b, beta, u, w, c, s):
        """One FGMRES on the bordered system, preconditioned by the gauged
        Jacobian's own factorisation, or by the latest one while reusing it
        is cheaper (as for plain solves); a reuse that does not converge
        within its iteration budget is redone after a fresh factorisation."""
        self._count_solve(op)
        own = op.jac.lu
        if isinstance(own, Factorization) and own.valid() and own.precision == self.precision:
            fac, limit = own, self.maxit
        else:
            prec = self._prec
            limit = self._reuse_limit() if self.reuse else 0
            if (limit >= 2 and prec is not None and prec.valid() and prec.precision == self.precision
                    and (self.reuse_policy == 'always' or self._drift(op) <= self._drift_tol)):
                fac = prec
            else:
                fac, limit = self.factorize(op), self.maxit
        x, its, rr = self._bordered_fgmres(op, fac, u, w, c, b, beta, limit)
        if fac is not op.jac.lu and (not math.isfinite(rr) or rr > self.tol):
            self.stats['refactored_after_reuse'] += 1
            self._drift_tol *= 0.5
            x, its, rr = self._bordered_fgmres(op, self.factorize(op), u, w, c, b, beta, self.maxit)
        elif fac is not op.jac.lu:
            self.stats['reused'] += 1
        if not math.isfinite(rr) or rr > max(self.tol, 1e-6):
            raise RuntimeError('GMRES did not converge in a bordered solve: relative residual %.3e' % rr)
        n = op.n
        y = torch.empty(n, dtype=torch.float64, device=b.device)
        self._copy(x[:n], y)
        return DeviceVector(y), float(x[n].item()) * s


def _to_tensor(v, device):
    if isinstance(v, DeviceVector):
        return v.data
    if isinstance(v, torch.Tensor):
        return v.to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(v, dtype=np.float64)).to(device)


def _dot_t(a, b):
    from .vector import _dot
    return _dot(DeviceVector(a), DeviceVector(b))
