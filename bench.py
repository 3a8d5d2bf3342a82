"""Benchmark: seconds to reach the Reynolds-number target on one GB300.

Workload (the plain-GPU configuration of the headline metric): 2D
lid-driven cavity, nx = ny = 256 (196,608 unknowns), FP64 assembly,
Newton at Re = 0 from the zero state, then pseudo-arclength continuation in
the Reynolds number from 0 to 5000 with ds = 200 and ||F|| <= 1e-8 at every
point; linear solves by FP64 GMRES to 1e-10 relative residual, preconditioned
by the nested-dissection LU of the gauged Jacobian.  One step = one complete
branch.  Synthetic: the branch starts from the zero state (no dataset).

  value      seconds per branch, the initial state already on the device
  e2e        the same through the public API with host buffers: the initial
             state is copied from pinned host memory and the final state read
             back inside the timed region
  roofline   the dominant kernel, timed live with CUDA events
  cpu_baseline  the CPU oracle (NumPy assembly + SuperLU) per call on this
             host, scaled by the branch's call counts

``--impl reference`` times the reference algorithm's CPU implementation on
this host (the oracle restatement: the reference package itself is not
installable on the GPU machine) on the same workload, one bounded sample per
step.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
import io
import contextlib

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 's to Re target: learned+mixed vs plain FP64 on same GB300 at ||F||<=1e-8'


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--nx', type=int, default=256)
    ap.add_argument('--target', type=float, default=5000.0)
    ap.add_argument('--ds', type=float, default=200.0)
    ap.add_argument('--precision', default='fp64', choices=['fp64', 'fp32'])
    ap.add_argument('--tol', type=float, default=1e-10)
    ap.add_argument('--no-baseline', action='store_true')
    ap.add_argument('--profile', default=None, choices=['factor', 'solve', 'assemble'],
                    help='run only a few launches of one stage (for ncu captures)')
    ap.add_argument('--nz', type=int, default=1, help='cells in z (1: the 2D grid)')
    ap.add_argument('--batched', type=int, default=0,
                    help='time this many random lid-driven cavities (nx from 32..192, Re from [100, 4000], '
                         'seed 2) solved concurrently and one after the other, then exit')
    ap.add_argument('--re', type=float, default=1000.0, help='Reynolds number of the --profile state')
    ap.add_argument('--apply', default='levels', choices=['flow', 'levels', 'sweep'],
                    help='application of the inverted factors: one dataflow launch or one launch per tree height')
    ap.add_argument('--flow-fuse', type=int, default=48, help='dataflow apply: most factor tiles of a warp-task front')
    ap.add_argument('--flow-chunk', type=int, default=24, help='dataflow apply: target tiles per CTA task')
    ap.add_argument('--leaf-cells', type=int, default=48, help='grid cells at which nested dissection stops')
    ap.add_argument('--reuse-its', type=int, default=None, help="'Reuse Iterations' (default: the backend's)")
    ap.add_argument('--no-inverse', action='store_true', help="'Inverse Apply': False (substitution solves)")
    ap.add_argument('--reuse-drift', type=float, default=None, help="'Reuse Drift' (default: the backend's)")
    ap.add_argument('--learned', action='store_true',
                    help='train the learned predictor on plain branches of the --train-grids, then time the '
                         'branch at --nx/--nz plain (FP64 factors) and learned (FP32 factors), then exit')
    ap.add_argument('--train-grids', default='32,48', help='--learned: training grid sizes (cubes when --nz > 1)')
    ap.add_argument('--train-seeds', default='3,4,5,6', help='--learned: one training branch per seed and grid')
    ap.add_argument('--train-target', type=float, default=2500.0, help='--learned: Re at the end of training branches')
    ap.add_argument('--train-steps', type=int, default=100, help='--learned: Adam steps per grid and round')
    ap.add_argument('--train-rounds', type=int, default=4, help='--learned: rounds over the training grids')
    ap.add_argument('--sweep-heights', type=int, default=0,
                    help='with --apply sweep: tree heights nearest the root in the cooperative launch (0: all)')
    return ap.parse_args()


def config(args):
    if args.nz > 1:
        n = 4 * args.nx * args.nx * args.nz
        grid = '3D lid-driven cavity %dx%dx%d, dof 4' % (args.nx, args.nx, args.nz)
    else:
        n = 3 * args.nx * args.nx
        grid = '2D lid-driven cavity %dx%d, dof 3' % (args.nx, args.nx)
    return {'workload': '%s (%d unknowns), Newton at Re=0 then continuation '
                        'Re 0->%g, ds=%g, ||F||<=1e-8, FP64 GMRES to %g + ND-LU (%s factors)'
                        % (grid, n, args.target, args.ds, args.tol, args.precision),
            'nx': args.nx, 'ny': args.nx, 'nz': args.nz, 'dof': 4 if args.nz > 1 else 3, 'unknowns': n,
            'target_re': args.target, 'ds': args.ds, 'newton_tolerance': 1e-8,
            'l2': 'working set larger than L2 (1.1 GB of frontal matrices at 256^2)',
            'parallelism': 'replicas (one instance per GPU)'}


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ('clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in self.lines:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_branch(itf, Continuation, x0, args):
    cont = Continuation(itf, newton_tolerance=1e-8)
    with contextlib.redirect_stdout(io.StringIO()):
        itf.set_parameter('Reynolds Number', 0.0)
        x = cont.newton(x0)
        x, mu = cont.continuation(x, 'Reynolds Number', 0.0, args.target, args.ds)
    return x, mu, cont


def gpu_arm(args, rank, world, local):
    import torch
    from transiflow_gb300 import Continuation, Interface, _lib, dist
    torch.cuda.set_device(local)
    lib = _lib.load()
    tuning = {}
    if args.reuse_its is not None:
        tuning['Reuse Iterations'] = args.reuse_its
    if args.reuse_drift is not None:
        tuning['Reuse Drift'] = args.reuse_drift
    if args.no_inverse:
        tuning['Inverse Apply'] = False
    params = {'CUDA': {**tuning, 'Factor Precision': args.precision, 'Tolerance': args.tol,
                       'Dataflow Apply': args.apply == 'flow', 'Sweep Apply': (args.sweep_heights or True) if args.apply == 'sweep' else False,
                       'Dataflow Fuse Tiles': args.flow_fuse,
                       'Dataflow Chunk Tiles': args.flow_chunk, 'Leaf Cells': args.leaf_cells}}
    itf = Interface(params, args.nx, args.nx, args.nz)
    n = itf.n
    stream = torch.cuda.current_stream()

    # warm-up branches (the first one also builds the elimination plan)
    for _ in range(args.warmup):
        x, mu, cont = run_branch(itf, Continuation, itf.vector(), args)
    calls = dict(cont.stats)
    calls['factorizations'] = None
    fac0 = itf.solver.stats['factorizations']
    x, mu, cont = run_branch(itf, Continuation, itf.vector(), args)
    calls['factorizations'] = itf.solver.stats['factorizations'] - fac0
    calls['gmres_iterations_last'] = itf.solver.stats['gmres_iterations']
    itf.set_parameter('Reynolds Number', mu)
    fnorm_end = itf.rhs(x).norm()

    # ---- value: device-resident start state ----
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    l0 = lib.tf_launch_count()
    g0 = itf.solver.stats['graph_kernel_launches']
    s0 = dict(itf.solver.stats)
    t_dev = []
    for _ in range(args.steps):
        x0 = itf.vector()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        x, mu, _ = run_branch(itf, Continuation, x0, args)
        ev1.record(stream)
        torch.cuda.synchronize()
        t_dev.append(ev0.elapsed_time(ev1) / 1000.0)
    launches = lib.tf_launch_count() - l0 + itf.solver.stats['graph_kernel_launches'] - g0
    s1 = itf.solver.stats
    solver_stats = {k: (s1[k] - s0[k]) / args.steps for k in ('factorizations', 'solves', 'gmres_iterations',
                                                               'reused', 'refactored_after_reuse')}
    dist.barrier()
    clk = clocks.stop()
    t_step = dist.max_over_ranks(statistics.mean(t_dev))

    # ---- e2e: host buffers through the public API ----
    host0 = torch.zeros(n, dtype=torch.float64).pin_memory()
    t_e2e = []
    dist.barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        x0 = itf.vector_from_array(host0.numpy())
        x, mu, _ = run_branch(itf, Continuation, x0, args)
        out = itf.array_from_vector(x)
        torch.cuda.synchronize()
        t_e2e.append(time.perf_counter() - t0)
    e2e = dist.max_over_ranks(statistics.mean(t_e2e))
    dist.barrier()

    roof = roofline(itf, x, args, lib)
    result = {'metric': METRIC, 'value': t_step, 'unit': 's', 'n_gpus': world, 'steps': args.steps,
              'warmup': args.warmup, 'ms_per_step': t_step * 1000.0, 'higher_is_better': False,
              'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64' if args.precision == 'fp64' else 'f64+f32',
              'data': 'synthetic (zero initial state; no dataset)', 'config': config(args),
              'e2e': {'value': e2e, 'unit': 's', 'h2d_bytes_per_step': 8 * n, 'd2h_bytes_per_step': 8 * n},
              'roofline': roof, 'clocks': clk, 'gpu_launches': int(launches),
              'branch': {'points': calls.get('points'), 'rhs': calls.get('rhs'), 'jacobian': calls.get('jacobian'),
                         'solve': calls.get('solve'), 'factorizations': calls.get('factorizations'),
                         'final_re': mu, 'final_fnorm': fnorm_end, 'per_step_solver': solver_stats,
                         'newton_steps_per_s': (calls.get('jacobian') or 0) / t_step}}
    if rank == 0 and not args.no_baseline:
        result['cpu_baseline'] = cpu_baseline(args, calls)
    return result


def _peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def fp64_peak():
    """FP64 dense throughput of this GPU measured live: cuBLAS DGEMM 4096^3
    through torch (best of 5), the denominator for FP64-bound kernels."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device='cuda')
    b = torch.randn(4096, 4096, dtype=torch.float64, device='cuda')
    c = a @ b
    best = None
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1000.0
        best = t if best is None else min(best, t)
    del a, b, c
    return 2.0 * 4096 ** 3 / best / 1e12


# DRAM bytes (read + write) of one factorisation with the inversion of its own
# blocks, summed over its launches in one ncu capture of
# `bench.py --profile factor` on a GB300.
FACTOR_TRAFFIC = {(256, 1, 'fp64'): 6.353e9}


def roofline(itf, x, args, lib):
    """Live CUDA-event timing of the dominant kernels over rotating buffers
    larger than L2 (129 MB)."""
    import torch
    from transiflow_gb300.vector import _stream
    n = itf.n
    nnz = itf.pattern.nnz
    prob = itf._problem()
    reps = 8
    # rotating states and Jacobian value buffers: reps x (8n + 8 nnz) > L2
    states = [x.data.clone() for _ in range(reps)]
    rhs = [torch.empty(n, dtype=torch.float64, device=itf.device) for _ in range(reps)]
    jv = [torch.empty(nnz, dtype=torch.float64, device=itf.device) for _ in range(reps)]
    st = torch.cuda.current_stream()

    def timed(fn, count):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for i in range(count):
            fn(i % reps)
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0 / count

    def asm(i):
        lib.tf_assemble(ctypes.byref(prob), states[i].data_ptr(), rhs[i].data_ptr(), jv[i].data_ptr(), _stream())

    timed(asm, reps)
    t_asm = timed(asm, 40)
    bytes_asm = 16 * n + 8 * nnz          # read x + write F, write J values
    rp, cp = itf.pattern.rowptr, itf.pattern.cols

    def spmv(i):
        lib.tf_spmv_f64(n, rp.data_ptr(), cp.data_ptr(), jv[i].data_ptr(), states[i].data_ptr(),
                        rhs[i].data_ptr(), 1.0, 0.0, _stream())

    timed(spmv, reps)
    t_spmv = timed(spmv, 40)
    bytes_spmv = 12 * nnz + 4 * (n + 1) + 16 * n
    # factorisation and solve of the current Jacobian
    J = itf.jacobian(itf.vector_from_array(x.numpy()))
    fac = itf.solver.factorization(J)
    torch.cuda.synchronize()
    f_time = []
    for _ in range(3):
        J.lu = None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fac = itf.solver.factorization(J)
        e1.record(st)
        torch.cuda.synchronize()
        f_time.append(e0.elapsed_time(e1) / 1000.0)
    t_fac = min(f_time)
    v = torch.ones(n, dtype=torch.float64, device=itf.device)
    t_sol = timed(lambda i: fac.apply(v), 10)
    peak, which = _peaks()
    flops = itf.solver.plan.flops
    f64 = fp64_peak()
    kernels = {
        'tf_assemble (F + J, fused)': {'s_per_launch': t_asm, 'bytes': bytes_asm,
                                       'GB/s': bytes_asm / t_asm / 1e9, 'frac_hbm': bytes_asm / t_asm / 1e9 / peak},
        'tf_spmv_f64': {'s_per_launch': t_spmv, 'bytes': bytes_spmv, 'GB/s': bytes_spmv / t_spmv / 1e9,
                        'frac_hbm': bytes_spmv / t_spmv / 1e9 / peak},
        'tf_nd_factor (%s)' % args.precision: {'s_per_call': t_fac, 'flops': flops,
                                                'TFLOP/s': flops / t_fac / 1e12},
        'tf_nd_solve (%s)' % args.precision: {'s_per_call': t_sol},
    }
    # The dominant work of a branch is the multifrontal factorisation, one
    # CUDA-graph launch per Jacobian; its trailing-update GEMMs are FP64
    # issue bound, so it is compared with this GPU's dense FP64 GEMM rate
    # (cuBLAS DGEMM measured live; MEASURED_PEAKS.json has no FP64 figure).
    a = flops / t_fac / 1e12
    return {'bound': 'tensor', 'kernel': 'tf_nd_factor_%s: multifrontal LU graph (%dx%d, %.2f GFLOP per launch)'
            % (args.precision, args.nx, args.nx, flops / 1e9),
            'achieved': a, 'peak': f64 if args.precision == 'fp64' else None, 'unit': 'TFLOP/s',
            'frac': a / f64 if args.precision == 'fp64' else None,
            'peak_source': 'FP64 dense GEMM of this GPU measured in this run (cuBLAS DGEMM 4096^3)',
            'traffic': FACTOR_TRAFFIC.get((args.nx, args.nz, args.precision)),
            'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum over the launches of one '
                              'factorisation (caches flushed per kernel: an upper bound)',
            'algorithmic_flops': flops, 'hbm_peak_gbs': peak,
            'hbm_peak_source': '%s (MEASURED_PEAKS.json hbm_gbs)' % which, 'kernels': kernels}


# ---------------------------------------------------------------------------
# CPU oracle timings (the reference algorithm on this host's cores)
# ---------------------------------------------------------------------------
def oracle_sample(nx, seed=1):
    from oracle.solve import Interface as OracleInterface
    itf = OracleInterface({'Reynolds Number': 1000}, nx, nx)
    s = 0.1 * np.random.default_rng(seed).standard_normal(itf.vector().size)
    t = {}
    t0 = time.perf_counter()
    f = itf.rhs(s)
    t['rhs'] = time.perf_counter() - t0
    t0 = time.perf_counter()
    J = itf.jacobian(s)
    t['jacobian'] = time.perf_counter() - t0
    t0 = time.perf_counter()
    itf.solve(J, f)
    t['factor_solve'] = time.perf_counter() - t0
    t0 = time.perf_counter()
    itf.solve(J, f)
    t['solve'] = time.perf_counter() - t0
    return t


# Call counts of the branch (2D LDC 256^2, Re 0 -> 5000, ds = 200,
# newton_tolerance 1e-8) as run by the continuation driver; the GPU arm
# recomputes them live and the reference arm uses these.
# Interface calls of the 256^2 branch (Re 0 -> 5000, ds = 200, ||F|| <= 1e-8) as
# the reference's Continuation makes them on an exact solver; the SciPy
# interface factors every Jacobian once (the LU is cached on the matrix).
BRANCH_CALLS_256 = {'rhs': 111, 'jacobian': 47, 'solve': 92, 'factorizations': 47}


def extrapolate(t, calls):
    """Seconds of the reference's SciPy path for these call counts: one
    SuperLU factorisation per Jacobian (SciPy.py:151, cached on the matrix)."""
    nfac = calls['jacobian']
    return (calls['rhs'] * t['rhs'] + calls['jacobian'] * t['jacobian'] + nfac * t['factor_solve']
            + max(calls['solve'] - nfac, 0) * t['solve'])


def cpu_baseline(args, calls):
    t = oracle_sample(args.nx)
    est = extrapolate(t, calls)
    return {'value': est, 'unit': 's', 'cores': 1, 'kind': 'port',
            'sample': 'oracle (vectorised NumPy restatement of Discretization + SciPy SuperLU, '
                      'single-threaded splu) at %dx%d: 1 rhs %.2fs, 1 jacobian %.2fs, 1 factor+solve %.2fs, '
                      '1 solve %.2fs, scaled by the branch call counts %s (one factorisation per jacobian)'
                      % (args.nx, args.nx, t['rhs'], t['jacobian'], t['factor_solve'], t['solve'],
                         {k: calls[k] for k in ('rhs', 'jacobian', 'solve')}),
            'host_cpus': os.cpu_count()}


def reference_arm(args, rank):
    if rank != 0:
        return None
    calls = dict(BRANCH_CALLS_256)
    if args.nx != 256 or args.nz != 1:
        return {'impl': 'reference', 'unavailable': 'branch call counts are known for the 256x256 branch only'}
    for _ in range(args.warmup):
        oracle_sample(args.nx)
    vals = []
    for _ in range(args.steps):
        t = oracle_sample(args.nx)
        vals.append(extrapolate(t, calls))
    v = statistics.mean(vals)
    return {'metric': METRIC, 'value': v, 'unit': 's', 'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': v * 1000.0, 'higher_is_better': False, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference', 'config': config(args),
            'cpu_baseline': {'value': v, 'unit': 's', 'cores': 1, 'kind': 'port',
                             'sample': 'per step one rhs, one jacobian, one SuperLU factor+solve and one solve '
                                       'of the oracle at %dx%d on this host, scaled by the branch call counts %s'
                                       % (args.nx, args.nx, calls)},
            'e2e': {'value': v, 'unit': 's', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}


def profile_stage(args):
    """A short, fixed sequence of one stage for profiler captures: the
    Jacobian of a random state (Re from --re, 2D unless --nz > 1), then 3
    factorisations, 3 preconditioner applications or 3 fused assemblies,
    each timed with CUDA events on the launching stream."""
    import torch
    from transiflow_gb300 import Interface
    p = {'Reynolds Number': args.re, 'CUDA': {'Factor Precision': args.precision, 'CUDA Graphs': False,
                                              'Dataflow Apply': args.apply == 'flow',
                                              'Sweep Apply': ((args.sweep_heights or True)
                                                              if args.apply == 'sweep' else False),
                                              'Dataflow Fuse Tiles': args.flow_fuse,
                                              'Dataflow Chunk Tiles': args.flow_chunk, 'Leaf Cells': args.leaf_cells}}
    itf = Interface(p, args.nx, args.nx, args.nz)
    s = 0.1 * np.random.default_rng(1).standard_normal(itf.n)
    x = itf.vector_from_array(s)
    J = itf.jacobian(x)
    t0 = time.perf_counter()
    fac = itf.solver.factorization(J)
    torch.cuda.synchronize()
    first = time.perf_counter() - t0
    st = torch.cuda.current_stream()
    times = []
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        if args.profile == 'factor':
            J.lu = None
            fac = itf.solver.factorization(J)
        elif args.profile == 'solve':
            fac.apply(x.data)
        else:
            itf.rhs(x)
            itf.jacobian(x)
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1000.0)
    plan = itf.solver.plan
    print(json.dumps({'profile': args.profile, 'nx': args.nx, 'nz': args.nz, 'unknowns': itf.n,
                      'precision': args.precision, 's_per_call': times, 'first_factor_s': first,
                      'factor_gflop': plan.flops / 1e9, 'front_gb': plan.front_elems * (8 if args.precision == 'fp64' else 4) / 1e9}))


def batched(args):
    """The batched configuration: many independent lid-driven cavities of
    uneven size and Reynolds number, each by Newton at Re = 0 and continuation
    to its Re with ||F|| <= 1e-10, solved concurrently (one stream per
    instance) and one after the other on the same GPU."""
    import torch
    from transiflow_gb300.batch import solve_instance, solve_many
    rng = np.random.default_rng(2)
    specs = [{'nx': int(rng.choice(np.arange(32, 193, 16))), 'target': float(rng.uniform(100, 4000)),
              'ds': 200.0, 'tolerance': 1e-10} for _ in range(args.batched)]
    solve_many(specs[:4])                      # plans and kernels warm
    for sp in {s['nx']: s for s in specs}.values():
        solve_instance(dict(sp, target=100.0))  # every grid shape's plan built before timing
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = solve_many(specs)
    torch.cuda.synchronize()
    t_conc = time.perf_counter() - t0
    t0 = time.perf_counter()
    for sp in specs:
        solve_instance(sp)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    print(json.dumps({'batched': args.batched, 'concurrent_s': t_conc, 'sequential_s': t_seq,
                      'max_fnorm': max(r['fnorm'] for r in res),
                      'unknowns': int(sum(3 * s['nx'] ** 2 for s in specs))}))


def learned(args):
    """The learned + mixed configuration against plain FP64 on one GPU.
    Training: one plain FP64 branch (Re 0 -> --train-target, ||F|| <= 1e-8)
    per training grid and seed, the seed drawing the initial step from
    [0.5, 1.5] x --ds; the learned predictor is trained on all their points
    (Adam, --train-rounds rounds of --train-steps steps per grid).  Timed:
    Newton at Re = 0 and the branch to --target at --nx/--nz, plain (secant
    predictor, FP64 factors) and learned (learned predictor, FP32 factors),
    each after a short warm-up branch on the same grid; every point at
    ||F|| <= 1e-8, the end points compared after Newton polishing at the
    target."""
    import torch
    from transiflow_gb300 import Continuation, Interface
    from transiflow_gb300.surrogate import LearnedPredictor, Recorder, Surrogate
    three_d = args.nz > 1

    def make(n, precision):
        return Interface({'CUDA': {'Factor Precision': precision, 'Tolerance': args.tol}},
                         n, n, n if three_d else 1)

    t0 = time.perf_counter()
    groups = []
    for n in [int(v) for v in args.train_grids.split(',')]:
        for seed in [int(v) for v in args.train_seeds.split(',')]:
            itf = make(n, 'fp64')
            rec = Recorder()
            cont = Continuation(itf, newton_tolerance=1e-8, quiet=True, predictor=rec.predictor, log=rec.log)
            itf.set_parameter('Reynolds Number', 0.0)
            x0 = cont.newton(itf.vector())
            ds = args.ds * float(np.random.default_rng(seed).uniform(0.5, 1.5))
            cont.continuation(x0, 'Reynolds Number', 0.0, args.train_target, ds)
            groups.append(((n, n, n if three_d else 1), rec.samples))
    branches_s = time.perf_counter() - t0
    net = Surrogate(4 if three_d else 3)
    net.fit_scales([smp for _, g in groups for smp in g])
    t1 = time.perf_counter()
    for r in range(args.train_rounds):
        for dims, g in groups:
            if g:
                net.train(g, dims, steps=args.train_steps, lr=2e-3, batch=4, seed=r)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1

    def branch(precision, predictor):
        itf = make(args.nx, precision)
        fn = []
        cont = Continuation(itf, newton_tolerance=1e-8, quiet=True, predictor=predictor,
                            log=lambda rec: fn.append(rec['fnorm']))
        itf.set_parameter('Reynolds Number', 0.0)
        cont.continuation(cont.newton(itf.vector()), 'Reynolds Number', 0.0, min(args.target, 2 * args.ds),
                          args.ds)                                  # warm-up: plans, graphs
        itf.set_parameter('Reynolds Number', 0.0)
        fn.clear()
        cont = Continuation(itf, newton_tolerance=1e-8, quiet=True, predictor=predictor,
                            log=lambda rec: fn.append(rec['fnorm']))
        torch.cuda.synchronize()
        t = time.perf_counter()
        x = cont.newton(itf.vector())
        x, mu = cont.continuation(x, 'Reynolds Number', 0.0, args.target, args.ds)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t
        itf.set_parameter('Reynolds Number', args.target)
        xp = Continuation(itf, quiet=True).newton(x, 1e-12).numpy()
        return wall, dict(cont.stats), max(f for f in fn if f is not None), xp

    plain_s, plain_stats, plain_f, xa = branch('fp64', None)
    learned_s, learned_stats, learned_f, xb = branch('fp32', LearnedPredictor(net))
    print(json.dumps({'learned': True, 'nx': args.nx, 'nz': args.nz, 'target_re': args.target, 'ds': args.ds,
                      'plain_fp64_s': plain_s, 'learned_mixed_s': learned_s, 'speedup': plain_s / learned_s,
                      'plain_stats': plain_stats, 'learned_stats': learned_stats,
                      'max_fnorm': max(plain_f, learned_f),
                      'end_point_rel_diff': float(np.linalg.norm(xb - xa) / np.linalg.norm(xa)),
                      'train_grids': args.train_grids, 'train_seeds': args.train_seeds,
                      'train_samples': sum(len(g) for _, g in groups), 'train_branches_s': branches_s,
                      'train_s': train_s, 'parameters': net.parameters()}))


def main():
    args = parse()
    if args.profile:
        profile_stage(args)
        return
    if args.batched:
        batched(args)
        return
    if args.learned:
        learned(args)
        return
    from transiflow_gb300 import dist
    rank, world, local = dist.init_from_env()
    try:
        if args.impl == 'reference':
            res = reference_arm(args, rank)
        else:
            res = gpu_arm(args, rank, world, local)
        if rank == 0 and res is not None:
            print(json.dumps(res), flush=True)
    finally:
        dist.finalize()


if __name__ == '__main__':
    main()
