"""Benchmark: seconds to reach the Reynolds-number target on one GB300,
learned predictor + mixed precision against the plain FP64 GPU backend.

Workload: 3D lid-driven cavity 64x64x64 (dof 4, 1,048,576 unknowns, lid on
top), Newton at Re = 0 from the zero state, then pseudo-arclength
continuation in the Reynolds number from 0 to 2000 with ds = 100, every
accepted point at ||F|| <= 1e-8.  Two arms on the same GPU:

  learned+mixed  the learned continuation predictor (three-point quadratic
                 extrapolation plus a residual from a 4-layer 3D CNN with 32
                 channels, BF16 weights, FP32 accumulation, used while it
                 clearly beats the secant predictor), FP32 multifrontal
                 factors with tensor-core trailing updates as the
                 preconditioner of FP64 flexible GMRES to 1e-10 (the
                 residual, the Newton update and the arclength scalars in
                 FP64).  One step = one complete branch; `value` is the mean
                 over the timed steps.
  plain FP64     the secant predictor and FP64 factors; run once per bench
                 invocation and reported beside the learned arm.

The predictor is trained before the timed region on the points of plain
continuations of 32^3 and 48^3 cavities (Re 0 -> 2500, one branch per seed
3..6 and grid, the seed drawing the branch's first step from [0.8, 1.2] x
--ds, later steps at most --train-ds), run with the mixed solver.  Inputs are synthetic (the zero
start state; no dataset).  The frontal matrices (77 GB in FP32) are far
larger than L2, so no flush is needed between steps.

  value      seconds per learned+mixed branch, start state already on the GPU
  e2e        the same steps through the public API: the start state copied
             from pinned host memory and the final state read back inside the
             timed region
  roofline   the dominant step of the learned+mixed branch, one FP32
             preconditioner application (HBM-bound), timed live, with the
             factorisation, the tensor-core update, the assembly and the SpMV
             beside it
  cpu_baseline  the oracle's CPU rhs / jacobian (a restatement of the
             reference's discretisation) on this host, sampled at 32^3 and
             scaled by the cell count, times the plain branch's call counts;
             the reference's SuperLU solve at 1,048,576 3D unknowns does not
             finish on a CPU, so this is a lower bound

``--impl reference`` times the reference algorithm's CPU implementation (the
oracle restatement: the reference package cannot travel to the GPU machine)
on the same workload, one bounded sample per step.  ``--workload ldc2d``
times the plain FP64 2D 256^2 branch (Re 0 -> 5000, ds = 200) instead.
"""

import argparse
import ctypes
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

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
    ap.add_argument('--workload', default='ldc3d', choices=['ldc3d', 'ldc2d'],
                    help='ldc3d: the headline learned+mixed vs plain FP64 comparison; ldc2d: the plain 2D branch')
    ap.add_argument('--nx', type=int, default=None, help='cells per direction (64 for ldc3d, 256 for ldc2d)')
    ap.add_argument('--target', type=float, default=None, help='Re at the branch end (2000 / 5000)')
    ap.add_argument('--ds', type=float, default=None, help='initial arclength step (100 / 200)')
    ap.add_argument('--tol', type=float, default=1e-10, help='FGMRES relative tolerance')
    ap.add_argument('--precision', default='fp64', choices=['fp64', 'fp32'], help='ldc2d: factor precision')
    ap.add_argument('--no-plain', action='store_true', help='ldc3d: skip the plain FP64 arm')
    ap.add_argument('--no-baseline', action='store_true')
    ap.add_argument('--train-grids', default='32,48', help='training grid sizes (cubes)')
    ap.add_argument('--train-seeds', default='3,4,5,6', help='one training branch per seed and grid')
    ap.add_argument('--train-target', type=float, default=2500.0, help='Re at the end of the training branches')
    ap.add_argument('--train-ds', type=float, default=50.0,
                    help='training branches: largest step (the first is drawn from [0.8, 1.2] x --ds)')
    ap.add_argument('--train-tol', type=float, default=1e-7, help='training branches: Newton tolerance on ||F||')
    ap.add_argument('--train-steps', type=int, default=150, help='Adam steps per grid and round')
    ap.add_argument('--train-rounds', type=int, default=4, help='rounds over the training grids')
    ap.add_argument('--reuse-its', type=int, default=None, help="'Reuse Iterations' (default: the backend's)")
    ap.add_argument('--reuse-drift', type=float, default=None, help="'Reuse Drift' (default: the backend's)")
    ap.add_argument('--no-tc', action='store_true', help='FP32 factors without tensor-core updates')
    ap.add_argument('--profile', default=None, choices=['factor', 'solve', 'assemble', 'tc', 'spmv', 'conv'],
                    help='run only a few launches of one stage (for ncu captures)')
    ap.add_argument('--nz', type=int, default=None, help='--profile: cells in z (1: the 2D grid)')
    ap.add_argument('--re', type=float, default=1000.0, help='Reynolds number of the --profile state')
    ap.add_argument('--batched', type=int, default=0,
                    help='time this many random lid-driven cavities (nx from 32..192, Re from [100, 4000], '
                         'seed 2) solved concurrently and one after the other, then exit')
    ap.add_argument('--leaf-cells', type=int, default=48, help='grid cells at which nested dissection stops')
    a = ap.parse_args()
    three = a.workload == 'ldc3d'
    a.nx = a.nx or (64 if three else 256)
    a.target = a.target or (2000.0 if three else 5000.0)
    a.ds = a.ds or (100.0 if three else 200.0)
    if a.nz is None:
        a.nz = a.nx if three else 1
    return a


# Factor reuse of the 3D workload (both arms): a 64^3 factorisation costs
# seconds (FP32) to a minute (FP64) against milliseconds per GMRES
# iteration, so a reused factorisation may take up to the restart length in
# iterations and the Jacobian may drift further before a refactorisation.
REUSE_3D = {'Reuse Iterations': 50, 'Reuse Drift': 0.2}


def solver_options(args, precision):
    o = {'Factor Precision': precision, 'Tolerance': args.tol, 'Leaf Cells': args.leaf_cells}
    if args.workload == 'ldc3d':
        o.update(REUSE_3D)
    if args.reuse_its is not None:
        o['Reuse Iterations'] = args.reuse_its
    if args.reuse_drift is not None:
        o['Reuse Drift'] = args.reuse_drift
    if args.no_tc:
        o['Tensor Cores'] = False
    return o


def config(args):
    n3 = args.nx * args.nx * args.nz
    if args.workload == 'ldc3d':
        n = 4 * n3
        return {'workload': '3D lid-driven cavity %dx%dx%d, dof 4 (%d unknowns), Newton at Re=0 then continuation '
                            'Re 0->%g, ds=%g, ||F||<=1e-8; timed: learned predictor + FP32/tensor-core factors '
                            'under FP64 FGMRES to %g; beside it once: secant predictor + FP64 factors'
                            % (args.nx, args.nx, args.nz, n, args.target, args.ds, args.tol),
                'nx': args.nx, 'ny': args.nx, 'nz': args.nz, 'dof': 4, 'unknowns': n, 'target_re': args.target,
                'ds': args.ds, 'newton_tolerance': 1e-8,
                'training': 'plain continuations at %s^3, Re 0->%g, seeds %s' % (args.train_grids, args.train_target,
                                                                                args.train_seeds),
                'l2': 'working set larger than L2 (77 GB of FP32 frontal matrices at 64^3)',
                'parallelism': 'replicas (one instance per GPU)'}
    n = 3 * n3
    return {'workload': '2D lid-driven cavity %dx%d, dof 3 (%d unknowns), Newton at Re=0 then continuation '
                        'Re 0->%g, ds=%g, ||F||<=1e-8, FP64 GMRES to %g + ND-LU (%s factors)'
                        % (args.nx, args.nx, n, args.target, args.ds, args.tol, args.precision),
            'nx': args.nx, 'ny': args.nx, 'nz': 1, 'dof': 3, 'unknowns': n, 'target_re': args.target,
            'ds': args.ds, 'newton_tolerance': 1e-8,
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
# headline: learned + mixed against plain FP64 (3D lid-driven cavity)
# ---------------------------------------------------------------------------
def _free():
    import torch
    gc.collect()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def _branch(itf, x0, args, predictor=None, log=None):
    from transiflow_gb300 import Continuation
    if predictor is not None:
        predictor.reset()       # a new branch: no history
    cont = Continuation(itf, newton_tolerance=1e-8, quiet=True, predictor=predictor, log=log)
    itf.set_parameter('Reynolds Number', 0.0)
    x = cont.newton(x0)
    x, mu = cont.continuation(x, 'Reynolds Number', 0.0, args.target, args.ds)
    return x, mu, cont


def _polish(itf, x, mu):
    """The branch end polished by Newton to ||F|| <= 1e-12 (outside any timed
    region), as a host array."""
    from transiflow_gb300 import Continuation
    itf.set_parameter('Reynolds Number', mu)
    return itf.array_from_vector(Continuation(itf, quiet=True).newton(x, 1e-12))


def train_predictor(args):
    """Plain continuations at the training grids (mixed solver), then the
    learned predictor trained on all of their points."""
    import torch
    from transiflow_gb300 import Continuation, Interface
    from transiflow_gb300.surrogate import Recorder, Surrogate, regular_steps
    t0 = time.perf_counter()
    groups = []
    stalls = []
    dropped = 0
    for n in [int(v) for v in args.train_grids.split(',')]:
        for seed in [int(v) for v in args.train_seeds.split(',')]:
            itf = Interface({'CUDA': solver_options(args, 'fp32')}, n, n, n)
            rec = Recorder()
            # training points need not meet the timed branch's 1e-8: near
            # Re 2300 at 32^3 ||F|| has a rounding floor of about 1e-8
            cont = Continuation(itf, newton_tolerance=args.train_tol, quiet=True, predictor=rec.predictor,
                                log=rec.log)
            itf.set_parameter('Reynolds Number', 0.0)
            x0 = cont.newton(itf.vector(), args.train_tol)
            # first step near the bench's own (a first step of a few tens from
            # Re = 0 lands where the reference's Re = 0 -> 1 viscosity
            # substitution makes the secant tangent useless), later steps at
            # most --train-ds so that the branch yields many regular points
            # (with the timed branch's own step rule, up to 1000, the 32^3 and
            # 48^3 branches left 15 steps the three-point history describes)
            ds = args.ds * float(np.random.default_rng(seed).uniform(0.8, 1.2))
            try:
                cont.continuation(x0, 'Reynolds Number', 0.0, args.train_target, ds, ds_max=args.train_ds)
            except Exception as e:
                # a singular point before the target (on the 32^3 branch near
                # Re 2338 the corrector cannot converge at any step size):
                # the branch ends there, its points so far are kept
                if 'stalled' not in str(e):
                    raise
                stalls.append((n, seed, float(itf.get_parameter('Reynolds Number'))))
            # regular steps only: near a singular point the accepted steps
            # shrink to ~0.01; the first steps from Re = 0 (the reference's
            # Re = 0 -> 1 viscosity substitution) and other steps the
            # three-point history does not describe are dropped by
            # regular_steps
            kept = regular_steps([smp for smp in rec.samples
                                  if smp['ds'] >= 0.25 * args.train_ds and (smp['its'] or 0) >= 1])
            dropped += len(rec.samples) - len(kept)
            groups.append(((n, n, n), kept))
            del itf, cont, x0
            _free()
    branches_s = time.perf_counter() - t0
    net = Surrogate(4)
    net.fit_scales([smp for _, g in groups for smp in g])
    t1 = time.perf_counter()
    losses = []
    for r in range(args.train_rounds):
        for dims, g in groups:
            if g:
                losses.append(float(net.train(g, dims, steps=args.train_steps, lr=2e-3, batch=4, seed=r)[-1]))
    # the step-size proposal: the network's error relative to the secant
    # predictor and the secant error plain steps handled comfortably
    step_model = net.calibrate_steps([(dims, g) for dims, g in groups if g])
    torch.cuda.synchronize()
    info = {'branches': len(groups), 'points': sum(len(g) for _, g in groups), 'branches_s': branches_s,
            'step_model': step_model,
            'ended_at_singular_point': stalls, 'irregular_points_dropped': dropped,
            'train_s': time.perf_counter() - t1, 'adam_steps': args.train_rounds * args.train_steps * len(groups),
            'final_loss': losses[-1] if losses else None, 'parameters': net.parameters()}
    return net, info


def plain_arm(args):
    """The plain FP64 GPU backend on the same branch, once: secant
    predictor, FP64 factors (after one warm-up factorisation that builds the
    plan and the buffers)."""
    import torch
    from transiflow_gb300 import Interface
    itf = Interface({'CUDA': solver_options(args, 'fp64')}, args.nx, args.nx, args.nz)
    x0 = itf.vector()
    itf.set_parameter('Reynolds Number', 0.0)
    itf.solve(itf.jacobian(x0), itf.rhs(x0))
    torch.cuda.synchronize()
    s0 = dict(itf.solver.stats)
    log = []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    x, mu, cont = _branch(itf, itf.vector(), args, log=log.append)
    ev[1].record()
    torch.cuda.synchronize()
    t = ev[0].elapsed_time(ev[1]) / 1000.0
    s1 = itf.solver.stats
    out = {'value': t, 'unit': 's', 'points': cont.stats['points'], 'rhs': cont.stats['rhs'],
           'jacobian': cont.stats['jacobian'], 'solve': cont.stats['solve'],
           'factorizations': s1['factorizations'] - s0['factorizations'],
           'gmres_iterations': s1['gmres_iterations'] - s0['gmres_iterations'],
           'max_fnorm': max(r['fnorm'] for r in log if r['fnorm'] is not None),
           'mus': [r['mu'] for r in log], 'final_re': mu}
    xe = _polish(itf, x, mu)
    del itf, x, x0, cont
    _free()
    return out, xe


def learned_arm(args, net, rank, local):
    """W warm-up and K timed learned+mixed branches, each from the zero state
    copied from pinned host memory, the final state read back."""
    import torch
    from transiflow_gb300 import Interface, _lib, dist
    from transiflow_gb300.surrogate import LearnedPredictor
    lib = _lib.load()
    itf = Interface({'CUDA': solver_options(args, 'fp32')}, args.nx, args.nx, args.nz)
    pred = LearnedPredictor(net)
    n = itf.n
    host0 = torch.zeros(n, dtype=torch.float64).pin_memory()
    for _ in range(args.warmup):
        x, mu, cont = _branch(itf, itf.vector_from_array(host0.numpy()), args, pred)
        itf.array_from_vector(x)
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    l0 = lib.tf_launch_count()
    s0 = dict(itf.solver.stats)
    t_dev, t_e2e, logs = [], [], []
    for _ in range(args.steps):
        log = []
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        x0 = itf.vector_from_array(host0.numpy())
        ev0.record(stream)
        x, mu, cont = _branch(itf, x0, args, pred, log=log.append)
        ev1.record(stream)
        xh = itf.array_from_vector(x)
        torch.cuda.synchronize()
        t_e2e.append(time.perf_counter() - w0)
        t_dev.append(ev0.elapsed_time(ev1) / 1000.0)
        logs.append(log)
    launches = lib.tf_launch_count() - l0 + itf.solver.stats['graph_kernel_launches'] - s0['graph_kernel_launches']
    dist.barrier()
    clk = clocks.stop()
    s1 = itf.solver.stats
    per = {k: (s1[k] - s0[k]) / args.steps for k in ('factorizations', 'solves', 'gmres_iterations', 'reused',
                                                      'refactored_after_reuse')}
    fn = [r['fnorm'] for log in logs for r in log if r['fnorm'] is not None]
    out = {'t_dev': dist.max_over_ranks(statistics.mean(t_dev)), 't_e2e': dist.max_over_ranks(statistics.mean(t_e2e)),
           'launches': int(launches), 'clocks': clk, 'max_fnorm': max(fn), 'final_re': mu,
           'branch': {'points': cont.stats['points'], 'rhs': cont.stats['rhs'], 'jacobian': cont.stats['jacobian'],
                      'solve': cont.stats['solve'], 'learned_accepted': cont.stats['learned_accepted'],
                      'learned_rejected': cont.stats['learned_rejected'], 'per_step_solver': per,
                      'steps_proposed': pred.steps_proposed, 'learned_used': pred.used,
                      'learned_over_secant_error': [round(r, 4) for r in pred.ratios],
                      'mus': [r['mu'] for r in logs[-1]], 'step_s': t_dev}}
    out['end_state'] = _polish(itf, x, mu)
    return out, itf


def headline_arm(args, rank, world, local):
    """The learned+mixed arm timed per step, the plain FP64 arm once, the
    predictor trained first."""
    import torch
    from transiflow_gb300 import dist
    torch.cuda.set_device(local)
    net, training = train_predictor(args)
    plain, xp = (None, None) if args.no_plain else plain_arm(args)
    res, itf = learned_arm(args, net, rank, local)
    t_step, e2e = res['t_dev'], res['t_e2e']
    n = itf.n
    roof = roofline_3d(itf, args)
    xl = res.pop('end_state')
    diff = float(np.linalg.norm(xl - xp) / np.linalg.norm(xp)) if xp is not None else None
    max_fn = max(res['max_fnorm'], plain['max_fnorm'] if plain else 0.0)
    ok = max_fn <= 1e-8 and (diff is None or diff <= 1e-8)
    result = {'metric': METRIC, 'value': t_step, 'unit': 's', 'n_gpus': world, 'steps': args.steps,
              'warmup': args.warmup, 'ms_per_step': t_step * 1000.0, 'higher_is_better': False,
              'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64+f32 (split-TF32 tensor-core factor updates)',
              'data': 'synthetic (zero initial state; no dataset)', 'config': config(args),
              'e2e': {'value': e2e, 'unit': 's', 'h2d_bytes_per_step': 8 * n, 'd2h_bytes_per_step': 8 * n},
              'roofline': roof, 'clocks': res['clocks'], 'gpu_launches': res['launches'],
              'status': 'ok' if ok else 'failed: ||F|| %.3e, end-point difference %s' % (max_fn, diff),
              'plain_fp64': plain, 'speedup_vs_plain_fp64': (plain['value'] / t_step) if plain else None,
              'end_point_rel_diff_vs_plain': diff, 'max_fnorm': max_fn,
              'learned_mixed': res['branch'], 'training': training}
    if rank == 0 and not args.no_baseline:
        result['cpu_baseline'] = cpu_baseline_3d(args, plain or res['branch'])
    return result


def _peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), float(p['bf16_tflops']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, 'fallback'


def _timed(fn, count):
    import torch
    st = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for i in range(count):
        fn(i)
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0 / count


def _bandwidth_kernels(itf, reps=4):
    """Fused assembly and FP64 SpMV timed over `reps` rotating buffer sets
    (each larger than half of L2 at 64^3 and 256^2, together larger than L2)."""
    import torch
    from transiflow_gb300 import _lib
    from transiflow_gb300.vector import _stream
    lib = _lib.load()
    n, nnz = itf.n, itf.pattern.nnz
    prob = itf._problem()
    gen = torch.Generator(device=itf.device).manual_seed(1)
    states = [0.1 * torch.randn(n, dtype=torch.float64, device=itf.device, generator=gen) for _ in range(reps)]
    rhs = [torch.empty(n, dtype=torch.float64, device=itf.device) for _ in range(reps)]
    jv = [torch.empty(nnz, dtype=torch.float64, device=itf.device) for _ in range(reps)]

    def asm(i):
        lib.tf_assemble(ctypes.byref(prob), states[i % reps].data_ptr(), rhs[i % reps].data_ptr(),
                        jv[i % reps].data_ptr(), _stream())

    _timed(asm, reps)
    t_asm = _timed(asm, 20)
    rp, cp = itf.pattern.rowptr, itf.pattern.cols

    def spmv(i):
        lib.tf_spmv_f64(n, rp.data_ptr(), cp.data_ptr(), jv[i % reps].data_ptr(), states[i % reps].data_ptr(),
                        rhs[(i + 1) % reps].data_ptr(), 1.0, 0.0, _stream())

    _timed(spmv, reps)
    t_spmv = _timed(spmv, 20)
    hbm = _peaks()[0]
    b_asm = 16 * n + 8 * nnz
    b_spmv = 12 * nnz + 4 * (n + 1) + 16 * n
    return states[0], {
        'tf_assemble (F + J, fused)': {'s_per_launch': t_asm, 'bytes': b_asm, 'GB/s': b_asm / t_asm / 1e9,
                                       'frac_hbm': b_asm / t_asm / 1e9 / hbm},
        'tf_spmv_f64': {'s_per_launch': t_spmv, 'bytes': b_spmv, 'GB/s': b_spmv / t_spmv / 1e9,
                        'frac_hbm': b_spmv / t_spmv / 1e9 / hbm}}


# DRAM bytes (read + write) of the roofline unit -- one FP32 preconditioner
# application, summed over its apply_kernel launches -- keyed by (nx, nz).
# 64^3 is too large for a multi-metric capture: the ratio of DRAM traffic to
# algorithmic factor bytes measured over a whole sweep at 32^3 (1.0717:
# 698.9 MB for 652.3 MB, profiles/apply_kernel_ldc3d32.md) scaled to the
# 22.951 GB a 64^3 application streams.  Large fronts dominate at 64^3 and
# have the lowest ratios, so this is an upper estimate.
ROOF_TRAFFIC = {(64, 64): 1.0717 * 22.951191352e9}


def application_bytes(plan):
    """Factor bytes one FP32 application reads: per front the strict lower
    and the upper own triangle (n^2 in all) and L21 and U12 (2 n (f - n))."""
    p = plan.host
    n = p.n_own.astype(np.float64)
    f = p.f.astype(np.float64)
    return 4.0 * float(np.sum(n * n + 2.0 * n * (f - n)))


def roofline_3d(itf, args):
    """Live CUDA-event timings at the bench grid.  The roofline unit is the
    dominant step of the timed branch, one FP32 preconditioner application
    (apply_kernel, four launches per tree height, replayed from a CUDA
    graph): HBM-bound, the factor bytes it streams over its event-timed
    duration.  Beside it: the fused assembly, the SpMV, one factorisation and
    the tensor-core trailing update (tc_update_kernel) alone -- one launch at
    k0 = 0 over the tree height with the widest fronts, timed on the plan's
    own front buffer (which is scribbled on, so the factorisation is dropped
    afterwards)."""
    import torch
    from transiflow_gb300 import _lib
    from transiflow_gb300.vector import DeviceVector
    lib = _lib.load()
    hbm, bf16, which = _peaks()
    x, kernels = _bandwidth_kernels(itf)
    solver = itf.solver
    J = itf.jacobian(DeviceVector(x))
    fac = solver.factorization(J)
    torch.cuda.synchronize()
    t_fac = []
    for _ in range(2):
        J.lu = None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fac = solver.factorization(J)
        e1.record()
        torch.cuda.synchronize()
        t_fac.append(e0.elapsed_time(e1) / 1000.0)
    v = torch.ones(itf.n, dtype=torch.float64, device=itf.device)
    t_app = _timed(lambda i: fac.apply(v), 5)
    plan = solver.plan
    kernels['tf_nd_factor_inv_f32 (one factorisation, graph)'] = {
        's_per_call': min(t_fac), 'flops': plan.flops, 'TFLOP/s': plan.flops / min(t_fac) / 1e12}
    kernels['tf_nd_solve_inv_f32 (one preconditioner application, graph)'] = {'s_per_call': t_app}
    # the tensor-core update alone
    p = plan.host
    h = int(np.argmax(plan.max_f))
    nodes = p.levels[h]
    E = np.minimum(256, p.n_own[nodes]).astype(np.float64)
    rest = p.f[nodes].astype(np.float64) - E
    flops = float(np.sum(2.0 * E * rest * rest))
    c_bytes = float(np.sum(8.0 * rest * rest))
    eng = solver._engine('fp32')
    fronts, _ = solver._fronts_raw('fp32')
    sp = ctypes.cast(ctypes.pointer(eng.struct), ctypes.c_void_p)
    st = torch.cuda.current_stream().cuda_stream

    def tc(i):
        _lib.check(lib.tf_nd_tc_update_f32(sp, h, 0, solver.tc_terms, fronts.data_ptr(), solver.info.data_ptr(),
                                           ctypes.c_void_p(st)), 'tf_nd_tc_update_f32')

    tc(0)
    t_tc = _timed(tc, 5)
    solver._owner.pop('fp32', None)       # the fronts no longer hold a factorisation
    tc_rate = flops / t_tc / 1e12
    tf32 = bf16 / 2.0
    kernels['tc_update_kernel (alone)'] = {
        'what': 'tcgen05 rank-256 trailing update of the FP32 fronts, tree height %d (%d fronts), %.1f GFLOP'
                % (h, len(nodes), flops / 1e9),
        's_per_launch': t_tc, 'flops': flops, 'TFLOP/s': tc_rate, 'frac_tf32': tc_rate / tf32,
        'tf32_peak_source': 'half the measured BF16 dense rate (%s: MEASURED_PEAKS.json bf16_tflops %.1f); '
                            'split-TF32 issues %d tensor products per algorithmic one' % (which, bf16,
                                                                                          solver.tc_terms),
        'front_rw_bytes': c_bytes, 'GB/s': c_bytes / t_tc / 1e9}
    a_bytes = application_bytes(plan)
    achieved = a_bytes / t_app / 1e9
    return {'bound': 'hbm',
            'kernel': 'one FP32 preconditioner application: apply_kernel<float, 0..3>, four launches per tree '
                      'height (%d heights), %dx%dx%d, %.2f GB of factors streamed'
                      % (len(plan.host.levels), args.nx, args.nx, args.nz, a_bytes / 1e9),
            'achieved': achieved, 'peak': hbm, 'unit': 'GB/s', 'frac': achieved / hbm,
            'peak_source': '%s (MEASURED_PEAKS.json hbm_gbs, a copy timed alone)' % which,
            'traffic': ROOF_TRAFFIC.get((args.nx, args.nz)),
            'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum over the apply_kernel launches of '
                              'a backward sweep at 32^3 (1.0717 x its algorithmic bytes), scaled to this '
                              "application's algorithmic bytes (profiles/apply_kernel_ldc3d32.md)",
            'algorithmic_bytes': a_bytes, 's_per_application': t_app,
            'kernels': kernels}


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
# `bench.py --workload ldc2d --profile factor` on a GB300.
FACTOR_TRAFFIC = {(256, 1, 'fp64'): 6.353e9}


def roofline_2d(itf, x, args):
    """The 2D plain workload: the FP64 factorisation against this GPU's FP64
    GEMM rate (its trailing updates run on the FP64 pipe)."""
    import torch
    _, kernels = _bandwidth_kernels(itf)
    J = itf.jacobian(itf.vector_from_array(x.numpy()))
    fac = itf.solver.factorization(J)
    torch.cuda.synchronize()
    f_time = []
    for _ in range(3):
        J.lu = None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fac = itf.solver.factorization(J)
        e1.record()
        torch.cuda.synchronize()
        f_time.append(e0.elapsed_time(e1) / 1000.0)
    t_fac = min(f_time)
    v = torch.ones(itf.n, dtype=torch.float64, device=itf.device)
    t_sol = _timed(lambda i: fac.apply(v), 10)
    hbm, _, which = _peaks()
    flops = itf.solver.plan.flops
    f64 = fp64_peak()
    kernels['tf_nd_factor (%s)' % args.precision] = {'s_per_call': t_fac, 'flops': flops,
                                                      'TFLOP/s': flops / t_fac / 1e12}
    kernels['tf_nd_solve (%s)' % args.precision] = {'s_per_call': t_sol}
    a = flops / t_fac / 1e12
    return {'bound': 'fp64-pipe', 'kernel': 'tf_nd_factor_%s: multifrontal LU graph (%dx%d, %.2f GFLOP per launch)'
            % (args.precision, args.nx, args.nx, flops / 1e9),
            'achieved': a, 'peak': f64 if args.precision == 'fp64' else None, 'unit': 'TFLOP/s',
            'frac': a / f64 if args.precision == 'fp64' else None,
            'peak_source': 'FP64 dense GEMM of this GPU measured in this run (cuBLAS DGEMM 4096^3); the FP64 '
                           'factorisation runs on the FP64 pipe, not the tensor cores',
            'traffic': FACTOR_TRAFFIC.get((args.nx, args.nz, args.precision)),
            'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum over the launches of one '
                              'factorisation (caches flushed per kernel: an upper bound)',
            'algorithmic_flops': flops, 'hbm_peak_gbs': hbm,
            'hbm_peak_source': '%s (MEASURED_PEAKS.json hbm_gbs)' % which, 'kernels': kernels}


# ---------------------------------------------------------------------------
# the plain 2D workload
# ---------------------------------------------------------------------------
def plain2d_arm(args, rank, world, local):
    import torch
    from transiflow_gb300 import Interface, _lib, dist
    torch.cuda.set_device(local)
    lib = _lib.load()
    itf = Interface({'CUDA': solver_options(args, args.precision)}, args.nx, args.nx, 1)
    n = itf.n
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        x, mu, cont = _branch(itf, itf.vector(), args)
    calls = dict(cont.stats)
    fac0 = itf.solver.stats['factorizations']
    x, mu, cont = _branch(itf, itf.vector(), args)
    calls['factorizations'] = itf.solver.stats['factorizations'] - fac0
    itf.set_parameter('Reynolds Number', mu)
    fnorm_end = itf.rhs(x).norm()
    host0 = torch.zeros(n, dtype=torch.float64).pin_memory()
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    l0 = lib.tf_launch_count()
    s0 = dict(itf.solver.stats)
    t_dev, t_e2e = [], []
    for _ in range(args.steps):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        x0 = itf.vector_from_array(host0.numpy())
        ev0.record(stream)
        x, mu, _ = _branch(itf, x0, args)
        ev1.record(stream)
        itf.array_from_vector(x)
        torch.cuda.synchronize()
        t_e2e.append(time.perf_counter() - w0)
        t_dev.append(ev0.elapsed_time(ev1) / 1000.0)
    launches = lib.tf_launch_count() - l0 + itf.solver.stats['graph_kernel_launches'] - s0['graph_kernel_launches']
    s1 = itf.solver.stats
    per = {k: (s1[k] - s0[k]) / args.steps for k in ('factorizations', 'solves', 'gmres_iterations', 'reused',
                                                      'refactored_after_reuse')}
    dist.barrier()
    clk = clocks.stop()
    t_step = dist.max_over_ranks(statistics.mean(t_dev))
    e2e = dist.max_over_ranks(statistics.mean(t_e2e))
    roof = roofline_2d(itf, x, args)
    result = {'metric': METRIC, 'value': t_step, 'unit': 's', 'n_gpus': world, 'steps': args.steps,
              'warmup': args.warmup, 'ms_per_step': t_step * 1000.0, 'higher_is_better': False,
              'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64' if args.precision == 'fp64' else 'f64+f32',
              'data': 'synthetic (zero initial state; no dataset)', 'config': config(args),
              'e2e': {'value': e2e, 'unit': 's', 'h2d_bytes_per_step': 8 * n, 'd2h_bytes_per_step': 8 * n},
              'roofline': roof, 'clocks': clk, 'gpu_launches': int(launches),
              'branch': {'points': calls.get('points'), 'rhs': calls.get('rhs'), 'jacobian': calls.get('jacobian'),
                         'solve': calls.get('solve'), 'factorizations': calls.get('factorizations'),
                         'final_re': mu, 'final_fnorm': fnorm_end, 'per_step_solver': per,
                         'newton_steps_per_s': (calls.get('jacobian') or 0) / t_step}}
    if rank == 0 and not args.no_baseline:
        result['cpu_baseline'] = cpu_baseline_2d(args, calls)
    return result


# ---------------------------------------------------------------------------
# CPU oracle timings (the reference algorithm on this host's cores)
# ---------------------------------------------------------------------------
def oracle_sample(nx, nz=1, solve=True, seed=1):
    from oracle.solve import Interface as OracleInterface
    itf = OracleInterface({'Reynolds Number': 1000}, nx, nx, nz)
    s = 0.1 * np.random.default_rng(seed).standard_normal(itf.vector().size)
    t = {}
    t0 = time.perf_counter()
    f = itf.rhs(s)
    t['rhs'] = time.perf_counter() - t0
    t0 = time.perf_counter()
    J = itf.jacobian(s)
    t['jacobian'] = time.perf_counter() - t0
    if solve:
        t0 = time.perf_counter()
        itf.solve(J, f)
        t['factor_solve'] = time.perf_counter() - t0
        t0 = time.perf_counter()
        itf.solve(J, f)
        t['solve'] = time.perf_counter() - t0
    return t


def extrapolate_2d(t, calls):
    """Seconds of the reference's SciPy path for these call counts: one
    SuperLU factorisation per Jacobian (SciPy.py:151, cached on the matrix)."""
    nfac = calls['jacobian']
    return (calls['rhs'] * t['rhs'] + calls['jacobian'] * t['jacobian'] + nfac * t['factor_solve']
            + max(calls['solve'] - nfac, 0) * t['solve'])


def cpu_baseline_2d(args, calls):
    t = oracle_sample(args.nx)
    return {'value': extrapolate_2d(t, calls), 'unit': 's', 'cores': 1, 'kind': 'port',
            'sample': 'oracle (vectorised NumPy restatement of Discretization + SciPy SuperLU, single-threaded '
                      'splu) at %dx%d: 1 rhs %.2fs, 1 jacobian %.2fs, 1 factor+solve %.2fs, 1 solve %.2fs, scaled '
                      'by the branch call counts %s (one factorisation per jacobian)'
                      % (args.nx, args.nx, t['rhs'], t['jacobian'], t['factor_solve'], t['solve'],
                         {k: calls[k] for k in ('rhs', 'jacobian', 'solve')}),
            'host_cpus': os.cpu_count()}


# the oracle's rhs / jacobian scale with the cell count: they are sampled
# on the 32^3 grid and scaled to the bench grid
SAMPLE_3D = 32


def extrapolate_3d(t, calls, args):
    scale = args.nx * args.nx * args.nz / float(SAMPLE_3D ** 3)
    return (calls['rhs'] * t['rhs'] + calls['jacobian'] * t['jacobian']) * scale


def cpu_baseline_3d(args, calls):
    t = oracle_sample(SAMPLE_3D, SAMPLE_3D, solve=False)
    return {'value': extrapolate_3d(t, calls, args), 'unit': 's', 'cores': 1, 'kind': 'port',
            'sample': 'oracle (vectorised NumPy restatement of Discretization) at %d^3: 1 rhs %.2fs, 1 jacobian '
                      '%.2fs, scaled by the cell count to %dx%dx%d and by the plain branch call counts '
                      '(rhs %d, jacobian %d); the solves are left out: SuperLU on 1,048,576 3D unknowns does not '
                      'finish on a CPU, so this is a lower bound' % (SAMPLE_3D, t['rhs'], t['jacobian'], args.nx,
                                                                    args.nx, args.nz, calls['rhs'], calls['jacobian']),
            'host_cpus': os.cpu_count()}


# Interface calls of the reference-equivalent branches: 2D 256^2 (Re 0 ->
# 5000, ds = 200) as the reference's Continuation makes them on an exact
# solver (the SciPy interface factors every Jacobian once), and the plain
# 3D 64^3 branch (Re 0 -> 2000, ds = 100) as measured on the GPU.
BRANCH_CALLS_256 = {'rhs': 111, 'jacobian': 47, 'solve': 92, 'factorizations': 47}
BRANCH_CALLS_64 = {'rhs': 85, 'jacobian': 36, 'solve': 70}


def reference_arm(args, rank):
    if rank != 0:
        return None
    three = args.workload == 'ldc3d'
    if three:
        calls = dict(BRANCH_CALLS_64)
        if args.nx != 64 or args.nz != 64:
            return {'impl': 'reference', 'unavailable': 'branch call counts are known for the 64^3 branch only'}
        sample = lambda: extrapolate_3d(oracle_sample(SAMPLE_3D, SAMPLE_3D, solve=False), calls, args)
        text = ('per step one rhs and one jacobian of the oracle at %d^3 on this host, scaled by the cell count to '
                '64^3 and by the branch call counts %s; SuperLU solves at 1,048,576 3D unknowns do not finish on a '
                'CPU and are left out, so the value is a lower bound' % (SAMPLE_3D, calls))
    else:
        calls = dict(BRANCH_CALLS_256)
        if args.nx != 256:
            return {'impl': 'reference', 'unavailable': 'branch call counts are known for the 256x256 branch only'}
        sample = lambda: extrapolate_2d(oracle_sample(args.nx), calls)
        text = ('per step one rhs, one jacobian, one SuperLU factor+solve and one solve of the oracle at %dx%d on '
                'this host, scaled by the branch call counts %s' % (args.nx, args.nx, calls))
    for _ in range(args.warmup):
        sample()
    v = statistics.mean([sample() for _ in range(args.steps)])
    return {'metric': METRIC, 'value': v, 'unit': 's', 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': v * 1000.0, 'higher_is_better': False, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference', 'config': config(args),
            'cpu_baseline': {'value': v, 'unit': 's', 'cores': 1, 'kind': 'port', 'sample': text},
            'e2e': {'value': v, 'unit': 's', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}


def profile_stage(args):
    """A short, fixed sequence of one stage for profiler captures: the
    Jacobian of a random state (Re from --re, 2D unless --nz > 1), then 3
    factorisations, 3 preconditioner applications or 3 fused assemblies,
    each timed with CUDA events on the launching stream."""
    import torch
    from transiflow_gb300 import Interface
    opts = solver_options(args, args.precision)
    opts['CUDA Graphs'] = False
    p = {'Reynolds Number': args.re, 'CUDA': opts}
    itf = Interface(p, args.nx, args.nx, args.nz)
    s = 0.1 * np.random.default_rng(1).standard_normal(itf.n)
    x = itf.vector_from_array(s)
    J = itf.jacobian(x)
    fac, first = None, None
    if args.profile in ('factor', 'solve', 'tc'):
        # only these stages hold the frontal matrices on the device
        t0 = time.perf_counter()
        fac = itf.solver.factorization(J)
        torch.cuda.synchronize()
        first = time.perf_counter() - t0
    st = torch.cuda.current_stream()
    times = []
    if args.profile in ('spmv', 'conv'):
        from transiflow_gb300 import _lib
        from transiflow_gb300.vector import _stream
        lib = _lib.load()
        if args.profile == 'spmv':
            rp, cp = itf.pattern.rowptr, itf.pattern.cols
            y = torch.empty_like(x.data)

            def run():
                _lib.check(lib.tf_spmv_f64(itf.n, rp.data_ptr(), cp.data_ptr(), J.values.data_ptr(),
                                           x.data.data_ptr(), y.data_ptr(), 1.0, 0.0, _stream()), 'tf_spmv_f64')
        else:
            # one forward pass of the learned predictor's network on this grid
            from transiflow_gb300.surrogate import Surrogate
            net = Surrogate(itf.dof)
            net.fit_scales([{'x0': x.data, 't': x.data, 'x1': x.data, 'mu': 1.0, 'ds': 1.0}])
            dims = (itf.nx, itf.ny, itf.nz)

            def run():
                net.predict(x.data, x.data, 1.0, 1.0, dims)
        run()
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            run()
            e1.record(st)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
        print(json.dumps({'profile': args.profile, 'nx': args.nx, 'nz': args.nz, 's_per_call': times}))
        return
    if args.profile == 'tc':
        # the tensor-core update alone on the widest height (scribbles on the
        # fronts; nothing is solved afterwards)
        from transiflow_gb300 import _lib
        lib = _lib.load()
        plan = itf.solver.plan
        h = int(np.argmax(plan.max_f))
        eng = itf.solver._engine(args.precision)
        fronts, _ = itf.solver._fronts_raw(args.precision)
        sp = ctypes.cast(ctypes.pointer(eng.struct), ctypes.c_void_p)
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            _lib.check(lib.tf_nd_tc_update_f32(sp, h, 0, itf.solver.tc_terms, fronts.data_ptr(),
                                               itf.solver.info.data_ptr(), ctypes.c_void_p(st.cuda_stream)),
                       'tf_nd_tc_update_f32')
            e1.record(st)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
        print(json.dumps({'profile': 'tc', 'nx': args.nx, 'nz': args.nz, 'height': h, 's_per_call': times}))
        return
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
    out = {'profile': args.profile, 'nx': args.nx, 'nz': args.nz, 'unknowns': itf.n, 'precision': args.precision,
           's_per_call': times}
    plan = itf.solver.plan
    if plan is not None:
        out.update({'first_factor_s': first, 'factor_gflop': plan.flops / 1e9,
                    'front_gb': plan.front_elems * (8 if args.precision == 'fp64' else 4) / 1e9})
        eng = itf.solver._engines.get(args.precision)
        if eng is not None:
            out['apply_waves'] = int(eng.struct.apply_waves)
    print(json.dumps(out))


def batched(args):
    """The batched configuration: many independent lid-driven cavities of
    uneven size and Reynolds number, each by Newton at Re = 0 and continuation
    to its Re with ||F|| <= 1e-10, solved concurrently (one stream per
    instance) and one after the other on the same GPU.  Under torchrun the
    instances are sharded over the ranks (one GPU each, largest first to the
    least loaded rank) and the results gathered on every rank; the time is
    the slowest rank's."""
    import torch
    from transiflow_gb300 import dist
    from transiflow_gb300.batch import shard, solve_instance, solve_many, solve_sharded
    rank, world, local = dist.init_from_env()
    torch.cuda.set_device(local)
    try:
        rng = np.random.default_rng(2)
        specs = [{'nx': int(rng.choice(np.arange(32, 193, 16))), 'target': float(rng.uniform(100, 4000)),
                  'ds': 200.0, 'tolerance': 1e-10} for _ in range(args.batched)]
        mine = [specs[i] for i in shard(specs, world, rank)]
        solve_many(mine[:4])                       # plans and kernels warm
        for sp in {s['nx']: s for s in mine}.values():
            solve_instance(dict(sp, target=100.0))  # every grid shape's plan built before timing
        torch.cuda.synchronize()
        dist.barrier()
        t0 = time.perf_counter()
        res = solve_sharded(specs)
        torch.cuda.synchronize()
        t_conc = dist.max_over_ranks(time.perf_counter() - t0)
        out = {'batched': args.batched, 'n_gpus': world, 'concurrent_s': t_conc,
               'instances_per_rank': [len(shard(specs, world, r)) for r in range(world)],
               'max_fnorm': max(r['fnorm'] for r in res),
               'unknowns': int(sum(3 * s['nx'] ** 2 for s in specs))}
        if world == 1:
            t0 = time.perf_counter()
            for sp in specs:
                solve_instance(sp)
            torch.cuda.synchronize()
            out['sequential_s'] = time.perf_counter() - t0
        if rank == 0:
            print(json.dumps(out))
    finally:
        dist.finalize()


def main():
    args = parse()
    if args.profile:
        profile_stage(args)
        return
    if args.batched:
        batched(args)
        return
    from transiflow_gb300 import dist
    rank, world, local = dist.init_from_env()
    try:
        if args.impl == 'reference':
            res = reference_arm(args, rank)
        elif args.workload == 'ldc3d':
            res = headline_arm(args, rank, world, local)
        else:
            res = plain2d_arm(args, rank, world, local)
        if rank == 0 and res is not None:
            print(json.dumps(res), flush=True)
    finally:
        dist.finalize()


if __name__ == '__main__':
    main()
