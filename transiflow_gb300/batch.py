"""Many independent instances on one GPU.

The batched configuration of the hot path solves many unrelated problems --
for example lid-driven cavities with nx = ny drawn from {32, 48, ..., 192}
and Reynolds numbers drawn from [100, 4000] -- each to its own tolerance.
The instances share nothing but the device, so ``solve_many`` drives each
one from its own host thread on its own CUDA stream: Newton at the start
value of the parameter, then pseudo-arclength continuation to the instance's
target, exactly as a single instance would run (``Continuation.newton`` and
``Continuation.continuation``).  The kernels of small instances, which leave
most SMs idle on their own, overlap on the GPU; every libtfcuda call is
stream-ordered and the host synchronisations of one instance wait only for
its own stream.  Elimination plans are shared between instances of the same
grid shape.

Across GPUs the instances are sharded, not replicated: ``shard`` assigns
each instance to one rank (largest estimated cost first, to the least loaded
rank; the same on every rank, no communication), ``solve_sharded`` solves a
rank's share with ``solve_many`` and gathers every result on every rank in
the order of the specs -- the only exchange between ranks.
"""

import threading

import torch

from . import _lib, dist

from .continuation import Continuation
from .interface import Interface


def solve_instance(spec, stream=None):
    """Solve one instance described by ``spec`` (a dict):

    ``nx``, ``ny`` (default nx), ``nz`` (default 1), ``parameters`` (the
    interface parameters, default {}), ``name`` (the continuation parameter,
    default 'Reynolds Number'), ``start`` (default 0), ``target``, ``ds``
    (initial step, default 100), ``tolerance`` (Newton, default 1e-10).

    Returns a dict with the final state (NumPy), parameter value, ||F|| and
    the interface call counts."""
    stream = stream or torch.cuda.current_stream()
    with torch.cuda.stream(stream):
        params = dict(spec.get('parameters', {}))
        name = spec.get('name', 'Reynolds Number')
        start = float(spec.get('start', 0.0))
        target = float(spec['target'])
        tol = float(spec.get('tolerance', 1e-10))
        params[name] = start
        itf = Interface(params, spec['nx'], spec.get('ny', spec['nx']), spec.get('nz', 1))
        cont = Continuation(itf, newton_tolerance=tol, quiet=True)
        x = cont.newton(itf.vector(), tol=tol)
        mu = start
        if target != start:
            x, mu = cont.continuation(x, name, start, target, float(spec.get('ds', 100.0)))
        itf.set_parameter(name, mu)
        fnorm = itf.rhs(x).norm()
        out = itf.array_from_vector(x)
        stream.synchronize()
    return {'x': out, 'mu': mu, 'fnorm': fnorm, 'calls': dict(cont.stats),
            'factorizations': itf.solver.stats['factorizations']}


def solve_many(specs, concurrency=None):
    """Solve every instance of ``specs`` (see ``solve_instance``), up to
    ``concurrency`` at a time (default: all), each on its own stream.
    Returns the results in the order of ``specs``; an instance that fails
    re-raises its exception here."""
    specs = list(specs)
    results = [None] * len(specs)
    errors = [None] * len(specs)
    limit = threading.Semaphore(concurrency or max(1, len(specs)))
    device = torch.cuda.current_device()

    def work(i):
        with limit:
            try:
                torch.cuda.set_device(device)
                results[i] = solve_instance(specs[i], _lib.new_stream())
            except BaseException as e:   # re-raised on the calling thread
                errors[i] = e

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(specs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for e in errors:
        if e is not None:
            raise e
    return results


def instance_cost(spec):
    """Relative cost estimate of one instance: the multifrontal solve of a
    grid with N unknowns scales like N^1.5 in 2D and N^2 in 3D, times the
    continuation steps to the target (about target / ds, at least one)."""
    nx = int(spec['nx'])
    ny = int(spec.get('ny', nx))
    nz = int(spec.get('nz', 1))
    cells = nx * ny * nz
    work = cells ** (2.0 if nz > 1 else 1.5)
    steps = 1.0 + abs(float(spec['target']) - float(spec.get('start', 0.0))) / float(spec.get('ds', 100.0))
    return work * steps


def shard(specs, world, rank):
    """Indices (ascending) of the instances rank ``rank`` of ``world`` solves.
    Longest estimated cost first, each to the currently least loaded rank
    (ties: the lower rank); deterministic, so every rank computes the same
    partition without communicating."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError('rank %d outside a world of %d' % (rank, world))
    costs = [instance_cost(sp) for sp in specs]
    load = [0.0] * world
    owner = [0] * len(specs)
    for i in sorted(range(len(specs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(specs)) if owner[i] == rank]


def solve_sharded(specs, concurrency=None, solver=None):
    """Solve ``specs`` across the ranks of the initialised process group
    (one GPU each): every rank solves its shard concurrently on its GPU
    (``solve_many``, or ``solver`` -- a callable taking a list of specs and
    returning their results), then all results are gathered on every rank
    in the order of ``specs``.  Without a process group this is
    ``solve_many``."""
    import torch.distributed as tdist
    specs = list(specs)
    solver = solver or (lambda sp: solve_many(sp, concurrency))
    if not tdist.is_initialized():
        return solver(specs)
    world, rank = tdist.get_world_size(), tdist.get_rank()
    mine = shard(specs, world, rank)
    local = solver([specs[i] for i in mine]) if mine else []
    parts = [None] * world
    tdist.all_gather_object(parts, list(zip(mine, local)))
    out = [None] * len(specs)
    for part in parts:
        for i, res in part:
            out[i] = res
    dist.barrier()
    return out
