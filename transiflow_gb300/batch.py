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
"""

import threading

import torch

from . import _lib

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
