"""GPU linear solves against the reference SciPy backend (splu) fixtures and
against SciPy on larger grids."""

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _gauged(A, g):
    import scipy.sparse as sp
    A = A.tocoo()
    keep = (A.row != g) & (A.col != g)
    return sp.csr_matrix((np.append(A.data[keep], -1.0), (np.append(A.row[keep], g), np.append(A.col[keep], g))),
                         shape=A.shape)


def test_direct_solve_matches_reference():
    from transiflow_gb300 import Interface
    g = load_golden('solve_ldc2d_12')
    itf = Interface({'Reynolds Number': float(g['re'])}, 12, 12)
    J = itf.jacobian(itf.vector_from_array(g['state']))
    y = itf.solve(J, itf.vector_from_array(g['b'])).numpy()
    assert np.linalg.norm(y - g['y']) / np.linalg.norm(g['y']) < 1e-10


@pytest.mark.parametrize('method', ['krylov', 'elimination'])
@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_bordered_solve_matches_reference(method, precision):
    """The bordered system [J, V; W^T, C] against the reference's SuperLU
    solve of its bordered matrix, solved as one FGMRES on the bordered
    matrix (block preconditioner from the Jacobian's factorisation) or by
    block elimination.  The single Krylov solve takes about the iterations
    of one plain solve with the same factorisation."""
    from transiflow_gb300 import Interface
    g = load_golden('solve_ldc2d_12')
    itf = Interface({'Reynolds Number': float(g['re']),
                     'CUDA': {'Bordered Solve': method, 'Factor Precision': precision, 'Tolerance': 1e-12}},
                    12, 12)
    J = itf.jacobian(itf.vector_from_array(g['state']))
    st = itf.solver.stats
    itf.solve(J, itf.vector_from_array(g['b']))
    plain = st['gmres_iterations']
    y1, y2 = itf.solve(J, itf.vector_from_array(g['b']), float(g['rhs2']), itf.vector_from_array(g['V']),
                       itf.vector_from_array(g['W']), float(g['C']))
    bordered = st['gmres_iterations'] - plain
    assert np.linalg.norm(y1.numpy() - g['y1']) / np.linalg.norm(g['y1']) < 1e-9
    assert abs(y2 - float(g['y2'])) <= 1e-9 * abs(float(g['y2']))
    if method == 'krylov':
        assert bordered <= plain + 2, (plain, bordered)


@pytest.mark.parametrize('inverse', [True, False])
@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
@pytest.mark.parametrize('shape,params', [((48, 48, 1), {'Reynolds Number': 2000}),
                                          ((24, 20, 1), {'Problem Type': 'Differentially Heated Cavity',
                                                         'Rayleigh Number': 1e5, 'Prandtl Number': 1000,
                                                         'Reynolds Number': 1, 'Grid Stretching Factor': 1.5}),
                                          ((8, 8, 6), {'Reynolds Number': 300})])
def test_nd_gmres_solves_gauged_system(precision, shape, params, inverse):
    from transiflow_gb300 import Interface
    p = dict(params)
    p['CUDA'] = {'Factor Precision': precision, 'Tolerance': 1e-12, 'Inverse Apply': inverse}
    nx, ny, nz = shape
    itf = Interface(p, nx, ny, nz)
    rng = np.random.default_rng(3)
    x = itf.vector_from_array(0.5 * rng.standard_normal(itf.n))
    J = itf.jacobian(x)
    b = rng.standard_normal(itf.n)
    y = itf.solve(J, itf.vector_from_array(b)).numpy()
    A = _gauged(J.to_scipy(), itf.dim)
    bg = b.copy()
    bg[itf.dim] = 0
    assert np.linalg.norm(A @ y - bg) / np.linalg.norm(bg) < 1e-11
    ref = spla.spsolve(A.tocsc(), bg)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-8
    # the factorisation is cached on the matrix: a second solve reuses it
    nf = itf.solver.stats['factorizations']
    itf.solve(J, itf.vector_from_array(b))
    assert itf.solver.stats['factorizations'] == nf


def test_zero_rhs_gives_zero():
    from transiflow_gb300 import Interface
    itf = Interface({'Reynolds Number': 10}, 8, 8)
    J = itf.jacobian(itf.vector())
    y = itf.solve(J, itf.vector())
    assert np.all(y.numpy() == 0)


@pytest.mark.parametrize('shape,params', [((40, 36, 1), {'Reynolds Number': 1500}),
                                          ((7, 6, 6), {'Reynolds Number': 200}),
                                          ((16, 8, 1), {'Problem Type': 'AMOC', 'Rayleigh Number': 4e4,
                                                        'Prandtl Number': 2.25, 'X-max': 5,
                                                        'Temperature Forcing': 1.0})])
def test_one_application_of_the_inverted_factors_solves(shape, params):
    """One application of the FP64 factorisation (no Krylov iteration) with
    inverted own blocks agrees with the substitution sweeps and with a
    sparse direct solve: the inverses are exact up to rounding."""
    import torch
    from transiflow_gb300 import Interface
    nx, ny, nz = shape
    rng = np.random.default_rng(5)
    out = {}
    for inverse in (True, False):
        p = dict(params)
        p['CUDA'] = {'Inverse Apply': inverse, 'CUDA Graphs': False}
        itf = Interface(p, nx, ny, nz)
        st = 0.3 * np.random.default_rng(4).standard_normal(itf.n)
        J = itf.jacobian(itf.vector_from_array(st))
        fac = itf.solver.factorization(J)
        b = rng.standard_normal(itf.n) if inverse else out['b']
        b[itf.dim] = 0.0
        v = torch.as_tensor(b.copy()).to(itf.device)
        fac.apply(v)
        out['b'] = b
        out[inverse] = v.cpu().numpy()
        A = _gauged(J.to_scipy(), itf.dim)
    ref = spla.spsolve(A.tocsc(), out['b'])
    assert np.linalg.norm(out[True] - ref) <= 1e-9 * np.linalg.norm(ref)
    assert np.linalg.norm(out[True] - out[False]) <= 1e-9 * np.linalg.norm(ref)


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
@pytest.mark.parametrize('shape,params', [((40, 36, 1), {'Reynolds Number': 1500}),
                                          ((7, 6, 6), {'Reynolds Number': 200}),
                                          ((12, 10, 1), {'Problem Type': 'Rayleigh-Benard',
                                                         'Rayleigh Number': 1800, 'Prandtl Number': 10}),
                                          ((16, 8, 1), {'Problem Type': 'AMOC', 'Rayleigh Number': 4e4,
                                                        'Prandtl Number': 2.25, 'X-max': 5,
                                                        'Temperature Forcing': 1.0})])
def test_dataflow_application_matches_per_height_launches(shape, params, precision):
    """The one-launch dataflow application of the inverted factors (tasks over
    the tree) gives the per-height application's result (up to the order of
    the sums) for every split of the fronts into tasks -- all split into
    single strips, the defaults, all fused -- and its bounded waits report no
    time-out."""
    import torch
    from transiflow_gb300 import Interface
    nx, ny, nz = shape
    b = None
    results = {}
    for flow, fuse, chunk in [(False, 48, 24), (True, 0, 1), (True, 0, 24), (True, 48, 24), (True, 10 ** 6, 24)]:
        p = dict(params)
        p['CUDA'] = {'Factor Precision': precision, 'CUDA Graphs': False, 'Dataflow Apply': flow,
                     'Dataflow Fuse Tiles': fuse, 'Dataflow Chunk Tiles': chunk}
        itf = Interface(p, nx, ny, nz)
        st = 0.3 * np.random.default_rng(4).standard_normal(itf.n)
        J = itf.jacobian(itf.vector_from_array(st))
        fac = itf.solver.factorization(J)
        eng = itf.solver._engine(precision)
        assert (eng.flow is not None) == flow
        if b is None:
            b = np.random.default_rng(5).standard_normal(itf.n)
            b[itf.dim] = 0.0
        v = torch.as_tensor(b.copy()).to(itf.device)
        fac.apply(v)
        fac.apply(v)      # a second application reuses the cleared counters
        eng.check()
        results[(flow, fuse, chunk)] = v.cpu().numpy()
    base = results.pop((False, 48, 24))
    if precision == 'fp64':
        for key, r in results.items():
            assert np.all(np.isfinite(r)), key
            assert np.linalg.norm(r - base) <= 1e-11 * np.linalg.norm(base), key
    else:
        # single-precision factors: both orders of summation are equally
        # accurate against the FP64 sparse direct solution
        ref = spla.spsolve(_gauged(J.to_scipy(), itf.dim).tocsc(), b)
        err_base = np.linalg.norm(base - ref) / np.linalg.norm(ref)
        for key, r in results.items():
            assert np.all(np.isfinite(r)), key
            assert np.linalg.norm(r - ref) / np.linalg.norm(ref) <= 3 * err_base + 1e-6, key


def test_dataflow_wait_times_out_and_reports():
    """Failure detection of the bounded waits: one task of the dataflow
    application is made to wait for a counter value that no task produces.
    Its wait gives up after its poll limit (about a second), the others
    return through the abort word, tf_nd_flow_status reports TF_ERR_TIMEOUT
    once, and the context stays usable: re-preparing the task list gives the
    correct application again."""
    import ctypes
    import torch
    from transiflow_gb300 import Interface, _lib
    p = {'Reynolds Number': 500, 'CUDA': {'CUDA Graphs': False, 'Dataflow Apply': True,
                                          'Dataflow Fuse Tiles': 0, 'Dataflow Chunk Tiles': 8}}
    itf = Interface(p, 24, 24)
    rng = np.random.default_rng(11)
    J = itf.jacobian(itf.vector_from_array(0.3 * rng.standard_normal(itf.n)))
    fac = itf.solver.factorization(J)
    eng = itf.solver._engine('fp64')
    b = rng.standard_normal(itf.n)
    b[itf.dim] = 0.0
    good = torch.as_tensor(b.copy()).to(itf.device)
    fac.apply(good)
    eng.check()
    # header: err, ntasks, pad, pad (int32), then tasks_off (int64, bytes 16-23);
    # task: node, kind, r0, r1, wait, target, signal, pad (int32)
    words = eng.flow.view(torch.int32)
    ntasks = int(words[1])
    tasks_off = int(eng.flow.view(torch.int64)[2])
    assert tasks_off % 16 == 0 and tasks_off >= 56
    tasks = words[tasks_off // 4: tasks_off // 4 + 8 * ntasks].view(ntasks, 8)
    waiting = torch.nonzero(tasks[:, 5] > 0).flatten()
    assert len(waiting) > 0
    k = int(waiting[len(waiting) // 2])
    tasks[k, 5] += 1                      # a count no task reaches
    bad = torch.as_tensor(b.copy()).to(itf.device)
    fac.apply(bad)
    torch.cuda.synchronize()
    lib = _lib.load()
    assert lib.tf_nd_flow_status(ctypes.c_void_p(eng.flow.data_ptr())) == 5     # TF_ERR_TIMEOUT
    assert lib.tf_nd_flow_status(ctypes.c_void_p(eng.flow.data_ptr())) == 0     # sticky word cleared
    tasks[k, 5] -= 1
    again = torch.as_tensor(b.copy()).to(itf.device)
    fac.apply(again)
    eng.check()
    assert torch.allclose(again, good, rtol=1e-12, atol=1e-12 * float(good.abs().max()))


@pytest.mark.parametrize('shape,params', [((48, 48, 1), {'Reynolds Number': 2000}),
                                          ((24, 20, 1), {'Problem Type': 'Differentially Heated Cavity',
                                                         'Rayleigh Number': 1e5, 'Prandtl Number': 1000,
                                                         'Reynolds Number': 1, 'Grid Stretching Factor': 1.5}),
                                          ((10, 10, 8), {'Reynolds Number': 300})])
def test_fp32_inner_products_with_fp64_refinement(shape, params):
    """Mixed-precision Krylov: FP32 factors, Arnoldi products with an FP32
    copy of the gauged Jacobian, FP64 residuals between cycles -- the solve
    still meets the FP64 tolerance and matches the all-FP64-operator solve."""
    from transiflow_gb300 import Interface
    nx, ny, nz = shape
    ys = []
    for inner in ('fp64', 'fp32'):
        p = dict(params)
        p['CUDA'] = {'Factor Precision': 'fp32', 'Tolerance': 1e-12, 'Inner Precision': inner}
        itf = Interface(p, nx, ny, nz)
        rng = np.random.default_rng(11)
        x = itf.vector_from_array(0.5 * rng.standard_normal(itf.n))
        J = itf.jacobian(x)
        b = rng.standard_normal(itf.n)
        y = itf.solve(J, itf.vector_from_array(b)).numpy()
        A = _gauged(J.to_scipy(), itf.dim)
        bg = b.copy()
        bg[itf.dim] = 0
        assert np.linalg.norm(A @ y - bg) / np.linalg.norm(bg) < 1e-11
        ys.append(y)
    assert np.linalg.norm(ys[1] - ys[0]) / np.linalg.norm(ys[0]) < 1e-9


def test_tuned_application_solves_the_same_system(tmp_path, monkeypatch):
    """With 'Tune Application' the first FP32 factorisation times the
    application's launch shapes and keeps the fastest (cached per GPU, grid
    and precision); the solve agrees with the untuned one to the solver
    tolerance, and a second interface on the same grid reads the cache."""
    from transiflow_gb300 import Interface, solver
    monkeypatch.setattr(solver, '_TUNE_CACHE', solver.TuneCache(str(tmp_path / 'tune.json')))
    n = 10 * 10 * 8 * 4
    x0 = 0.5 * np.random.default_rng(3).standard_normal(n)
    b = np.random.default_rng(5).standard_normal(n)
    ys, waves = [], []
    for tune in (False, True, True):
        itf = Interface({'Reynolds Number': 300,
                         'CUDA': {'Factor Precision': 'fp32', 'Tolerance': 1e-12, 'Tune Application': tune}},
                        10, 10, 8)
        J = itf.jacobian(itf.vector_from_array(x0))
        ys.append(itf.solve(J, itf.vector_from_array(b)).numpy())
        waves.append(itf.solver._engine('fp32').struct.apply_waves)
    assert waves[0] == 0 and waves[1] in solver.APPLY_WAVES and waves[2] == waves[1]
    assert solver._TUNE_CACHE.get(itf.solver._tune_key('fp32')) == waves[1]
    for y in ys[1:]:
        assert np.linalg.norm(y - ys[0]) <= 1e-9 * np.linalg.norm(ys[0])
