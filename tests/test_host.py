"""Host-side logic of the CUDA backend, testable without a GPU: the
nested-dissection plan, the stencil template, the boundary program and the
C ABI of libtfcuda.so (symbols only -- no kernel is called)."""

import ctypes
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import ROOT
from oracle import fvm
from transiflow_gb300 import grid
from transiflow_gb300.ndplan import build_plan, numeric_reference


def _gauged(A, g):
    A = A.tocoo()
    keep = (A.row != g) & (A.col != g)
    r = np.append(A.row[keep], g)
    c = np.append(A.col[keep], g)
    v = np.append(A.data[keep], -1.0)
    M = sp.csr_matrix((v, (r, c)), shape=A.shape)
    M.sort_indices()
    return M


@pytest.mark.parametrize('case', [
    ({'Reynolds Number': 1000}, 16, 16, 1, 16),
    ({'Reynolds Number': 3000}, 12, 9, 1, 10),
    ({'Reynolds Number': 100}, 6, 5, 4, 12),
    ({'Problem Type': 'Differentially Heated Cavity', 'Rayleigh Number': 1e5, 'Prandtl Number': 1000,
      'Reynolds Number': 1, 'Grid Stretching Factor': 1.5}, 10, 10, 1, 16),
])
def test_nested_dissection_plan_solves_exactly(case):
    params, nx, ny, nz, leaf = case
    d = fvm.Discretization(dict(params), nx, ny, nz)
    s = np.random.default_rng(0).standard_normal(nx * ny * nz * d.dof)
    A = _gauged(d.jacobian(s).to_scipy(), d.dim)
    plan = build_plan(nx, ny, nz, d.dof, A.indptr, A.indices, leaf_cells=leaf, pressure_var=d.dim)
    assert plan.n_own.sum() == A.shape[0]
    b = np.random.default_rng(1).standard_normal(A.shape[0])
    b[d.dim] = 0
    x = numeric_reference(plan, A.data, b)
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-10


def test_plan_every_entry_routed_once():
    d = fvm.Discretization({'Reynolds Number': 100}, 9, 7)
    A = _gauged(d.jacobian(np.ones(9 * 7 * 3)).to_scipy(), 2)
    p = build_plan(9, 7, 1, 3, A.indptr, A.indices, leaf_cells=8, pressure_var=2)
    assert len(np.unique(p.scat_src)) == len(p.scat_src) == A.nnz
    # child boundaries land inside parent fronts
    for t in range(p.nnodes):
        if p.parent[t] >= 0:
            m = p.ea_map[p.ea_map_off[t]:p.ea_map_off[t + 1]]
            assert len(m) == p.n_bnd[t] and m.max(initial=-1) < p.f[p.parent[t]]


LAYOUT_CASES = [
    (2, 3, {'Reynolds Number': 1000}, (9, 8, 1)),
    (2, 4, {'Problem Type': 'Differentially Heated Cavity', 'Rayleigh Number': 1e4, 'Reynolds Number': 1}, (7, 6, 1)),
    (2, 4, {'Problem Type': 'Rayleigh-Benard Perturbation', 'Biot Number': 0.3, 'Reynolds Number': 1}, (7, 6, 1)),
    (3, 4, {'Reynolds Number': 100}, (5, 4, 4)),
    (3, 4, {'Reynolds Number': 100}, (5, 4, 1)),
    (3, 5, {'Problem Type': 'Rayleigh-Benard', 'Rayleigh Number': 1e3, 'Reynolds Number': 1}, (4, 4, 3)),
    (3, 5, {'Problem Type': 'Rayleigh-Benard Perturbation', 'Biot Number': 0.3, 'Reynolds Number': 1}, (4, 4, 3)),
    (2, 3, {'Problem Type': 'Double Gyre', 'Reynolds Number': 30, 'Rossby Parameter': 500,
            'Wind Stress Parameter': 700}, (7, 6, 1)),
    (2, 4, {'Problem Type': 'Double Gyre', 'Reynolds Number': 16, 'Rossby Parameter': 1000,
            'Wind Stress Parameter': 1000}, (5, 6, 1)),
    (2, 5, {'Problem Type': 'AMOC', 'Rayleigh Number': 4e4, 'Prandtl Number': 2.25, 'Temperature Forcing': 1,
            'Freshwater Flux': 0.3, 'X-max': 5}, (7, 5, 1)),
]


@pytest.mark.parametrize('dim,dof,params,shape', LAYOUT_CASES)
def test_stencil_template_covers_every_atom_entry(built_lib, dim, dof, params, shape):
    """Every atom entry the reference can produce (after boundary folding)
    has a slot in the fixed-width stencil CSR."""
    ro = np.zeros(dof + 1, dtype=np.int32)
    slot = np.zeros(dof * dof * 27, dtype=np.int32)
    assert built_lib.tf_stencil_layout(dim, dof, ro.ctypes.data, slot.ctypes.data) == 0
    slot = slot.reshape(dof, dof, 3, 3, 3)   # [d1, d2, oz, oy, ox]
    nx, ny, nz = shape
    d = fvm.Discretization(dict(params), nx, ny, nz, dim, dof)
    for seed in range(3):
        s = np.random.default_rng(seed).standard_normal(nx * ny * nz * dof)
        J, F = d.nonlinear_part(s)
        lin = d.linear_part()
        J += lin
        F += lin
        d.boundaries(J)
        d.boundaries(F)
        for A in (J, F):
            nz_ = np.abs(A).max(axis=(0, 1, 2)) != 0          # [d1, d2, ox, oy, oz]
            d1, d2, ox, oy, oz = np.nonzero(nz_)
            assert np.all(slot[d1, d2, oz, oy, ox] >= 0)


def test_c_abi_exports_every_declared_symbol(built_lib):
    hdr = open(os.path.join(ROOT, 'include', 'tfcuda.h')).read()
    names = set(re.findall(r'^\s*(?:int|size_t|long long|void|const char \*)\s*(tf_\w+)\s*\(', hdr, re.M))
    assert len(names) >= 20
    for name in sorted(names):
        assert hasattr(built_lib, name), name
        assert ctypes.cast(getattr(built_lib, name), ctypes.c_void_p).value


def test_plan_with_too_many_fronts_in_a_height_is_refused(built_lib):
    """A height with more fronts than a grid dimension holds (65535) makes
    every per-height entry point return TF_ERR_SIZE before any CUDA call (so
    this runs without a GPU; the device pointers are never read)."""
    from transiflow_gb300 import _lib
    fake = ctypes.c_void_p(16)
    level_ptr = (ctypes.c_int32 * 3)(0, 1, 70002)
    sizes = (ctypes.c_int32 * 2)(4, 8)
    p = _lib.NdPlan()
    p.n, p.nnodes, p.nlevels = 4 * 70002, 70002, 2
    p.level_ptr = ctypes.cast(level_ptr, ctypes.c_void_p)
    p.max_own = p.max_f = ctypes.cast(sizes, ctypes.c_void_p)
    for f in ('d_n_own', 'd_f', 'd_parent', 'd_front_off', 'd_idx_off', 'd_idx', 'd_ea_off', 'd_ea_map',
              'd_scat_pos', 'd_scat_src', 'd_piv_off', 'd_rank'):
        setattr(p, f, fake)
    fn = built_lib.tf_nd_solve_inv_f32
    fn.argtypes = [ctypes.c_void_p] * 6
    fn.restype = ctypes.c_int
    assert fn(ctypes.cast(ctypes.pointer(p), ctypes.c_void_p), fake, fake, fake, fake, None) == 4


def test_python_binding_matches_the_header():
    """Every entry point the ctypes binding declares is in the header with
    the same number of parameters and a matching return type (the binding
    cannot drift from the C ABI a foreign caller sees)."""
    from transiflow_gb300 import _lib
    hdr = open(os.path.join(ROOT, 'include', 'tfcuda.h')).read()
    hdr = re.sub(r'/\*.*?\*/', '', hdr, flags=re.S)
    protos = {}
    for m in re.finditer(r'^\s*(int|size_t|long long|void|const char \*)\s*(tf_\w+)\s*\(([^;]*?)\)\s*;', hdr, re.M | re.S):
        ret, name, args = m.group(1), m.group(2), ' '.join(m.group(3).split())
        n = 0 if args in ('', 'void') else args.count(',') + 1
        protos[name] = (ret, n)
    rets = {'int': ctypes.c_int, 'size_t': ctypes.c_size_t, 'long long': ctypes.c_longlong, 'void': None,
            'const char *': ctypes.c_char_p}
    for name, (args, res) in _lib._SIGNATURES.items():
        assert name in protos, name
        ret, n = protos[name]
        assert n == len(args), (name, n, len(args))
        assert rets[ret] is res, (name, ret, res)


def test_boundary_program_records_custom_callback():
    """The reference's test_custom_bc callback (tests/test_interface.py:118-148)."""
    def boundaries(bc, atom):
        bc.heat_flux_east(atom, 0)
        bc.heat_flux_west(atom, 0)
        bc.no_slip_east(atom)
        bc.no_slip_west(atom)
        bc.heat_flux_north(atom, 0)
        bc.heat_flux_south(atom, 0)
        bc.no_slip_north(atom)
        bc.no_slip_south(atom)
        bc.heat_flux_top(atom, 0, 0)
        bc.temperature_bottom(atom, 0)
        bc.free_slip_top(atom)
        bc.no_slip_bottom(atom)
        return bc.get_forcing()

    x = grid.uniform_coordinates(0, 1, 4)
    p = grid.make_problem({'Rayleigh Number': 100, 'Prandtl Number': 100}, 4, 4, 4, 3, 5, x, x, x, 0, 4,
                          boundary_conditions=boundaries)
    assert p.nops == 12
    kinds = [(p.ops[t].kind, p.ops[t].axis, p.ops[t].high) for t in range(p.nops)]
    assert kinds[:4] == [(2, 0, 1), (2, 0, 0), (1, 0, 1), (1, 0, 0)]
    assert (p.ops[10].kind, p.ops[10].var) == (1, 1)      # free slip: sign +1


def test_builtin_programs_match_oracle():
    for params, shape in [({'Reynolds Number': 1}, (4, 4, 1)), ({'Reynolds Number': 1}, (4, 4, 4)),
                          ({'Problem Type': 'Differentially Heated Cavity'}, (4, 4, 4)),
                          ({'Problem Type': 'Rayleigh-Benard', 'Biot Number': 0.2, 'Asymmetry Parameter': 0.3},
                           (5, 4, 3))]:
        nx, ny, nz = shape
        d = fvm.Discretization(dict(params), nx, ny, nz)
        ref = d.bc_program()
        p = grid.make_problem(dict(params), nx, ny, nz, d.dim, d.dof, d.x, d.y, d.z, 0, max(shape))
        assert p.nops == len(ref)
        for t, op in enumerate(ref):
            o = p.ops[t]
            if op[0] == 'wall':
                assert (o.kind, o.axis, bool(o.high), o.var) == (1, op[1], op[2], op[3])
            else:
                assert (o.kind, o.axis, bool(o.high), o.var, o.fc, o.ac) == (2,) + tuple(op[1:])


def test_metric_table_matches_oracle_spacings():
    p = {'Grid Stretching Factor': 1.5}
    x = grid.coordinate_vector(p, 0.0, 1.0, 12)
    assert np.array_equal(x, fvm.coordinate_vector(p, 0.0, 1.0, 12))
    t = grid.metric_table((x, x, x), (12, 12, 12))
    m = fvm._Metric(x, 12)
    assert np.array_equal(t[0, 0, :12], m.D) and np.array_equal(t[0, 3, :12], m.Hp)
    assert np.array_equal(t[0, 8, :12], m.w0) and np.array_equal(t[0, 9, :12], m.w1)


K_FOWN, K_FBND, K_BBND, K_BOWN, K_WFWD, K_WBWD = 0, 1, 3, 4, 5, 6


def _flow_tasks(lib, plan, fuse, chunk):
    import ctypes
    n = np.ascontiguousarray(plan.n_own, dtype=np.int32)
    f = np.ascontiguousarray(plan.f, dtype=np.int32)
    par = np.ascontiguousarray(plan.parent, dtype=np.int32)
    lp = np.cumsum([0] + [len(l) for l in plan.levels]).astype(np.int32)
    assert (np.concatenate(plan.levels) == np.arange(plan.nnodes)).all()
    cnt = ctypes.c_int(0)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    args = (plan.nnodes, ptr(n), ptr(f), ptr(par), len(plan.levels), ptr(lp), fuse, chunk)
    assert lib.tf_nd_flow_tasks_host(*args, None, None, 0, ctypes.byref(cnt)) == 0
    tasks = np.zeros((cnt.value, 8), np.int32)
    nodes = np.zeros((plan.nnodes, 8), np.int32)
    assert lib.tf_nd_flow_tasks_host(*args, ptr(tasks), ptr(nodes), cnt.value, ctypes.byref(cnt)) == 0
    return tasks, nodes


@pytest.mark.parametrize('fuse,chunk', [(0, 1), (0, 24), (12, 8), (48, 24), (10 ** 6, 24)])
@pytest.mark.parametrize('case', [({'Reynolds Number': 100}, 32, 24, 1),
                                  ({'Reynolds Number': 100}, 6, 6, 6)])
def test_dataflow_task_list_follows_the_elimination_tree(built_lib, case, fuse, chunk):
    """The task list of the one-launch dataflow application (built by the
    library's own host code) covers every row of every front once per part of
    each sweep, every counter is signalled exactly as often as its waiters
    expect and only by tasks earlier in the list (so the launch cannot
    deadlock whatever number of CTAs is resident), and the waits imply every
    dependency of the substitution: descendants before a front's forward,
    ancestors before its backward."""
    params, nx, ny, nz = case
    d = fvm.Discretization(dict(params), nx, ny, nz)
    A = _gauged(d.jacobian(np.random.default_rng(0).standard_normal(nx * ny * nz * d.dof)).to_scipy(), d.dim)
    plan = build_plan(nx, ny, nz, d.dof, A.indptr, A.indices, pressure_var=d.dim)
    T0, NF = _flow_tasks(built_lib, plan, fuse, chunk)
    n, f, par = plan.n_own, plan.f, plan.parent
    # expand warp bundles into one pseudo task per front (kinds 100 / 101)
    rows = []
    for t in T0:
        if t[1] in (K_WFWD, K_WBWD):
            assert 1 <= t[2] <= 8
            for i in range(t[0], t[0] + t[2]):
                w, tg, sg = NF[i, 0:3] if t[1] == K_WFWD else NF[i, 3:6]
                rows.append([i, 100 if t[1] == K_WFWD else 101, 0, 0, w, tg, sg, 0])
        else:
            rows.append(list(t))
    T = np.array(rows, np.int64)
    cov = {}
    for node, kind, r0, r1 in T[:, :4]:
        cov.setdefault((node, kind), []).append((r0, r1))
    for i in range(plan.nnodes):
        if (i, 100) in cov:
            assert len(cov[(i, 100)]) == 1 and len(cov[(i, 101)]) == 1
            continue
        for kind, lo, hi in [(K_FOWN, 0, n[i]), (K_FBND, n[i], f[i]), (K_BBND, 0, n[i]), (K_BOWN, 0, n[i])]:
            rs = sorted(cov.get((i, kind), []))
            if hi == lo:
                assert not rs
                continue
            assert rs[0][0] == lo and rs[-1][1] == hi
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
    sig = {}
    for k, t in enumerate(T):
        if t[6] >= 0:
            sig.setdefault(int(t[6]), []).append(k)
    done = [0] * len(T)
    for k, t in enumerate(T):
        if t[4] >= 0 and t[5] > 0:
            s = sig.get(int(t[4]), [])
            assert len(s) == t[5] and max(s) < k
            m = 0
            for j in s:
                m |= (1 << j) | done[j]
            done[k] = m
        else:
            assert t[5] == 0
    of = {}
    for k, t in enumerate(T):
        of.setdefault((int(t[0]), int(t[1])), []).append(k)

    def mask(fronts, kinds):
        m = 0
        for i in fronts:
            for kd in kinds:
                for k in of.get((i, kd), []):
                    m |= 1 << k
        return m

    kids = [[] for _ in range(plan.nnodes)]
    for i in range(plan.nnodes):
        if par[i] >= 0:
            kids[par[i]].append(i)

    def desc(i):
        out, st = [], list(kids[i])
        while st:
            c = st.pop()
            out.append(c)
            st.extend(kids[c])
        return out

    def anc(i):
        out, a = [], par[i]
        while a >= 0:
            out.append(a)
            a = par[a]
        return out

    fw = (K_FOWN, K_FBND, 100)
    for k, t in enumerate(T):
        i, kind = int(t[0]), int(t[1])
        if kind in (K_FOWN, 100):
            need = mask(desc(i), fw)
        elif kind == K_FBND:
            need = mask([i], (K_FOWN,))
        elif kind in (K_BBND, 101):
            need = mask(anc(i), (K_BOWN, 101)) | mask([i] + desc(i), fw)
        else:
            need = mask([i], (K_BBND,))
        assert need & ~done[k] == 0


def test_parameter_files_round_trip(tmp_path):
    """Parameters saved with a state (the reference's save_parameters /
    load_parameters format, BaseInterface.py:84-160) survive NumPy scalars,
    arrays and complex values."""
    from transiflow_gb300.interface import Interface
    params = {'Reynolds Number': np.float64(1500.0), 'Problem Type': 'Lid-driven Cavity',
              'Grid Stretching Factor': 1.5, 'Count': np.int32(3), 'Shift': 1 + 2j,
              'Profile': np.arange(3.0)}
    name = str(tmp_path / 'state')
    Interface.save_json(None, name + '.params', params)
    back = Interface.load_json(None, name + '.params')
    assert back['Reynolds Number'] == 1500.0 and back['Count'] == 3
    assert back['Shift'] == 1 + 2j
    assert back['Profile'] == [0.0, 1.0, 2.0]
    assert back['Problem Type'] == 'Lid-driven Cavity' and back['Grid Stretching Factor'] == 1.5


def test_tuner_picks_the_fastest_median_and_caches_it(tmp_path):
    """The application tuner's selection (median of repeated timings, ties to
    the earlier candidate) and its JSON cache: entries survive a new cache
    object on the same file, and an unreadable file only means no entries."""
    from transiflow_gb300.solver import APPLY_WAVES, TuneCache, pick_fastest
    times = {16: [3.0, 1.0, 3.0], 32: [2.0, 2.0, 9.0], 64: [2.0, 2.0, 2.0], 128: [5.0, 5.0, 5.0]}
    calls = {k: iter(v) for k, v in times.items()}
    assert pick_fastest(APPLY_WAVES, lambda c: next(calls[c])) == 32
    path = str(tmp_path / 'sub' / 'tune.json')
    c = TuneCache(path)
    assert c.get('k') is None
    c.put('k', 64)
    c.put('other', 16)
    assert TuneCache(path).get('k') == 64 and TuneCache(path).get('other') == 16
    with open(path, 'w') as f:
        f.write('{not json')
    assert TuneCache(path).get('k') is None
