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
