"""GPU parity of the fused assembly kernel against fixtures computed by the
reference (tests/golden).  Tolerance: 1e-12 relative for RHS and Jacobian
values, exact equality for CSR row pointers and column indices."""

import numpy as np
import pytest

from conftest import DISC_FIXTURES, golden_csr, golden_params, load_golden

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _interface(g):
    from transiflow_gb300 import Interface
    return Interface(golden_params(g), int(g['nx']), int(g['ny']), int(g['nz']), int(g['dim']), int(g['dof']))


@pytest.mark.parametrize('name', DISC_FIXTURES)
def test_rhs_and_jacobian_match_reference(name):
    g = load_golden(name)
    itf = _interface(g)
    exact = True
    for t, s in enumerate(g['states']):
        x = itf.vector_from_array(s)
        f = itf.rhs(x).numpy()
        ref = g['rhs'][t]
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(f - ref).max() <= RTOL * scale
        exact &= np.array_equal(f, ref)
        b, c, v = itf.jacobian(x).compact()
        rb, rc, rv = golden_csr(g, t)
        assert np.array_equal(b, rb), 'row pointers differ'
        assert np.array_equal(c, rc), 'column indices differ'
        assert np.all(np.abs(v - rv) <= RTOL * np.abs(rv))
        exact &= np.array_equal(v, rv)
    print('%s: bit-exact=%s' % (name, exact))


@pytest.mark.parametrize('name', ['ldc2d_16_re1000', 'ldc3d_5x4x3_stretched', 'dhc2d_8_stretched'])
def test_mass_matrix_matches_reference(name):
    g = load_golden(name)
    itf = _interface(g)
    d = itf.mass_matrix().diagonal()
    ref = np.zeros(len(d))
    rows = np.repeat(np.arange(len(d)), np.diff(g['mass_begA']))
    ref[rows] = g['mass_coA']
    assert np.array_equal(d, ref)


def test_fused_rhs_jacobian_equals_separate():
    g = load_golden('ldc2d_16_re1000')
    from transiflow_gb300 import Interface
    p = dict(golden_params(g))
    p['CUDA'] = {'Fuse Jacobian': True}
    itf = Interface(p, 16, 16)
    x = itf.vector_from_array(g['states'][3])
    f = itf.rhs(x)
    J = itf.jacobian(x)
    assert itf.calls['fused_jacobians'] == 1
    b, c, v = J.compact()
    rb, rc, rv = golden_csr(g, 3)
    assert np.array_equal(c, rc) and np.allclose(v, rv, rtol=RTOL, atol=0)
    assert np.allclose(f.numpy(), g['rhs'][3], rtol=0, atol=RTOL * np.abs(g['rhs'][3]).max())


def test_spmv_matches_scipy():
    g = load_golden('ldc2d_16_re1000')
    itf = _interface(g)
    x = itf.vector_from_array(g['states'][0])
    J = itf.jacobian(x)
    v = np.random.default_rng(5).standard_normal(itf.n)
    y = (J @ itf.vector_from_array(v)).numpy()
    ref = J.to_scipy() @ v
    assert np.allclose(y, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
