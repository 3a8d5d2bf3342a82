"""The learned continuation predictor: its convolution, gradients and Adam
step against the CPU oracle (PyTorch conv3d and autograd in FP32), what the
trained network gains over the secant predictor on a 2D lid-driven cavity
branch, and the continuation's fallback to the secant predictor."""

import ctypes
import time

import numpy as np
import pytest
import torch

from oracle import surrogate as ref


# -- CPU: the oracle's conventions and the continuation's fallback ----------------

@pytest.mark.parametrize('dims', [(4, 3, 2), (5, 4, 1), (3, 3, 3)])
def test_oracle_convolution_matches_explicit_loops(dims):
    """The torch conv3d route of the oracle agrees with explicit loops over
    cells and taps (cell = i + nx*(j + ny*k), tap = (ox+1) + 3(oy+1) + 9(oz+1))."""
    g = torch.Generator().manual_seed(0)
    ncell = dims[0] * dims[1] * dims[2]
    x = torch.randn(ncell, 16, generator=g, dtype=torch.float64)
    w = torch.randn(27, 16, 8, generator=g, dtype=torch.float64)
    b = torch.randn(8, generator=g, dtype=torch.float64)
    z = ref.conv(x, w, b, dims).numpy()
    assert np.allclose(z, ref.conv_loops(x.numpy(), w.numpy(), b.numpy(), dims), rtol=1e-12, atol=1e-12)


class _Cubic:
    """A two-unknown problem F(x, mu) = (x0^3 + x0 - mu, x1 - mu/2) with the
    interface calls the continuation makes, on NumPy vectors."""

    def __init__(self):
        self.mu = 0.0

    def set_parameter(self, name, value):
        self.mu = value

    def get_parameter(self, name):
        return self.mu

    def rhs(self, x):
        return np.array([x[0] ** 3 + x[0] - self.mu, x[1] - 0.5 * self.mu])

    def jacobian(self, x):
        return np.array([[3 * x[0] ** 2 + 1, 0.0], [0.0, 1.0]])

    def solve(self, jac, rhs, *args):
        return np.linalg.solve(jac, rhs)


@pytest.mark.parametrize('quality', ['exact', 'wrong'])
def test_continuation_falls_back_to_the_secant_predictor(quality):
    """A predictor the corrector accepts is counted as accepted; one whose
    corrector does not converge within the learned iteration limit is
    rejected and the step is redone from the secant predictor, reaching the
    same branch end."""
    from transiflow_gb300.continuation import Continuation

    def exact(interface, x0, mu0, dx, dmu, ds):
        mu = mu0 + ds * dmu
        r = np.roots([1, 0, 1, -mu]).real.max()
        return np.array([r, 0.5 * mu]), mu

    def wrong(interface, x0, mu0, dx, dmu, ds):
        return np.array([1e6, -1e6]), mu0 + ds * dmu

    itf = _Cubic()
    plain = Continuation(itf, newton_tolerance=1e-10, quiet=True)
    xp, mup = plain.continuation(np.zeros(2), 'mu', 0.0, 10.0, 0.5)
    itf = _Cubic()
    cont = Continuation(itf, newton_tolerance=1e-10, quiet=True,
                        predictor=exact if quality == 'exact' else wrong)
    x, mu = cont.continuation(np.zeros(2), 'mu', 0.0, 10.0, 0.5)
    assert abs(mu - 10.0) < 1e-4 and abs(mup - 10.0) < 1e-4
    for xx, mm in ((x, mu), (xp, mup)):
        r = np.roots([1, 0, 1, -mm]).real.max()
        assert np.allclose(xx, [r, 0.5 * mm], rtol=1e-9, atol=1e-9)
    if quality == 'exact':
        assert cont.stats['learned_accepted'] > 0 and cont.stats['learned_rejected'] == 0
    else:
        assert cont.stats['learned_accepted'] == 0 and cont.stats['learned_rejected'] > 0


def test_recorder_collects_consecutive_steps():
    """Recorder samples from a plain continuation: each sample's corrected
    point is the next sample's start, its step is the one the step was
    accepted with, and the secant predictor runs unchanged (same branch as
    a run without the recorder)."""
    from transiflow_gb300.continuation import Continuation
    from transiflow_gb300.surrogate import Recorder
    itf = _Cubic()
    plain = Continuation(itf, newton_tolerance=1e-10, quiet=True)
    xp, mup = plain.continuation(np.zeros(2), 'mu', 0.0, 10.0, 0.5)
    itf = _Cubic()
    rec = Recorder()
    steps = []
    cont = Continuation(itf, newton_tolerance=1e-10, quiet=True, predictor=rec.predictor,
                        log=lambda r: (steps.append(r), rec.log(r)))
    x, mu = cont.continuation(np.zeros(2), 'mu', 0.0, 10.0, 0.5)
    assert mu == mup and np.array_equal(x, xp)
    assert cont.stats['points'] == plain.stats['points']
    smp = rec.samples
    assert len(smp) >= 3
    for a, b in zip(smp, smp[1:]):
        assert torch.equal(a['x1'], b['x0'])
    for k, sm in enumerate(smp):
        assert sm['ds'] == steps[k]['ds']
    # the previous-correction input: zero at the first step, then the
    # previous sample's (x1 - x0 - ds t) / ds^2; its weight phi in the
    # quadratic extrapolation for the step taken (the first tangent is exact)
    assert torch.count_nonzero(smp[0]['p']) == 0 and smp[0]['phi'] == 0.0
    for k in range(1, len(smp)):
        h, h0, ds = smp[k - 1]['ds'], smp[k - 2]['ds'] if k >= 2 else 0.0, smp[k]['ds']
        assert smp[k]['phi'] == pytest.approx(h * (ds + h) / (ds * (h0 + h)), rel=1e-12)
    for a, b in zip(smp, smp[1:]):
        want = (a['x1'] - a['x0'] - a['ds'] * a['t']) / a['ds'] ** 2
        assert torch.allclose(b['p'], want, rtol=1e-9, atol=1e-12)
        # the tangent is the normalised secant of the previous step
        x1 = sm['x0'].numpy() + sm['ds'] * sm['t'].numpy()
        assert np.all(np.isfinite(x1))
        r = np.roots([1, 0, 1, -sm['mu']]).real.max()
        assert np.allclose(sm['x0'].numpy(), [r, 0.5 * sm['mu']], rtol=1e-9, atol=1e-9)


def test_quadratic_extrapolation_is_exact_on_a_parabola():
    """The history's p and phi reproduce a quadratic branch exactly: for
    x(s) = a + b s + c s^2 sampled at unequal steps, with the exact tangent
    at the first point and secant tangents after it, x_k + ds t_k + ds^2 phi
    p lands on x(s_k + ds) for every next step ds."""
    from transiflow_gb300.surrogate import _History
    g = torch.Generator().manual_seed(3)
    a, b, c = (torch.randn(5, dtype=torch.float64, generator=g) for _ in range(3))

    def x(s):
        return a + b * s + c * s * s
    s_pts = [0.0, 0.7, 1.9, 2.4, 3.9, 4.2]
    hist = _History()
    t = b.clone()                    # exact tangent at s = 0 (dmu = 1: mu is s)
    for k, sk in enumerate(s_pts):
        if k > 0:
            t = (x(sk) - x(s_pts[k - 1])) / (sk - s_pts[k - 1])
        p = hist.step(t, sk, 1.0)
        if k == 0:
            assert torch.count_nonzero(p) == 0 and hist.phi(1.0) == 0.0
            continue
        for ds in (0.3, 1.0, 2.5):
            pred = x(sk) + ds * t + ds * ds * hist.phi(ds) * p
            assert torch.allclose(pred, x(sk + ds), rtol=0, atol=1e-12), (k, ds)


def test_regular_steps_keep_what_the_history_describes():
    """regular_steps keeps the samples whose quadratic extrapolation beats the
    secant predictor -- here steps along a parabola, where it is exact -- and
    drops the first step of a branch (no history) and a step whose history
    points the wrong way."""
    from transiflow_gb300.surrogate import _History, regular_steps
    g = torch.Generator().manual_seed(7)
    a, b, c = (torch.randn(6, dtype=torch.float64, generator=g) for _ in range(3))

    def x(s):
        return a + b * s + c * s * s
    s_pts = [0.0, 0.5, 1.2, 1.8, 2.9]
    hist = _History()
    samples = []
    t = b.clone()
    for k in range(len(s_pts) - 1):
        if k > 0:
            t = (x(s_pts[k]) - x(s_pts[k - 1])) / (s_pts[k] - s_pts[k - 1])
        p = hist.step(t, s_pts[k], 1.0)
        ds = s_pts[k + 1] - s_pts[k]
        samples.append({'x0': x(s_pts[k]), 't': t, 'p': p, 'phi': hist.phi(ds), 'ds': ds, 'x1': x(s_pts[k + 1]),
                        'mu': s_pts[k]})
    bad = dict(samples[-1], p=-50.0 * samples[-1]['p'])
    kept = regular_steps(samples + [bad])
    assert [s['mu'] for s in kept] == [s['mu'] for s in samples[1:]]


def test_step_proposal_from_the_error_ratio():
    """The proposed step stretches ds by ratio^(-1/3) (the learned error,
    of third order in the step, then equals the secant error at ds), never
    shrinks it and at most doubles it; undefined ratios leave ds alone."""
    from transiflow_gb300.surrogate import Surrogate
    assert Surrogate.propose_step(100.0, 0.125) == pytest.approx(200.0)
    assert Surrogate.propose_step(100.0, 0.216) == pytest.approx(100.0 / 0.6)
    assert Surrogate.propose_step(-50.0, 0.216) == pytest.approx(-50.0 / 0.6)
    assert Surrogate.propose_step(100.0, 1e-6) == 200.0
    assert Surrogate.propose_step(100.0, 3.0) == 100.0
    for bad in (0.0, float('nan'), float('inf'), -1.0):
        assert Surrogate.propose_step(100.0, bad) == 100.0


# -- GPU: the kernels against the oracle ---------------------------------------

def _lib():
    from transiflow_gb300 import _lib as L
    return L, L.load()


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.gpu
@pytest.mark.parametrize('dims,kp,np_', [((7, 5, 3), 16, 32), ((9, 7, 1), 32, 32), ((6, 6, 2), 32, 16),
                                          ((5, 3, 4), 16, 16), ((33, 17, 1), 32, 32)])
def test_convolution_matches_the_oracle(dims, kp, np_):
    """Forward convolution (BF16 operands, FP32 accumulation) against the
    oracle on the same BF16 values: sums of exact products, so only the
    summation order differs (relative 1e-5)."""
    L, lib = _lib()
    g = torch.Generator().manual_seed(1)
    ncell = dims[0] * dims[1] * dims[2]
    x = ref.bf16(torch.randn(ncell, kp, generator=g))
    w = ref.bf16(torch.randn(27, kp, np_, generator=g) * 0.2)
    b = torch.randn(np_, generator=g)
    dx = x.to(torch.bfloat16).cuda()
    dwf = w.permute(0, 2, 1).contiguous().to(torch.bfloat16).cuda()
    db = b.cuda()
    z = torch.empty(ncell, np_, dtype=torch.float32, device='cuda')
    a = torch.empty(ncell, np_, dtype=torch.bfloat16, device='cuda')
    L.check(lib.tf_sg_conv(*dims, kp, np_, dx.data_ptr(), dwf.data_ptr(), db.data_ptr(), z.data_ptr(),
                           a.data_ptr(), 1, _stream()), 'tf_sg_conv')
    torch.cuda.synchronize()
    zr = ref.conv(x.double(), w.double(), b.double(), dims)
    zg = z.cpu().double()
    assert (zg - zr).abs().max() <= 1e-5 * zr.abs().max()
    assert torch.equal(a.cpu(), torch.relu(z.cpu()).to(torch.bfloat16))


def _surrogate(dof, seed, layers=4, channels=32):
    from transiflow_gb300.surrogate import Surrogate
    s = Surrogate(dof, channels=channels, layers=layers, seed=seed)
    # a non-zero last layer, so that gradients reach every layer
    g = torch.Generator().manual_seed(seed + 100)
    w = torch.zeros_like(s.w[-1], device='cpu')
    w[:, :, :dof] = (torch.rand(27, s.kp[-1], dof, generator=g) * 2 - 1) * 0.05
    s.w[-1].copy_(w)
    s.b[-1][:dof].copy_(torch.tensor([0.1, -0.2, 0.05, 0.3, -0.1][:dof]))
    s.export_weights()
    return s


@pytest.mark.gpu
@pytest.mark.parametrize('dims,dof', [((8, 6, 1), 3), ((5, 4, 3), 4), ((70, 20, 1), 3)])
def test_gradients_match_cpu_autograd(dims, dof):
    """Loss and the gradient of every weight and bias through the GPU
    backward kernels against CPU autograd of the oracle network.  The GPU
    path rounds the back-propagated gradient to BF16 before each
    transposed convolution; the oracle keeps it in FP32, hence 2e-2 on the
    relative norm of each gradient."""
    s = _surrogate(dof, seed=3)
    ncell = dims[0] * dims[1] * dims[2]
    g = torch.Generator().manual_seed(4)
    x = torch.randn(ncell * dof, generator=g, dtype=torch.float64).cuda()
    t = torch.randn(ncell * dof, generator=g, dtype=torch.float64).cuda()
    x1 = x + 0.3 * t + 0.01 * torch.randn(ncell * dof, generator=g, dtype=torch.float64).cuda()
    pv = torch.randn(ncell * dof, generator=g, dtype=torch.float64).cuda()
    sample = {'x0': x, 't': t, 'p': pv, 'phi': 0.7, 'mu': 250.0, 'ds': 0.3, 'x1': x1}
    s.fit_scales([sample])
    b = s._buffers(dims)
    ps = s._pack(b, x, t, sample['mu'], sample['ds'], pv, sample['phi'])
    s._target(b, sample, ps)
    s._forward(b)
    s._backward(b, ctypes.c_void_p(b['loss'].data_ptr()), False)
    torch.cuda.synchronize()
    # the packed input, exactly: the scaled state, tangent and previous
    # correction (at unit RMS per variable: the residual mode's per-sample
    # scale), then mu and ds
    x0 = b['x0'].view(ncell, s.kp[0]).float().cpu()
    sc = s.scales
    rms = pv.view(ncell, dof).pow(2).mean(dim=0).sqrt().cpu() * 0.7
    assert np.allclose(ps, rms.numpy(), rtol=1e-12)
    want = torch.zeros(ncell, s.kp[0])
    want[:, :dof] = (x.view(ncell, dof).float().cpu() * torch.tensor(sc['sx']).float())
    want[:, dof:2 * dof] = (t.view(ncell, dof).float().cpu() * torch.tensor(sc['st']).float())
    want[:, 2 * dof:3 * dof] = (pv.view(ncell, dof).float().cpu() * torch.tensor([0.7 / r for r in ps]).float())
    want[:, 3 * dof] = float(np.float32(sample['mu'] * sc['mu']))
    want[:, 3 * dof + 1] = float(np.float32(sample['ds'] * sc['ds']))
    assert torch.equal(x0, ref.bf16(want))
    tgt = b['tgt'].view(ncell, dof).cpu()
    loss, gw, gb = ref.loss_and_grads(x0, tgt, [w.cpu() for w in s.w], [bb.cpu() for bb in s.b], dims, dof)
    assert abs(float(b['loss'].item()) - loss) <= 1e-4 * loss
    for layer in range(s.layers):
        gr = s.grad[layer].view(28, s.kp[layer], s.np[layer]).cpu()
        e_w = (gr[:27] - gw[layer]).norm() / gw[layer].norm()
        e_b = (gr[27, 0] - gb[layer]).norm() / max(gb[layer].norm(), 1e-30)
        assert e_w <= 2e-2, (layer, float(e_w))
        assert e_b <= 2e-2, (layer, float(e_b))


@pytest.mark.gpu
def test_adam_step_and_weight_layouts():
    """One Adam step against its formula, and both BF16 layouts the
    convolutions read (forward [tap][co][ci], backward-data the mirrored tap
    [26 - tap][ci][co]) written from the updated master weights."""
    s = _surrogate(3, seed=5, layers=2)
    g = torch.Generator().manual_seed(6)
    w0 = [w.cpu().clone() for w in s.w]
    b0 = [b.cpu().clone() for b in s.b]
    grads = []
    for layer in range(2):
        gr = torch.randn(28, s.kp[layer], s.np[layer], generator=g)
        s.grad[layer].copy_(gr.view(-1))
        grads.append(gr * 0.5)
    s._adam(1e-2, 2)
    torch.cuda.synchronize()
    for layer in range(2):
        gr = grads[layer]
        upd = lambda p, gg: p - 1e-2 * ((0.1 * gg) / 0.1) / (torch.sqrt((0.001 * gg * gg) / 0.001) + 1e-8)
        w1 = upd(w0[layer], gr[:27])
        b1 = upd(b0[layer], gr[27, 0])
        assert torch.allclose(s.w[layer].cpu(), w1, rtol=1e-5, atol=1e-6)
        assert torch.allclose(s.b[layer].cpu(), b1, rtol=1e-5, atol=1e-6)
        wq = s.w[layer].cpu().to(torch.bfloat16)
        kp, np_ = s.kp[layer], s.np[layer]
        assert torch.equal(s.wf[layer].view(27, np_, kp).cpu(), wq.permute(0, 2, 1))
        assert torch.equal(s.wb[layer].view(27, kp, np_).cpu(), wq.flip(0))


def _branch_samples():
    from transiflow_gb300 import Interface
    from transiflow_gb300.continuation import Continuation
    from transiflow_gb300.surrogate import Recorder
    itf = Interface({}, 16, 16)
    rec = Recorder()
    cont = Continuation(itf, newton_tolerance=1e-8, quiet=True, predictor=rec.predictor, log=rec.log)
    x0 = cont.newton(itf.vector())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x, mu = cont.continuation(x0.copy(), 'Reynolds Number', 0, 2000, 100)
    torch.cuda.synchronize()
    stats = dict(cont.stats, wall_s=time.perf_counter() - t0)
    return itf, x0, x, stats, rec.samples


@pytest.fixture(scope='module')
def trained():
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    from transiflow_gb300.surrogate import Surrogate, regular_steps
    itf, x0, x_plain, stats, samples = _branch_samples()
    samples = regular_steps(samples)
    s = Surrogate(itf.dof, seed=0)
    s.fit_scales(samples)
    before = s.evaluate(samples, (16, 16, 1))
    losses = s.train(samples, (16, 16, 1), steps=400, lr=2e-3, batch=4)
    after = s.evaluate(samples, (16, 16, 1))
    return {'itf': itf, 'x0': x0, 'x_plain': x_plain, 'stats': stats, 'samples': samples, 's': s,
            'before': before, 'after': after, 'losses': losses}


@pytest.mark.gpu
def test_training_reduces_the_predictor_error(trained):
    """Trained on the regular branch points of a plain continuation (2D
    lid-driven cavity 16x16, Re 0 -> 2000, ds = 100), the network's
    predictor is closer to the corrected points than the quadratic
    extrapolation it starts from (the untrained network's scaled error is
    the quadratic's residual relative to its correction)."""
    before, after = trained['before'], trained['after']
    print('samples %d, secant error %.4f, learned error %.4f, final training loss %.4f'
          % (len(trained['samples']), before.mean(), after.mean(), trained['losses'][-10:].mean()))
    assert len(trained['samples']) >= 8
    assert np.all(np.isfinite(after))
    assert after.mean() < 0.8 * before.mean()


@pytest.mark.gpu
def test_learned_continuation_reaches_the_same_branch_end(trained):
    """Continuation with the learned predictor reaches Re = 2000 at the same
    solution as the plain run (both polished by Newton to ||F|| <= 1e-12),
    every accepted point has ||F|| <= 1e-8, and the learned predictions are
    used.  The solve counts of both runs are printed: the gain of the
    network over the secant predictor on this branch."""
    from transiflow_gb300.continuation import Continuation
    from transiflow_gb300.surrogate import LearnedPredictor
    itf = trained['itf']
    itf.set_parameter('Reynolds Number', 0)
    fn = []
    cont = Continuation(itf, newton_tolerance=1e-8, quiet=True, predictor=LearnedPredictor(trained['s']),
                        log=lambda r: fn.append(r['fnorm']))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x, mu = cont.continuation(trained['x0'].copy(), 'Reynolds Number', 0, 2000, 100)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    assert abs(mu - 2000) < 1e-3
    assert all(f is not None and f <= 1e-8 for f in fn)
    assert cont.stats['learned_accepted'] > 0
    print('plain: %s\nlearned: %s, wall_s %.3f' % (trained['stats'], cont.stats, wall))
    itf.set_parameter('Reynolds Number', 2000)
    polish = Continuation(itf, quiet=True)
    xa = polish.newton(x, 1e-12).numpy()
    xb = polish.newton(trained['x_plain'], 1e-12).numpy()
    assert np.linalg.norm(xa - xb) <= 1e-8 * np.linalg.norm(xb)


def test_surrogate_rejects_fields_its_kernels_cannot_read():
    """The surrogate's kernels take raw device pointers: host tensors, other
    dtypes, strided views and fields of another grid size are refused before
    any launch (checked here without a GPU)."""
    from transiflow_gb300.surrogate import check_field
    n = 4 * 27
    with pytest.raises(ValueError, match='GPU'):
        check_field(torch.zeros(n, dtype=torch.float64), n)
    with pytest.raises(ValueError, match='torch tensor'):
        check_field(np.zeros(n), n)
    if torch.cuda.is_available():
        with pytest.raises(ValueError, match='float64'):
            check_field(torch.zeros(n, dtype=torch.float32, device='cuda'), n)
        with pytest.raises(ValueError, match='contiguous'):
            check_field(torch.zeros(2 * n, dtype=torch.float64, device='cuda')[::2], n)
        with pytest.raises(ValueError, match='values'):
            check_field(torch.zeros(n + 1, dtype=torch.float64, device='cuda'), n)


@pytest.mark.gpu
def test_samples_from_two_grid_sizes_train_one_network():
    """Recorder samples (device vectors) of two branches on grids of
    different sizes: fit_scales equals NumPy RMS values over the concatenated
    samples, and training steps run on each grid with finite losses."""
    import contextlib
    import io
    from transiflow_gb300 import Continuation, Interface
    from transiflow_gb300.surrogate import Recorder, Surrogate
    groups = []
    for n in (10, 14):
        itf = Interface({'CUDA': {'Tolerance': 1e-10}}, n, n)
        rec = Recorder()
        cont = Continuation(itf, newton_tolerance=1e-8, predictor=rec.predictor, log=rec.log)
        with contextlib.redirect_stdout(io.StringIO()):
            cont.continuation(cont.newton(itf.vector()), 'Reynolds Number', 0.0, 600.0, 100.0)
        assert len(rec.samples) >= 3
        assert all(s['x0'].is_cuda and s['x0'].numel() == itf.n for s in rec.samples)
        groups.append(((n, n, 1), rec.samples))
    samples = [s for _, g in groups for s in g]
    net = Surrogate(3)
    net.fit_scales(samples)

    def rms(key):
        a = np.concatenate([s[key].cpu().numpy().reshape(-1, 3) for s in samples])
        return np.sqrt((a ** 2).mean(axis=0))
    xr, tr = rms('x0'), rms('t')
    # residual mode: the target is what the quadratic extrapolation misses
    d = np.concatenate([((s['x1'] - s['x0'] - s['ds'] * s['t']) / s['ds'] ** 2 - s['phi'] * s['p'])
                        .cpu().numpy().reshape(-1, 3) for s in samples])
    dr = np.sqrt((d ** 2).mean(axis=0))
    assert np.allclose(net.scales['sx'], 1.0 / xr, rtol=1e-6)
    assert np.allclose(net.scales['st'], 1.0 / tr, rtol=1e-6)
    assert np.allclose(net.scales['sd'], dr, rtol=1e-6)
    for dims, g in groups:
        losses = net.train(g, dims, steps=5, lr=1e-3, batch=2)
        assert np.all(np.isfinite(losses))


@pytest.mark.parametrize('quality', ['exact', 'wrong'])
def test_predictor_can_propose_the_step_size(quality):
    """A predictor returning (x, mu, ds') sets the step it is corrected on:
    exact proposals of twice the step are accepted and the branch needs
    fewer points; wrong ones are rejected and the step is redone from the
    secant predictor with the original step, giving the plain branch."""
    from transiflow_gb300.continuation import Continuation

    def exact(interface, x0, mu0, dx, dmu, ds):
        mu = mu0 + 2 * ds * dmu
        r = np.roots([1, 0, 1, -mu]).real.max()
        return np.array([r, 0.5 * mu]), mu, 2 * ds

    def wrong(interface, x0, mu0, dx, dmu, ds):
        return np.array([1e6, -1e6]), mu0 + ds * dmu, 3 * ds

    plain = Continuation(_Cubic(), newton_tolerance=1e-10, quiet=True)
    xp, mup = plain.continuation(np.zeros(2), 'mu', 0.0, 10.0, 0.5, ds_max=0.5)
    cont = Continuation(_Cubic(), newton_tolerance=1e-10, quiet=True,
                        predictor=exact if quality == 'exact' else wrong)
    x, mu = cont.continuation(np.zeros(2), 'mu', 0.0, 10.0, 0.5, ds_max=0.5 if quality == 'wrong' else 1.0)
    assert abs(mu - 10.0) < 1e-4
    r = np.roots([1, 0, 1, -mu]).real.max()
    assert np.allclose(x, [r, 0.5 * mu], rtol=1e-9, atol=1e-9)
    if quality == 'exact':
        assert cont.stats['learned_rejected'] == 0
        assert cont.stats['points'] < plain.stats['points']
    else:
        assert cont.stats['learned_accepted'] == 0
        assert cont.stats['points'] == plain.stats['points'] and mu == mup and np.array_equal(x, xp)


@pytest.mark.gpu
def test_learned_predictor_on_an_unseen_grid():
    """Trained on the regular steps of plain branches of 2D lid-driven
    cavities 12^2 and 16^2 (Re 0 -> 2000, ds = 100), the predictor is used on
    a 24^2 cavity it has not seen, with steps growing past the trained ones:
    the branch ends at the plain branch's solution, every point has ||F||
    <= 1e-8, the calibrated error is below the secant predictor's, and on
    the unseen grid the learned prediction of a step is typically (median
    over the branch) well below the secant's error.  The corrector work of
    both runs is printed."""
    import contextlib
    import io
    from transiflow_gb300 import Continuation, Interface
    from transiflow_gb300.surrogate import LearnedPredictor, Recorder, Surrogate, regular_steps
    groups = []
    for n in (12, 16):
        itf = Interface({'CUDA': {'Tolerance': 1e-10}}, n, n)
        rec = Recorder()
        cont = Continuation(itf, newton_tolerance=1e-8, predictor=rec.predictor, log=rec.log)
        with contextlib.redirect_stdout(io.StringIO()):
            cont.continuation(cont.newton(itf.vector()), 'Reynolds Number', 0.0, 2000.0, 100.0, ds_max=100.0)
        groups.append(((n, n, 1), regular_steps(rec.samples)))
    net = Surrogate(3)
    net.fit_scales([s for _, g in groups for s in g])
    for r in range(4):
        for dims, g in groups:
            net.train(g, dims, steps=150, lr=2e-3, batch=4, seed=r)
    model = net.calibrate_steps(groups)
    runs = {}
    for name, pred in (('plain', None), ('learned', LearnedPredictor(net))):
        itf = Interface({'CUDA': {'Tolerance': 1e-10}}, 24, 24)
        fn = []
        cont = Continuation(itf, newton_tolerance=1e-8, quiet=True, predictor=pred,
                            log=lambda r: fn.append(r['fnorm']))
        itf.set_parameter('Reynolds Number', 0.0)
        x, mu = cont.continuation(cont.newton(itf.vector()), 'Reynolds Number', 0.0, 2000.0, 100.0)
        assert abs(mu - 2000.0) < 1e-3 and max(f for f in fn if f is not None) <= 1e-8
        itf.set_parameter('Reynolds Number', mu)
        xe = Continuation(itf, quiet=True).newton(x, 1e-12).numpy()
        runs[name] = (dict(cont.stats), xe, pred)
    print('step model', model)
    for name, (st, _, pred) in runs.items():
        print(name, {k: st[k] for k in ('points', 'jacobian', 'solve', 'learned_accepted', 'learned_rejected')},
              'steps proposed', getattr(pred, 'steps_proposed', 0))
    ratios = runs['learned'][2].ratios
    print('learned / secant error on the unseen grid, per step:', [round(r, 3) for r in ratios])
    assert model['eps'] < 1.0
    assert len(ratios) >= 5 and float(np.median(ratios)) < 0.7
    assert np.linalg.norm(runs['learned'][1] - runs['plain'][1]) <= 1e-8 * np.linalg.norm(runs['plain'][1])
    assert runs['learned'][0]['learned_accepted'] > 0
