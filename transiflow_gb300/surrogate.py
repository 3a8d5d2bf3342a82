"""Learned continuation predictor: a convolutional surrogate trained on the
branch points that plain continuation computes.

The predictor is a three-point quadratic extrapolation of the branch plus a
learned residual.  With the secant tangents t_{k-1}, t_k of the last two
steps (lengths h0, h) the quadratic through the last three points corrects
the secant predictor ``x + ds*t`` by ``ds**2 * phi * p`` with
``p = (t_k - t_{k-1}) / h`` (the previous step's correction per unit step
squared) and ``phi = h (ds + h) / (ds (h0 + h))`` (1 for equal steps; after
the first, exact tangent h0 = 0).  The network reads the current state
``x``, the secant tangent ``t``, ``p``, the parameter ``mu`` and the step
``ds`` on the cell grid and proposes what the quadratic still misses; a
3x3x3 stencil network alone sees only a few cells of what is a global
curvature, the extrapolation carries it.  From its measured accuracy it
also stretches the next step.  The Newton corrector of the
continuation judges every point; the secant predictor is the fallback
whenever the corrector started from the learned predictor does not converge
within ``Continuation(learned_newton_iterations=4)`` iterations, and
``LearnedPredictor`` uses the network only while its prediction of the last
step beat the secant's.

Architecture: ``layers`` 3x3x3 convolutions over the cell grid (a 2D grid is
a grid one cell thick), ``channels`` channels between them, ReLU after every
layer but the last.  Inputs are ``3*dof + 2`` channels (x, t and p per
variable, mu and ds as constant fields; ``2*dof + 2`` without p), outputs
``dof`` channels.  Forward,
backward and Adam run in libtfcuda kernels (``tf_sg_*``): BF16 operands with
FP32 accumulation on the tensor cores, FP32 master weights.  Inputs and
targets are scaled per variable with statistics of the training samples; the
target is the corrector's displacement from the quadratic predictor divided
by ``ds**2`` (the order of the secant predictor's error), so the
zero-initialised last layer starts the network at exactly the quadratic
predictor (the secant one without ``p``).

The reference has no counterpart: its continuation predicts with the secant
only (transiflow/Continuation.py:258-260).
"""

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .vector import DeviceVector, _stream

__all__ = ['Surrogate', 'Recorder', 'LearnedPredictor', 'regular_steps']


def _pad16(c):
    return 16 if c <= 16 else 32


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _snapshot(v):
    """A copy of a continuation vector as a tensor (DeviceVector or NumPy;
    NumPy vectors stay in host memory until the surrogate moves them)."""
    if isinstance(v, DeviceVector):
        return v.data.clone()
    return torch.tensor(np.asarray(v, dtype=np.float64))


def check_field(t, n, name='field'):
    """Raises ValueError unless t is a contiguous FP64 CUDA tensor of n
    values: the surrogate's kernels read and write raw device pointers, so a
    host tensor or a field of another grid must never reach them."""
    if not isinstance(t, torch.Tensor):
        raise ValueError('%s must be a torch tensor, not %s' % (name, type(t).__name__))
    if t.device.type != 'cuda':
        raise ValueError('%s must be on the GPU (got %s)' % (name, t.device))
    if t.dtype != torch.float64:
        raise ValueError('%s must be float64 (got %s)' % (name, t.dtype))
    if not t.is_contiguous():
        raise ValueError('%s must be contiguous' % name)
    if t.numel() != n:
        raise ValueError('%s has %d values, the grid needs %d' % (name, t.numel(), n))


def _phi(h, h0, ds):
    """Weight of p in the quadratic extrapolation through the last three
    points for the next step ds (h: the last step, h0: the one before, 0
    when the earlier tangent was the exact one at the first point)."""
    if h is None or h0 is None or ds == 0 or abs(h0 + h) <= 1e-12 * abs(h):
        return 0.0
    return h * (ds + h) / (ds * (h0 + h))


class _History:
    """The previous step's correction of the secant predictor, per unit
    step squared.  Consecutive secant tangents t_{k-1}, t_k of a branch
    satisfy x_k - x_{k-1} = ds_{k-1} t_k, so the correction
    (x_k - x_{k-1} - ds_{k-1} t_{k-1}) / ds_{k-1}^2 is (t_k - t_{k-1}) /
    ds_{k-1}, with ds_{k-1} = (mu_k - mu_{k-1}) / dmu_k; zero at the first
    step of a branch.  Also keeps the last two step lengths for phi."""

    def __init__(self):
        self.t = None
        self.mu = None
        self.h = None
        self.h0 = None

    def step(self, t, mu, dmu):
        prev_t, prev_mu = self.t, self.mu
        self.t, self.mu = t, mu
        if prev_t is None or dmu == 0 or mu == prev_mu or prev_t.shape != t.shape:
            self.h = self.h0 = None
            return torch.zeros_like(t)
        ds_prev = (mu - prev_mu) / float(dmu)
        # the first tangent of a branch is exact: a double node, h0 = 0
        self.h0, self.h = (self.h if self.h is not None else 0.0), ds_prev
        return (t - prev_t) / ds_prev

    def phi(self, ds):
        return _phi(self.h, self.h0, ds)


class Recorder:
    """Collects training samples from a plain continuation: pass
    ``recorder.predictor`` as the continuation's predictor (it proposes
    nothing, so the secant predictor runs) and ``recorder.log`` as its log.
    A sample is (x0, t, p, phi, mu0, ds, x1, its): the state, tangent,
    previous correction and parameter a step started from, the weight of p
    in the quadratic extrapolation for the step it was accepted with, that
    step, the point it converged to and the corrector iterations it took."""

    def __init__(self):
        self.samples = []
        self._pending = None
        self._ds = None
        self._its = None
        self._history = _History()

    def predictor(self, interface, x0, mu0, dx, dmu, ds):
        if self._pending is not None and self._ds is not None:
            px, pt, pp, pmu, h, h0 = self._pending
            self.samples.append({'x0': px, 't': pt, 'p': pp, 'phi': _phi(h, h0, self._ds), 'mu': pmu,
                                 'ds': self._ds, 'x1': _snapshot(x0), 'its': self._its})
        t = _snapshot(dx)
        pp = self._history.step(t, float(mu0), dmu)
        self._pending = (_snapshot(x0), t, pp, float(mu0), self._history.h, self._history.h0)
        self._ds = None
        return None

    def log(self, record):
        self._ds = float(record['ds'])
        self._its = record.get('newton_iterations')


def regular_steps(samples):
    """The samples a three-point history describes: a nonzero quadratic
    correction phi p that brings the predictor closer to the converged point
    than the secant predictor.  This drops the first steps of a branch and
    steps across irregular stretches (from a Stokes state, at a fold), whose
    corrections are unrelated to the history; the predictor's online guard
    keeps the secant there."""
    out = []
    for smp in samples:
        p, phi = smp.get('p'), smp.get('phi', 0.0)
        if p is None or not phi:
            continue
        xs = smp['x0'] + smp['ds'] * smp['t']
        es = float((smp['x1'] - xs).pow(2).mean().sqrt())
        eq = float((smp['x1'] - xs - (smp['ds'] ** 2 * phi) * p).pow(2).mean().sqrt())
        if eq < es:
            out.append(smp)
    return out


class Surrogate:
    """The network, its Adam state and its scratch buffers (per grid shape)."""

    def __init__(self, dof, channels=32, layers=4, seed=0, device=None, history=True, residual=True):
        if channels not in (16, 32):
            raise ValueError('channels must be 16 or 32')
        if layers < 2:
            raise ValueError('the surrogate needs at least two layers')
        # inputs: state, tangent, (previous correction,) mu, ds
        self.history = bool(history)
        # learn the residual of the quadratic extrapolation (needs p)
        self.residual = bool(residual) and self.history
        cin = (3 if self.history else 2) * dof + 2
        if cin > 32:
            raise ValueError('too many variables per cell for the input layer')
        self.lib = _lib.load()
        self.device = torch.device(device or 'cuda')
        self.dof = dof
        self.layers = layers
        self.kp = [_pad16(cin)] + [channels] * (layers - 1)
        self.np = [channels] * (layers - 1) + [_pad16(dof)]
        real_in = [cin] + [channels] * (layers - 1)
        real_out = [channels] * (layers - 1) + [dof]
        gen = torch.Generator().manual_seed(seed)
        self.w, self.b, self.grad, self.m, self.v, self.wf, self.wb = [], [], [], [], [], [], []
        for layer in range(layers):
            kp, np_ = self.kp[layer], self.np[layer]
            w = torch.zeros(27, kp, np_, dtype=torch.float32)
            if layer < layers - 1:
                # He-uniform for the ReLU layers; the last layer starts at zero
                bound = math.sqrt(6.0 / (27 * real_in[layer]))
                w[:, :real_in[layer], :real_out[layer]] = \
                    (torch.rand(27, real_in[layer], real_out[layer], generator=gen) * 2 - 1) * bound
            dev = dict(device=self.device)
            self.w.append(w.to(self.device).contiguous())
            self.b.append(torch.zeros(np_, dtype=torch.float32, **dev))
            for lst in (self.grad, self.m, self.v):
                lst.append(torch.zeros(28 * kp * np_, dtype=torch.float32, **dev))
            self.wf.append(torch.empty(27 * np_ * kp, dtype=torch.bfloat16, **dev))
            self.wb.append(torch.empty(27 * kp * np_, dtype=torch.bfloat16, **dev))
        self.step = 0
        self.scales = None
        # step-size model, set by calibrate_steps
        self.step_model = None
        self._bufs = {}
        self.export_weights()

    # -- weights ----------------------------------------------------------------
    def export_weights(self):
        """Write both BF16 layouts of every layer from the master weights
        (after construction or an edit of ``w`` / ``b``)."""
        s = _stream()
        for layer in range(self.layers):
            _lib.check(self.lib.tf_sg_adam(self.kp[layer], self.np[layer], _ptr(self.w[layer]), _ptr(self.b[layer]),
                                           None, None, None, 0.0, 0.0, 0.0, 0.0, 0, 1.0,
                                           _ptr(self.wf[layer]), _ptr(self.wb[layer]), s), 'tf_sg_adam')

    def parameters(self):
        return sum(int(w.numel()) + int(b.numel()) for w, b in zip(self.w, self.b))

    # -- scratch ------------------------------------------------------------------
    def _buffers(self, dims):
        dims = tuple(int(d) for d in dims)
        if dims in self._bufs:
            return self._bufs[dims]
        nx, ny, nz = dims
        ncell = nx * ny * nz
        dev = dict(device=self.device)
        L = self.layers
        b = {'dims': dims, 'ncell': ncell,
             'x0': torch.empty(ncell * self.kp[0], dtype=torch.bfloat16, **dev),
             'z': [torch.empty(ncell * n, dtype=torch.float32, **dev) for n in self.np],
             'a': [torch.empty(ncell * n, dtype=torch.bfloat16, **dev) for n in self.np[:L - 1]],
             'dzf': [torch.empty(ncell * n, dtype=torch.float32, **dev) for n in self.np],
             'dzh': [torch.empty(ncell * n, dtype=torch.bfloat16, **dev) for n in self.np],
             'da': [torch.empty(ncell * n, dtype=torch.float32, **dev) for n in self.np[:L - 1]],
             'tgt': torch.empty(ncell * self.dof, dtype=torch.float32, **dev),
             'xb': torch.empty(ncell * self.dof, dtype=torch.float64, **dev),
             'loss': torch.zeros(1, dtype=torch.float64, **dev)}
        lw = self.lib.tf_sg_loss_workspace_bytes(ncell, self.np[-1])
        ww = max(self.lib.tf_sg_wgrad_workspace_bytes(ncell, kp, np_) for kp, np_ in zip(self.kp, self.np))
        b['lwork'] = torch.empty(lw, dtype=torch.uint8, **dev)
        b['wwork'] = torch.empty(ww, dtype=torch.uint8, **dev)
        self._bufs[dims] = b
        return b

    # -- the kernels in order ------------------------------------------------------
    def _on_device(self, sample):
        """The sample's fields on this surrogate's GPU (samples recorded from
        NumPy continuation vectors are host tensors)."""
        keys = [k for k in ('x0', 't', 'x1', 'p') if k in sample]
        if all(sample[k].device == self.device for k in keys):
            return sample
        out = dict(sample)
        for k in keys:
            out[k] = sample[k].to(self.device, dtype=torch.float64).contiguous()
        return out

    def _based(self, b, x, ds, p, phi):
        """x + ds^2 phi p (into the scratch) when the network learns the
        residual of the quadratic extrapolation, else x."""
        if not self.residual or p is None or not phi:
            return x
        n = b['ncell'] * self.dof
        check_field(p, n, 'previous correction')
        _lib.check(self.lib.tf_vec_axpby(n, 1.0, _ptr(x), float(ds * ds * phi), _ptr(p), _ptr(b['xb']), _stream()),
                   'tf_vec_axpby')
        return b['xb']

    def _pscale(self, p, phi):
        """Per-variable RMS of the quadratic correction phi p (the scale of
        the residual the network learns), or None when it is zero."""
        if not self.residual or p is None or not phi:
            return None
        r = (p.view(-1, self.dof).pow(2).mean(dim=0).sqrt() * abs(phi)).cpu().tolist()
        return r if max(r) > 0 else None

    def _pack(self, b, x, t, mu, ds, p=None, phi=0.0, ps='auto'):
        """Packs the network input; returns the per-variable residual scales
        of this sample (residual mode; None when the quadratic correction is
        zero, and then the network's output is not used).  ``ps`` may pass
        scales computed before (training reuses them every step)."""
        n = b['ncell'] * self.dof
        check_field(x, n, 'state')
        check_field(t, n, 'tangent')
        sc = self.scales
        sx = (ctypes.c_float * self.dof)(*sc['sx'])
        st = (ctypes.c_float * self.dof)(*sc['st'])
        pp, sp = None, None
        if not (self.history and self.residual):
            ps = None
        if self.history:
            if p is None:
                p = torch.zeros_like(x)
            check_field(p, n, 'previous correction')
            pp = p
            if self.residual:
                # p at unit RMS per variable: the network sees the shape of
                # the curvature, whatever its size
                ps = self._pscale(p, phi) if isinstance(ps, str) else ps
                sp = (ctypes.c_float * self.dof)(*[abs(phi) / r if ps and r > 0 else 0.0
                                                   for r in (ps or [0.0] * self.dof)])
            else:
                sp = (ctypes.c_float * self.dof)(*sc['sp'])
        _lib.check(self.lib.tf_sg_pack(b['ncell'], self.dof, self.kp[0], _ptr(x), _ptr(t), _ptr(pp), sx, st, sp,
                                       float(mu * sc['mu']), float(ds * sc['ds']), _ptr(b['x0']), _stream()),
                   'tf_sg_pack')
        return ps

    def _out_scales(self, ds, ps):
        """Per-variable factors from the network's output to the state: ds^2
        times the residual scale (residual mode) or the global target scale."""
        if self.residual:
            return [ds * ds * r for r in (ps or [0.0] * self.dof)]
        return [ds * ds * v for v in self.scales['sd']]

    def _target(self, b, sample, ps=None):
        n = b['ncell'] * self.dof
        for k in ('x0', 't', 'x1'):
            check_field(sample[k], n, 'sample ' + k)
        ds = sample['ds']
        x0 = self._based(b, sample['x0'], ds, sample.get('p'), sample.get('phi', 0.0))
        inv = (ctypes.c_double * self.dof)(*[1.0 / v if v > 0 else 0.0 for v in self._out_scales(ds, ps)])
        _lib.check(self.lib.tf_sg_target(b['ncell'], self.dof, _ptr(x0), _ptr(sample['t']),
                                         _ptr(sample['x1']), float(ds), inv, _ptr(b['tgt']), _stream()),
                   'tf_sg_target')

    def _forward(self, b):
        nx, ny, nz = b['dims']
        s = _stream()
        inp = b['x0']
        for layer in range(self.layers):
            last = layer == self.layers - 1
            _lib.check(self.lib.tf_sg_conv(nx, ny, nz, self.kp[layer], self.np[layer], _ptr(inp),
                                           _ptr(self.wf[layer]), _ptr(self.b[layer]), _ptr(b['z'][layer]),
                                           None if last else _ptr(b['a'][layer]), 0 if last else 1, s),
                       'tf_sg_conv')
            if not last:
                inp = b['a'][layer]

    def _backward(self, b, loss_ptr, accumulate):
        nx, ny, nz = b['dims']
        ncell = b['ncell']
        s = _stream()
        L = self.layers
        _lib.check(self.lib.tf_sg_loss(ncell, self.dof, self.np[-1], _ptr(b['z'][-1]), _ptr(b['tgt']),
                                       _ptr(b['dzf'][-1]), _ptr(b['dzh'][-1]), loss_ptr,
                                       _ptr(b['lwork']), b['lwork'].numel(), s), 'tf_sg_loss')
        for layer in range(L - 1, -1, -1):
            inp = b['x0'] if layer == 0 else b['a'][layer - 1]
            _lib.check(self.lib.tf_sg_wgrad(nx, ny, nz, self.kp[layer], self.np[layer], _ptr(inp),
                                            _ptr(b['dzf'][layer]), _ptr(self.grad[layer]), 1 if accumulate else 0,
                                            _ptr(b['wwork']), b['wwork'].numel(), s), 'tf_sg_wgrad')
            if layer > 0:
                # gradient with respect to the layer's input: the same
                # convolution over dZ with the mirrored, transposed weights
                _lib.check(self.lib.tf_sg_conv(nx, ny, nz, self.np[layer], self.kp[layer], _ptr(b['dzh'][layer]),
                                               _ptr(self.wb[layer]), None, _ptr(b['da'][layer - 1]), None, 0, s),
                           'tf_sg_conv')
                _lib.check(self.lib.tf_sg_act_grad(ncell * self.np[layer - 1], _ptr(b['da'][layer - 1]),
                                                   _ptr(b['z'][layer - 1]), _ptr(b['dzf'][layer - 1]),
                                                   _ptr(b['dzh'][layer - 1]), s), 'tf_sg_act_grad')

    def _adam(self, lr, batch):
        self.step += 1
        s = _stream()
        for layer in range(self.layers):
            _lib.check(self.lib.tf_sg_adam(self.kp[layer], self.np[layer], _ptr(self.w[layer]), _ptr(self.b[layer]),
                                           _ptr(self.grad[layer]), _ptr(self.m[layer]), _ptr(self.v[layer]),
                                           float(lr), 0.9, 0.999, 1e-8, self.step, 1.0 / batch,
                                           _ptr(self.wf[layer]), _ptr(self.wb[layer]), s), 'tf_sg_adam')

    # -- training -----------------------------------------------------------------
    def fit_scales(self, samples):
        """Per-variable input and target scales from the training samples."""
        dof = self.dof

        def rms(vs):
            # samples may come from grids of different sizes
            a = torch.cat([v.view(-1, dof) for v in vs]).pow(2).mean(dim=0).sqrt().cpu().numpy()
            return [float(v) if v > 1e-300 else 1.0 for v in a]
        xr = rms([s['x0'] for s in samples])
        tr = rms([s['t'] for s in samples])
        pr = rms([s['p'] if 'p' in s else torch.zeros_like(s['t']) for s in samples])
        def base(s):
            if self.residual and 'p' in s and s.get('phi'):
                return s['phi'] * s['p']
            return 0.0
        dr = rms([(s['x1'] - s['x0'] - s['ds'] * s['t']) / (s['ds'] ** 2) - base(s) for s in samples])
        mu = max(abs(s['mu']) for s in samples) or 1.0
        ds = max(abs(s['ds']) for s in samples) or 1.0
        self.scales = {'sx': [1.0 / v for v in xr], 'st': [1.0 / v for v in tr], 'sp': [1.0 / v for v in pr],
                       'sd': dr, 'mu': 1.0 / mu, 'ds': 1.0 / ds}

    def train(self, samples, dims, steps=300, lr=1e-3, batch=4, seed=0):
        """Adam on the mean-squared scaled target; returns the loss per step
        (mean over its batch), read back once at the end."""
        if not samples:
            raise ValueError('no training samples')
        samples = [self._on_device(smp) for smp in samples]
        if self.scales is None:
            self.fit_scales(samples)
        b = self._buffers(dims)
        rng = np.random.default_rng(seed)
        batch = min(batch, len(samples))
        losses = torch.zeros(steps * batch, dtype=torch.float64, device=self.device)
        scales = [self._pscale(smp.get('p'), smp.get('phi', 0.0)) for smp in samples]
        for it in range(steps):
            for j, i in enumerate(rng.choice(len(samples), size=batch, replace=False)):
                sample = samples[i]
                ps = self._pack(b, sample['x0'], sample['t'], sample['mu'], sample['ds'], sample.get('p'),
                                sample.get('phi', 0.0), scales[i])
                self._target(b, sample, ps)
                self._forward(b)
                self._backward(b, ctypes.c_void_p(losses.data_ptr() + 8 * (it * batch + j)), j > 0)
            self._adam(lr, batch)
        return losses.view(steps, batch).mean(dim=1).cpu().numpy()

    def evaluate(self, samples, dims):
        """Scaled mean-squared error of the network per sample: of the
        residual of the quadratic extrapolation relative to the quadratic
        correction (residual mode), else of the secant predictor's
        correction relative to its training RMS (1.0: the secant
        predictor's error level)."""
        if self.scales is None:
            raise RuntimeError('fit_scales() or train() sets the scales first')
        samples = [self._on_device(smp) for smp in samples]
        b = self._buffers(dims)
        out = torch.zeros(len(samples), dtype=torch.float64, device=self.device)
        for k, sample in enumerate(samples):
            ps = self._pack(b, sample['x0'], sample['t'], sample['mu'], sample['ds'], sample.get('p'),
                            sample.get('phi', 0.0))
            self._target(b, sample, ps)
            self._forward(b)
            _lib.check(self.lib.tf_sg_loss(b['ncell'], self.dof, self.np[-1], _ptr(b['z'][-1]), _ptr(b['tgt']),
                                           _ptr(b['dzf'][-1]), _ptr(b['dzh'][-1]),
                                           ctypes.c_void_p(out.data_ptr() + 8 * k), _ptr(b['lwork']),
                                           b['lwork'].numel(), _stream()), 'tf_sg_loss')
        return out.cpu().numpy()

    def calibrate_steps(self, groups, quantile=0.75):
        """Measures the predictor on samples given as ``[(dims, samples),
        ...]``: for every sample the RMS errors of the secant predictor
        (e_s), of the quadratic extrapolation alone (e_q) and of the learned
        predictor (e_l) against the converged point; ``eps`` is the given
        quantile of e_l / e_s (how much of the secant error the network
        removes, read conservatively) and ``eps_quadratic`` the same for
        e_q / e_s.  A network with eps >= 1 is not used by
        ``LearnedPredictor``.  Returns the model."""
        ratios, qratios = [], []
        for dims, g in groups:
            for smp in g:
                smp = self._on_device(smp)
                ds, p, phi = smp['ds'], smp.get('p'), smp.get('phi', 0.0)
                xs = smp['x0'] + ds * smp['t']
                xq = xs + (ds * ds * phi) * p if (p is not None and phi) else xs
                xl = self.predict(smp['x0'], smp['t'], smp['mu'], ds, dims, p, phi)
                es = float((smp['x1'] - xs).pow(2).mean().sqrt())
                eq = float((smp['x1'] - xq).pow(2).mean().sqrt())
                el = float((smp['x1'] - xl).pow(2).mean().sqrt())
                if es > 0:
                    ratios.append(el / es)
                    qratios.append(eq / es)
        if not ratios:
            raise ValueError('no samples with a nonzero secant error')
        self.step_model = {'eps': float(np.quantile(ratios, quantile)),
                           'eps_quadratic': float(np.quantile(qratios, quantile))}
        return self.step_model

    @staticmethod
    def propose_step(ds, ratio):
        """The step for a predictor whose error is ``ratio`` times the secant
        predictor's at ds and of third order in the step (the quadratic
        extrapolation's order): ds ratio^(-1/3), where its error equals the
        secant predictor's error at ds -- the step the Newton-count rule
        chose for the secant predictor -- within [1, 2] times ds (the upper
        bound of that rule's growth)."""
        if not ratio > 0 or not math.isfinite(ratio):
            return ds
        return ds * min(max(ratio ** (-1.0 / 3.0), 1.0), 2.0)

    # -- inference ------------------------------------------------------------------
    def predict(self, x, t, mu, ds, dims, p=None, phi=0.0):
        """The learned predictor x + ds t + ds^2 phi p + correction (FP64
        tensor); p is the previous step's correction per unit step squared
        (zero if None) and phi its weight in the quadratic extrapolation for
        this ds (the phi p term only when the network learns the residual)."""
        if self.scales is None:
            raise RuntimeError('the surrogate has not been trained')
        b = self._buffers(dims)
        ps = self._pack(b, x, t, mu, ds, p, phi)
        self._forward(b)
        xb = self._based(b, x, ds, p, phi)
        xp = torch.empty_like(x)
        sc = (ctypes.c_double * self.dof)(*self._out_scales(ds, ps))
        _lib.check(self.lib.tf_sg_unpack(b['ncell'], self.dof, self.np[-1], _ptr(b['z'][-1]), _ptr(xb), _ptr(t),
                                         float(ds), sc, _ptr(xp), _stream()), 'tf_sg_unpack')
        return xp


class LearnedPredictor:
    """The continuation's ``predictor`` hook over a trained surrogate: the
    state from the network, the parameter from the secant, and -- with
    ``propose_steps`` -- the step size.

    Online guard: the network predicts every step, but its prediction is
    used only when its prediction of the previous step (same step length)
    was clearly closer to the point the corrector then found than the secant
    predictor was (error below TRUST_BELOW = 0.8 of the secant's; the first
    two steps of a branch, which have no such record, use the secant).  Irregular stretches of a branch -- the first
    steps from a Stokes state, a fold -- thus fall back to the secant by
    themselves.  A network whose calibrated error is not below the secant
    predictor's (eps >= 1, ``Surrogate.calibrate_steps``) is not used.

    Step size: while the prediction is used, the step the continuation's
    Newton-count rule chose (for the secant predictor) is stretched by
    ``Surrogate.propose_step`` from the learned / secant error ratio measured
    on the last judged step, and the network predicts again at that step.
    The reference picks steps by Newton counts only (Continuation.py:197-209).
    """

    def __init__(self, surrogate, propose_steps=True):
        self.surrogate = surrogate
        self.propose_steps = propose_steps
        self.reset()

    def reset(self):
        """Forget the branch (history, guard and counts): call before the
        predictor serves another branch."""
        self.calls = 0
        self.steps_proposed = 0
        self.used = 0
        self._history = _History()
        self._last = None       # (learned, secant prediction, step) of the previous call
        self._trust = False
        # learned / secant error of every judged step (out of sample when the
        # branch's grid was not trained on)
        self.ratios = []

    # a calibrated network no better than the secant predictor is not used
    USE_BELOW = 1.0
    # the prediction is used while its last judged error was below this
    # fraction of the secant predictor's: one barely better does not pay for
    # the corrector iterations a rejected prediction costs
    TRUST_BELOW = 0.8

    def _judge(self, x0, h):
        """Compares the previous step's predictions with the point reached."""
        last, self._last = self._last, None
        if last is None or h is None:
            self._trust = False
            return
        xl, xs, step = last
        if step == 0 or abs(h / step - 1.0) > 1e-9:
            return      # the step was shortened: no comparison
        el = float((x0 - xl).pow(2).mean().sqrt())
        es = float((x0 - xs).pow(2).mean().sqrt())
        if es > 0:
            self.ratios.append(el / es)
        self._trust = el < self.TRUST_BELOW * es

    def _predict(self, x0, dx, mu0, ds, dims, p):
        xp = self.surrogate.predict(x0.data, dx.data, mu0, ds, dims, p, self._history.phi(ds))
        # the corrector may update its start in place: judge on a copy
        self._last = (xp.clone(), x0.data + ds * dx.data, ds)
        return xp

    def __call__(self, interface, x0, mu0, dx, dmu, ds):
        net = self.surrogate
        if net.scales is None:
            return None
        sm = net.step_model
        p = self._history.step(dx.data.clone(), float(mu0), dmu) if net.history else None
        if sm is not None and not sm['eps'] < self.USE_BELOW:
            return None
        self._judge(x0.data, self._history.h)
        self.calls += 1
        dims = (interface.nx, interface.ny, interface.nz)
        if self._trust and self.propose_steps and self.ratios:
            ds_new = net.propose_step(ds, self.ratios[-1])
            if abs(ds_new / ds - 1.0) > 0.05:
                self.steps_proposed += 1
                self.used += 1
                xp = self._predict(x0, dx, mu0, ds_new, dims, p)
                return DeviceVector(xp), mu0 + ds_new * dmu, ds_new
        xp = self._predict(x0, dx, mu0, ds, dims, p)
        if not self._trust:
            return None
        self.used += 1
        return DeviceVector(xp), mu0 + ds * dmu
