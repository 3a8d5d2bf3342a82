"""CPU oracle of the learned continuation predictor.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker of the GPU
network kernels, never by the ``transiflow_gb300`` package.

The predictor has no counterpart in the reference (its continuation uses the
secant predictor only, transiflow/Continuation.py:258-260); the gradient
oracle for its kernels is PyTorch's CPU convolution and autograd in FP32,
with the BF16 rounding the GPU kernels apply to weights and activations
reproduced by straight-through rounding (forward values rounded, gradients
passed unchanged).

Layouts follow the GPU kernels: activations ``[cell][channel]`` with
``cell = i + nx*(j + ny*k)``; weights ``w[tap][ci][co]`` with
``tap = (ox+1) + 3*(oy+1) + 9*(oz+1)``; a convolution computes
``z[c][co] = sum_tap sum_ci x[c + off(tap)][ci] * w[tap][ci][co] + b[co]``
with zero padding outside the grid.
"""

import numpy as np
import torch
import torch.nn.functional as F

__all__ = ['bf16', 'bf16_st', 'conv', 'conv_loops', 'forward', 'loss_and_grads']


def bf16(t):
    """Round to the nearest BF16 value (ties to even), returned as FP32."""
    return t.to(torch.bfloat16).to(torch.float32)


def bf16_st(t):
    """BF16 rounding in the forward pass, identity in the backward pass."""
    return t + (bf16(t) - t).detach()


def conv(x, w, b, dims):
    """One 3x3x3 convolution in the kernels' layouts (x [ncell, kp], w [27,
    kp, np], b [np] or None) through torch's conv3d."""
    nx, ny, nz = dims
    kp, np_ = w.shape[1], w.shape[2]
    xi = x.t().reshape(1, kp, nz, ny, nx)
    wt = w.reshape(3, 3, 3, kp, np_).permute(4, 3, 0, 1, 2)   # [co, ci, oz, oy, ox]
    z = F.conv3d(xi, wt, bias=b, padding=1)
    return z.reshape(np_, nx * ny * nz).t()


def conv_loops(x, w, b, dims):
    """The same convolution by explicit loops over cells and taps (NumPy);
    pins the tap and cell conventions of ``conv`` on small grids."""
    nx, ny, nz = dims
    x = np.asarray(x, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    z = np.zeros((nx * ny * nz, w.shape[2]))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                c = i + nx * (j + ny * k)
                for tap in range(27):
                    a, bb, cc = i + tap % 3 - 1, j + (tap // 3) % 3 - 1, k + tap // 9 - 1
                    if 0 <= a < nx and 0 <= bb < ny and 0 <= cc < nz:
                        z[c] += x[a + nx * (bb + ny * cc)] @ w[tap]
    if b is not None:
        z += np.asarray(b, dtype=np.float64)
    return z


def forward(x0, weights, biases, dims):
    """The network: BF16 weights, FP32 accumulation, ReLU between layers with
    the activations rounded to BF16, the last layer linear.  Returns the last
    layer's FP32 output [ncell, np_last]."""
    a = bf16_st(x0)
    n = len(weights)
    for layer, (w, b) in enumerate(zip(weights, biases)):
        z = conv(a, bf16_st(w), b, dims)
        if layer < n - 1:
            a = bf16_st(torch.relu(z))
        else:
            return z


def loss_and_grads(x0, tgt, weights, biases, dims, dof):
    """Mean-squared loss over the first ``dof`` output channels and its
    gradients with respect to every weight and bias (CPU autograd)."""
    ws = [w.detach().clone().requires_grad_(True) for w in weights]
    bs = [b.detach().clone().requires_grad_(True) for b in biases]
    out = forward(x0, ws, bs, dims)
    loss = ((out[:, :dof] - tgt) ** 2).mean()
    loss.backward()
    return float(loss.detach()), [w.grad for w in ws], [b.grad for b in bs]
