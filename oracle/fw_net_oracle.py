"""CPU reference of the learned coarse-grid correction network (test
infrastructure: only the tests use it, to check the GPU's forward pass and
gradients).  numpy, channels-last, the same architecture, padding and
parameter layout as funwave-tvd_gb300/csrc/fw_learn.cu:

  input (eta, u, v, depth/10, MASK) padded to 8 channels -> conv3x3 32 ReLU
  -> conv3x3 32 ReLU -> conv3x3 32 ReLU -> conv3x3 3

with weights w[9][cin][cout] (tap k = (ky+1)*3 + (kx+1) reads (x+kx, y+ky)),
then b[cout], per layer.  With bf16=True the weights, the packed input and
the hidden activations are rounded to BF16 (round to nearest even) as the
GPU stores them, and the convolutions accumulate in float32 (bias, then
taps, then input channels; the tensor cores add in another order, which the
tests' tolerances cover).  The backward pass runs in float64 on the stored
values and rounds, as the GPU stores them, the output gradient and each
hidden activation's gradient (with its ReLU mask applied) to BF16.  With
bf16=False everything is float64, for finite-difference checks.

No reference counterpart: the network is an extension of the reference.
"""
import numpy as np

LAYERS = [(8, 32, True), (32, 32, True), (32, 32, True), (32, 3, False)]
NIN = 5


def bf16_round(a):
    """float32 values rounded to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def num_params():
    return sum(9 * ci * co + co for ci, co, _ in LAYERS)


def unpack(params):
    out, off = [], 0
    for ci, co, relu in LAYERS:
        w = params[off:off + 9 * ci * co].reshape(9, ci, co)
        off += 9 * ci * co
        b = params[off:off + co]
        off += co
        out.append((w, b, relu))
    return out


def _shift(x, kx, ky):
    """x[b, y+ky, x+kx, :] with zeros outside (x: [B, H, W, C])."""
    B, H, W, C = x.shape
    out = np.zeros_like(x)
    ys = slice(max(0, -ky), min(H, H - ky))
    xs = slice(max(0, -kx), min(W, W - kx))
    yd = slice(max(0, ky), min(H, H + ky))
    xd = slice(max(0, kx), min(W, W + kx))
    out[:, ys, xs, :] = x[:, yd, xd, :]
    return out


def forward(params, x, bf16=True):
    """x: [B, H, W, 5] -> (y [B, H, W, 3], stored activations per layer input)."""
    B, H, W, _ = x.shape
    a = np.zeros((B, H, W, 8), dtype=np.float32 if bf16 else np.float64)
    a[..., :NIN] = x
    if bf16:
        a = bf16_round(a)
    acts = []
    for w, b, relu in unpack(params):
        acts.append(a)
        if bf16:
            wq = bf16_round(w).astype(np.float32)
            acc = np.broadcast_to(b.astype(np.float32), (B, H, W, w.shape[2])).copy()
            for k in range(9):
                kx, ky = k % 3 - 1, k // 3 - 1
                xs = _shift(a, kx, ky)
                for ci in range(w.shape[1]):
                    acc = (acc + xs[..., ci:ci + 1] * wq[k, ci][None, None, None, :]).astype(np.float32)
        else:
            acc = np.broadcast_to(b, (B, H, W, w.shape[2])).astype(np.float64).copy()
            for k in range(9):
                kx, ky = k % 3 - 1, k // 3 - 1
                acc += _shift(a, kx, ky) @ w[k].astype(np.float64)
        if relu:
            acc = np.maximum(acc, 0.0)
            a = bf16_round(acc) if bf16 else acc
        else:
            a = acc
    return a, acts


def loss_grad(params, x, target, wmask, bf16=True):
    """Masked MSE sum(w (y-t)^2) / (B*H*W) and its gradient w.r.t. params."""
    y, acts = forward(params, x, bf16)
    n = y.shape[0] * y.shape[1] * y.shape[2]
    d = y.astype(np.float64) - target
    loss = float(np.sum(wmask[..., None] * d * d) / n)
    dy = 2.0 * wmask[..., None] * d / n
    if bf16:
        dy = bf16_round(dy.astype(np.float32)).astype(np.float64)
    grads = []
    layers = unpack(params)
    for li in range(len(layers) - 1, -1, -1):
        w, b, relu = layers[li]
        wq = bf16_round(w).astype(np.float64) if bf16 else w.astype(np.float64)
        xin = acts[li].astype(np.float64)
        gw = np.zeros_like(wq)
        dx = np.zeros_like(xin)
        for k in range(9):
            kx, ky = k % 3 - 1, k // 3 - 1
            xs = _shift(xin, kx, ky)
            gw[k] = np.einsum("bhwc,bhwo->co", xs, dy)
            # the output at q read the input at q + (kx, ky)
            dx += _shift(dy @ wq[k].T, -kx, -ky)
        gb = dy.sum(axis=(0, 1, 2))
        grads.append(np.concatenate([gw.ravel(), gb]))
        if li > 0:
            prev_relu = layers[li - 1][2]
            dy = dx * (acts[li] > 0) if prev_relu else dx
            if bf16:
                dy = bf16_round(dy.astype(np.float32)).astype(np.float64)
    g = np.concatenate(grads[::-1])
    # the padding input channels carry no gradient
    w0 = g[:9 * 8 * 32].reshape(9, 8, 32)
    w0[:, NIN:, :] = 0.0
    return loss, g
