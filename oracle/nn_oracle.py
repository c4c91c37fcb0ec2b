"""CPU oracle for the surrogate network — TEST INFRASTRUCTURE ONLY.

float64 NumPy restatement of the network's layers (3x3x3 "same" convolution
with dilation, bias, ReLU, residual add, soft-target cross entropy) and of
their gradients, used to check the CUDA forward and backward kernels. The
oracle rounds activations to bfloat16 between layers where the GPU stores
bfloat16, so the remaining differences are accumulation order only.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a):
    """Round float values to the nearest bfloat16 (ties to even), as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def offsets(dil):
    return [((t // 9 - 1) * dil, ((t // 3) % 3 - 1) * dil, (t % 3 - 1) * dil) for t in range(27)]


def _shift(x, dz, dy, dx):
    """x[n, z+dz, y+dy, x+dx, c] with zeros outside (x: [N, D, H, W, C])."""
    N, D, H, W, C = x.shape
    out = np.zeros_like(x)
    zs, ze = max(0, -dz), min(D, D - dz)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ze > zs and ye > ys and xe > xs:
        out[:, zs:ze, ys:ye, xs:xe] = x[:, zs + dz:ze + dz, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv_fwd(x, w, b=None, dil=1):
    """x [N,D,H,W,Cin], w [27,Cout,Cin] -> [N,D,H,W,Cout] (float64)."""
    y = np.zeros(x.shape[:4] + (w.shape[1],))
    for t, (dz, dy, dx) in enumerate(offsets(dil)):
        y += _shift(x, dz, dy, dx) @ w[t].T
    if b is not None:
        y += b
    return y


def conv_wgrad(x, dy, dil=1):
    """dW[t][co][ci] = sum_v dy[v][co] x[v + off_t][ci]."""
    cout, cin = dy.shape[-1], x.shape[-1]
    dw = np.zeros((27, cout, cin))
    dyf = dy.reshape(-1, cout)
    for t, (dz, dyo, dx) in enumerate(offsets(dil)):
        dw[t] = dyf.T @ _shift(x, dz, dyo, dx).reshape(-1, cin)
    return dw


def conv_dgrad(dy, w, dil=1):
    """dX[u][ci] = sum_t sum_co dy[u - off_t][co] w[t][co][ci]."""
    dx = np.zeros(dy.shape[:4] + (w.shape[2],))
    for t, (dz, dyo, ddx) in enumerate(offsets(dil)):
        dx += _shift(dy @ w[t], -dz, -dyo, -ddx)
    return dx


def xent(logits, target, weight, nol):
    """Mean soft cross entropy over weighted voxels and its logits gradient."""
    z = logits[..., :nol]
    m = z.max(-1, keepdims=True)
    lse = m + np.log(np.exp(z - m).sum(-1, keepdims=True))
    q = np.exp(z - lse)
    wsum = max(weight.sum(), 1.0)
    loss = -(weight[..., None] * target * (z - lse)).sum() / wsum
    g = np.zeros_like(logits)
    g[..., :nol] = weight[..., None] * (q - target) / wsum
    return loss, g


def network_grads(x, ws, bs, dils, target, weight, nol, rounding=True):
    """Forward + backward of the surrogate network (stem, residual blocks,
    head) with bf16 rounding of stored activations and gradients and fp32
    logits, as the GPU stores them; returns (loss, logits, [dW], [db]).
    rounding=False keeps everything in float64 (exact derivatives of the
    loss, for finite-difference checks of the oracle itself)."""
    bf16_round = globals()["bf16_round"] if rounding else (lambda a: np.asarray(a, np.float64))
    acts = [x]
    a = bf16_round(np.maximum(conv_fwd(x, ws[0], bs[0]), 0))
    acts.append(a)
    for i, d in enumerate(dils):
        t = bf16_round(np.maximum(conv_fwd(a, ws[1 + 2 * i], bs[1 + 2 * i], d), 0))
        a = bf16_round(np.maximum(conv_fwd(t, ws[2 + 2 * i], bs[2 + 2 * i], d) + a, 0))
        acts += [t, a]
    logits = conv_fwd(a, ws[-1], bs[-1])
    if rounding:
        logits = logits.astype(np.float32).astype(np.float64)
    loss, dl = xent(logits, target, weight, nol)
    dl = bf16_round(dl)
    dws, dbs = [None] * len(ws), [None] * len(ws)
    dws[-1], dbs[-1] = conv_wgrad(acts[-1], dl), dl.reshape(-1, dl.shape[-1]).sum(0)
    da = bf16_round(conv_dgrad(dl, ws[-1]))
    for i in reversed(range(len(dils))):
        d = dils[i]
        a_in, t, a_out = acts[1 + 2 * i], acts[2 + 2 * i], acts[3 + 2 * i]
        g = bf16_round(np.where(a_out > 0, da, 0.0))
        dws[2 + 2 * i], dbs[2 + 2 * i] = conv_wgrad(t, g, d), g.reshape(-1, g.shape[-1]).sum(0)
        dt = bf16_round(conv_dgrad(g, ws[2 + 2 * i], d))
        dt = bf16_round(np.where(t > 0, dt, 0.0))
        dws[1 + 2 * i], dbs[1 + 2 * i] = conv_wgrad(a_in, dt, d), dt.reshape(-1, dt.shape[-1]).sum(0)
        da = bf16_round(conv_dgrad(dt, ws[1 + 2 * i], d) + g)
    g0 = bf16_round(np.where(acts[1] > 0, da, 0.0))
    dws[0], dbs[0] = conv_wgrad(acts[0], g0), g0.reshape(-1, g0.shape[-1]).sum(0)
    return loss, logits, dws, dbs
