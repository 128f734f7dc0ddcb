"""CPU reference of the learned motion-vector proposer's net (test
infrastructure only: the gradient checks compare the GPU forward and backward
kernels of govid_gb300/csrc/mvnet_kernels.cu with this file).

The net has no counterpart in the reference project; this restates the
mathematics the kernels implement, in float64 numpy:

* input: two channels (current, reference luma), each the 4x4 box average
  (sum + 8) >> 4 of the padded plane, as (v - 128) / 64;
* four 3x3 convolutions with zero padding 1 (2->32->32->32->34 channels),
  ReLU after the first three; weights are used at BF16 precision and hidden
  activations are stored at BF16 (round to nearest even), as on the GPU;
* the 34 head channels are averaged over each macroblock's 4x4 pixels and
  split into 17 x and 17 y logits over displacement bins of 2 full pixels
  (-16..16); the loss is the mean over macroblocks of the two softmax
  cross-entropies against the bin of the exhaustive-search vector.

With bf16=False every rounding is skipped, which is what the
finite-difference check of the backward pass uses.
"""
from __future__ import annotations

import numpy as np

IN_CH, HIDDEN, BINS, RANGE = 2, 32, 17, 16
HEAD = 2 * BINS
SHAPES = [(HIDDEN, IN_CH), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HEAD, HIDDEN)]
N_PARAMS = sum(co * ci * 9 + co for co, ci in SHAPES)


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (u.astype(np.uint32)).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray):
    """Flat parameter vector -> [(W [co][ci][9], b [co])] per layer."""
    out, off = [], 0
    for co, ci in SHAPES:
        w = params[off: off + co * ci * 9].reshape(co, ci, 9)
        off += co * ci * 9
        b = params[off: off + co]
        off += co
        out.append((w, b))
    return out


def downsample(plane: np.ndarray) -> np.ndarray:
    h, w = plane.shape[0] // 4, plane.shape[1] // 4
    s = plane[: h * 4, : w * 4].astype(np.int64).reshape(h, 4, w, 4).sum(axis=(1, 3))
    return ((s + 8) >> 4).astype(np.float64) / 64.0 - 2.0


def bin_of(d: int) -> int:
    return min(BINS - 1, max(0, (int(d) + RANGE + 1) >> 1))


def conv(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    """x [B][ci][h][w], w [co][ci][9] -> [B][co][h][w] (zero padding 1)."""
    B, _, h, wd = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    out = np.zeros((B, w.shape[0], h, wd))
    for k in range(9):
        ky, kx = divmod(k, 3)
        out += np.einsum("oc,bchw->bohw", w[:, :, k], xp[:, :, ky: ky + h, kx: kx + wd])
    return out


def conv_wgrad(x: np.ndarray, g: np.ndarray) -> np.ndarray:
    """dW[co][ci][k] = sum g[b][co][p] * x[b][ci][p + k - 1]."""
    _, _, h, wd = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    dw = np.zeros((g.shape[1], x.shape[1], 9))
    for k in range(9):
        ky, kx = divmod(k, 3)
        dw[:, :, k] = np.einsum("bohw,bchw->oc", g, xp[:, :, ky: ky + h, kx: kx + wd])
    return dw


def conv_dgrad(g: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Gradient of conv with respect to its input."""
    B, _, h, wd = g.shape
    dxp = np.zeros((B, w.shape[1], h + 2, wd + 2))
    for k in range(9):
        ky, kx = divmod(k, 3)
        dxp[:, :, ky: ky + h, kx: kx + wd] += np.einsum("oc,bohw->bchw", w[:, :, k], g)
    return dxp[:, :, 1:-1, 1:-1]


def forward(params: np.ndarray, x0: np.ndarray, bf16: bool = True):
    """Returns (head [B][34][h][w], stored activations [x0, a1, a2, a3])."""
    rnd = bf16_round if bf16 else (lambda v: v)
    acts = [x0]
    a = x0
    layers = unpack(params)
    for i, (w, b) in enumerate(layers):
        z = conv(a, rnd(w)) + b[None, :, None, None]
        if i < len(layers) - 1:
            a = rnd(np.maximum(z, 0.0))
            acts.append(a)
        else:
            return z, acts
    raise AssertionError


def pool(head: np.ndarray) -> np.ndarray:
    """[B][34][h][w] -> per-macroblock logits [B][mbs][34] (raster order)."""
    B, C, h, w = head.shape
    p = head.reshape(B, C, h // 4, 4, w // 4, 4).mean(axis=(3, 5))
    return p.reshape(B, C, -1).transpose(0, 2, 1)


def loss_and_grads(params: np.ndarray, x0: np.ndarray, labels: np.ndarray, bf16: bool = True):
    """labels [B][mbs][2] full-pel vectors.  Returns (loss, flat gradient)."""
    rnd = bf16_round if bf16 else (lambda v: v)
    head, acts = forward(params, x0, bf16)
    B, C, h, w = head.shape
    lg = pool(head)
    n = lg.shape[0] * lg.shape[1]
    loss = 0.0
    dlg = np.zeros_like(lg)
    for a in range(2):
        z = lg[:, :, a * BINS: (a + 1) * BINS]
        m = z.max(axis=2, keepdims=True)
        lse = m + np.log(np.exp(z - m).sum(axis=2, keepdims=True))
        p = np.exp(z - lse)
        lab = np.vectorize(bin_of)(labels[:, :, a])
        onehot = np.zeros_like(p)
        np.put_along_axis(onehot, lab[:, :, None], 1.0, axis=2)
        loss += float((lse[:, :, 0] - np.take_along_axis(z, lab[:, :, None], axis=2)[:, :, 0]).sum()) / n
        dlg[:, :, a * BINS: (a + 1) * BINS] = (p - onehot) / n
    # un-pool: each of a macroblock's 16 pixels gets 1/16 of its gradient
    g = dlg.transpose(0, 2, 1).reshape(B, C, h // 4, 1, w // 4, 1)
    g = np.broadcast_to(g / 16.0, (B, C, h // 4, 4, w // 4, 4)).reshape(B, C, h, w)
    layers = unpack(params)
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        w_, _ = layers[i]
        dw = conv_wgrad(acts[i], g)
        db = g.sum(axis=(0, 2, 3))
        grads.append((dw, db))
        if i > 0:
            g = conv_dgrad(g, rnd(w_)) * (acts[i] > 0)
    grads.reverse()
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return loss, flat
