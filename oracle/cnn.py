"""Residual CNN channel estimator (oracle side, float64 accumulation).

TEST INFRASTRUCTURE ONLY. The learned estimator has no counterpart in the
reference; this restates the engine's definition of its inference
(``hpx_cnn_refine``) in numpy with the engine's BF16 rounding points, so that the
learned link's BER can be checked against an independent CPU computation on the
same drops:

    s   = sqrt(mean |LS|^2) over the 16 antenna pairs, words and used columns
    x0  = bf16(LS / s) as 32 channels (pair p -> channels 2p = re, 2p + 1 = im)
    h_l = bf16(relu(conv3x3(h_{l-1}; bf16(W_l)) + b_l)),  l = 1..5
    out = LS + s (conv3x3(h_5; bf16(W_6)) + b_6)

Each conv3x3 is zero-padded over (word, column); weights are laid out
[layer][32 out][9 taps][32 in] with tap = 3 dy + dx, dy along words and dx along
columns, followed by the biases [layer][32] (the engine's parameter vector).
Products and sums run in float64 here (FP32 accumulation on the tensor cores), so
the two differ only by accumulation rounding.
"""

from __future__ import annotations

import numpy as np

LAYERS, CHANNELS, PAIRS = 6, 32, 16


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""

    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32)
    r = ((a >> 16) & np.uint32(1)) + np.uint32(0x7FFF)
    return ((a + r) & np.uint32(0xFFFF0000)).view(np.float32)


def split(params: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(weights [6][32][9][32] rounded to bf16, biases [6][32]) of a parameter vector."""

    p = np.asarray(params, dtype=np.float32).reshape(-1)
    nw = LAYERS * CHANNELS * 9 * CHANNELS
    w = bf16(p[:nw]).reshape(LAYERS, CHANNELS, 9, CHANNELS)
    return w.astype(np.float64), p[nw:].reshape(LAYERS, CHANNELS).astype(np.float64)


def conv3x3(x: np.ndarray, w: np.ndarray, b: np.ndarray) -> np.ndarray:
    """x (H, W, 32) -> (H, W, 32): zero-padded 3x3 convolution plus bias."""

    H, W, _ = x.shape
    xp = np.zeros((H + 2, W + 2, CHANNELS))
    xp[1:-1, 1:-1] = x
    cols = np.concatenate([xp[dy:dy + H, dx:dx + W] for dy in range(3) for dx in range(3)], axis=2)
    return cols @ w.reshape(CHANNELS, 9 * CHANNELS).T + b


def refine(params: np.ndarray, ls: np.ndarray) -> np.ndarray:
    """(Nrx, Ntx, words, C) LS estimate of a 4 x 4 link -> refined estimate (same shape)."""

    w, b = split(params)
    nrx, ntx, H, W = ls.shape
    z = ls.reshape(nrx * ntx, H, W)
    if z.shape[0] != PAIRS:
        raise ValueError("the network refines 16 antenna pairs")
    s = np.sqrt(np.sum(np.abs(z) ** 2) / (PAIRS * H * W))
    x = np.empty((H, W, CHANNELS))
    x[..., 0::2] = np.moveaxis(z.real, 0, 2)
    x[..., 1::2] = np.moveaxis(z.imag, 0, 2)
    h = bf16(x / s).astype(np.float64)
    for layer in range(LAYERS - 1):
        h = bf16(np.maximum(conv3x3(h, w[layer], b[layer]), 0.0)).astype(np.float64)
    d = conv3x3(h, w[-1], b[-1]) * s
    out = z + np.moveaxis(d[..., 0::2] + 1j * d[..., 1::2], 2, 0)
    return out.reshape(ls.shape)
