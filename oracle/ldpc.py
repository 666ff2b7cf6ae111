"""LDPC encoding and belief-propagation decoding (oracle side; test infrastructure only).

The reference wraps aff3ct (fec/aff3ct/ldpc.cpp: Encoder_LDPC_from_H, Decoder_LDPC_BP_flooding
with Update_rule_SPA, decode_hiho); the aff3ct sources are not part of the reference
checkout, so this module restates the published algorithms the wrapper names, in
float64 numpy. Parity against aff3ct itself is unpinned.

* ``read_alist``: MacKay's alist format (N M / max degrees / column and row degrees /
  1-based check indices per column / variable indices per row), the format of the
  reference's ``modem/resources/ofdm_ldpc.alist``.
* ``systematic``: reduced row-echelon form of H over GF(2); data bits at the non-pivot
  columns, pivot bit i = parity of row i over the data bits.
* ``decode``: flooding belief propagation, sum-product check update in the
  phi(x) = -log tanh(x / 2) form, argument clamped to [1e-6, 30]; hard input bit b ->
  channel LLR ``HARD_LLR`` (1 - 2b); syndrome stop after ``min_iterations``.
"""

from __future__ import annotations

import numpy as np


def read_alist(path: str) -> tuple[int, int, np.ndarray, np.ndarray]:
    """(N, M, edge_var, edge_chk) of the parity-check matrix in an alist file."""

    with open(path) as f:
        lines = [ln.split() for ln in f.read().splitlines() if ln.strip()]
    N, M = int(lines[0][0]), int(lines[0][1])
    ev, ec = [], []
    for v in range(N):  # one line per column, zero entries pad to the maximum degree
        for t in lines[4 + v]:
            if int(t) > 0:
                ev.append(v)
                ec.append(int(t) - 1)
    return N, M, np.asarray(ev, np.int32), np.asarray(ec, np.int32)


def dense_h(N: int, M: int, edge_var: np.ndarray, edge_chk: np.ndarray) -> np.ndarray:
    h = np.zeros((M, N), np.uint8)
    h[edge_chk, edge_var] = 1
    return h


def systematic(h: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(info positions, parity positions, rows) with parity[i] = rows[i] . data (mod 2)."""

    a = h.copy().astype(np.uint8)
    M, N = a.shape
    pivots = []
    row = 0
    for col in range(N):
        if row == M:
            break
        sel = np.nonzero(a[row:, col])[0]
        if sel.size == 0:
            continue
        r = row + sel[0]
        if r != row:
            a[[row, r]] = a[[r, row]]
        others = np.nonzero(a[:, col])[0]
        for o in others:
            if o != row:
                a[o] ^= a[row]
        pivots.append(col)
        row += 1
    info = np.array([c for c in range(N) if c not in set(pivots)], np.int32)
    rows = a[: len(pivots)][:, info]
    return info, np.asarray(pivots, np.int32), rows


def encode(h: np.ndarray, data: np.ndarray) -> np.ndarray:
    info, piv, rows = systematic(h)
    data = np.atleast_2d(np.asarray(data, np.uint8))
    code = np.zeros((data.shape[0], h.shape[1]), np.uint8)
    code[:, info] = data
    code[:, piv] = (data.astype(np.int64) @ rows.T.astype(np.int64)) % 2
    return code


HARD_LLR = 4.0  # channel LLR magnitude of a hard input bit (the engine's choice)


def hard_llr(bits: np.ndarray) -> np.ndarray:
    return HARD_LLR * (1.0 - 2.0 * np.asarray(bits, np.float64))


def _phi(x: np.ndarray) -> np.ndarray:
    x = np.clip(x, 1e-6, 30.0)
    return np.log((np.exp(x) + 1.0) / (np.exp(x) - 1.0))


def decode(h: np.ndarray, llr: np.ndarray, iterations: int, syndrome: bool = True,
           min_iterations: int = 1) -> tuple[np.ndarray, int]:
    """Hard decisions of every code bit and the iterations run, for one block of LLRs."""

    M, N = h.shape
    chk, var = np.nonzero(h)  # edges in check order
    L = np.asarray(llr, np.float64)
    v2c = L[var].copy()
    hard = (L < 0).astype(np.uint8)
    it = 0
    while it < iterations:
        c2v = np.empty_like(v2c)
        for c in range(M):
            e = np.nonzero(chk == c)[0]
            m = v2c[e]
            ph = _phi(np.abs(m))
            s = ph.sum()
            neg = np.bitwise_xor.reduce((m < 0).astype(np.int64)) if e.size else 0
            mag = _phi(np.maximum(s - ph, 0.0))
            c2v[e] = np.where(np.bitwise_xor(neg, (m < 0).astype(np.int64)) == 1, -mag, mag)
        tot = L.copy()
        np.add.at(tot, var, c2v)
        v2c = tot[var] - c2v
        hard = (tot < 0).astype(np.uint8)
        it += 1
        if syndrome and it >= min_iterations and not np.any((h.astype(np.int64) @ hard) % 2):
            break
    return hard, it
