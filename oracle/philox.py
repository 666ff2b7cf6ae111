"""Philox4x32-10 in numpy (oracle side).

Philox is the counter-based generator of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC'11). One call maps a
128-bit counter and a 64-bit key to 128 random bits through ten rounds of

    (hi0, lo0) = mulhilo32(M0, c0); (hi1, lo1) = mulhilo32(M1, c2)
    c = (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0)
    k = (k0 + W0, k1 + W1)            (between rounds)

The engine's device implementation must produce identical words; the tests
check both against the published known-answer vectors.
"""

from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)
_SHIFT = np.uint64(32)


def philox4x32(counters: np.ndarray, key, rounds: int = 10) -> np.ndarray:
    """Apply Philox4x32-``rounds`` to an (n, 4) uint32 counter array.

    Args:
        counters: (n, 4) array of uint32 counter words (c0, c1, c2, c3).
        key: pair of uint32 key words (k0, k1).
        rounds: number of rounds (10 for Philox4x32-10).

    Returns: (n, 4) uint32 array of output words.
    """

    c = np.array(counters, dtype=np.uint32, copy=True).reshape(-1, 4)
    c0, c1, c2, c3 = (c[:, i].astype(np.uint64) for i in range(4))
    k0 = np.uint32(key[0])
    k1 = np.uint32(key[1])
    for r in range(rounds):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> _SHIFT, p0 & _MASK
        hi1, lo1 = p1 >> _SHIFT, p1 & _MASK
        c0 = hi1 ^ c1 ^ np.uint64(k0)
        c1 = lo1
        c2 = hi0 ^ c3 ^ np.uint64(k1)
        c3 = lo0
        if r + 1 < rounds:
            with np.errstate(over="ignore"):
                k0 = np.uint32(k0 + W0)
                k1 = np.uint32(k1 + W1)
    out = np.stack([c0, c1, c2, c3], axis=1).astype(np.uint32)
    return out


def seed_key(seed: int) -> tuple[int, int]:
    """Split a 64-bit campaign seed into the two Philox key words."""

    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return seed & 0xFFFFFFFF, seed >> 32
