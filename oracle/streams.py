"""The engine's random-stream layout, restated in numpy.

Every random quantity of a drop is a pure function of (campaign seed, drop
index, stream id, element index) through Philox4x32-10, so the engine can
regenerate any draw anywhere (bits are regenerated by the detector instead of
being stored) and the oracle can reproduce every draw exactly.

Counter layout of one Philox call: ``c0`` = block index, ``c1`` = stream id
(antenna / data stream), ``c2`` = drop index (low 32 bits), ``c3`` = domain in
the low byte and drop index bits 32..55 above it. The key is the 64-bit
campaign seed.

Domains
-------
BITS    Data bits. Packed 32-bit word ``j`` of stream ``s`` is output word
        ``j % 4`` of block ``j // 4``; bit ``b`` is bit ``b % 32`` of word ``b // 32``.
        Replaces ``RandomBitsSource.generate_bits`` (modem/bits_source.py:62-63):
        iid Bernoulli(1/2) bits, stream ``s`` taking the ``s``-th contiguous chunk
        as in ``TransmittingModemBase.__map`` (modem/modem.py:747-763).
FADING  The uniforms of one fading realization, ``u = (w + 0.5) * 2**-32``.
        Replaces ``ConsistentGenerator.realize`` with infinite decorrelation
        distance (channel/consistent.py:431-432) followed by
        ``ConsistentUniform.sample`` (:475-485), whose output is uniform on (0, 1).
NOISE   Complex AWGN sample ``k`` of receive antenna ``r`` is a Box-Muller pair
        from words (0, 1) (``k`` even) or (2, 3) (``k`` odd) of block ``k // 2``.
        Replaces ``AWGNRealization.add_to`` (simulation/rf/noise/model.py:143-160).
"""

from __future__ import annotations

import numpy as np

from .philox import philox4x32, seed_key

DOMAIN_BITS = 1
DOMAIN_FADING = 2
DOMAIN_NOISE = 3

_TWO_M32 = 2.0**-32


def _counters(blocks: np.ndarray, stream: int, drop: int, domain: int) -> np.ndarray:
    blocks = np.asarray(blocks, dtype=np.uint64)
    c = np.empty((blocks.size, 4), dtype=np.uint32)
    c[:, 0] = (blocks & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    c[:, 1] = np.uint32(stream)
    c[:, 2] = np.uint32(int(drop) & 0xFFFFFFFF)
    c[:, 3] = np.uint32((domain & 0xFF) | (((int(drop) >> 32) & 0xFFFFFF) << 8))
    return c


def words(seed: int, drop: int, stream: int, domain: int, num_words: int) -> np.ndarray:
    """First ``num_words`` 32-bit output words of one (drop, stream, domain) sequence."""

    num_blocks = (num_words + 3) // 4
    out = philox4x32(_counters(np.arange(num_blocks), stream, drop, domain), seed_key(seed))
    return out.reshape(-1)[:num_words]


def data_bits(seed: int, drop: int, stream: int, num_bits: int) -> np.ndarray:
    """uint8 0/1 data bits of one transmit stream."""

    w = words(seed, drop, stream, DOMAIN_BITS, (num_bits + 31) // 32)
    bits = (w[:, None] >> np.arange(32, dtype=np.uint32)[None, :]) & np.uint32(1)
    return bits.reshape(-1)[:num_bits].astype(np.uint8)


def fading_uniforms(seed: int, drop: int, num: int) -> np.ndarray:
    """float64 uniforms on (0, 1) of one fading realization."""

    w = words(seed, drop, 0, DOMAIN_FADING, num)
    return (w.astype(np.float64) + 0.5) * _TWO_M32


def noise_normals(seed: int, drop: int, antenna: int, num_samples: int) -> np.ndarray:
    """Unit-variance-per-dimension complex normals (re, im ~ N(0, 1)) of one antenna."""

    num_blocks = (num_samples + 1) // 2
    w = philox4x32(_counters(np.arange(num_blocks), antenna, drop, DOMAIN_NOISE), seed_key(seed))
    pairs = w.reshape(-1, 2)[:num_samples]  # (w0,w1), (w2,w3), ...
    u1 = (pairs[:, 0].astype(np.float64) + 0.5) * _TWO_M32
    u2 = (pairs[:, 1].astype(np.float64) + 0.5) * _TWO_M32
    r = np.sqrt(-2.0 * np.log(u1))
    return r * np.cos(2 * np.pi * u2) + 1j * r * np.sin(2 * np.pi * u2)


def awgn(seed: int, drop: int, num_antennas: int, num_samples: int, power: float) -> np.ndarray:
    """AWGN of total power ``power`` per complex sample, shape (antennas, samples)."""

    n = np.stack([noise_normals(seed, drop, r, num_samples) for r in range(num_antennas)])
    return np.sqrt(0.5 * power) * n
