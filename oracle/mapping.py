"""3GPP Gray PSK/QAM mapping and hard demapping (oracle side).

Restates ``PskQamMapping`` (modem/tools/psk_qam_mapping.py):

* ``get_symbols``  follows :104-169 with the PAM amplitude rules of
  ``generate_pam_symbol_3gpp`` (:261-298).
* ``detect_bits``  follows :171-259 with the piecewise-linear LLRs of
  ``get_llr_3gpp`` (:300-497); a hard bit is ``llr > 0`` (:259), so an LLR of
  exactly zero (a tie on a decision boundary) and any NaN give bit 0.
* ``get_mapping``  follows :499-525.

Only the default complex constellations used on the OFDM path are restated:
BPSK (2), QPSK (4), 16-, 64- and 256-QAM.
"""

from __future__ import annotations

import numpy as np

SUPPORTED_ORDERS = (2, 4, 16, 64, 256)
_SCALE = {2: 1.0, 4: np.sqrt(2), 16: np.sqrt(10), 64: np.sqrt(42), 256: np.sqrt(170)}


def bits_per_symbol(order: int) -> int:
    if order not in SUPPORTED_ORDERS:
        raise ValueError(f"Unsupported modulation order ({order})")
    return int(np.log2(order))


def pam_3gpp(order: int, bits: np.ndarray) -> np.ndarray:
    """PAM amplitudes of ``generate_pam_symbol_3gpp`` (psk_qam_mapping.py:261-298)."""

    b = bits.astype(np.float64)
    if order == 2:
        return 1.0 - 2 * b[0]
    if order == 4:
        return (1 - 2 * b[0]) * (1 + 2 * b[1])
    if order == 8:
        return (2 * b[0] - 1) * ((1 - 2 * b[1]) * (1 + 2 * b[2]) - 4)
    if order == 16:
        return ((((1 - 2 * b[2]) * (1 + 2 * b[3]) - 4) * (-1 + 2 * b[1])) - 8) * (-1 + 2 * b[0])
    raise ValueError(order)


def get_symbols(order: int, bits: np.ndarray) -> np.ndarray:
    """Map MSB-first bit groups to unit-energy symbols (psk_qam_mapping.py:104-169)."""

    m = bits_per_symbol(order)
    bits = np.asarray(bits, dtype=np.uint8).reshape(-1)
    k = bits.size // m
    sb = bits[: k * m].reshape((m, k), order="F")
    if order == 2:
        return pam_3gpp(2, sb) + 0j
    if order == 4:
        return (pam_3gpp(2, sb[0:1]) + 1j * pam_3gpp(2, sb[1:2])) / np.sqrt(2)
    half = m // 2
    re = pam_3gpp(2**half, sb[0::2])
    im = pam_3gpp(2**half, sb[1::2])
    return (re + 1j * im) / _SCALE[order]


def get_mapping(order: int) -> np.ndarray:
    """Constellation in symbol-index order (psk_qam_mapping.py:499-525)."""

    m = bits_per_symbol(order)
    idx = np.arange(order)
    bits = ((idx[:, None] >> (m - 1 - np.arange(m))[None, :]) & 1).astype(np.uint8)
    return get_symbols(order, bits.reshape(-1))


def _llr_pam(order: int, r: np.ndarray) -> np.ndarray:
    """Piecewise-linear LLRs of ``get_llr_3gpp`` (psk_qam_mapping.py:331-497),
    complex case, unit noise variance. Returns (bits, K)."""

    nv = 1.0
    r = r * np.sqrt(2)
    band = np.bitwise_and
    with np.errstate(invalid="ignore"):
        if order == 2:
            return (-2 * r / nv)[None, :] / 2
        if order == 4:
            r = r * np.sqrt(5)
            llr = np.zeros([2, r.size])
            llr[0] = 2 * ((r <= -2) * (-4 * (1 + r)) + np.logical_and(r > -2, r <= 2) * (-2 * r)
                          + (r > 2) * (4 * (1 - r))) / nv
            llr[1] = 2 * ((r <= 0) * (-2 * (2 + r)) + (r > 0) * (-2 * (2 - r))) / nv
            return llr / 5 / 2
        if order == 8:
            r = r * np.sqrt(21)
            llr = np.zeros([3, r.size])
            llr[0] = 4 * ((r <= -6) * (-4 * (3 + r)) + band(r > -6, r <= -4) * (-3 * (2 + r))
                          + band(r > -4, r <= -2) * (-2 * (1 + r)) + band(r > -2, r <= 2) * (-r)
                          + band(r > 2, r <= 4) * (2 * (1 - r)) + band(r > 4, r <= 6) * (3 * (2 - r))
                          + (r > 6) * (4 * (3 - r))) / nv
            llr[1] = 4 * ((r <= -6) * (-2 * (5 + r)) + band(r > -6, r <= -2) * (-(4 + r))
                          + band(r > -2, r <= 0) * (-2 * (3 + r)) + band(r > 0, r <= 2) * (-2 * (3 - r))
                          + band(r > 2, r <= 6) * (-(4 - r)) + (r > 6) * (-2 * (5 - r))) / nv
            llr[2] = 4 * ((r <= -4) * (-(6 + r)) + band(r > -4, r <= 0) * (2 + r)
                          + band(r > 0, r <= 4) * (2 - r) + (r > 4) * (-(6 - r))) / nv
            return llr / 21 / 2
        if order == 16:
            r = r * np.sqrt(85)
            llr = np.zeros([4, r.size])
            llr[0] = 8 * ((r <= -14) * (-4 * (7 + r)) - band(r > -14, r <= -12) * 3.5 * (6 + r)
                          - band(r > -12, r <= -10) * 3 * (5 + r) - band(r > -10, r <= -8) * 2.5 * (4 + r)
                          - band(r > -8, r <= -6) * 2 * (3 + r) - band(r > -6, r <= -4) * 1.5 * (2 + r)
                          - band(r > -4, r <= -2) * (1 + r) - band(r > -2, r <= 2) * 0.5 * r
                          + band(r > 2, r <= 4) * (1 - r) + band(r > 4, r <= 6) * 1.5 * (2 - r)
                          + band(r > 6, r <= 8) * 2 * (3 - r) + band(r > 8, r <= 10) * 2.5 * (4 - r)
                          + band(r > 10, r <= 12) * 3 * (5 - r) + band(r > 12, r <= 14) * 3.5 * (6 - r)
                          + (r > 14) * 4 * (7 - r)) / nv
            llr[1] = 8 * ((r <= -14) * (-2 * (11 + r)) - band(r > -14, r <= -12) * 1.5 * (10 + r)
                          - band(r > -12, r <= -10) * (9 + r) - band(r > -10, r <= -6) * 0.5 * (8 + r)
                          - band(r > -6, r <= -4) * (7 + r) - band(r > -4, r <= -2) * 1.5 * (6 + r)
                          - band(r > -2, r <= 0) * 2 * (5 + r) - band(r > 0, r <= 2) * 2 * (5 - r)
                          - band(r > 2, r <= 4) * 1.5 * (6 - r) - band(r > 4, r <= 6) * (7 - r)
                          - band(r > 6, r <= 10) * 0.5 * (8 - r) - band(r > 10, r <= 12) * (9 - r)
                          - band(r > 12, r <= 14) * 1.5 * (10 - r) - (r > 14) * 2 * (11 - r)) / nv
            llr[2] = 8 * ((r <= -14) * (-13 - r) - band(r > -14, r <= -10) * 0.5 * (12 + r)
                          - band(r > -10, r <= -8) * (11 + r) + band(r > -8, r <= -6) * (5 + r)
                          + band(r > -6, r <= -2) * 0.5 * (4 + r) + band(r > -2, r <= 0) * (3 + r)
                          + band(r > 0, r <= 2) * (3 - r) + band(r > 2, r <= 6) * 0.5 * (4 - r)
                          + band(r > 6, r <= 8) * (5 - r) - band(r > 8, r <= 10) * (11 - r)
                          - band(r > 10, r <= 14) * 0.5 * (12 - r) - (r > 14) * (13 - r)) / nv
            llr[3] = 8 * ((r <= -12) * (-0.5 * (14 + r)) + band(r > -12, r <= -8) * 0.5 * (10 + r)
                          - band(r > -8, r <= -4) * 0.5 * (6 + r) + band(r > -4, r <= 0) * 0.5 * (2 + r)
                          + band(r > 0, r <= 4) * 0.5 * (2 - r) - band(r > 4, r <= 8) * 0.5 * (6 - r)
                          + band(r > 8, r <= 12) * 0.5 * (10 - r) - (r > 12) * 0.5 * (14 - r)) / nv
            return llr / 85 / 2
    raise ValueError(order)


def detect_bits(order: int, symbols: np.ndarray) -> np.ndarray:
    """Hard-decision bits (uint8) of ``PskQamMapping.detect_bits`` (psk_qam_mapping.py:171-259)."""

    m = bits_per_symbol(order)
    s = np.asarray(symbols, dtype=np.complex128).reshape(-1)
    llr = np.zeros(s.size * m)
    if order == 2:
        # BPSK: real-valued 2-PAM without the complex sqrt(2) scaling (:229-231)
        with np.errstate(invalid="ignore"):
            llr = -2 * np.real(s) / 1.0
    elif order == 4:
        llr[0::2] = _llr_pam(2, np.real(s)).ravel("F")
        llr[1::2] = _llr_pam(2, np.imag(s)).ravel("F")
    else:
        pam = 2 ** (m // 2)
        llr[0::2] = _llr_pam(pam, np.real(s)).ravel("F")
        llr[1::2] = _llr_pam(pam, np.imag(s)).ravel("F")
    return (llr > 0).astype(np.uint8)
