"""Frame synchronization and preambles (oracle side; test infrastructure only).

Restates with numpy / scipy, oversampling factor 1:

* ``PilotSection._pilot_sequence`` / ``generate`` (modem/waveforms/orthogonal/
  waveform.py:822-878): the frame mapping's symbols of ``default_rng(50)`` bits,
  transformed like a data word without prefix (ofdm.py:98-130).
* ``SchmidlCoxPilotSection._pilot_sequence`` (ofdm.py:190-205): those symbols on
  every second subcarrier, the lower half rolled by one under DC suppression.
* ``SchmidlCoxSynchronization.synchronize`` (ofdm.py:226-257): delay metric
  ``sum_s |sum_k conj(x[d+k]) x[d+k+N/2]|`` with a leading zero, ``find_peaks``
  at 0.75 of the maximum and 0.9 frames apart, indices minus one.
* ``CorrelationSynchronization.synchronize``
  (modem/waveform_correlation_synchronization.py:119-170): stream-summed
  ``|correlate(x, pilot, "full")|``, normalized, ``find_peaks`` at 0.9 and 0.8
  frames apart, shifted by the pilot length and clipped into the signal.
"""

from __future__ import annotations

import numpy as np
from numpy.lib.stride_tricks import sliding_window_view
from scipy.signal import correlate, find_peaks

from . import mapping


def forward_transform(symbols: np.ndarray, dc_suppression: bool) -> np.ndarray:
    """One OFDM symbol of N subcarriers -> N samples (ofdm.py:98-130, oversampling 1)."""

    n = symbols.shape[-1]
    x = np.asarray(symbols, dtype=np.complex128) / np.sqrt(n)
    if dc_suppression:
        dc = int(0.5 * n)
        x = x.copy()
        x[dc:] = np.roll(x[dc:], 1)
    return np.fft.ifft(np.fft.ifftshift(x), n, norm="forward")


def pilot_sequence(order: int, num_symbols: int) -> np.ndarray:
    rng = np.random.default_rng(50)
    bits = rng.integers(0, 2, num_symbols * mapping.bits_per_symbol(order), np.uint8).flatten()
    return mapping.get_symbols(order, bits)[:num_symbols]


def schmidl_cox_sequence(order: int, n: int, dc_suppression: bool) -> np.ndarray:
    stuffed = np.zeros(n, dtype=np.complex128)
    stuffed[::2] = pilot_sequence(order, int(np.ceil(0.5 * n)))
    if dc_suppression:
        dc = int(0.5 * n)
        stuffed[:dc] = np.roll(stuffed[:dc], 1)
    return stuffed


def preamble(order: int, n: int, dc_suppression: bool, schmidl_cox: bool) -> np.ndarray:
    seq = schmidl_cox_sequence(order, n, dc_suppression) if schmidl_cox else pilot_sequence(order, n)
    return forward_transform(seq, dc_suppression)


def schmidl_cox_metric(signal: np.ndarray, symbol_length: int) -> np.ndarray:
    """The reference's ``delay_powers`` (length n - L + 2, first entry 0)."""

    x = np.atleast_2d(np.asarray(signal, dtype=np.complex128))
    n = x.shape[1]
    half = int(0.5 * symbol_length)
    nd = n - symbol_length + 1
    prod = x[:, : n - half].conj() * x[:, half:]
    windows = sliding_window_view(prod, half, axis=1)[:, :nd].sum(axis=-1)
    return np.concatenate([[0.0], np.abs(windows).sum(axis=0)])


def schmidl_cox_synchronize(signal: np.ndarray, symbol_length: int, samples_per_frame: int) -> list[int]:
    x = np.atleast_2d(signal)
    if x.shape[1] < symbol_length:
        return []
    powers = schmidl_cox_metric(x, symbol_length)
    peaks, _ = find_peaks(powers, distance=int(0.9 * samples_per_frame), height=0.75 * np.max(powers))
    return (peaks - 1).tolist()


def correlation_profile(signal: np.ndarray, pilot: np.ndarray) -> np.ndarray:
    x = np.atleast_2d(np.asarray(signal, dtype=np.complex128))
    out = np.zeros(len(pilot) + x.shape[1] - 1)
    for stream in x:
        out += np.abs(correlate(stream, pilot, mode="full", method="direct"))
    return out


def correlation_synchronize(signal: np.ndarray, pilot: np.ndarray, frame_length: int) -> list[int]:
    x = np.atleast_2d(signal)
    corr = correlation_profile(x, pilot)
    corr /= corr.max()
    idx, _ = find_peaks(np.abs(corr), height=0.9, distance=int(0.8 * frame_length))
    if len(idx) < 1:
        return []
    idx = idx - (len(pilot) - 1)
    idx = np.where(idx < 0, 0, idx)
    idx = np.where(idx > (x.shape[1] - frame_length), abs(x.shape[1] - frame_length), idx)
    return idx.tolist()
