"""OFDM place / modulate / demodulate / pick (oracle side).

Restates, for one stream, with oversampling factor 1:

* ``OrthogonalWaveform.place``   (modem/waveforms/orthogonal/waveform.py:1221-1258)
* ``OrthogonalWaveform.modulate`` (:1292-1323) with ``SymbolSection.place_samples``
  (:520-565) and ``OFDMWaveform._forward_transformation`` (ofdm.py:98-130):
  ``X / sqrt(N)`` -> DC roll -> ``ifftshift`` -> ``ifft(norm="forward")`` -> prefix.
* ``OrthogonalWaveform.demodulate`` (:1325-1364) with ``SymbolSection.pick_samples``
  (:567-614) and ``OFDMWaveform._backward_transformation`` (ofdm.py:133-161):
  strip prefix -> ``fft(norm="backward")`` -> ``fftshift`` -> DC roll -> ``* N**-0.5``.
* ``OrthogonalWaveform.pick``    (:1260-1290): data resource elements in grid order.
"""

from __future__ import annotations

import numpy as np

from .frame import FrameLayout


def place(layout: FrameLayout, data_symbols: np.ndarray, stream: int = 0) -> np.ndarray:
    """Data symbols -> (words, N) grid with reference symbols inserted (the
    stream's own under a pilot comb)."""

    data_symbols = np.asarray(data_symbols).reshape(-1)
    if data_symbols.size != layout.num_data:
        raise ValueError(
            f"Number of provided data symbols does not match the number of symbols in the frame "
            f"({data_symbols.size} != {layout.num_data})"
        )
    grid = np.zeros((layout.num_words, layout.N), dtype=np.complex128)
    grid[layout.ref_mask] = layout.stream_pilot_symbols(stream)
    grid[layout.data_mask] = data_symbols
    return grid


def modulate_grid(layout: FrameLayout, grid: np.ndarray) -> np.ndarray:
    """(words, N) grid -> frame samples (T,)."""

    n = layout.N
    spectrum = np.zeros((layout.num_words, n), dtype=np.complex128)
    spectrum[:, layout.bins()] = grid / np.sqrt(n)
    symbols = np.fft.ifft(spectrum, axis=-1, norm="forward")
    out = np.empty(layout.samples_per_frame, dtype=np.complex128)
    for w in range(layout.num_words):
        p = int(layout.prefix[w])
        s = int(layout.word_start[w])
        if p > 0:
            out[s : s + p] = 0 if layout.zero_prefix[w] else symbols[w, -p:]
        out[s + p : s + p + n] = symbols[w]
    return out


def modulate(layout: FrameLayout, data_symbols: np.ndarray, stream: int = 0) -> np.ndarray:
    return modulate_grid(layout, place(layout, data_symbols, stream))


def demodulate(layout: FrameLayout, samples: np.ndarray) -> np.ndarray:
    """Frame samples (>= T,) -> (words, N) grid."""

    n = layout.N
    windows = np.stack([samples[int(s) : int(s) + n] for s in layout.window_start])
    spectrum = np.fft.fft(windows, axis=-1, norm="backward")
    return spectrum[:, layout.bins()] * n**-0.5


def pick(layout: FrameLayout, grid: np.ndarray) -> np.ndarray:
    """Data resource elements of a (..., words, N) grid in frame order."""

    return grid[..., layout.data_mask]
