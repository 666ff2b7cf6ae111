"""OFDM resource-grid description (oracle side).

Restates the grid bookkeeping of the reference's orthogonal waveforms
(modem/waveforms/orthogonal/waveform.py):

* ``GridResource.mask``             :205-222  element masks, repeated along frequency
* ``SymbolSection.resource_mask``   :616-624  per-word masks from the pattern
* ``SymbolSection.num_samples``     :626-635  N + int(N * prefix_ratio) per word
* ``OrthogonalWaveform.resource_mask`` :1196-1211  frame mask over (words, N)
* ``GridSection.place_symbols``     :357-376  ``grid[mask] = symbols`` (row-major order)
* ``ConfigurablePilotWaveform.pilot_symbols`` (modem/waveform.py:797-820) with
  ``MappedPilotSymbolSequence`` (:748-758): reference symbol ``k`` is constellation
  point ``k mod M`` in ``get_mapping`` order.

Only symbol sections without sample offset and without a preamble pilot
section are described (the configurations of the hot path use neither).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import mapping

NULL, REFERENCE, DATA = 2, 0, 1  # ElementType values (waveform.py:39-49)


@dataclass
class Resource:
    """``GridResource`` (waveform.py:96-238)."""

    repetitions: int = 1
    prefix_ratio: float = 0.0
    elements: list = field(default_factory=list)  # [(ElementType value, repetitions)]
    prefix_type: str = "CYCLIC"  # CYCLIC | ZEROPAD | NONE

    @property
    def num_subcarriers(self) -> int:
        return self.repetitions * sum(r for _, r in self.elements)

    def mask(self) -> np.ndarray:
        base = np.concatenate([np.full(r, t, dtype=np.int8) for t, r in self.elements])
        return np.tile(base, self.repetitions)


@dataclass
class Section:
    """``SymbolSection`` (waveform.py:514-651) with zero sample offset."""

    num_repetitions: int
    pattern: list


@dataclass
class FrameSpec:
    num_subcarriers: int
    resources: list
    sections: list
    modulation_order: int = 16
    dc_suppression: bool = True
    # Engine extension for MIMO pilots (the reference has no MIMO reference
    # scheme): with pilot_comb = P > 1, stream s transmits the reference element at
    # grid column c only if c % P == s % P and sends zero there otherwise, so each
    # stream's pilots are alone on their subcarriers.
    pilot_comb: int = 0


class FrameLayout:
    """Everything the kernels need to know about one frame, as flat tables."""

    def __init__(self, spec: FrameSpec) -> None:
        n = spec.num_subcarriers
        self.spec = spec
        self.N = n
        self.order = spec.modulation_order
        self.bits_per_symbol = mapping.bits_per_symbol(self.order)
        word_resources = []
        for sec in spec.sections:
            word_resources += list(sec.pattern) * sec.num_repetitions
        self.word_resource = np.asarray(word_resources, dtype=np.int32)
        self.num_words = len(word_resources)
        kind = np.full((self.num_words, n), NULL, dtype=np.int8)
        prefix = np.zeros(self.num_words, dtype=np.int32)
        prefix_type = []
        for w, r in enumerate(word_resources):
            res = spec.resources[r]
            m = res.mask()
            kind[w, : m.size] = m
            prefix[w] = int(n * res.prefix_ratio) if res.prefix_type != "NONE" else 0
            prefix_type.append(res.prefix_type)
        self.kind = kind
        self.prefix = prefix
        self.zero_prefix = np.array([t == "ZEROPAD" for t in prefix_type])
        self.num_used = int(max(spec.resources[r].num_subcarriers for r in set(word_resources)))
        self.data_mask = kind == DATA
        self.ref_mask = kind == REFERENCE
        self.num_data = int(self.data_mask.sum())
        self.num_refs = int(self.ref_mask.sum())
        # sample offsets: word w occupies [word_start[w], word_start[w] + prefix[w] + N)
        lengths = prefix + n
        self.word_start = np.concatenate([[0], np.cumsum(lengths)[:-1]]).astype(np.int64)
        self.window_start = self.word_start + prefix  # FFT window (CP stripped)
        self.samples_per_frame = int(lengths.sum())

    # --- grid column <-> FFT bin --------------------------------------------------
    def bins(self) -> np.ndarray:
        """FFT bin of every grid column.

        ``OFDMWaveform._forward_transformation`` (ofdm.py:98-130) rolls the upper
        half of the grid by one when ``dc_suppression`` is set and then applies
        ``ifftshift``; ``_backward_transformation`` (:133-161) undoes both.
        """

        n = self.N
        c = np.arange(n)
        if self.spec.dc_suppression:
            b = np.where(c < n // 2, c + n // 2, c + 1 - n // 2)
            b[n - 1] = 0
        else:
            b = (c + n // 2) % n
        return b.astype(np.int64)

    def pilot_symbols(self) -> np.ndarray:
        seq = mapping.get_mapping(self.order)
        reps = int(np.ceil(max(self.num_refs, 1) / seq.size))
        return np.tile(seq, reps)[: self.num_refs]

    def stream_ref_mask(self, stream: int) -> np.ndarray:
        """Reference elements stream ``stream`` actually transmits (``pilot_comb``)."""

        comb = self.spec.pilot_comb
        if comb <= 1:
            return self.ref_mask.copy()
        cols = np.arange(self.N)[None, :] % comb == stream % comb
        return self.ref_mask & cols

    def stream_pilot_symbols(self, stream: int) -> np.ndarray:
        """Reference symbols of one stream in frame order, zero where it is silent."""

        keep = self.stream_ref_mask(stream)[self.ref_mask]
        return np.where(keep, self.pilot_symbols(), 0)

    def bits_per_frame(self) -> int:
        return self.num_data * self.bits_per_symbol
