"""OFDM waveform of the drop-in API, backed by the engine's CUDA kernels.

Mirrors the reference's grid description and ``OFDMWaveform``
(modem/waveforms/orthogonal/waveform.py, modem/waveforms/orthogonal/ofdm.py):
``GridElement``, ``GridResource``, ``SymbolSection``, ``ElementType``,
``PrefixType`` keep their names, arguments and validation; ``OFDMWaveform``
keeps ``map / unmap / place / pick / modulate / demodulate``,
``estimate_channel / equalize_symbols`` and the frame bookkeeping properties.
The frame's tables live on the GPU (one ``hpx_frame`` handle per layout).
A ``PilotSection`` / ``SchmidlCoxPilotSection`` preamble (waveform.py:719-903,
ofdm.py:184-205) is modulated once by the transmit kernel and prepended to every
frame; ``demodulate`` skips it, and ``synchronization`` (``Synchronization``,
``SchmidlCoxSynchronization``, ``OFDMCorrelationSynchronization``) finds frame
starts with the metric kernels of ``hpx_sync_*``. Oversampling factors other than 1
and symbol sections with a sample offset are not part of the engine and raise
``NotImplementedError``.
"""

from __future__ import annotations

import ctypes
import enum
from typing import Sequence

import numpy as np
import torch

from . import _lib
from .containers import StatedSymbols, Symbols, to_device, to_numpy
from .mapping import PskQamMapping


class ElementType(enum.Enum):
    REFERENCE = 0
    DATA = 1
    NULL = 2


class PrefixType(enum.Enum):
    CYCLIC = 0
    ZEROPAD = 1
    NONE = 2


class GridElement:
    def __init__(self, type: str | ElementType, repetitions: int = 1) -> None:
        self.type = ElementType[type] if isinstance(type, str) else type
        self.repetitions = int(repetitions)


class GridResource:
    """One frequency-domain resource pattern (waveform.py:96-238)."""

    def __init__(self, repetitions: int = 1, prefix_type: PrefixType | str = PrefixType.CYCLIC,
                 prefix_ratio: float = 0.0, elements: list[GridElement] | None = None) -> None:
        if repetitions < 1:
            raise ValueError("Number of frame resource repetitions must be greater or equal to one")
        if prefix_ratio < 0.0:
            raise ValueError(f"Cyclic prefix ratio must be non-negative (not {prefix_ratio})")
        self.repetitions = int(repetitions)
        self.prefix_ratio = float(prefix_ratio)
        self.prefix_type = PrefixType[prefix_type] if isinstance(prefix_type, str) else prefix_type
        self.elements = elements if elements is not None else []

    @property
    def num_subcarriers(self) -> int:
        return self.repetitions * sum(e.repetitions for e in self.elements)

    @property
    def num_symbols(self) -> int:
        return self.repetitions * sum(e.repetitions for e in self.elements if e.type == ElementType.DATA)

    @property
    def num_references(self) -> int:
        return self.repetitions * sum(e.repetitions for e in self.elements if e.type == ElementType.REFERENCE)

    @property
    def mask(self) -> np.ndarray:
        base = np.concatenate([np.full(e.repetitions, e.type.value, dtype=np.int8) for e in self.elements]) \
            if self.elements else np.zeros(0, np.int8)
        kinds = np.tile(base, self.repetitions)
        mask = np.zeros((len(ElementType), kinds.size), dtype=bool)
        for t in ElementType:
            mask[t.value] = kinds == t.value
        return mask


class SymbolSection:
    """A repeated pattern of grid resources in time (waveform.py:514-651)."""

    def __init__(self, num_repetitions: int = 1, pattern: list[int] | None = None, sample_offset: int = 0,
                 wave: "OFDMWaveform | None" = None) -> None:
        if num_repetitions < 1:
            raise ValueError("OFDM frame number of repetitions must be greater or equal to one")
        if sample_offset != 0:
            raise NotImplementedError("symbol sections with a sample offset are not part of the engine")
        self.num_repetitions = int(num_repetitions)
        self.pattern = list(pattern) if pattern is not None else []
        self.sample_offset = 0
        self.wave = wave

    @property
    def num_words(self) -> int:
        return self.num_repetitions * len(self.pattern)


class PilotSection:
    """Static preamble of one OFDM symbol without prefix (waveform.py:719-903).

    Its N subcarriers carry ``pilot_elements`` (tiled), or by default the frame
    mapping's symbols of ``numpy.random.default_rng(50)`` bits, as in the reference.
    """

    def __init__(self, pilot_elements: Symbols | None = None, wave=None) -> None:
        self.pilot_elements = pilot_elements
        self.wave = wave
        self._cache = None

    @property
    def pilot_elements(self) -> Symbols | None:
        return self._pilot_elements

    @pilot_elements.setter
    def pilot_elements(self, value: Symbols | None) -> None:
        if value is not None:
            if value.num_streams != 1:
                raise ValueError("Subsymbol pilot configuration may only contain a single stream")
            if value.num_symbols < 1:
                raise ValueError("Subsymbol pilot configuration must contain at least one symbol")
        self._pilot_elements = value
        self._cache = None

    @property
    def num_repetitions(self) -> int:
        return 1

    @num_repetitions.setter
    def num_repetitions(self, value: int) -> None:
        if value != 1:
            raise ValueError("Pilot sections may not be repeated")

    @property
    def sample_offset(self) -> int:
        return 0

    @sample_offset.setter
    def sample_offset(self, value: int) -> None:
        if value != 0:
            raise ValueError("Pilot sections may not have a sample offset")

    def num_samples(self, bandwidth: float = 1.0, oversampling_factor: int = 1) -> int:
        return self.wave.num_subcarriers * oversampling_factor

    @property
    def num_words(self) -> int:
        return 1

    @property
    def num_symbols(self) -> int:
        return 0

    @property
    def num_references(self) -> int:
        if self._pilot_elements is not None or self.wave is None:
            return 0
        return self.wave.num_subcarriers

    def _pilot_sequence(self, num_symbols: int | None = None) -> np.ndarray:
        n = self.wave.num_subcarriers if num_symbols is None else int(num_symbols)
        if self._pilot_elements is None:
            rng = np.random.default_rng(50)
            bits = rng.integers(0, 2, n * self.wave.mapping.bits_per_symbol, np.uint8).flatten()
            symbols = self.wave.mapping.get_symbols(bits)
        else:
            flat = self._pilot_elements.raw.reshape(-1)
            symbols = np.tile(flat, int(np.ceil(n / flat.size)))
        return np.asarray(symbols, dtype=np.complex128)[:n]

    def generate_device(self) -> torch.Tensor:
        """The preamble's N time-domain samples (the transmit kernel on a one-word,
        N-column, prefix-free frame), cached per subcarrier count."""

        n = self.wave.num_subcarriers
        key = (n, self.wave.dc_suppression, self.wave.modulation_order)
        if self._cache is None or self._cache[0] != key:
            grid = to_device(self._pilot_sequence(n)).reshape(1, 1, n)
            kind = np.full((1, n), ElementType.REFERENCE.value, dtype=np.int8)
            prefix = np.zeros(1, dtype=np.int32)
            desc = _lib.FrameDesc(n, 1, n, self.wave.modulation_order, int(self.wave.dc_suppression),
                                  prefix.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                  prefix.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                  kind.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), 0)
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_frame_create(ctypes.byref(desc), ctypes.byref(h)))
            try:
                out = torch.empty((1, n), dtype=torch.complex64, device=grid.device)
                _lib.call("hpx_ofdm_modulate_grid", h, _lib.ptr(grid), n, 1, _lib.ptr(out), _lib.stream_ptr())
                torch.cuda.current_stream().synchronize()
            finally:
                _lib.call("hpx_frame_destroy", h)
            self._cache = (key, out[0])
        return self._cache[1]

    def generate(self, oversampling_factor: int = 1) -> np.ndarray:
        if self.wave is None:
            raise RuntimeError("Pilot section must be associated with a waveform")
        if oversampling_factor != 1:
            raise NotImplementedError("the engine runs OFDM frames without oversampling")
        return to_numpy(self.generate_device())


class SchmidlCoxPilotSection(PilotSection):
    """Schmidl-Cox preamble: pilots on every second subcarrier, so the symbol's two
    halves repeat in time (ofdm.py:184-205)."""

    def _pilot_sequence(self, num_symbols: int | None = None) -> np.ndarray:
        if self.wave is None:
            raise RuntimeError("Waveform not set for pilot section")
        n = self.wave.num_subcarriers
        stuffed = np.zeros(n, dtype=np.complex128)
        stuffed[::2] = PilotSection._pilot_sequence(self, int(np.ceil(0.5 * n)))
        if self.wave.dc_suppression:
            dc = int(0.5 * n)
            stuffed[:dc] = np.roll(stuffed[:dc], 1)
        return stuffed


class OFDMWaveform:
    """Orthogonal frequency-division multiplexing waveform (ofdm.py:33-181)."""

    def __init__(self, grid_resources: Sequence[GridResource], grid_structure: Sequence[SymbolSection],
                 num_subcarriers: int = 1024, dc_suppression: bool = True, pilot_section=None,
                 pilot_sequence=None, repeat_pilot_sequence: bool = True, modulation_order: int = 16,
                 oversampling_factor: int = 1, pilot_comb: int = 0, **kwargs) -> None:
        if num_subcarriers < 1:
            raise ValueError("Number of subcarriers must be greater or equal to one")
        if pilot_sequence is not None:
            raise NotImplementedError("custom pilot symbol sequences are not part of the engine")
        self.num_subcarriers = int(num_subcarriers)
        self.grid_resources = list(grid_resources)
        self.grid_structure = list(grid_structure)
        for s in self.grid_structure:
            s.wave = self
        self.dc_suppression = bool(dc_suppression)
        self.modulation_order = int(modulation_order)
        self.oversampling_factor = int(oversampling_factor)
        # Engine extension for MIMO channel estimation (no counterpart in the
        # reference): with pilot_comb = P > 1 stream s sends the reference element
        # of grid column c only if c % P == s % P.
        self.pilot_comb = int(pilot_comb)
        self.pilot_section = pilot_section
        self._synchronization = None
        self._channel_estimation = None
        self._channel_equalization = None
        self._handle = None
        self._key = None
        self._tables = None

    # ---------------------------------------------------------------- mapping
    @property
    def mapping(self) -> PskQamMapping:
        return PskQamMapping(self.modulation_order)

    @property
    def bits_per_symbol(self) -> int:
        return int(np.log2(self.modulation_order))

    def bits_per_frame(self, num_data_symbols: int | None = None) -> int:
        n = self.num_data_symbols if num_data_symbols is None else num_data_symbols
        return n * self.bits_per_symbol

    # ------------------------------------------------------------------ frame
    def _layout(self) -> dict:
        key = (self.num_subcarriers, self.dc_suppression, self.modulation_order, self.pilot_comb,
               tuple((r.repetitions, r.prefix_ratio, r.prefix_type, tuple((e.type, e.repetitions) for e in r.elements))
                     for r in self.grid_resources),
               tuple((s.num_repetitions, tuple(s.pattern)) for s in self.grid_structure))
        if self._tables is not None and self._key == key:
            return self._tables
        n = self.num_subcarriers
        words = []
        for sec in self.grid_structure:
            words += list(sec.pattern) * sec.num_repetitions
        if not words:
            raise ValueError("frame has no words")
        cols = max(self.grid_resources[r].num_subcarriers for r in set(words))
        if cols > n:
            raise ValueError("grid resources exceed the number of subcarriers")
        kind = np.full((len(words), cols), ElementType.NULL.value, dtype=np.int8)
        prefix = np.zeros(len(words), dtype=np.int32)
        zero = np.zeros(len(words), dtype=np.int32)
        for w, r in enumerate(words):
            res = self.grid_resources[r]
            m = res.mask
            for t in ElementType:
                kind[w, : m.shape[1]][m[t.value]] = t.value
            prefix[w] = int(n * self.oversampling_factor * res.prefix_ratio) if res.prefix_type != PrefixType.NONE else 0
            zero[w] = 1 if res.prefix_type == PrefixType.ZEROPAD else 0
        self._tables = {"kind": kind, "prefix": prefix, "zero": zero, "num_words": len(words), "num_columns": cols}
        self._key = key
        if self._handle is not None:
            _lib.call("hpx_frame_destroy", self._handle)
            self._handle = None
        return self._tables

    def _frame(self):
        """The engine's frame handle (created on first use)."""

        t = self._layout()
        if self.oversampling_factor != 1:
            raise NotImplementedError("the engine runs OFDM frames without oversampling")
        if self._handle is None:
            _lib.load()
            kind = np.ascontiguousarray(t["kind"])
            prefix = np.ascontiguousarray(t["prefix"])
            zero = np.ascontiguousarray(t["zero"])
            desc = _lib.FrameDesc(self.num_subcarriers, t["num_words"], t["num_columns"], self.modulation_order,
                                  int(self.dc_suppression), prefix.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                  zero.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                  kind.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), self.pilot_comb)
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_frame_create(ctypes.byref(desc), ctypes.byref(h)))
            self._handle = h
        return self._handle

    def __del__(self):
        try:
            if self._handle is not None and _lib._lib is not None:
                _lib._lib.hpx_frame_destroy(self._handle)
        except Exception:
            pass

    @property
    def resource_mask(self) -> np.ndarray:
        t = self._layout()
        mask = np.zeros((len(ElementType), t["num_words"], self.num_subcarriers), dtype=bool)
        for e in ElementType:
            mask[e.value, :, : t["num_columns"]] = t["kind"] == e.value
        mask[ElementType.NULL.value, :, t["num_columns"]:] = False
        return mask

    @property
    def words_per_frame(self) -> int:
        return self._layout()["num_words"]

    @property
    def num_data_symbols(self) -> int:
        return int((self._layout()["kind"] == ElementType.DATA.value).sum())

    @property
    def references_per_frame(self) -> int:
        return int((self._layout()["kind"] == ElementType.REFERENCE.value).sum())

    @property
    def symbols_per_frame(self) -> int:
        return self.num_data_symbols + self.references_per_frame

    @property
    def pilot_section(self) -> PilotSection | None:
        return self._pilot_section

    @pilot_section.setter
    def pilot_section(self, value: PilotSection | None) -> None:
        self._pilot_section = value
        if value is not None and value.wave is not self:
            value.wave = self

    def _preamble_length(self) -> int:
        return self.num_subcarriers if self._pilot_section is not None else 0

    def pilot_signal(self, bandwidth: float = 1.0, oversampling_factor: int = 1):
        """The preamble as a signal (empty without a pilot section)."""

        from .containers import Signal

        self._check_osf(oversampling_factor)
        if self._pilot_section is None:
            return Signal.Empty(bandwidth * oversampling_factor)
        return Signal.Create(self._pilot_section.generate_device()[None], bandwidth * oversampling_factor)

    @property
    def synchronization(self):
        if self._synchronization is None:
            from .synchronization import Synchronization

            self._synchronization = Synchronization(self)
        return self._synchronization

    @synchronization.setter
    def synchronization(self, value) -> None:
        self._synchronization = value
        if value is not None and value.waveform is not self:
            value.waveform = self

    def samples_per_frame(self, bandwidth: float = 1.0, oversampling_factor: int = 1) -> int:
        t = self._layout()
        return int(t["num_words"] * self.num_subcarriers * oversampling_factor + t["prefix"].sum()) + \
            self._preamble_length() * oversampling_factor

    def _grid_samples(self) -> int:
        return self.samples_per_frame() - self._preamble_length()

    def frame_duration(self, bandwidth: float) -> float:
        return self.samples_per_frame(bandwidth, 1) / bandwidth

    def symbol_energy(self, bandwidth: float = 1.0, oversampling_factor: int = 1) -> float:
        return float(oversampling_factor)

    def bit_energy(self, bandwidth: float = 1.0, oversampling_factor: int = 1) -> float:
        return self.symbol_energy(bandwidth, oversampling_factor) / self.bits_per_symbol

    @property
    def power(self) -> float:
        return 1.0

    def pilot_symbols(self, num_symbols: int) -> np.ndarray:
        seq = self.mapping.get_mapping()
        reps = int(np.ceil(max(num_symbols, 1) / seq.size))
        return np.tile(seq, reps)[:num_symbols]

    # ------------------------------------------------------------- operators
    def map(self, data_bits) -> Symbols:
        return Symbols(self.mapping.get_symbols_device(data_bits)[None, :, None])

    def unmap(self, symbols: Symbols) -> np.ndarray:
        return to_numpy(self.mapping.detect_bits_device(symbols.device_raw.reshape(-1))).astype(np.uint8)

    def _check_osf(self, oversampling_factor: int) -> None:
        if oversampling_factor != 1:
            raise NotImplementedError("the engine runs OFDM frames without oversampling")

    def place(self, symbols: Symbols) -> Symbols:
        data = symbols.device_raw.reshape(-1)
        if data.numel() != self.num_data_symbols:
            raise ValueError(
                f"Number of provided data symbols does not match the number of symbols in the frame "
                f"({data.numel()} != {self.num_data_symbols})")
        t = self._layout()
        dev = data.device
        grid = torch.zeros((t["num_words"], self.num_subcarriers), dtype=torch.complex64, device=dev)
        kind = torch.from_numpy(t["kind"]).to(dev)
        sub = grid[:, : t["num_columns"]]
        refs = to_device(self.pilot_symbols(self.references_per_frame))
        sub[kind == ElementType.REFERENCE.value] = refs
        sub[kind == ElementType.DATA.value] = data
        return Symbols(grid[None])

    def pick(self, placed_symbols: StatedSymbols) -> StatedSymbols:
        t = self._layout()
        kind = torch.from_numpy(t["kind"]).to(placed_symbols.device_raw.device) == ElementType.DATA.value
        raw = placed_symbols.device_raw[:, :, : t["num_columns"]][:, kind][:, :, None]
        st = placed_symbols.device_states[:, :, :, : t["num_columns"]][:, :, kind][..., None]
        return StatedSymbols(raw, st, placed_symbols.noise_variance)

    def modulate_device(self, grid: torch.Tensor) -> torch.Tensor:
        """(batch, words, G) placed grids -> (batch, T) samples."""

        grid = grid.contiguous()
        out = torch.empty((grid.shape[0], self._grid_samples()), dtype=torch.complex64, device=grid.device)
        _lib.call("hpx_ofdm_modulate_grid", self._frame(), _lib.ptr(grid), grid.shape[-1], grid.shape[0],
                  _lib.ptr(out), _lib.stream_ptr())
        return self._with_preamble(out)

    def _with_preamble(self, frames: torch.Tensor) -> torch.Tensor:
        if self._pilot_section is None:
            return frames
        pre = self._pilot_section.generate_device()
        return torch.cat([pre[None].expand(frames.shape[0], -1), frames], dim=1)

    def modulate_data_device(self, data: torch.Tensor) -> torch.Tensor:
        """(batch, num_data) data symbols -> (batch, T) samples (place + modulate fused)."""

        data = to_device(data).reshape(-1, self.num_data_symbols).contiguous()
        out = torch.empty((data.shape[0], self._grid_samples()), dtype=torch.complex64, device=data.device)
        _lib.call("hpx_ofdm_modulate", self._frame(), _lib.ptr(data), data.shape[0], _lib.ptr(out), _lib.stream_ptr())
        return self._with_preamble(out)

    def modulate(self, data_symbols: Symbols, bandwidth: float = 1.0, oversampling_factor: int = 1) -> np.ndarray:
        self._check_osf(oversampling_factor)
        grid = data_symbols.device_raw
        if grid.ndim == 3 and grid.shape[0] == 1 and grid.shape[1] == self.words_per_frame:
            return to_numpy(self.modulate_device(grid[0][None])[0])
        return to_numpy(self.modulate_data_device(grid.reshape(1, -1))[0])

    def demodulate_device(self, samples: torch.Tensor, num_columns: int | None = None) -> torch.Tensor:
        """(batch, >= T) samples -> (batch, words, num_columns) grid."""

        pre = self._preamble_length()
        if pre:  # skip the preamble (waveform.py:1328-1330)
            samples = samples[:, pre:]
        samples = samples.contiguous()
        cols = self.num_subcarriers if num_columns is None else num_columns
        out = torch.empty((samples.shape[0], self.words_per_frame, cols), dtype=torch.complex64, device=samples.device)
        _lib.call("hpx_ofdm_demodulate", self._frame(), _lib.ptr(samples), samples.shape[-1], samples.shape[0], cols,
                  _lib.ptr(out), _lib.stream_ptr())
        return out

    def demodulate(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> Symbols:
        self._check_osf(oversampling_factor)
        s = to_device(signal).reshape(1, -1)
        if s.shape[1] < self.samples_per_frame():
            s = torch.nn.functional.pad(s, (0, self.samples_per_frame() - s.shape[1]))
        return Symbols(self.demodulate_device(s)[0][None])

    # --------------------------------------------------- estimation plumbing
    @property
    def channel_estimation(self):
        if self._channel_estimation is None:
            from .estimation import ChannelEstimation

            self._channel_estimation = ChannelEstimation(self)
        return self._channel_estimation

    @channel_estimation.setter
    def channel_estimation(self, value) -> None:
        self._channel_estimation = value
        if value is not None:
            value.waveform = self

    @property
    def channel_equalization(self):
        if self._channel_equalization is None:
            from .estimation import ChannelEqualization

            self._channel_equalization = ChannelEqualization(self)
        return self._channel_equalization

    @channel_equalization.setter
    def channel_equalization(self, value) -> None:
        self._channel_equalization = value
        if value is not None:
            value.waveform = self

    def estimate_channel(self, symbols: Symbols, bandwidth: float = 1.0, oversampling_factor: int = 1,
                         delay: float = 0.0) -> StatedSymbols:
        return self.channel_estimation.estimate_channel(symbols, bandwidth, oversampling_factor, delay)

    def equalize_symbols(self, symbols: StatedSymbols) -> Symbols:
        return self.channel_equalization.equalize_channel(symbols)
