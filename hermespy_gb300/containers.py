"""Signal and symbol containers of the drop-in API.

They mirror the reference's signal model (core/signal_model.py: ``SignalBlock``
:395-745, ``Signal`` :746-1185, ``DenseSignal`` :1187-1596, ``SparseSignal``
:1598-2659), ``Symbols`` and ``StatedSymbols`` (modem/symbols.py:136-411): the
engine keeps the samples on the GPU as complex64 torch tensors; ``.raw`` /
``.samples`` return numpy complex128 copies for code written against the
reference, ``.device_*`` accessors give the tensors without a copy, and dense
signals and blocks are DLPack producers (zero-copy exchange with torch, CuPy,
JAX or any other consumer on the same device).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib


def to_device(x, dtype=torch.complex64) -> torch.Tensor:
    """numpy array or tensor -> contiguous CUDA tensor of ``dtype``."""

    dev = _lib.require_cuda()
    if isinstance(x, torch.Tensor):
        t = x.to(device=dev, dtype=dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x).astype(
            {torch.complex64: np.complex64, torch.float32: np.float32, torch.uint8: np.uint8,
             torch.float64: np.float64}[dtype]))).to(dev)
    return t.contiguous()


def to_numpy(t: torch.Tensor, complex128: bool = True) -> np.ndarray:
    a = t.detach().cpu().numpy()
    if complex128 and np.iscomplexobj(a):
        return a.astype(np.complex128)
    return a


class SignalBlock:
    """One dense piece of a signal: a (streams, samples) complex64 CUDA tensor at an
    integer sample offset from the signal start (signal_model.py:395-745).

    The block exposes ``__dlpack__`` / ``__dlpack_device__`` of its tensor, so
    ``torch.from_dlpack(block)`` (or any DLPack consumer) views the device samples
    without a copy; ``.samples`` is a numpy complex128 copy.
    """

    def __init__(self, samples, offset: int = 0) -> None:
        t = to_device(samples)
        if t.ndim == 1:
            t = t[None, :]
        if t.ndim != 2:
            raise ValueError("HermesPy signal models must be two-dimensional")
        self._t = t.contiguous()
        self.offset = offset

    @property
    def offset(self) -> int:
        return self._offset

    @offset.setter
    def offset(self, value: int) -> None:
        if value < 0:
            raise ValueError("Offset must be non-zero")
        self._offset = int(value)

    @property
    def num_streams(self) -> int:
        return int(self._t.shape[0])

    @property
    def num_samples(self) -> int:
        return int(self._t.shape[1])

    @property
    def shape(self) -> tuple[int, int]:
        return (self.num_streams, self.num_samples)

    @property
    def end(self) -> int:
        return self._offset + self.num_samples

    @property
    def device_samples(self) -> torch.Tensor:
        return self._t

    @property
    def samples(self) -> np.ndarray:
        return to_numpy(self._t)

    @property
    def energy(self) -> np.ndarray:
        """Sum of squared magnitudes per stream."""

        return (self._t.abs().double() ** 2).sum(dim=1).cpu().numpy()

    @property
    def power(self) -> np.ndarray:
        return self.energy / self.num_samples

    def copy(self) -> "SignalBlock":
        return SignalBlock(self._t.clone(), self._offset)

    def __dlpack__(self, *args, **kwargs):
        return self._t.__dlpack__(*args, **kwargs)

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def _blocks_from(samples, offsets) -> list[SignalBlock]:
    """Blocks of ``Signal.Create`` input with the reference's offset rules
    (signal_model.py:2490-2574): SignalBlocks keep their offsets; arrays take the
    given offsets or follow each other; arrays may not overlap."""

    if isinstance(samples, SignalBlock):
        return [samples]
    if isinstance(samples, (list, tuple)):
        items = list(samples)
    else:
        t = samples if isinstance(samples, torch.Tensor) else np.asarray(samples)
        items = list(t) if t.ndim == 3 else [t]
    if offsets is not None and len(offsets) != len(items):
        raise ValueError(f"samples and offsets legthes do not match ({len(items)} and {len(offsets)})")
    if items and all(isinstance(b, SignalBlock) for b in items) and offsets is None:
        return items
    blocks, cursor = [], 0
    for i, item in enumerate(items):
        if isinstance(item, SignalBlock):
            off = item.offset if offsets is None else int(offsets[i])
            b = SignalBlock(item.device_samples, off)
        else:
            b = SignalBlock(item, cursor if offsets is None else int(offsets[i]))
        if blocks:
            if b.num_streams != blocks[0].num_streams:
                raise ValueError("At least one if the samples blocks contains different number of streams")
            if b.offset < blocks[-1].end:
                raise ValueError(f"One of the blocks contains incorrect offset in this sequence (previous block "
                                 f"ends on {blocks[-1].end}, this block's offset is {b.offset})")
        blocks.append(b)
        cursor = b.end
    return blocks


class Signal:
    """Multi-stream baseband samples at one sampling rate (signal_model.py:746-1185).

    ``Signal.Create`` returns a ``DenseSignal`` for one block and a ``SparseSignal``
    for several; both keep their samples as CUDA tensors. Calling ``Signal(...)``
    directly builds a ``DenseSignal`` (the engine's own call sites).
    """

    def __new__(cls, *args, **kwargs):
        if cls is Signal:
            return super().__new__(DenseSignal)
        return super().__new__(cls)

    def _init_meta(self, sampling_rate, carrier_frequency, noise_power, delay) -> None:
        if sampling_rate <= 0.0:
            raise ValueError("Sampling rate must be greater than zero")
        self.sampling_rate = float(sampling_rate)
        self.carrier_frequency = float(carrier_frequency)
        self.noise_power = float(noise_power)
        self.delay = float(delay)

    @staticmethod
    def Create(samples, sampling_rate: float = 1.0, carrier_frequency: float = 0.0, noise_power: float = 0.0,
               delay: float = 0.0, offsets=None) -> "Signal":
        if isinstance(samples, (list, tuple)) and len(samples) != 1:
            return SparseSignal(_blocks_from(samples, offsets), sampling_rate, carrier_frequency, noise_power, delay)
        first = samples[0] if isinstance(samples, (list, tuple)) else samples
        if offsets is not None and len(offsets) > 0:
            delay = delay + offsets[0] / sampling_rate
        t = first.device_samples if isinstance(first, SignalBlock) else first
        return DenseSignal(t, sampling_rate, carrier_frequency, noise_power, delay=delay)

    @staticmethod
    def Empty(sampling_rate: float, num_streams: int = 0, num_samples: int = 0, **kwargs) -> "Signal":
        return Signal.Create(torch.zeros((num_streams, num_samples), dtype=torch.complex64,
                                         device=_lib.require_cuda()), sampling_rate, **kwargs)

    @staticmethod
    def from_dlpack(obj, sampling_rate: float, carrier_frequency: float = 0.0, noise_power: float = 0.0,
                    delay: float = 0.0) -> "DenseSignal":
        """A dense signal viewing a DLPack producer's (streams, samples) complex64 CUDA
        buffer without a copy (other dtypes or host memory are converted)."""

        return DenseSignal(torch.from_dlpack(obj), sampling_rate, carrier_frequency, noise_power, delay=delay)

    # ----------------------------------------------------------- block model
    @property
    def blocks(self) -> list[SignalBlock]:  # pragma: no cover - interface
        raise NotImplementedError

    @property
    def block_offsets(self) -> list[int]:
        return [b.offset for b in self.blocks]

    @property
    def num_blocks(self) -> int:
        return len(self.blocks)

    @property
    def num_streams(self) -> int:
        return self.blocks[0].num_streams if self.blocks else 0

    @property
    def num_samples(self) -> int:
        return self.blocks[-1].end if self.blocks else 0

    @property
    def shape(self) -> tuple[int, int]:
        return (self.num_streams, self.num_samples)

    @property
    def timestamps(self) -> np.ndarray:
        return np.arange(self.num_samples) / self.sampling_rate

    @property
    def duration(self) -> float:
        return self.num_samples / self.sampling_rate

    def to_dense(self) -> "DenseSignal":
        out = torch.zeros(self.shape, dtype=torch.complex64, device=_lib.require_cuda())
        for b in self.blocks:
            out[:, b.offset:b.end] = b.device_samples
        return DenseSignal(out, self.sampling_rate, self.carrier_frequency, self.noise_power, delay=self.delay)

    @property
    def device_samples(self) -> torch.Tensor:
        """Dense (streams, samples) device tensor (a view for dense signals)."""

        return self.to_dense().device_samples

    @property
    def samples(self) -> np.ndarray:
        return to_numpy(self.device_samples)

    def view(self, _type=np.ndarray) -> np.ndarray:
        return self.samples

    def superimpose(self, added: "Signal") -> "DenseSignal":
        """Dense sum of two signals at the same sampling and carrier frequency, the
        shorter one zero-extended (the same-rate case of signal_model.py:1075-1107)."""

        if added.sampling_rate != self.sampling_rate or added.carrier_frequency != self.carrier_frequency:
            raise NotImplementedError("superimposing signals of different sampling rates or carriers")
        if added.num_streams != self.num_streams:
            raise ValueError("Superimposed signals must have the same number of streams")
        n = max(self.num_samples, added.num_samples)
        out = torch.zeros((self.num_streams, n), dtype=torch.complex64, device=_lib.require_cuda())
        for sig in (self, added):
            for b in sig.blocks:
                out[:, b.offset:b.end] += b.device_samples
        return DenseSignal(out, self.sampling_rate, self.carrier_frequency, self.noise_power + added.noise_power,
                           delay=self.delay)


class DenseSignal(Signal):
    """One block at offset 0 (signal_model.py:1187-1596); DLPack-exportable."""

    def __init__(self, samples, sampling_rate: float, carrier_frequency: float = 0.0, noise_power: float = 0.0,
                 offset: int = 0, delay: float = 0.0) -> None:
        self._block = SignalBlock(samples, 0)
        self._init_meta(sampling_rate, carrier_frequency, noise_power, delay)
        self.offset = int(offset)  # sample offset of the frame inside a received signal

    @staticmethod
    def FromNDArray(array, sampling_rate: float = 1.0, carrier_frequency: float = 0.0, noise_power: float = 0.0,
                    delay: float = 0.0) -> "DenseSignal":
        return DenseSignal(array, sampling_rate, carrier_frequency, noise_power, delay=delay)

    @staticmethod
    def Zeros(num_streams: int, num_samples: int, sampling_rate: float = 1.0, **kwargs) -> "DenseSignal":
        return DenseSignal(torch.zeros((num_streams, num_samples), dtype=torch.complex64,
                                       device=_lib.require_cuda()), sampling_rate, **kwargs)

    @property
    def blocks(self) -> list[SignalBlock]:
        return [self._block]

    @property
    def device_samples(self) -> torch.Tensor:
        return self._block.device_samples

    @property
    def energy(self) -> np.ndarray:
        return self._block.energy

    @property
    def power(self) -> np.ndarray:
        return self._block.power if self.num_samples else np.zeros(self.num_streams)

    def __mul__(self, value: complex) -> "DenseSignal":
        return DenseSignal(self.device_samples * value, self.sampling_rate, self.carrier_frequency, self.noise_power,
                           self.offset, self.delay)

    def append_samples(self, value) -> "DenseSignal":
        t = value.device_samples if isinstance(value, Signal) else to_device(value)
        if t.ndim == 1:
            t = t[None]
        if t.shape[0] != self.num_streams:
            raise ValueError("Number of streams do not match")
        return DenseSignal(torch.cat([self.device_samples, t], 1), self.sampling_rate, self.carrier_frequency,
                           self.noise_power, self.offset, self.delay)

    def append_streams(self, value) -> "DenseSignal":
        t = value.device_samples if isinstance(value, Signal) else to_device(value)
        if t.ndim == 1:
            t = t[None]
        if t.shape[1] != self.num_samples:
            raise ValueError("Number of samples do not match")
        return DenseSignal(torch.cat([self.device_samples, t], 0), self.sampling_rate, self.carrier_frequency,
                           self.noise_power, self.offset, self.delay)

    def copy(self) -> "DenseSignal":
        return DenseSignal(self.device_samples.clone(), self.sampling_rate, self.carrier_frequency, self.noise_power,
                           self.offset, self.delay)

    def __dlpack__(self, *args, **kwargs):
        return self._block.__dlpack__(*args, **kwargs)

    def __dlpack_device__(self):
        return self._block.__dlpack_device__()


class SparseSignal(Signal):
    """Sorted, non-overlapping blocks separated by zeros (signal_model.py:1598-2659).

    As in the reference, ``energy`` is the total over blocks and streams and
    ``power`` the mean of the blocks' per-stream powers.
    """

    def __init__(self, samples, sampling_rate: float = 1.0, carrier_frequency: float = 0.0,
                 noise_power: float = 0.0, delay: float = 0.0) -> None:
        self._blocks = _blocks_from(samples, None)
        self._init_meta(sampling_rate, carrier_frequency, noise_power, delay)
        self.offset = 0

    @property
    def blocks(self) -> list[SignalBlock]:
        return self._blocks

    @property
    def energy(self) -> np.ndarray:
        return np.sum([b.energy for b in self._blocks])

    @property
    def power(self) -> np.ndarray:
        return np.mean([b.power for b in self._blocks], axis=0)

    def __mul__(self, value: complex) -> "SparseSignal":
        return SparseSignal([SignalBlock(b.device_samples * value, b.offset) for b in self._blocks],
                            self.sampling_rate, self.carrier_frequency, self.noise_power, self.delay)

    def copy(self) -> "SparseSignal":
        return SparseSignal([b.copy() for b in self._blocks], self.sampling_rate, self.carrier_frequency,
                            self.noise_power, self.delay)


class Symbols:
    """Communication symbols, shape (streams, blocks, symbols per block)."""

    def __init__(self, symbols=None) -> None:
        if symbols is None:
            self._raw = None
            return
        t = to_device(symbols)
        if t.ndim == 1:
            t = t[None, :, None]
        elif t.ndim == 2:
            t = t[:, :, None]
        self._raw = t.contiguous()

    @property
    def device_raw(self) -> torch.Tensor:
        return self._raw

    @property
    def raw(self) -> np.ndarray:
        return to_numpy(self._raw)

    @property
    def num_streams(self) -> int:
        return int(self._raw.shape[0])

    @property
    def num_blocks(self) -> int:
        return int(self._raw.shape[1])

    @property
    def num_symbols(self) -> int:
        return int(self._raw.shape[2])

    def append_stream(self, symbols: "Symbols") -> None:
        self._raw = symbols.device_raw if self._raw is None else torch.cat([self._raw, symbols.device_raw], 0)


class StatedSymbols(Symbols):
    """Symbols with channel states of shape (rx streams, tx streams, blocks, symbols)."""

    def __init__(self, symbols, states, noise_variance: float = 0.0) -> None:
        Symbols.__init__(self, symbols)
        s = to_device(states)
        self._states = s.contiguous()
        self.noise_variance = float(noise_variance)

    @property
    def device_states(self) -> torch.Tensor:
        return self._states

    @property
    def states(self) -> np.ndarray:
        return to_numpy(self._states)

    def dense_states(self) -> np.ndarray:
        return self.states

    @property
    def num_transmit_streams(self) -> int:
        return int(self._states.shape[1])
