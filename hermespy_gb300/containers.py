"""Signal and symbol containers of the drop-in API.

They mirror the reference's ``Signal`` (core/signal_model.py:866-911),
``Symbols`` and ``StatedSymbols`` (modem/symbols.py:136-411): the engine keeps
the samples on the GPU as complex64 torch tensors; ``.raw`` / ``.samples``
return numpy complex128 copies for code written against the reference, and
``.device`` accessors give the tensors without a copy.
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


class Signal:
    """Multi-stream baseband samples at one sampling rate (``Signal.Create``)."""

    def __init__(self, samples, sampling_rate: float, carrier_frequency: float = 0.0, noise_power: float = 0.0,
                 offset: int = 0) -> None:
        t = to_device(samples)
        if t.ndim == 1:
            t = t[None, :]
        self._samples = t.contiguous()
        self.sampling_rate = float(sampling_rate)
        self.carrier_frequency = float(carrier_frequency)
        self.noise_power = float(noise_power)
        self.offset = int(offset)

    @classmethod
    def Create(cls, samples, sampling_rate: float, carrier_frequency: float = 0.0, noise_power: float = 0.0,
               offset: int = 0) -> "Signal":
        return cls(samples, sampling_rate, carrier_frequency, noise_power, offset)

    @property
    def num_streams(self) -> int:
        return int(self._samples.shape[0])

    @property
    def num_samples(self) -> int:
        return int(self._samples.shape[1])

    @property
    def device_samples(self) -> torch.Tensor:
        return self._samples

    @property
    def samples(self) -> np.ndarray:
        return to_numpy(self._samples)

    def view(self, _type=np.ndarray) -> np.ndarray:
        return self.samples

    def copy(self) -> "Signal":
        return Signal(self._samples.clone(), self.sampling_rate, self.carrier_frequency, self.noise_power, self.offset)


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
