"""Noise models and levels of the drop-in API.

* ``AWGN`` / ``AWGNRealization`` mirror simulation/rf/noise/model.py:140-187:
  ``realize(power).add_to(signal)`` adds ``sqrt(P/2) (n_re + j n_im)`` with unit
  normals from the engine's Philox stream (Box-Muller), on the GPU.
* ``EBN0`` mirrors simulation/modem/noise.py:93-103: ``bit_energy / level``.
* ``SNR`` mirrors simulation/rf/noise/level.py:200-275: ``power / snr`` times the
  channel's expected energy scale when a channel is given.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .containers import Signal


class AWGNRealization:
    def __init__(self, power: float, seed: int, drop: int) -> None:
        self.power = float(power)
        self.seed = int(seed)
        self.drop = int(drop)

    def add_to(self, signal: Signal) -> Signal:
        """Noise of the signal's whole (streams, samples) extent, added to every
        block at its offset (model.py:143-160)."""

        if self.power == 0.0:
            return signal
        out = signal.copy()
        dense = out.num_blocks == 1 and out.blocks[0].offset == 0 and out.blocks[0].num_samples == out.num_samples
        x = out.blocks[0].device_samples if dense else torch.zeros(out.shape, dtype=torch.complex64,
                                                                    device=_lib.require_cuda())
        p = torch.tensor([self.power], dtype=torch.float32, device=x.device)
        _lib.call("hpx_awgn_add", _lib.ptr(x), 1, x.shape[0], x.shape[1], _lib.ptr(p), self.seed, self.drop,
                  _lib.stream_ptr())
        if not dense:
            for b in out.blocks:
                b.device_samples.add_(x[:, b.offset:b.end])
        out.noise_power = self.power
        return out


class AWGN:
    def __init__(self, seed: int | None = None) -> None:
        self.seed = int(np.random.SeedSequence(seed).generate_state(1, np.uint64)[0]) if seed is None else int(seed)
        self.drop_counter = 0

    def realize(self, power: float) -> AWGNRealization:
        r = AWGNRealization(power, self.seed, self.drop_counter)
        self.drop_counter += 1
        return r

    def add_noise(self, signal: Signal, power: float) -> Signal:
        return self.realize(power).add_to(signal)


class NoiseLevel:
    def get_power(self, bandwidth: float = 1.0) -> float:  # pragma: no cover - interface
        raise NotImplementedError


class EBN0(NoiseLevel):
    """Noise power from the reference waveform's bit energy: ``E_b / level``."""

    def __init__(self, reference, level: float = float("inf")) -> None:
        if level <= 0:
            raise ValueError("Noise level must be greater than zero")
        self.reference = reference
        self.level = float(level)

    def _waveform(self):
        wf = getattr(self.reference, "waveform", self.reference)
        if wf is None:
            raise RuntimeError("The reference modem has no waveform configured. Noise level cannot be determined.")
        return wf

    def get_power(self, bandwidth: float = 1.0) -> float:
        return self._waveform().bit_energy(bandwidth, 1) / self.level


class ESN0(EBN0):
    def get_power(self, bandwidth: float = 1.0) -> float:
        return self._waveform().symbol_energy(bandwidth, 1) / self.level


class SNR(NoiseLevel):
    """Noise power ``reference.power / snr``, scaled by the channel's expected energy."""

    def __init__(self, snr: float, reference, channel=None) -> None:
        if snr <= 0:
            raise ValueError("Signal to noise ratio must be greater than zero")
        self.snr = float(snr)
        self.reference = reference
        self.channel = channel

    @property
    def level(self) -> float:
        return self.snr

    def get_power(self, bandwidth: float = 1.0) -> float:
        scale = 1.0
        if self.channel is not None:
            scale = self.channel.gain * float(np.sum(self.channel.power_profile))
        power = getattr(self.reference, "power", 1.0)
        return power / self.snr * scale
