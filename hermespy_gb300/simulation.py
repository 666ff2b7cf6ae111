"""Devices, simplex link, scenario drop and bit-error evaluation of the drop-in API.

A compact mirror of the per-drop chain of the reference
(``SimulationScenario._drop``, simulation/scenario.py:772-804) for one
transmitting and one receiving device linked by a ``MultipathFadingChannel``:

transmit   ``RandomBitsSource.generate_bits`` -> ``PskQamMapping.get_symbols`` ->
           ``OrthogonalWaveform.place/modulate`` (modem/modem.py:747-888)
propagate  ``MultipathFadingSample.propagate`` (channel/fading/fading.py:371-406)
receive    AWGN (``SimulatedDevice._generate_receiver_input``,
           simulation/simulated_device.py:1786-1830), frame = first T samples,
           demodulate -> estimate -> pick -> equalize -> unmap (modem/modem.py:1192-1267)
evaluate   ``BitErrorEvaluator`` (modem/evaluators.py:236-258)

Every array stays on the GPU; only what the caller reads is copied to the host.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .channel import MultipathFadingChannel
from .containers import Signal, StatedSymbols, Symbols, to_numpy
from .noise import AWGN


class _Antennas:
    def __init__(self, num: int) -> None:
        self.num_antennas = int(num)
        self.num_transmit_antennas = self.num_receive_antennas = int(num)


class SimulatedDevice:
    def __init__(self, bandwidth: float, antennas: int = 1, oversampling_factor: int = 1,
                 carrier_frequency: float = 0.0, noise_level=None, noise_model=None) -> None:
        if oversampling_factor != 1:
            raise NotImplementedError("the engine runs OFDM frames without oversampling")
        self.bandwidth = self.sampling_rate = float(bandwidth)
        self.antennas = _Antennas(antennas)
        self.carrier_frequency = float(carrier_frequency)
        self.noise_level = noise_level
        self.noise_model = noise_model if noise_model is not None else AWGN()
        self.transmitters: list = []
        self.receivers: list = []

    @property
    def num_antennas(self) -> int:
        return self.antennas.num_antennas


class RandomBitsSource:
    """Data bits from the engine's Philox stream (domain 1)."""

    def __init__(self, seed: int | None = None) -> None:
        self.seed = int(np.random.SeedSequence(seed).generate_state(1, np.uint64)[0]) if seed is None else int(seed)
        self.drop = 0

    def generate_bits_device(self, num_streams: int, bits_per_stream: int) -> torch.Tensor:
        out = torch.empty((num_streams, bits_per_stream), dtype=torch.uint8, device=_lib.require_cuda())
        _lib.call("hpx_bits_generate", self.seed, self.drop, 1, num_streams, bits_per_stream, _lib.ptr(out),
                  _lib.stream_ptr())
        return out

    def generate_bits(self, num_bits: int, num_streams: int = 1) -> np.ndarray:
        return to_numpy(self.generate_bits_device(num_streams, num_bits // num_streams)).reshape(-1)


class SimplexLink:
    """One transmitting and one receiving OFDM modem (modem/modem.py:1480-1604)."""

    def __init__(self, waveform=None, seed: int | None = None) -> None:
        self.waveform = waveform
        self.bits_source = RandomBitsSource(seed)
        self.transmission = None
        self.reception = None

    def transmit(self, device: SimulatedDevice) -> Signal:
        wf = self.waveform
        ns = device.num_antennas
        bits = self.bits_source.generate_bits_device(ns, wf.bits_per_frame())
        symbols = wf.mapping.get_symbols_device(bits.reshape(-1)).reshape(ns, -1)
        samples = wf.modulate_data_device(symbols)
        self.transmission = {"bits": bits.reshape(-1), "symbols": symbols, "samples": samples}
        return Signal(samples, device.sampling_rate, device.carrier_frequency)

    def receive(self, signal: Signal, device: SimulatedDevice) -> torch.Tensor:
        wf = self.waveform
        T = wf.samples_per_frame()
        # frame start from the waveform's synchronization (modem.py:1085-1146); the
        # default routine puts frames back to back from sample 0
        start = None
        for block in signal.blocks:
            found = wf.synchronization.synchronize(block.device_samples, device.bandwidth, 1)
            if found:
                start = (block, int(found[0]))
                break
        if start is None:
            self.reception = {"bits": torch.zeros(0, dtype=torch.uint8, device=signal.device_samples.device)}
            return self.reception["bits"]
        block, s0 = start
        frame = block.device_samples[:, s0:s0 + T]
        if frame.shape[1] < T:
            frame = torch.nn.functional.pad(frame, (0, T - frame.shape[1]))
        frame = frame.contiguous()
        grids = wf.demodulate_device(frame)  # (Nrx, W, N)
        stated = wf.estimate_channel(Symbols(grids), device.bandwidth, 1)
        stated.noise_variance = signal.noise_power
        picked = wf.pick(stated)
        equalized = wf.equalize_symbols(picked)
        raw = equalized.device_raw
        bits = torch.cat([wf.mapping.detect_bits_device(raw[s].reshape(-1)) for s in range(raw.shape[0])])
        self.reception = {"bits": bits, "equalized": raw, "grid": grids}
        return bits


class BitErrorArtifact:
    def __init__(self, ber: float) -> None:
        self.ber = float(ber)

    def to_scalar(self) -> float:
        return self.ber


class BitErrorEvaluation:
    def __init__(self, errors: torch.Tensor) -> None:
        self._errors = errors

    @property
    def evaluation(self) -> np.ndarray:
        return to_numpy(self._errors)

    def artifact(self) -> BitErrorArtifact:
        return BitErrorArtifact(float(self._errors.float().mean().item()) if self._errors.numel() else 0.0)


class BitErrorEvaluator:
    """Bit errors between the last transmission and reception of a link."""

    def __init__(self, transmitting_modem: SimplexLink, receiving_modem: SimplexLink | None = None) -> None:
        self.tx = transmitting_modem
        self.rx = receiving_modem if receiving_modem is not None else transmitting_modem

    @staticmethod
    def count(tx_bits: torch.Tensor, rx_bits: torch.Tensor) -> int:
        """Number of differing bits after zero-padding the shorter sequence (on the GPU)."""

        a = tx_bits.reshape(-1).contiguous()
        b = rx_bits.reshape(-1).contiguous()
        out = torch.empty(1, dtype=torch.int64, device=a.device)
        _lib.call("hpx_count_errors", _lib.ptr(a), a.numel(), _lib.ptr(b), b.numel(), 1, _lib.ptr(out),
                  _lib.stream_ptr())
        return int(out.item())

    def evaluate(self) -> BitErrorEvaluation:
        a = self.tx.transmission["bits"].to(torch.int8)
        b = self.rx.reception["bits"].to(torch.int8)
        n = max(a.numel(), b.numel())
        a = torch.nn.functional.pad(a, (0, n - a.numel()))
        b = torch.nn.functional.pad(b, (0, n - b.numel()))
        return BitErrorEvaluation((a - b).abs())


class SimulationScenario:
    """Two-device drop loop over one fading channel."""

    def __init__(self, seed: int | None = None) -> None:
        self.seed = seed
        self.devices: list[SimulatedDevice] = []
        self.channel: MultipathFadingChannel | None = None
        self.links: list[SimplexLink] = []
        self.drop_counter = 0

    def new_device(self, *args, **kwargs) -> SimulatedDevice:
        d = SimulatedDevice(*args, **kwargs)
        self.devices.append(d)
        return d

    def set_channel(self, alpha: SimulatedDevice, beta: SimulatedDevice, channel: MultipathFadingChannel) -> None:
        if alpha not in self.devices or beta not in self.devices:
            raise ValueError("Provided device is not registered with this scenario")
        self.channel = channel
        self._pair = (alpha, beta)

    def drop(self) -> dict:
        tx, rx = self._pair
        link: SimplexLink = tx.transmitters[0]
        drop = self.drop_counter
        self.drop_counter += 1
        link.bits_source.drop = drop
        signal = link.transmit(tx)
        sample = self.channel.realize().sample(tx, rx)
        received = sample.propagate(signal)
        if rx.noise_level is not None:
            power = rx.noise_level.get_power(rx.bandwidth)
            received = rx.noise_model.realize(power).add_to(received)
        bits = link.receive(received, rx)
        return {"transmitted_bits": link.transmission["bits"], "received_bits": bits, "sample": sample}
