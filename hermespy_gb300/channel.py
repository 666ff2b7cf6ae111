"""Statistical multipath fading channel of the drop-in API.

Mirrors ``hermespy/channel/fading/fading.py``: ``MultipathFadingChannel``
(:585-972) realizes ``MultipathFadingRealization`` objects (:425-583) whose
``sample(transmitter, receiver)`` returns a ``MultipathFadingSample`` (:147-422)
with ``propagate`` and ``state``. Angles, phases and the spatial response of a
realization come from the engine's Philox stream (campaign seed, drop index),
so a realization is reproducible and identical in the batched engine; the
arithmetic runs in the CUDA kernels (sum of sinusoids with 64-bit fixed-point
phases, fused tap convolution, spatial mixing and AWGN).

Model quirks of the reference that the engine keeps: the Doppler argument has
no 2*pi (``f_D t / f_s cos(.)`` radians); the tap coefficient is indexed by the
transmit time; MIMO is one SISO fading process times a random-phase spatial
matrix; antenna correlation multiplies by the covariance itself; the power
profile is not normalized.
"""

from __future__ import annotations

import ctypes
from typing import Callable

import numpy as np
import torch

from . import _lib
from .containers import DenseSignal, Signal, SignalBlock, to_device, to_numpy


class AntennaCorrelation:
    def sample_covariance(self, num_antennas: int) -> np.ndarray:  # pragma: no cover - interface
        raise NotImplementedError


class CustomAntennaCorrelation(AntennaCorrelation):
    """A fixed Hermitian positive definite covariance (fading.py:92-144)."""

    def __init__(self, covariance: np.ndarray) -> None:
        self.covariance = covariance

    @property
    def covariance(self) -> np.ndarray:
        return self._cov

    @covariance.setter
    def covariance(self, value: np.ndarray) -> None:
        value = np.asarray(value)
        if value.ndim != 2 or not np.allclose(value, value.T.conj()):
            raise ValueError("Antenna correlation must be a hermitian matrix")
        if np.any(np.linalg.eigvals(value) <= 0.0):
            raise ValueError("Antenna correlation matrix must be positive definite")
        self._cov = value.astype(np.complex128)

    def sample_covariance(self, num_antennas: int) -> np.ndarray:
        if self._cov.shape[0] < num_antennas:
            raise ValueError("Antenna correlation matrix does not match the number of antennas")
        return self._cov[:num_antennas, :num_antennas]


class ExponentialAntennaCorrelation(AntennaCorrelation):
    """Exponential correlation model: covariance entry (i, j) = rho^|i-j|.

    ``modes`` selects the array sides it describes, like the antenna mode the
    reference passes to ``sample_covariance`` (fading.py:480-489): a base station
    with correlated receive antennas serving independent single-antenna users
    uses ``modes=("rx",)``; the other side is then uncorrelated (identity).
    """

    def __init__(self, rho: float, modes: tuple = ("rx", "tx")) -> None:
        if not 0.0 <= rho < 1.0:
            raise ValueError("correlation coefficient must be in [0, 1)")
        self.rho = float(rho)
        self.modes = tuple(modes)

    def sample_covariance(self, num_antennas: int, mode: str = "rx") -> np.ndarray:
        i = np.arange(num_antennas)
        if mode not in self.modes:
            return np.eye(num_antennas, dtype=np.complex128)
        return (self.rho ** np.abs(i[:, None] - i[None, :])).astype(np.complex128)


def _covariance(model, num_antennas: int, mode: str) -> np.ndarray:
    try:
        return model.sample_covariance(num_antennas, mode)
    except TypeError:  # models without an antenna-mode argument describe both sides
        return model.sample_covariance(num_antennas)


def _num_antennas(device) -> int:
    if isinstance(device, int):
        return device
    ant = getattr(device, "antennas", None)
    if ant is not None:
        return int(getattr(ant, "num_antennas", ant))
    return int(getattr(device, "num_antennas"))


def _sampling_rate(device) -> float:
    return float(getattr(device, "sampling_rate"))


class LinkState:
    """Transmitter / receiver antenna counts and the sampling rate of one link."""

    def __init__(self, num_transmit_antennas: int, num_receive_antennas: int, sampling_rate: float,
                 transmitter=None, receiver=None) -> None:
        self.num_transmit_antennas = int(num_transmit_antennas)
        self.num_receive_antennas = int(num_receive_antennas)
        self.bandwidth = self.sampling_rate = float(sampling_rate)
        self.transmitter = transmitter
        self.receiver = receiver


class _FadingHandle:
    """An ``hpx_fading`` handle for one (channel parameters, antennas, rate) set."""

    def __init__(self, delays, power, rice, S, doppler, los_doppler, gain, nrx, ntx, fs, rx_cov=None, tx_cov=None,
                 los_gains=None, nlos_gains=None) -> None:
        lib = _lib.load()
        self._keep = []

        def arr(a, dtype=np.float64):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
            self._keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

        def carr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128)).view(np.float64)
            self._keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

        desc = _lib.FadingDesc(len(delays), int(S), int(nrx), int(ntx), float(fs), float(doppler), float(los_doppler),
                               float(gain), arr(delays), arr(power), arr(rice), carr(rx_cov), carr(tx_cov),
                               arr(los_gains), arr(nlos_gains))
        h = ctypes.c_void_p()
        _lib.check(lib.hpx_fading_create(ctypes.byref(desc), ctypes.byref(h)))
        self.handle = h
        nbytes = ctypes.c_int64()
        _lib.check(lib.hpx_fading_state_bytes(h, 1, ctypes.byref(nbytes)))
        self.state_bytes = int(nbytes.value)
        d = ctypes.c_int32()
        _lib.check(lib.hpx_fading_max_delay(h, ctypes.byref(d)))
        self.max_delay = int(d.value)
        self.L, self.S, self.nrx, self.ntx = len(delays), int(S), int(nrx), int(ntx)
        self.num_draws = nrx * ntx + 2 * self.L * (1 + self.S)

    def __del__(self):
        try:
            if _lib._lib is not None:
                _lib._lib.hpx_fading_destroy(self.handle)
        except Exception:
            pass

    def new_state(self, num_drops: int) -> torch.Tensor:
        return torch.empty(self.state_bytes * num_drops, dtype=torch.uint8, device=_lib.require_cuda())


class MultipathFadingSample:
    """One sample of the fading channel for one link (fading.py:147-422)."""

    def __init__(self, power_profile, delay_profile, los_angles, nlos_angles, los_phases, nlos_phases, los_gains,
                 nlos_gains, los_doppler, nlos_doppler, spatial_response, gain, state: LinkState,
                 _handle: _FadingHandle | None = None, _device_state: torch.Tensor | None = None) -> None:
        self.power_profile = np.asarray(power_profile, dtype=np.float64)
        self.delay_profile = np.asarray(delay_profile, dtype=np.float64)
        self.los_angles = np.asarray(los_angles, dtype=np.float64)
        self.nlos_angles = np.asarray(nlos_angles, dtype=np.float64)
        self.los_phases = np.asarray(los_phases, dtype=np.float64)
        self.nlos_phases = np.asarray(nlos_phases, dtype=np.float64)
        self.los_gains = np.asarray(los_gains, dtype=np.float64)
        self.nlos_gains = np.asarray(nlos_gains, dtype=np.float64)
        self.los_doppler = float(los_doppler)
        self.nlos_doppler = float(nlos_doppler)
        self.spatial_response = np.asarray(spatial_response, dtype=np.complex128)
        self.gain = float(gain)
        self.state_info = state
        self.bandwidth = self.sampling_rate = state.sampling_rate
        self.num_receive_antennas = state.num_receive_antennas
        self.num_transmit_antennas = state.num_transmit_antennas
        if _handle is None:
            nrx, ntx = self.spatial_response.shape
            order = np.argsort(self.delay_profile, kind="stable")
            _handle = _FadingHandle(self.delay_profile[order], self.power_profile[order],
                                    np.zeros(order.size), self.nlos_angles.shape[1] if self.nlos_angles.ndim == 2 else 0,
                                    self.nlos_doppler, self.los_doppler, self.gain, nrx, ntx, self.sampling_rate,
                                    los_gains=self.los_gains[order], nlos_gains=self.nlos_gains[order])
            dev_state = _handle.new_state(1)
            la = to_device(self.los_angles[order], torch.float64)
            na = to_device(self.nlos_angles[order].reshape(-1), torch.float64)
            lp = to_device(self.los_phases[order], torch.float64)
            np_ = to_device(self.nlos_phases[order].reshape(-1), torch.float64)
            sp = to_device(np.ascontiguousarray(self.spatial_response).view(np.float64).reshape(-1), torch.float64)
            _lib.call("hpx_fading_load", _handle.handle, 1, _lib.ptr(la), _lib.ptr(na), _lib.ptr(lp), _lib.ptr(np_),
                      _lib.ptr(sp), _lib.ptr(dev_state), _lib.stream_ptr())
            _device_state = dev_state
        self._handle = _handle
        self._state = _device_state

    @property
    def max_delay(self) -> float:
        return float(self.delay_profile.max())

    @property
    def expected_energy_scale(self) -> float:
        return self.gain * float(np.sum(self.power_profile))

    def path_impulses_device(self, num_samples: int) -> torch.Tensor:
        out = torch.empty((self._handle.L, num_samples), dtype=torch.complex64, device=self._state.device)
        _lib.call("hpx_fading_taps", self._handle.handle, _lib.ptr(self._state), 1, num_samples, _lib.ptr(out),
                  _lib.stream_ptr())
        return out

    def propagate_device(self, samples: torch.Tensor, noise_power: float | None = None, seed: int = 0,
                         drop: int = 0) -> torch.Tensor:
        """(Ntx, T) -> (Nrx, T + D) on the GPU, optionally with AWGN from the Philox stream."""

        x = to_device(samples)
        if x.ndim == 1:
            x = x[None]
        if x.shape[0] != self._handle.ntx:
            raise ValueError(
                f"Number of signal streams ({x.shape[0]}) does not match the number of transmit antennas "
                f"({self._handle.ntx})")
        T = x.shape[1]
        y = torch.empty((self._handle.nrx, T + self._handle.max_delay), dtype=torch.complex64, device=x.device)
        npow = None
        if noise_power is not None:
            npow = torch.tensor([float(noise_power)], dtype=torch.float32, device=x.device)
        _lib.call("hpx_fading_propagate", self._handle.handle, _lib.ptr(self._state), 1, _lib.ptr(x.contiguous()), T,
                  _lib.ptr(y), _lib.ptr(npow), seed, drop, _lib.stream_ptr())
        return y

    def propagate(self, signal, interpolation_mode=None) -> Signal:
        """Propagate every block of ``signal`` (channel.py:306-379, fading.py:371-406).

        As in the reference, each block is convolved with the taps from time zero
        of the realization and keeps its offset; several blocks give a sparse
        signal. A channel with zero expected energy returns an empty signal.
        """

        if not isinstance(signal, Signal):
            return Signal(self.propagate_device(signal), self.sampling_rate)
        if self.expected_energy_scale <= 0.0:
            return Signal.Empty(signal.sampling_rate, self.num_receive_antennas, 0,
                                carrier_frequency=signal.carrier_frequency, noise_power=signal.noise_power,
                                delay=signal.delay)
        if signal.num_streams != self.num_transmit_antennas:
            raise ValueError(f"Number of signal streams to be propagated does not match the number of transmitter "
                             f"antennas ({signal.num_streams} != {self.num_transmit_antennas}))")
        if signal.num_blocks == 1 and isinstance(signal, DenseSignal):
            y = self.propagate_device(signal.device_samples)
            return DenseSignal(y, signal.sampling_rate, signal.carrier_frequency, signal.noise_power, signal.offset,
                               signal.delay)
        blocks = [SignalBlock(self.propagate_device(b.device_samples), b.offset) for b in signal.blocks]
        return Signal.Create(blocks, self.sampling_rate, signal.carrier_frequency, signal.noise_power, signal.delay,
                             offsets=[b.offset for b in blocks])

    def state_device(self, num_samples: int, max_num_taps: int) -> torch.Tensor:
        ntaps = min(1 + self._handle.max_delay, int(max_num_taps))
        out = torch.empty((self._handle.nrx, self._handle.ntx, num_samples, ntaps), dtype=torch.complex64,
                          device=self._state.device)
        _lib.call("hpx_fading_csi", self._handle.handle, _lib.ptr(self._state), 1, num_samples, max_num_taps,
                  _lib.ptr(out), _lib.stream_ptr())
        return out

    def state(self, num_samples: int, max_num_taps: int, interpolation_mode=None) -> "ChannelStateInformation":
        return ChannelStateInformation(self.state_device(num_samples, max_num_taps))


class ChannelStateInformation:
    """Impulse-response channel state (core/channel.py:42-551), dense."""

    def __init__(self, state: torch.Tensor) -> None:
        self._state = state

    @property
    def device_state(self) -> torch.Tensor:
        return self._state

    def dense_state(self) -> np.ndarray:
        return to_numpy(self._state)

    @property
    def num_delay_taps(self) -> int:
        return int(self._state.shape[3])


class MultipathFadingRealization:
    """A channel realization: the draws of one drop (fading.py:425-583)."""

    def __init__(self, channel: "MultipathFadingChannel", drop: int) -> None:
        self.channel = channel
        self.drop = int(drop)

    def sample(self, transmitter, receiver, timestamp: float = 0.0, carrier_frequency: float = 0.0,
               sampling_rate: float | None = None) -> MultipathFadingSample:
        ntx, nrx = _num_antennas(transmitter), _num_antennas(receiver)
        fs = float(sampling_rate) if sampling_rate is not None else _sampling_rate(transmitter)
        state = LinkState(ntx, nrx, fs, transmitter, receiver)
        sample = self.channel._sample(self.drop, state)
        for hook, tx, rx in self.channel._hooks:
            if (tx is None or tx is transmitter) and (rx is None or rx is receiver):
                hook(sample)
        return sample


class MultipathFadingChannel:
    """Statistical multipath fading channel (fading.py:585-972)."""

    def __init__(self, delays, power_profile, rice_factors, correlation_distance: float = float("inf"),
                 num_sinusoids: int = 20, los_angle: float | None = None, doppler_frequency: float = 0.0,
                 los_doppler_frequency: float | None = None, antenna_correlation: AntennaCorrelation | None = None,
                 gain: float = 1.0, seed: int | None = None) -> None:
        delays = np.asarray(delays, dtype=np.float64)
        power_profile = np.asarray(power_profile, dtype=np.float64)
        rice_factors = np.asarray(rice_factors, dtype=np.float64)
        if delays.ndim != 1 or power_profile.ndim != 1 or rice_factors.ndim != 1:
            raise ValueError("Delays, power profile and rice factors must be vectors")
        if len(delays) < 1:
            raise ValueError("Configuration must contain at least one delay tap")
        if len(delays) != len(power_profile) or len(power_profile) != len(rice_factors):
            raise ValueError("Delays, power profile and rice factor vectors must be of equal length")
        if np.any(delays < 0.0):
            raise ValueError("Delays must be greater or equal to zero")
        if np.any(power_profile < 0.0):
            raise ValueError("Power profile factors must be greater or equal to zero")
        if np.any(rice_factors < 0.0):
            raise ValueError("Rice factors must be greater or equal to zero")
        if num_sinusoids < 0:
            raise ValueError("Number of sinusoids must be greater or equal to zero")
        if correlation_distance != float("inf"):
            raise NotImplementedError("the engine realizes spatially static channels (infinite correlation distance)")
        order = np.argsort(delays, kind="stable")
        self.delays = delays[order]
        self.power_profile = power_profile[order]
        self.rice_factors = rice_factors[order]
        self.num_sinusoids = int(num_sinusoids)
        self.correlation_distance = correlation_distance
        self.los_angle = los_angle
        self.doppler_frequency = float(doppler_frequency)
        self._los_doppler = los_doppler_frequency
        self.antenna_correlation = antenna_correlation
        self.gain = float(gain)
        self.seed = int(np.random.SeedSequence(seed).generate_state(1, np.uint64)[0]) if seed is None else int(seed)
        self.drop_counter = 0
        self._handles: dict = {}
        self._hooks: list = []

    @property
    def los_doppler_frequency(self) -> float:
        return self.doppler_frequency if self._los_doppler is None else float(self._los_doppler)

    @los_doppler_frequency.setter
    def los_doppler_frequency(self, value: float | None) -> None:
        self._los_doppler = value

    @property
    def max_delay(self) -> float:
        return float(self.delays.max())

    @property
    def num_resolvable_paths(self) -> int:
        return int(self.delays.size)

    def gains(self) -> tuple[np.ndarray, np.ndarray]:
        k = self.rice_factors
        inf = np.isposinf(k)
        los = np.ones_like(k)
        nlos = np.zeros_like(k)
        los[~inf] = np.sqrt(k[~inf] / (1 + k[~inf]))
        nlos[~inf] = np.sqrt(1 / ((1 + k[~inf]) * self.num_sinusoids)) if self.num_sinusoids else 0.0
        return los, nlos

    def add_sample_hook(self, callback: Callable, transmitter=None, receiver=None) -> None:
        self._hooks.append((callback, transmitter, receiver))

    def handle(self, num_rx: int, num_tx: int, sampling_rate: float) -> _FadingHandle:
        key = (num_rx, num_tx, float(sampling_rate), self.doppler_frequency, self.los_doppler_frequency, self.gain)
        h = self._handles.get(key)
        if h is None:
            rx_cov = tx_cov = None
            if self.antenna_correlation is not None:
                rx_cov = _covariance(self.antenna_correlation, num_rx, "rx")
                tx_cov = _covariance(self.antenna_correlation, num_tx, "tx")
            h = _FadingHandle(self.delays, self.power_profile, self.rice_factors, self.num_sinusoids,
                              self.doppler_frequency, self.los_doppler_frequency, self.gain, num_rx, num_tx,
                              sampling_rate, rx_cov, tx_cov)
            self._handles[key] = h
        return h

    def realize(self) -> MultipathFadingRealization:
        r = MultipathFadingRealization(self, self.drop_counter)
        self.drop_counter += 1
        return r

    def draws(self, drop: int, num_rx: int, num_tx: int, sampling_rate: float) -> np.ndarray:
        """The float64 uniforms of one drop in the realization's draw layout."""

        h = self.handle(num_rx, num_tx, sampling_rate)
        out = torch.empty(h.num_draws, dtype=torch.float64, device=_lib.require_cuda())
        _lib.call("hpx_fading_draws", h.handle, self.seed, drop, 1, _lib.ptr(out), _lib.stream_ptr())
        return out.cpu().numpy()

    def _sample(self, drop: int, state: LinkState) -> MultipathFadingSample:
        nrx, ntx, fs = state.num_receive_antennas, state.num_transmit_antennas, state.sampling_rate
        h = self.handle(nrx, ntx, fs)
        dev_state = h.new_state(1)
        _lib.call("hpx_fading_realize", h.handle, self.seed, drop, 1, _lib.ptr(dev_state), _lib.stream_ptr())
        u = self.draws(drop, nrx, ntx, fs)
        L, S = self.num_resolvable_paths, self.num_sinusoids
        o = nrx * ntx
        spatial = np.exp(2j * np.pi * u[:o].reshape(nrx, ntx))
        if self.antenna_correlation is not None:
            spatial = _covariance(self.antenna_correlation, nrx, "rx") @ spatial @ \
                _covariance(self.antenna_correlation, ntx, "tx")
        los_angles = 2 * np.pi * u[o:o + L]
        nlos_angles = -np.pi + 2 * np.pi * u[o + L:o + L + L * S].reshape(L, S)
        los_phases = -np.pi + 2 * np.pi * u[o + L + L * S:o + 2 * L + L * S]
        nlos_phases = -np.pi + 2 * np.pi * u[o + 2 * L + L * S:].reshape(L, S)
        los_g, nlos_g = self.gains()
        return MultipathFadingSample(self.power_profile, self.delays, los_angles, nlos_angles, los_phases, nlos_phases,
                                     los_g, nlos_g, self.los_doppler_frequency, self.doppler_frequency, spatial,
                                     self.gain, state, _handle=h, _device_state=dev_state)

    def propagate(self, signal: Signal, transmitter, receiver) -> Signal:
        return self.realize().sample(transmitter, receiver).propagate(signal)


class Exponential(MultipathFadingChannel):
    """Exponential power-delay profile (channel/fading/exponential.py:22-169)."""

    def __init__(self, tap_interval: float, rms_delay: float, **kwargs) -> None:
        if tap_interval <= 0.0:
            raise ValueError("Tap interval must be greater than zero")
        if rms_delay <= 0.0:
            raise ValueError("Root-mean-squared delay must be greater than zero")
        rms_norm = rms_delay / tap_interval
        alpha = -2 * np.log((-1 + np.sqrt(1 + 4 * rms_norm**2)) / (2 * rms_norm))
        max_delay_in_samples = int(-np.ceil(np.log(1e-5) / alpha))
        delays = np.arange(max_delay_in_samples + 1) * tap_interval
        power = np.exp(-alpha * np.arange(max_delay_in_samples + 1))
        MultipathFadingChannel.__init__(self, delays, power, np.zeros(delays.size), **kwargs)
