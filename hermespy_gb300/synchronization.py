"""Frame synchronization of the drop-in API.

Mirrors ``Synchronization`` (modem/waveform.py:30-108), the OFDM Schmidl-Cox
routine (modem/waveforms/orthogonal/ofdm.py:208-257) and the pilot-correlation
routine (modem/waveform_correlation_synchronization.py:27-186). The metric over
every candidate delay and the ``scipy.signal.find_peaks`` search the reference
runs on it (same height and distance rules, plateau midpoints, index offsets and
clipping) both run on the GPU (``hpx_sync_schmidl_cox`` / ``hpx_sync_correlation``
then ``hpx_sync_peaks``); only the frame start indices come back to the host. The
``*_batch`` methods synchronize many received signals in one launch each.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .containers import Signal, to_device

MAX_FRAMES = 64  # frame starts returned per signal


def _peaks(metric: torch.Tensor, normalize: bool, height: float, distance: int, offset: int, clip: bool = False,
           clip_max: int = 0, clip_value: int = 0, max_frames: int = MAX_FRAMES) -> list[list[int]]:
    """Device find_peaks over each row of ``metric`` (batch, length)."""

    metric = metric.contiguous()
    batch, length = metric.shape
    starts = torch.empty((batch, max_frames), dtype=torch.int64, device=metric.device)
    counts = torch.empty(batch, dtype=torch.int32, device=metric.device)
    _lib.call("hpx_sync_peaks", _lib.ptr(metric), batch, length, int(normalize), float(height), int(distance),
              int(offset), int(clip), int(clip_max), int(clip_value), max_frames, _lib.ptr(starts), _lib.ptr(counts),
              _lib.stream_ptr())
    c = counts.cpu().numpy()
    if np.any(c < 0):
        raise RuntimeError("synchronization: more than 512 candidate peaks above the detection height")
    if np.any(c > max_frames):
        raise RuntimeError(f"synchronization: more than {max_frames} frames in one signal")
    st = starts.cpu().numpy()
    return [st[b, : c[b]].tolist() for b in range(batch)]


def _batch_tensor(signals) -> torch.Tensor:
    t = signals if isinstance(signals, torch.Tensor) else to_device(signals)
    t = t.to(torch.complex64)
    if t.ndim == 2:
        t = t[:, None, :]
    if t.ndim != 3:
        raise ValueError("batched synchronization expects (signals, streams, samples)")
    return t.contiguous()


def _signal_tensor(signal) -> torch.Tensor:
    t = signal.device_samples if isinstance(signal, Signal) else to_device(signal)
    if t.ndim == 1:
        t = t[None, :]
    return t.contiguous()


class Synchronization:
    """Frames back to back from sample 0 (waveform.py:67-99)."""

    def __init__(self, waveform=None) -> None:
        self._waveform = None
        self.waveform = waveform

    @property
    def waveform(self):
        return self._waveform

    @waveform.setter
    def waveform(self, value) -> None:
        self._waveform = value
        if value is not None and getattr(value, "_synchronization", None) is not self:
            value._synchronization = self

    def _require_waveform(self):
        if self._waveform is None:
            raise RuntimeError("Trying to synchronize with a floating synchronization routine")
        return self._waveform

    def synchronize(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> list[int]:
        wf = self._require_waveform()
        n = _signal_tensor(signal).shape[1]
        spf = wf.samples_per_frame(bandwidth, oversampling_factor)
        num_frames = n // spf
        if num_frames < 1:
            return []
        return list(range(0, num_frames * spf, spf))


class OFDMSynchronization(Synchronization):
    """Synchronization routine base of OFDM waveforms (ofdm.py:208-211)."""


class SchmidlCoxSynchronization(OFDMSynchronization):
    """Schmidl-Cox timing: the delay whose two half-symbol windows correlate best.

    Needs a ``SchmidlCoxPilotSection`` on the waveform (ofdm.py:214-257).
    """

    def metric_batch(self, signals, bandwidth: float = 1.0, oversampling_factor: int = 1) -> torch.Tensor:
        """``delay_powers`` (leading zero included) of (signals, streams, samples) on the GPU."""

        wf = self._require_waveform()
        x = _batch_tensor(signals)
        L = oversampling_factor * wf.num_subcarriers
        B, S, n = x.shape
        out = torch.empty((B, max(n - L + 2, 0)), dtype=torch.float64, device=x.device)
        if n >= L:
            _lib.call("hpx_sync_schmidl_cox", _lib.ptr(x), B, S, n, L, _lib.ptr(out), _lib.stream_ptr())
        return out

    def metric_device(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> torch.Tensor:
        """The reference's ``delay_powers`` vector of one signal on the GPU."""

        return self.metric_batch(_signal_tensor(signal)[None], bandwidth, oversampling_factor)[0]

    def synchronize_batch(self, signals, bandwidth: float = 1.0, oversampling_factor: int = 1) -> list[list[int]]:
        wf = self._require_waveform()
        x = _batch_tensor(signals)
        if x.shape[2] < oversampling_factor * wf.num_subcarriers:
            return [[] for _ in range(x.shape[0])]
        spf = wf.samples_per_frame(bandwidth, oversampling_factor)
        return _peaks(self.metric_batch(x, bandwidth, oversampling_factor), False, 0.75, int(0.9 * spf), -1)

    def synchronize(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> list[int]:
        return self.synchronize_batch(_signal_tensor(signal)[None], bandwidth, oversampling_factor)[0]


class CorrelationSynchronization(Synchronization):
    """Cross-correlation with the waveform's pilot signal (waveform_correlation_synchronization.py:27-186).

    As in the reference, detection uses a normalized height of 0.9 and a peak
    distance of 0.8 frames; ``threshold`` and ``guard_ratio`` are validated and,
    with ``peak_prominence``, stored.
    """

    def __init__(self, threshold: float = 0.9, guard_ratio: float = 0.8, peak_prominence: float = 0.2,
                 waveform=None) -> None:
        self.threshold = threshold
        self.guard_ratio = guard_ratio
        self.peak_prominence = peak_prominence
        Synchronization.__init__(self, waveform)

    @property
    def threshold(self) -> float:
        return self._threshold

    @threshold.setter
    def threshold(self, value: float) -> None:
        if value < 0.0 or value > 1.0:
            raise ValueError("Synchronization threshold must be between zero and one.")
        self._threshold = float(value)

    @property
    def guard_ratio(self) -> float:
        return self._guard_ratio

    @guard_ratio.setter
    def guard_ratio(self, value: float) -> None:
        if value < 0.0 or value > 1.0:
            raise ValueError("Synchronization guard ratio must be between zero and one.")
        self._guard_ratio = float(value)

    def _pilot(self, bandwidth: float, oversampling_factor: int) -> torch.Tensor:
        wf = self._require_waveform()
        pilot = wf.pilot_signal(bandwidth, oversampling_factor).device_samples.reshape(-1).contiguous()
        if pilot.numel() < 1:
            raise RuntimeError("No pilot sequence configured, time-domain correlation synchronization impossible")
        return pilot

    def correlation_batch(self, signals, bandwidth: float = 1.0, oversampling_factor: int = 1) -> torch.Tensor:
        """Un-normalized correlation profiles (signals, samples + pilot - 1) on the GPU."""

        x = _batch_tensor(signals)
        pilot = self._pilot(bandwidth, oversampling_factor)
        B, S, n = x.shape
        out = torch.empty((B, n + pilot.numel() - 1), dtype=torch.float64, device=x.device)
        _lib.call("hpx_sync_correlation", _lib.ptr(x), B, S, n, _lib.ptr(pilot), pilot.numel(), _lib.ptr(out),
                  _lib.stream_ptr())
        return out

    def correlation_device(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> torch.Tensor:
        return self.correlation_batch(_signal_tensor(signal)[None], bandwidth, oversampling_factor)[0]

    def synchronize_batch(self, signals, bandwidth: float = 1.0, oversampling_factor: int = 1) -> list[list[int]]:
        wf = self._require_waveform()
        x = _batch_tensor(signals)
        if x.numel() < 1:
            return [[] for _ in range(x.shape[0])]
        frame_length = wf.samples_per_frame(bandwidth, oversampling_factor)
        pilot_length = self._pilot(bandwidth, oversampling_factor).numel()
        n = x.shape[2]
        return _peaks(self.correlation_batch(x, bandwidth, oversampling_factor), True, 0.9, int(0.8 * frame_length),
                      1 - pilot_length, True, n - frame_length, abs(n - frame_length))

    def synchronize(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> list[int]:
        return self.synchronize_batch(_signal_tensor(signal)[None], bandwidth, oversampling_factor)[0]


class OFDMCorrelationSynchronization(CorrelationSynchronization):
    """Correlation-based pilot detection for OFDM waveforms (ofdm.py:214-216)."""
