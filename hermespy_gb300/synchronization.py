"""Frame synchronization of the drop-in API.

Mirrors ``Synchronization`` (modem/waveform.py:30-108), the OFDM Schmidl-Cox
routine (modem/waveforms/orthogonal/ofdm.py:208-257) and the pilot-correlation
routine (modem/waveform_correlation_synchronization.py:27-186). The metric over
every candidate delay — the part whose cost grows with the signal length times the
symbol (or pilot) length — runs in the ``hpx_sync_*`` kernels; the peak search on
the FP64 metric is the reference's own ``scipy.signal.find_peaks`` call with the
same height and distance rules, on the host.
"""

from __future__ import annotations

import numpy as np
import torch
from scipy.signal import find_peaks

from . import _lib
from .containers import Signal, to_device


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

    def metric_device(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> torch.Tensor:
        """The reference's ``delay_powers`` vector (leading zero included) on the GPU."""

        wf = self._require_waveform()
        x = _signal_tensor(signal)
        L = oversampling_factor * wf.num_subcarriers
        n = x.shape[1]
        out = torch.empty(max(n - L + 2, 0), dtype=torch.float64, device=x.device)
        if n >= L:
            _lib.call("hpx_sync_schmidl_cox", _lib.ptr(x), 1, x.shape[0], n, L, _lib.ptr(out), _lib.stream_ptr())
        return out

    def synchronize(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> list[int]:
        wf = self._require_waveform()
        if _signal_tensor(signal).shape[1] < oversampling_factor * wf.num_subcarriers:
            return []
        powers = self.metric_device(signal, bandwidth, oversampling_factor).cpu().numpy()
        spf = wf.samples_per_frame(bandwidth, oversampling_factor)
        peaks, _ = find_peaks(powers, distance=int(0.9 * spf), height=0.75 * np.max(powers))
        return (peaks - 1).tolist()


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

    def correlation_device(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> torch.Tensor:
        """Un-normalized correlation profile (length samples + pilot - 1) on the GPU."""

        wf = self._require_waveform()
        x = _signal_tensor(signal)
        pilot = wf.pilot_signal(bandwidth, oversampling_factor).device_samples.reshape(-1).contiguous()
        if pilot.numel() < 1:
            raise RuntimeError("No pilot sequence configured, time-domain correlation synchronization impossible")
        n = x.shape[1]
        out = torch.empty(n + pilot.numel() - 1, dtype=torch.float64, device=x.device)
        _lib.call("hpx_sync_correlation", _lib.ptr(x), 1, x.shape[0], n, _lib.ptr(pilot), pilot.numel(),
                  _lib.ptr(out), _lib.stream_ptr())
        return out

    def synchronize(self, signal, bandwidth: float = 1.0, oversampling_factor: int = 1) -> list[int]:
        wf = self._require_waveform()
        x = _signal_tensor(signal)
        if x.numel() < 1:
            return []
        correlation = self.correlation_device(x, bandwidth, oversampling_factor).cpu().numpy()
        correlation /= correlation.max()
        frame_length = wf.samples_per_frame(bandwidth, oversampling_factor)
        indices, _ = find_peaks(np.abs(correlation), height=0.9, distance=int(0.8 * frame_length))
        if len(indices) < 1:
            return []
        pilot_length = wf.pilot_signal(bandwidth, oversampling_factor).num_samples
        indices = indices - (pilot_length - 1)
        indices = np.where(indices < 0, 0, indices)
        n = x.shape[1]
        indices = np.where(indices > (n - frame_length), abs(n - frame_length), indices)
        return indices.tolist()


class OFDMCorrelationSynchronization(CorrelationSynchronization):
    """Correlation-based pilot detection for OFDM waveforms (ofdm.py:214-216)."""
