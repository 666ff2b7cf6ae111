"""Batched Monte Carlo drop engine.

``LinkEngine`` runs whole drops of a simplex OFDM link over a
``MultipathFadingChannel`` in batches on the GPU through ``hpx_link_run``: one
call realizes the channels, generates and modulates the Philox bits, propagates
with AWGN, demodulates, estimates (ideal CSI or LS), equalizes (ZF or LMMSE),
demaps and counts bit errors per drop. It replaces the reference's per-drop
Python loop (``MonteCarloActor.__run_batch``, core/pymonte/actors.py:367-452,
running ``SimulationScenario._drop`` and ``BitErrorEvaluator`` per sample) for
throughput runs; every drop is the same drop the per-drop API simulates for the
same (seed, drop index).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch
from scipy.stats import beta

from . import _lib
from .channel import MultipathFadingChannel
from .estimation import ls_interpolation_table
from .waveform import OFDMWaveform


def clopper_pearson(errors: int, trials: int, confidence: float = 0.95) -> tuple[float, float]:
    """Exact binomial confidence interval of a bit-error rate."""

    a = 1.0 - confidence
    lo = 0.0 if errors == 0 else float(beta.ppf(a / 2, errors, trials - errors + 1))
    hi = 1.0 if errors == trials else float(beta.ppf(1 - a / 2, errors + 1, trials - errors))
    return lo, hi


@dataclass
class BerPoint:
    level_db: float
    errors: int
    bits: int

    @property
    def ber(self) -> float:
        return self.errors / self.bits if self.bits else 0.0

    @property
    def interval(self) -> tuple[float, float]:
        return clopper_pearson(self.errors, self.bits)


class LinkEngine:
    def __init__(self, waveform: OFDMWaveform, channel: MultipathFadingChannel, num_tx: int, num_rx: int,
                 sampling_rate: float, estimator: str = "ideal", equalizer: str = "lmmse", noise: str = "snr",
                 max_drops: int = 4096, seed: int = 0) -> None:
        if estimator not in ("ideal", "ls"):
            raise ValueError("estimator must be 'ideal' or 'ls'")
        if equalizer not in ("zf", "lmmse"):
            raise ValueError("equalizer must be 'zf' or 'lmmse'")
        if noise not in ("snr", "ebn0"):
            raise ValueError("noise must be 'snr' or 'ebn0'")
        self.waveform = waveform
        self.channel = channel
        self.num_tx, self.num_rx = int(num_tx), int(num_rx)
        self.sampling_rate = float(sampling_rate)
        self.estimator, self.equalizer, self.noise = estimator, equalizer, noise
        self.max_drops = int(max_drops)
        self.seed = int(seed)
        self.device = _lib.require_cuda()
        self._fading = channel.handle(num_rx, num_tx, sampling_rate)
        self._frame = waveform._frame()
        self._ls = None
        if estimator == "ls" and (num_tx != 1 or num_rx != 1):
            raise NotImplementedError("Least-Squares channel estimation is only implemented for SISO links")
        if estimator == "ls":
            mask = waveform.resource_mask[0]
            indptr, indices, weights = ls_interpolation_table(mask[:, : waveform._layout()["num_columns"]])
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_ls_create(self._frame, mask[:, : waveform._layout()["num_columns"]].shape[1],
                                                 indptr.ctypes.data_as(ctypes.c_void_p),
                                                 indices.ctypes.data_as(ctypes.c_void_p),
                                                 weights.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)))
            self._ls = h
        h = ctypes.c_void_p()
        _lib.check(_lib.load().hpx_link_create(self._frame, self._fading.handle, self._ls,
                                               _lib.EST_IDEAL if estimator == "ideal" else _lib.EST_LS,
                                               _lib.EQ_ZF if equalizer == "zf" else _lib.EQ_LMMSE, self.max_drops,
                                               ctypes.byref(h)))
        self._link = h
        self.bits_per_drop = waveform.bits_per_frame() * num_tx

    def __del__(self):
        try:
            if _lib._lib is not None:
                _lib._lib.hpx_link_destroy(self._link)
                if self._ls is not None:
                    _lib._lib.hpx_ls_destroy(self._ls)
        except Exception:
            pass

    def noise_power(self, level_db) -> np.ndarray:
        """Noise power of EBN0 / SNR levels in dB (simulation/modem/noise.py:97-98,
        simulation/rf/noise/level.py:258-259)."""

        level = 10.0 ** (np.asarray(level_db, dtype=np.float64) / 10.0)
        if self.noise == "ebn0":
            return self.waveform.bit_energy(self.sampling_rate, 1) / level
        scale = self.channel.gain * float(np.sum(self.channel.power_profile))
        return self.waveform.power / level * scale

    def run(self, drop0: int, noise_power: torch.Tensor, errors: torch.Tensor | None = None,
            stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        """Enqueue drops [drop0, drop0 + len(noise_power)) on the stream; returns per-drop
        bit errors (uint32 on the GPU). Does not synchronize."""

        n = noise_power.numel()
        if errors is None:
            errors = torch.empty(n, dtype=torch.int32, device=self.device)
        _lib.call("hpx_link_run", self._link, self.seed, int(drop0), n, _lib.ptr(noise_power), _lib.ptr(errors),
                  _lib.stream_ptr(stream))
        return errors

    def simulate(self, noise_power_host: np.ndarray, drop0: int = 0) -> np.ndarray:
        """Host noise powers in, host per-drop bit errors out (batched by max_drops)."""

        p = np.ascontiguousarray(np.asarray(noise_power_host, dtype=np.float32))
        out = np.empty(p.size, dtype=np.int64)
        for s in range(0, p.size, self.max_drops):
            chunk = torch.from_numpy(p[s:s + self.max_drops]).to(self.device, non_blocking=True)
            e = self.run(drop0 + s, chunk)
            out[s:s + chunk.numel()] = e.cpu().numpy().astype(np.int64)
        return out

    def ber_curve(self, levels_db, drops_per_level: int, drop0: int = 0) -> list[BerPoint]:
        levels_db = list(levels_db)
        powers = np.repeat(self.noise_power(levels_db), drops_per_level)
        errs = self.simulate(powers, drop0)
        pts = []
        for i, lv in enumerate(levels_db):
            e = int(errs[i * drops_per_level:(i + 1) * drops_per_level].sum())
            pts.append(BerPoint(float(lv), e, drops_per_level * self.bits_per_drop))
        return pts
