"""Batched Monte Carlo drop engine.

``LinkEngine`` runs whole drops of a simplex OFDM link over a
``MultipathFadingChannel`` in batches on the GPU. With ideal CSI or SISO LS one
``hpx_link_run`` call realizes the channels, generates and modulates the Philox
bits, propagates with AWGN, demodulates, estimates, equalizes (ZF or LMMSE),
demaps and counts bit errors per drop. The MIMO estimators of a pilot-comb frame
(per-stream LS, tap-domain LMMSE, the learned estimator) run the same stages as
separate launches with the estimate materialized as a CSI grid, followed by
``hpx_detect_csi``. It replaces the reference's per-drop
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
from .estimation import ls_interpolation_table, ls_stream_tables, robust_statistics
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
    drops: int = 0
    confident: bool = False

    @property
    def ber(self) -> float:
        return self.errors / self.bits if self.bits else 0.0

    @property
    def interval(self) -> tuple[float, float]:
        return clopper_pearson(self.errors, self.bits)


class LinkEngine:
    def __init__(self, waveform: OFDMWaveform, channel: MultipathFadingChannel, num_tx: int, num_rx: int,
                 sampling_rate: float, estimator: str = "ideal", equalizer: str = "lmmse", noise: str = "snr",
                 max_drops: int = 4096, seed: int = 0, model=None, also: tuple = ()) -> None:
        if estimator not in ("ideal", "ls", "lmmse", "lmmse_robust", "learned"):
            raise ValueError("estimator must be 'ideal', 'ls', 'lmmse', 'lmmse_robust' or 'learned'")
        if estimator == "learned" and model is None:
            raise ValueError("the learned estimator needs a model")
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
        self._lmmse = None
        self._lmmse_robust = None
        self._link = None
        self.model = model
        comb = waveform.pilot_comb
        cols = waveform._layout()["num_columns"]
        mask = waveform.resource_mask[0][:, :cols]
        siso = num_tx == 1 and num_rx == 1
        if estimator == "ls" and not siso and comb < max(num_tx, 2):
            raise NotImplementedError("Least-Squares channel estimation is only implemented for SISO links")
        self.staged = estimator in ("lmmse", "lmmse_robust", "learned") or (estimator == "ls" and not siso)
        # `also`: further estimators whose tables are built too, for estimate(estimator=...)
        wanted = {estimator, *also}
        if self.staged and wanted & {"ls", "learned"} or estimator in ("ls", "learned"):
            streams = num_tx if self.staged else 1
            if self.staged:
                indptr, indices, weights = ls_stream_tables(mask, comb, streams)
            else:
                indptr, indices, weights = ls_interpolation_table(mask)
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_ls_create_streams(self._frame, cols, streams,
                                                         indptr.ctypes.data_as(ctypes.c_void_p),
                                                         indices.ctypes.data_as(ctypes.c_void_p),
                                                         weights.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)))
            self._ls = h
        if "lmmse" in wanted:
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_lmmse_create(self._frame, self._fading.handle, cols, ctypes.byref(h)))
            self._lmmse = h
        if "lmmse_robust" in wanted:
            # the non-genie counterpart: design statistics instead of the channel's
            design, ridge = robust_statistics(channel, sampling_rate)
            self._robust_fading = design.handle(num_rx, num_tx, sampling_rate)
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_lmmse_create_regularized(self._frame, self._robust_fading.handle, cols,
                                                                float(ridge), ctypes.byref(h)))
            self._lmmse_robust = h
        self.num_columns = cols
        if self.staged:
            self._alloc(self.max_drops)
        else:
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_link_create(self._frame, self._fading.handle, self._ls,
                                                   _lib.EST_IDEAL if estimator == "ideal" else _lib.EST_LS,
                                                   _lib.EQ_ZF if equalizer == "zf" else _lib.EQ_LMMSE,
                                                   self.max_drops, ctypes.byref(h)))
            self._link = h
        self.bits_per_drop = waveform.bits_per_frame() * num_tx

    def _alloc(self, n: int) -> None:
        """Stage buffers of the staged estimators for batches of up to n drops."""

        wf, dev = self.waveform, self.device
        T = wf.samples_per_frame()
        D = self._fading.max_delay
        W = wf.words_per_frame
        C = self.num_columns
        self._T, self._D = T, D
        self._state = self._fading.new_state(n)
        self._x = torch.empty((n, self.num_tx, T), dtype=torch.complex64, device=dev)
        self._y = torch.empty((n, self.num_rx, T + D), dtype=torch.complex64, device=dev)
        self._grid = torch.empty((n, self.num_rx, W, C), dtype=torch.complex64, device=dev)
        self._csi = torch.empty((n, self.num_rx, self.num_tx, W, C), dtype=torch.complex64, device=dev)

    def __del__(self):
        try:
            if _lib._lib is not None:
                if self._link is not None:
                    _lib._lib.hpx_link_destroy(self._link)
                if self._ls is not None:
                    _lib._lib.hpx_ls_destroy(self._ls)
                if self._lmmse is not None:
                    _lib._lib.hpx_lmmse_destroy(self._lmmse)
                if self._lmmse_robust is not None:
                    _lib._lib.hpx_lmmse_destroy(self._lmmse_robust)
        except Exception:
            pass

    def receive(self, drop0: int, noise_power: torch.Tensor, stream: torch.cuda.Stream | None = None) -> None:
        """Staged transmit, channel and receive of drops [drop0, drop0 + n): leaves the
        received grids in ``self._grid[:n]`` (and the channel state in ``self._state``)."""

        n = noise_power.numel()
        if n > self.max_drops:
            raise ValueError(f"at most {self.max_drops} drops per call")
        sp = _lib.stream_ptr(stream)
        fh = self._fading.handle
        _lib.call("hpx_fading_realize", fh, self.seed, int(drop0), n, _lib.ptr(self._state), sp)
        _lib.call("hpx_ofdm_modulate_bits", self._frame, self.seed, int(drop0), n, self.num_tx, _lib.ptr(self._x), sp)
        _lib.call("hpx_fading_propagate", fh, _lib.ptr(self._state), n, _lib.ptr(self._x), self._T,
                  _lib.ptr(self._y), _lib.ptr(noise_power), self.seed, int(drop0), sp)
        _lib.call("hpx_ofdm_demodulate", self._frame, _lib.ptr(self._y), self._T + self._D, n * self.num_rx,
                  self.num_columns, _lib.ptr(self._grid), sp)

    def estimate(self, n: int, noise_power: torch.Tensor, stream: torch.cuda.Stream | None = None,
                 estimator: str | None = None) -> torch.Tensor:
        """Channel estimate of the received grids of the last ``receive`` call:
        (n, Nrx, Ntx, W, C) on the device."""

        est = estimator or self.estimator
        sp = _lib.stream_ptr(stream)
        C = self.num_columns
        out = self._csi[:n]
        if est == "ideal":
            _lib.call("hpx_fading_ideal_csi", self._fading.handle, _lib.ptr(self._state), n, self._frame, C,
                      _lib.ptr(out), sp)
        elif est == "ls":
            _lib.call("hpx_ls_estimate_streams", self._ls, _lib.ptr(self._grid), C, self.num_rx, n, _lib.ptr(out), sp)
        elif est in ("lmmse", "lmmse_robust"):
            _lib.call("hpx_lmmse_estimate", self._lmmse if est == "lmmse" else self._lmmse_robust,
                      _lib.ptr(self._grid), C, self.num_rx, n, _lib.ptr(noise_power), _lib.ptr(out), sp)
        elif est == "learned":
            _lib.call("hpx_ls_estimate_streams", self._ls, _lib.ptr(self._grid), C, self.num_rx, n, _lib.ptr(out), sp)
            self.model.refine(out, stream)
        else:
            raise ValueError(f"unknown estimator {est}")
        return out

    def detect(self, drop0: int, n: int, noise_power: torch.Tensor, errors: torch.Tensor,
               stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        C = self.num_columns
        _lib.call("hpx_detect_csi", self._frame, self.num_rx, self.num_tx,
                  _lib.EQ_ZF if self.equalizer == "zf" else _lib.EQ_LMMSE, _lib.ptr(self._grid), C,
                  _lib.ptr(self._csi), C, _lib.ptr(noise_power), self.seed, int(drop0), n, _lib.ptr(errors),
                  _lib.stream_ptr(stream))
        return errors

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
        if self.staged:
            self.receive(drop0, noise_power, stream)
            lm = {"lmmse": self._lmmse, "lmmse_robust": self._lmmse_robust}.get(self.estimator)
            if lm is not None:
                # fused: the LMMSE estimate stays on chip (hpx_detect_lmmse)
                _lib.call("hpx_detect_lmmse", lm, self.num_rx,
                          _lib.EQ_ZF if self.equalizer == "zf" else _lib.EQ_LMMSE, _lib.ptr(self._grid),
                          self.num_columns, _lib.ptr(noise_power), self.seed, int(drop0), n, _lib.ptr(errors),
                          _lib.stream_ptr(stream))
                return errors
            self.estimate(n, noise_power, stream)
            return self.detect(drop0, n, noise_power, errors, stream)
        _lib.call("hpx_link_run", self._link, self.seed, int(drop0), n, _lib.ptr(noise_power), _lib.ptr(errors),
                  _lib.stream_ptr(stream))
        return errors

    def status(self, clear: bool = True, stream: torch.cuda.Stream | None = None) -> None:
        """Raise RuntimeError if a bounded tensor-core wait of the engine's kernels (the
        LMMSE receiver, the learned estimator's network) ran out since the last check;
        ``clear`` resets the handles' sticky status words. Synchronizes the stream."""

        sp = _lib.stream_ptr(stream)
        try:
            for lm in (self._lmmse, self._lmmse_robust):
                if lm is not None:
                    _lib.call("hpx_lmmse_status", lm, int(clear), sp)
        finally:
            if self.model is not None:
                self.model.status(clear, stream)

    def counts(self, errors: torch.Tensor, stream: torch.cuda.Stream | None = None) -> np.ndarray:
        """Host int64 bit-error counts of a ``run``'s per-drop words, after checking the
        device status (``status``) and every drop's failure flags (``_lib.drop_counts``):
        a drop whose wait ran out or whose equalizer met NaN / inf raises instead of being
        counted."""

        words = errors.cpu().numpy()
        self.status(True, stream)
        return _lib.drop_counts(words)

    def simulate(self, noise_power_host: np.ndarray, drop0: int = 0) -> np.ndarray:
        """Host noise powers in, host per-drop bit errors out (batched by max_drops)."""

        p = np.ascontiguousarray(np.asarray(noise_power_host, dtype=np.float32))
        out = np.empty(p.size, dtype=np.int64)
        for s in range(0, p.size, self.max_drops):
            chunk = torch.from_numpy(p[s:s + self.max_drops]).to(self.device, non_blocking=True)
            e = self.run(drop0 + s, chunk)
            out[s:s + chunk.numel()] = self.counts(e)
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

    def ber_campaign(self, levels_db, accuracy: float = 1e-3, confidence: float = 0.05, min_samples: int = 64,
                     max_drops_per_level: int = 1 << 20, batch: int | None = None, max_batches: int = 1 << 20,
                     check_every: int = 4, drop0: int = 0) -> list[BerPoint]:
        """Device-resident Monte Carlo over noise levels with the reference's
        confidence stopping rule (``ScalarEvaluationResult.add_artifact``,
        core/pymonte/scalar.py:101-125, on the per-drop BER): every level runs until
        2 (1 - Phi(sqrt(n) accuracy / std)) < confidence or it holds
        ``max_drops_per_level`` drops. The fused engines (ideal CSI, SISO LS) run the
        whole loop in ``hpx_campaign_run``; the staged estimators (tap-domain LMMSE,
        per-stream LS, the learned estimator) enqueue ``hpx_campaign_assign``, their
        ``run`` and ``hpx_campaign_accumulate`` per batch, with the host reading the
        number of active levels (``hpx_campaign_poll``) every ``check_every`` batches.
        A drop whose device wait ran out or whose equalizer met NaN / inf stops the
        campaign with RuntimeError."""

        levels_db = [float(v) for v in levels_db]
        batch = min(self.max_drops, batch or self.max_drops)
        power = np.ascontiguousarray(self.noise_power(levels_db).astype(np.float32))
        h = ctypes.c_void_p()
        _lib.check(_lib.load().hpx_campaign_create(len(levels_db), power.ctypes.data_as(ctypes.c_void_p),
                                                   float(accuracy), float(confidence), int(min_samples),
                                                   int(max_drops_per_level), batch, float(self.bits_per_drop),
                                                   ctypes.byref(h)))
        try:
            active = ctypes.c_int32(len(levels_db))
            sp = _lib.stream_ptr()
            if self._link is not None:
                done = ctypes.c_int64()
                _lib.call("hpx_campaign_run", h, self.link_handle, self.seed, int(drop0), batch, int(max_batches),
                          int(check_every), ctypes.byref(done), ctypes.byref(active), sp)
            else:
                noise = torch.empty(batch, dtype=torch.float32, device=self.device)
                errors = torch.empty(batch, dtype=torch.int32, device=self.device)
                done = 0
                for b in range(int(max_batches)):
                    _lib.call("hpx_campaign_assign", h, batch, _lib.ptr(noise), sp)
                    self.run(int(drop0) + done, noise, errors)
                    _lib.call("hpx_campaign_accumulate", h, batch, _lib.ptr(errors), sp)
                    done += batch
                    if (b + 1) % int(check_every) == 0 or b + 1 == int(max_batches):
                        self.status()
                        _lib.call("hpx_campaign_poll", h, ctypes.byref(active), sp)
                        if active.value == 0:
                            break
            L = len(levels_db)
            drops = np.zeros(L, dtype=np.int64)
            errs = np.zeros(L, dtype=np.int64)
            conf = np.zeros(L, dtype=np.int32)
            _lib.call("hpx_campaign_results", h, drops.ctypes.data_as(ctypes.c_void_p),
                      errs.ctypes.data_as(ctypes.c_void_p), None, None, conf.ctypes.data_as(ctypes.c_void_p))
        finally:
            _lib.load().hpx_campaign_destroy(h)
        return [BerPoint(lv, int(e), int(d) * self.bits_per_drop, int(d), bool(c))
                for lv, e, d, c in zip(levels_db, errs, drops, conf)]

    @property
    def link_handle(self):
        return self._link

