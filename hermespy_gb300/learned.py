"""Learned channel estimator: a residual CNN over per-stream LS estimates.

No counterpart in the reference (its only trainable parts are outside the link
path). The network refines the LS + interpolation estimate of every antenna pair
of a 4x4 pilot-comb frame into the full (word, subcarrier) channel grid:

    x0 = LS estimate, 32 channels = 16 antenna pairs x (re, im)
    h_l = relu(conv3x3(h_{l-1}) + b_l), l = 1..5;   H = x0 + conv3x3(h_5) + b_6

Forward, backward and Adam run in ``libhpx.so`` (``hpx_cnn_*``: BF16 tensor-core
implicit GEMMs with FP32 accumulation). Training pairs (LS estimate, true channel)
come from the engine's own drops over random channels: 4-23 taps with an
exponential power-delay profile, Doppler U[0, 1000] Hz and SNR U[-5, 30] dB.

``LearnedChannelEstimation`` keeps the tap-domain LMMSE estimator as fallback and
yardstick: the network is used only while its validation NMSE is within 0.5 dB of
LMMSE's on the link's channel.
"""

from __future__ import annotations

import ctypes
import math
import os
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")


class CnnChannelEstimator:
    """Handle of one ``hpx_cnn`` (parameters, Adam state and activation buffers)."""

    LAYERS = 6
    CHANNELS = 32
    PAIRS = 16

    def __init__(self, num_words: int, num_columns: int, max_batch: int = 64, params: np.ndarray | None = None,
                 seed: int = 0) -> None:
        lib = _lib.load()
        _lib.require_cuda()
        self.num_words, self.num_columns, self.max_batch = int(num_words), int(num_columns), int(max_batch)
        self.num_params = int(lib.hpx_cnn_num_params())
        p = None
        if params is not None:
            params = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(-1))
            if params.size != self.num_params:
                raise ValueError(f"expected {self.num_params} parameters, got {params.size}")
            p = params.ctypes.data_as(ctypes.c_void_p)
        h = ctypes.c_void_p()
        _lib.check(lib.hpx_cnn_create(self.num_words, self.num_columns, self.max_batch, p, int(seed), ctypes.byref(h)))
        self.handle = h
        self._loss = torch.zeros(1, dtype=torch.float64, device="cuda")

    def __del__(self):
        try:
            if _lib._lib is not None and getattr(self, "handle", None) is not None:
                _lib._lib.hpx_cnn_destroy(self.handle)
        except Exception:
            pass

    # ------------------------------------------------------------- parameters
    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        _lib.call("hpx_cnn_get_params", self.handle, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def grads(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        _lib.call("hpx_cnn_get_grads", self.handle, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def split(self, params: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
        """(weights [6][32 out][9 taps][32 in], biases [6][32])."""

        p = self.params() if params is None else params
        nw = self.LAYERS * self.CHANNELS * 9 * self.CHANNELS
        return p[:nw].reshape(self.LAYERS, self.CHANNELS, 9, self.CHANNELS), p[nw:].reshape(self.LAYERS, self.CHANNELS)

    def save(self, path: str, **meta) -> None:
        np.savez(path, params=self.params(), num_words=self.num_words, num_columns=self.num_columns, **meta)

    @classmethod
    def load(cls, path: str, max_batch: int = 64) -> "CnnChannelEstimator":
        z = np.load(path)
        return cls(int(z["num_words"]), int(z["num_columns"]), max_batch, z["params"])

    # --------------------------------------------------------------- compute
    def refine(self, csi: torch.Tensor, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        """In place on (B, Nrx, Ntx, W, C) or (B, 16, W, C) complex64 LS estimates."""

        if csi.dtype != torch.complex64 or not csi.is_contiguous():
            raise ValueError("csi must be contiguous complex64")
        B = csi.shape[0]
        C = csi.shape[-1]
        if csi[0].numel() != self.PAIRS * self.num_words * C:
            raise ValueError("csi must hold 16 antenna pairs of the network's grid")
        _lib.call("hpx_cnn_refine", self.handle, _lib.ptr(csi), C, B, _lib.stream_ptr(stream))
        return csi

    def status(self, clear: bool = True, stream: torch.cuda.Stream | None = None) -> None:
        """Raise RuntimeError if a bounded TMA / tensor-core wait of ``refine`` ran out
        since the last check (its estimates are then NaN); ``clear`` resets the word."""

        _lib.call("hpx_cnn_status", self.handle, int(clear), _lib.stream_ptr(stream))

    def train_step(self, ls: torch.Tensor, truth: torch.Tensor, lr: float,
                   stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        """One Adam step; returns the device scalar sum |out - truth|^2 (not synchronized)."""

        _lib.call("hpx_cnn_train_step", self.handle, _lib.ptr(ls), _lib.ptr(truth), ls.shape[-1], ls.shape[0],
                  float(lr), _lib.ptr(self._loss), _lib.stream_ptr(stream))
        return self._loss


# ---------------------------------------------------------------- training data


@dataclass
class ChannelDraw:
    num_taps: int
    decay_db: float      # power decay per tap
    doppler: float       # Hz

    def profile(self, tap_spacing: float) -> tuple[np.ndarray, np.ndarray]:
        k = np.arange(self.num_taps)
        return k * tap_spacing, 10.0 ** (-self.decay_db * k / 10.0)


def random_channels(n: int, seed: int, taps=(4, 23), doppler=(0.0, 1000.0), decay_db=(0.2, 3.0)) -> list[ChannelDraw]:
    rng = np.random.default_rng(seed)
    return [ChannelDraw(int(rng.integers(taps[0], taps[1] + 1)), float(rng.uniform(*decay_db)),
                        float(rng.uniform(*doppler))) for _ in range(n)]


class PairSource:
    """(LS estimate, true channel) pairs from the engine's drops over random channels.

    One staged ``LinkEngine`` (estimator "ls") per channel draw shares the frame;
    every batch draws its channel from the pool, its SNRs uniformly, and runs
    transmit, fading + AWGN, receive, per-stream LS and the ideal CSI.
    """

    def __init__(self, waveform, sampling_rate: float, channels: list[ChannelDraw], batch: int, seed: int,
                 snr_db=(-5.0, 30.0), tap_spacing: float = 50e-9, num_antennas: int = 4) -> None:
        from .channel import MultipathFadingChannel
        from .engine import LinkEngine

        self.batch = int(batch)
        self.snr_db = snr_db
        self.rng = np.random.default_rng(seed + 1)
        self.engines = []
        for i, cd in enumerate(channels):
            d, p = cd.profile(tap_spacing)
            ch = MultipathFadingChannel(list(d), list(p), [0.0] * cd.num_taps, doppler_frequency=cd.doppler)
            self.engines.append(LinkEngine(waveform, ch, num_antennas, num_antennas, sampling_rate, "ls", "lmmse",
                                           "snr", max_drops=self.batch, seed=seed + 7919 * i))
        self.truth = torch.empty_like(self.engines[0]._csi)
        self.drop = 0

    def next(self) -> tuple[torch.Tensor, torch.Tensor, int]:
        eng = self.engines[int(self.rng.integers(len(self.engines)))]
        snr = self.rng.uniform(self.snr_db[0], self.snr_db[1], self.batch)
        p = torch.from_numpy(eng.noise_power(snr).astype(np.float32)).to("cuda", non_blocking=True)
        n = self.batch
        eng.receive(self.drop, p)
        ls = eng.estimate(n, p, estimator="ls")
        _lib.call("hpx_fading_ideal_csi", eng._fading.handle, _lib.ptr(eng._state), n, eng._frame, eng.num_columns,
                  _lib.ptr(self.truth), _lib.stream_ptr())
        self.drop += n
        return ls, self.truth, n


def nmse_db(err: float, power: float) -> float:
    return 10.0 * math.log10(max(err, 1e-300) / max(power, 1e-300))


def csi_error(frame, est: torch.Tensor, truth: torch.Tensor, pairs: int = 16) -> tuple[float, float]:
    """Sums of |est - truth|^2 and |truth|^2 over the data elements (hpx_csi_error)."""

    B = est.shape[0]
    err = torch.empty(B, dtype=torch.float64, device="cuda")
    pw = torch.empty(B, dtype=torch.float64, device="cuda")
    _lib.call("hpx_csi_error", frame, _lib.ptr(est), _lib.ptr(truth), est.shape[-1], pairs, B, _lib.ptr(err),
              _lib.ptr(pw), _lib.stream_ptr())
    return float(err.sum().item()), float(pw.sum().item())


def train(model: CnnChannelEstimator, source: PairSource, num_pairs: int, lr: float = 2e-3,
          log_every: int = 500, log=print) -> dict:
    """Adam over ``num_pairs`` simulator pairs (drops) with a cosine learning-rate decay."""

    steps = max(1, num_pairs // source.batch)
    t0 = time.perf_counter()
    hist = []
    acc = torch.zeros(1, dtype=torch.float64, device="cuda")
    for s in range(steps):
        ls, truth, n = source.next()
        rate = lr * 0.5 * (1.0 + math.cos(math.pi * s / steps))
        loss = model.train_step(ls, truth, rate)
        acc += loss
        if (s + 1) % log_every == 0 or s == steps - 1:
            torch.cuda.synchronize()
            per = float(acc.item()) / (log_every * n * model.PAIRS * model.num_words * model.num_columns)
            hist.append((s + 1, per))
            log(f"step {s + 1}/{steps}  mse/element {per:.4e}  {time.perf_counter() - t0:.1f}s")
            acc.zero_()
    torch.cuda.synchronize()
    return {"steps": steps, "pairs": steps * source.batch, "seconds": time.perf_counter() - t0, "history": hist}
