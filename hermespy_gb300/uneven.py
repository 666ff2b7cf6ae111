"""Uneven drop batches in one persistent launch, with an autotuned launch shape.

No counterpart in the reference, whose Monte Carlo actors simulate one drop at a
time (core/pymonte/actors.py:367-452). ``UnevenBatch`` hands a list of drops with
different antenna counts, FFT sizes, frame lengths, modulation orders, channels and
SNRs to ``hpx_uneven_*``: one persistent kernel in which every CTA takes whole drops
from an atomic counter (longest first) and runs each drop end to end with the
homogeneous engine's arithmetic. ``tune`` times the launch shapes that fit (threads
per CTA x CTAs per SM x register variant) and keeps the fastest; ``capture`` records the launch as a
CUDA graph that ``replay`` re-launches.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib


class UnevenDrop(ctypes.Structure):
    _fields_ = [
        ("num_rx", ctypes.c_int32), ("num_tx", ctypes.c_int32), ("fft_size", ctypes.c_int32),
        ("num_words", ctypes.c_int32), ("modulation_order", ctypes.c_int32), ("num_taps", ctypes.c_int32),
        ("tap_decay_db", ctypes.c_double), ("doppler_frequency", ctypes.c_double),
    ]


@dataclass
class DropConfig:
    num_rx: int
    num_tx: int
    fft_size: int
    num_words: int
    modulation_order: int
    num_taps: int
    tap_decay_db: float
    doppler_frequency: float
    snr_db: float

    def power_profile(self) -> np.ndarray:
        k = np.arange(self.num_taps)
        return 10.0 ** (-self.tap_decay_db * k / 10.0)

    def noise_power(self) -> float:
        """Noise power of the drop's SNR relative to the channel's expected energy
        (simulation/rf/noise/level.py:258-259 with unit waveform power)."""

        return float(np.sum(self.power_profile())) / 10.0 ** (self.snr_db / 10.0)


def random_drops(n: int, seed: int, antennas=(1, 2, 4, 8), fft_sizes=(128, 256, 512, 1024, 2048),
                 words=(4, 7, 14), orders=(4, 16, 64, 256), taps=(1, 23), doppler=(0.0, 1000.0),
                 snr_db=(-5.0, 30.0), decay_db=(1.0, 3.0)) -> list[DropConfig]:
    """Drops drawn uniformly over the given sets and ranges."""

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        out.append(DropConfig(int(rng.choice(antennas)), int(rng.choice(antennas)), int(rng.choice(fft_sizes)),
                              int(rng.choice(words)), int(rng.choice(orders)), int(rng.integers(taps[0], taps[1] + 1)),
                              float(rng.uniform(*decay_db)), float(rng.uniform(*doppler)),
                              float(rng.uniform(*snr_db))))
    return out


class UnevenBatch:
    def __init__(self, drops: list[DropConfig], subcarrier_spacing: float = 30e3, tap_spacing: float = 50e-9,
                 num_sinusoids: int = 20, max_slots: int | None = None) -> None:
        lib = _lib.load()
        self.device = _lib.require_cuda()
        self.drops = list(drops)
        self.subcarrier_spacing, self.tap_spacing, self.num_sinusoids = subcarrier_spacing, tap_spacing, num_sinusoids
        arr = (UnevenDrop * len(self.drops))(*[UnevenDrop(d.num_rx, d.num_tx, d.fft_size, d.num_words,
                                                          d.modulation_order, d.num_taps, d.tap_decay_db,
                                                          d.doppler_frequency) for d in self.drops])
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.max_slots = int(max_slots or 4 * sms)
        h = ctypes.c_void_p()
        _lib.check(lib.hpx_uneven_create(arr, len(self.drops), float(subcarrier_spacing), float(tap_spacing),
                                         int(num_sinusoids), self.max_slots, ctypes.byref(h)))
        self.handle = h
        bits = np.zeros(len(self.drops), dtype=np.int64)
        _lib.call("hpx_uneven_bits", h, bits.ctypes.data_as(ctypes.c_void_p))
        self.bits = bits
        self.noise_power = torch.tensor([d.noise_power() for d in self.drops], dtype=torch.float32,
                                        device=self.device)
        self.errors = torch.zeros(len(self.drops), dtype=torch.int32, device=self.device)
        self.tuning: list[dict] = []

    def __del__(self):
        try:
            if _lib._lib is not None and getattr(self, "handle", None) is not None:
                _lib._lib.hpx_uneven_destroy(self.handle)
        except Exception:
            pass

    # ------------------------------------------------------------- launch shape
    def config(self) -> dict:
        t, b, v = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _lib.call("hpx_uneven_get_config", self.handle, 0, 0, ctypes.byref(t), ctypes.byref(b), ctypes.byref(v), None)
        return {"threads": t.value, "blocks_per_sm": b.value, "variant": v.value}

    def fit(self, threads: int, variant: int) -> int:
        """CTAs of this shape that fit one SM."""

        f = ctypes.c_int32()
        _lib.call("hpx_uneven_get_config", self.handle, int(threads), int(variant), None, None, None, ctypes.byref(f))
        return f.value

    def set_config(self, threads: int, blocks_per_sm: int, variant: int = 0) -> None:
        _lib.call("hpx_uneven_config", self.handle, int(threads), int(blocks_per_sm), int(variant))

    def tune(self, seed: int = 0, drop0: int = 0, repeats: int = 2) -> dict:
        """Time every launch shape that fits (kernel variant x threads in {128, 256} x
        CTAs per SM up to the occupancy and slot limits) on this batch; keep the fastest."""

        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        best = None
        self.tuning = []
        for variant in (0, 1, 2):  # 2 exists only for batches of at most 4 antennas (fit 0 otherwise)
            for threads in (128, 256):
                fit = min(self.fit(threads, variant), max(1, self.max_slots // sms))
                for bps in range(1, fit + 1):
                    self.set_config(threads, bps, variant)
                    self.run(seed, drop0)  # warm
                    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    start.record()
                    for _ in range(repeats):
                        self.run(seed, drop0)
                    end.record()
                    torch.cuda.synchronize()
                    ms = start.elapsed_time(end) / repeats
                    cand = {"variant": variant, "threads": threads, "blocks_per_sm": bps, "ms": ms}
                    self.tuning.append(cand)
                    if best is None or ms < best["ms"]:
                        best = cand
        self.set_config(best["threads"], best["blocks_per_sm"], best["variant"])
        return best

    # ------------------------------------------------------------------ running
    def run(self, seed: int, drop0: int = 0, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        _lib.call("hpx_uneven_run", self.handle, int(seed), int(drop0), _lib.ptr(self.noise_power),
                  _lib.ptr(self.errors), _lib.stream_ptr(stream))
        return self.errors

    def capture(self, seed: int, drop0: int = 0) -> None:
        _lib.call("hpx_uneven_capture", self.handle, int(seed), int(drop0), _lib.ptr(self.noise_power),
                  _lib.ptr(self.errors))

    def replay(self, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        _lib.call("hpx_uneven_replay", self.handle, _lib.stream_ptr(stream))
        return self.errors
