"""One full simulated drop, bits to bit errors (oracle side, float64).

Restates the per-drop chain of ``SimulationScenario._drop``
(simulation/scenario.py:772-804) for a single-link OFDM modem over a
``MultipathFadingChannel``:

1. bits           ``RandomBitsSource.generate_bits`` (modem/bits_source.py:62-63),
                  one contiguous chunk per stream (modem/modem.py:747-763)
2. map + place    ``PskQamMapping.get_symbols``, ``OrthogonalWaveform.place``
3. modulate       ``OrthogonalWaveform.modulate`` per stream (modem/modem.py:765-795)
4. fading         ``MultipathFadingSample._propagate`` (channel/fading/fading.py:371-406)
5. AWGN           ``AWGNRealization.add_to`` (simulation/rf/noise/model.py:143-160) with
                  ``EBN0.get_power`` (simulation/modem/noise.py:97-98) or ``SNR.get_power``
                  (simulation/rf/noise/level.py:258-259)
6. frame          default synchronization: the first T samples (modem/modem.py:1085-1146)
7. demodulate, estimate, pick, equalize, unmap (modem/modem.py:1192-1267)
8. bit errors     ``BitErrorEvaluator.evaluate`` (modem/evaluators.py:239-258)

All random draws come from the engine's Philox streams (``oracle.streams``), so
the oracle and the engine simulate the very same drop.
"""

from __future__ import annotations

from dataclasses import dataclass

import time

import numpy as np

from . import cnn, estimation, fading, mapping, ofdm, streams
from .frame import FrameLayout, FrameSpec


@dataclass
class LinkConfig:
    frame: FrameSpec
    channel: fading.FadingConfig
    sampling_rate: float
    num_tx: int = 1
    num_rx: int = 1
    estimator: str = "ls"        # "ls" | "ideal" | "lmmse" (tap-domain LMMSE) | "learned" (LS + CNN)
    equalizer: str = "zf"        # "zf" | "lmmse"
    noise: str = "ebn0"          # "ebn0" | "snr"
    cnn_params: np.ndarray | None = None  # parameter vector of the learned estimator
    estimation_channel: fading.FadingConfig | None = None  # statistics the LMMSE estimator assumes (default: true)
    estimation_ridge: float = 0.0  # design noise variance regularizing the estimator's tap LS (0: plain LS)


def noise_power(cfg: LinkConfig, layout: FrameLayout, level_db: float) -> float:
    level = 10 ** (level_db / 10)
    if cfg.noise == "ebn0":
        # bit_energy = symbol_energy / bits_per_symbol with symbol_energy = 1
        # (modem/waveform.py:393-408, orthogonal/waveform.py:1086-1088)
        return (1.0 / layout.bits_per_symbol) / level
    # SNR relative to the waveform power (1.0) scaled by the channel's expected energy
    return 1.0 / level * cfg.channel.gain * float(np.sum(cfg.channel.power_profile))


def simulate_drop(cfg: LinkConfig, seed: int, drop: int, level_db: float, keep: bool = False,
                  timings: dict | None = None) -> dict:
    """One drop of the link. `timings`, if given, accumulates the seconds spent per
    stage (transmit, fading realization, propagation, AWGN, receive, estimation,
    detection) for the CPU baseline's split."""

    clock = [time.perf_counter()]

    def lap(stage: str) -> None:
        if timings is not None:
            now = time.perf_counter()
            timings[stage] = timings.get(stage, 0.0) + now - clock[0]
            clock[0] = now

    layout = FrameLayout(cfg.frame)
    fs = cfg.sampling_rate
    M = layout.order
    nbits = layout.bits_per_frame()
    tx_bits = np.stack([streams.data_bits(seed, drop, s, nbits) for s in range(cfg.num_tx)])
    x = np.stack([ofdm.modulate(layout, mapping.get_symbols(M, tx_bits[s]), s) for s in range(cfg.num_tx)])
    lap("transmit")
    sample = fading.realize(cfg.channel, seed, drop, cfg.num_rx, cfg.num_tx)
    lap("fading_realize")
    y = fading.propagate(sample, x, fs)
    lap("fading_propagate")
    p = noise_power(cfg, layout, level_db)
    if p > 0:
        y = y + streams.awgn(seed, drop, cfg.num_rx, y.shape[1], p)
    lap("awgn")
    T = layout.samples_per_frame
    frame = y[:, :T]
    grids = np.stack([ofdm.demodulate(layout, frame[r]) for r in range(cfg.num_rx)])  # (Nrx, W, N)
    lap("receive")
    if cfg.estimator in ("ls", "learned"):
        if (cfg.num_rx != 1 or cfg.num_tx != 1) and layout.spec.pilot_comb < max(cfg.num_tx, 2):
            raise NotImplementedError("Least-Squares channel estimation is only implemented for SISO links")
        H = estimation.mimo_ls_estimate(layout, grids, cfg.num_tx)
        if cfg.estimator == "learned":
            U = layout.num_used
            H[..., :U] = cnn.refine(cfg.cnn_params, H[..., :U])
    elif cfg.estimator == "lmmse":
        stats = cfg.estimation_channel if cfg.estimation_channel is not None else cfg.channel
        H = estimation.tap_lmmse_estimate(layout, grids, stats, fs, p, cfg.num_tx, cfg.estimation_ridge)
    else:
        H = estimation.ideal_csi(layout, sample, fs)
    lap("estimate")
    ydata = ofdm.pick(layout, grids)           # (Nrx, K)
    hdata = ofdm.pick(layout, H)               # (Nrx, Ntx, K)
    if cfg.equalizer == "zf":
        xhat = estimation.zf_equalize(ydata, hdata)
    else:
        xhat = estimation.lmmse_equalize(ydata, hdata, p)
    rx_bits = np.stack([mapping.detect_bits(M, xhat[s]) for s in range(xhat.shape[0])])
    errors = int(np.sum(np.abs(tx_bits.astype(np.int8) - rx_bits.astype(np.int8))))
    lap("detect")
    out = {"errors": errors, "bits": int(tx_bits.size), "noise_power": p}
    if keep:
        out.update(tx_bits=tx_bits, x=x, y=y, grids=grids, H=H, xhat=xhat, rx_bits=rx_bits, sample=sample)
    return out
