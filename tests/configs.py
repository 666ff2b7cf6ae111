"""Workload definitions shared by the tests (frames and channels of the named workloads)."""

import numpy as np

from oracle import fading as ofad
from oracle.frame import DATA, REFERENCE, FrameSpec, Resource, Section


def siso_frame(order: int = 16) -> FrameSpec:
    """SISO 256-point frame: 200 used subcarriers, CP 18, 14 words, comb pilots on
    every 4th subcarrier of words 0 and 7."""

    N, U, CP = 256, 200, 18
    res = [Resource(1, CP / N, [(DATA, U)]), Resource(U // 4, CP / N, [(REFERENCE, 1), (DATA, 3)])]
    return FrameSpec(N, res, [Section(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])], order, True)


def mimo_frame(order: int = 64) -> FrameSpec:
    """1024-point frame: 600 used data subcarriers, CP 72, 14 words."""

    N, U, CP = 1024, 600, 72
    return FrameSpec(N, [Resource(1, CP / N, [(DATA, U)])], [Section(14, [0])], order, True)


def pilot_frame(order: int = 64, comb: int = 4) -> FrameSpec:
    """1024-point 4x4 frame with per-stream pilots: words 0 and 7 carry reference
    elements on all 600 used subcarriers, stream s transmitting on columns
    c % 4 == s (pilot comb 4); the other 12 words carry data."""

    N, U, CP = 1024, 600, 72
    res = [Resource(1, CP / N, [(DATA, U)]), Resource(1, CP / N, [(REFERENCE, U)])]
    return FrameSpec(N, res, [Section(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])], order, True, comb)


def massive_frame(N: int = 4096, used: int = 3300, cp: int = 288, order: int = 16) -> FrameSpec:
    """Massive-MIMO uplink frame: 14 data words (ideal CSI, no pilots)."""

    return FrameSpec(N, [Resource(1, cp / N, [(DATA, used)])], [Section(14, [0])], order, True)


def massive_channel(nrx: int = 64, rho: float = 0.7, fs: float = 61.44e6, taps: int = 8,
                    doppler: float = 50.0) -> ofad.FadingConfig:
    """8 taps at one-sample spacing with an exponential profile (3 dB per tap),
    receive correlation rho^|i-j| at the base station, 50 Hz Doppler."""

    k = np.arange(taps)
    i = np.arange(nrx)
    rx = rho ** np.abs(i[:, None] - i[None, :]).astype(np.complex128)
    return ofad.FadingConfig(k / fs, 10 ** (-0.3 * k), np.zeros(taps), 20, doppler, None, 1.0, rx, None)


# name: (delays [samples], power, rice, S, doppler, los_doppler, gain, Nrx, Ntx, T, fs)
FADING_CASES = {
    "c1": (np.arange(6), 10 ** (-0.3 * np.arange(6)), np.zeros(6), 20, 100.0, None, 1.0, 1, 1, 3836, 15.36e6),
    "c2": (np.rint(np.arange(23) * 50e-9 * 30.72e6), 10 ** (-0.04 * np.arange(23)), np.zeros(23), 20, 500.0,
           None, 1.0, 4, 4, 3000, 30.72e6),
    "fast": (np.array([0, 3, 7, 19]), np.array([1.0, 0.5, 0.3, 0.1]), np.array([0.0, 1.0, 0.0, 2.0]), 5,
             50 * 1e6, 20 * 1e6, 0.987, 2, 3, 700, 1e6),
    "los": (np.array([0, 2]), np.array([1.0, 0.2]), np.array([np.inf, 3.0]), 7, 1e5, 3e4, 1.0, 1, 2, 500, 1e6),
    # taps rounding to one sample delay (groups at 0, 1 and 3 samples), LOS and NLOS
    # taps mixed inside a group; slow Doppler (Taylor tiles) and fast (direct sums)
    "grp": (np.array([0.0, 0.4, 1.2, 1.4, 3.0, 3.3, 3.45]), np.array([1.0, 0.7, 0.5, 0.4, 0.3, 0.2, 0.1]),
            np.array([np.inf, 0.0, 1.5, 0.0, 0.0, 2.0, np.inf]), 9, 100.0, 50.0, 1.0, 2, 2, 900, 1e6),
    "grp_fast": (np.array([0.0, 0.4, 1.2, 1.4, 3.0, 3.3, 3.45]), np.array([1.0, 0.7, 0.5, 0.4, 0.3, 0.2, 0.1]),
                 np.array([np.inf, 0.0, 1.5, 0.0, 0.0, 2.0, np.inf]), 9, 2e4, 1e4, 1.0, 2, 2, 900, 1e6),
}


def fading_case(name):
    d, p, k, S, fd, flos, g, nrx, ntx, T, fs = FADING_CASES[name]
    cfg = ofad.FadingConfig(np.asarray(d, float) / fs, p, k, S, fd, flos, g)
    return cfg, nrx, ntx, T, fs


def siso_channel(fs: float = 15.36e6) -> ofad.FadingConfig:
    """6 taps at 0..5 samples, 3 dB/tap decay, 20 sinusoids, 100 Hz Doppler (Rayleigh)."""

    return ofad.FadingConfig(np.arange(6) / fs, 10 ** (-0.3 * np.arange(6)), np.zeros(6), 20, 100.0)


def mimo_channel(fs: float = 30.72e6) -> ofad.FadingConfig:
    """23 taps at k*50 ns with -0.4k dB power, 20 sinusoids, 500 Hz Doppler (Rayleigh)."""

    k = np.arange(23)
    return ofad.FadingConfig(k * 50e-9, 10 ** (-0.04 * k), np.zeros(23), 20, 500.0)


def robust_design(cfg: ofad.FadingConfig, fs: float, num_delays: int = 64, doppler: float = 1000.0,
                  design_snr_db: float = 20.0) -> tuple[ofad.FadingConfig, float]:
    """Statistics of the robust (non-genie) tap-domain LMMSE estimator: a uniform
    profile over `num_delays` sample delays carrying the channel's expected energy,
    design Doppler `doppler`, and the prior noise variance of `design_snr_db`
    (hermespy_gb300.estimation.robust_statistics). Returns (design config, ridge)."""

    energy = cfg.gain * float(np.sum(cfg.power_profile))
    k = np.arange(num_delays)
    design = ofad.FadingConfig(k / fs, np.full(num_delays, energy / num_delays), np.zeros(num_delays), 20, doppler)
    return design, energy * 10.0 ** (-design_snr_db / 10.0)
