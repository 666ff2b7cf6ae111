"""Sum-of-sinusoids multipath fading (oracle side, float64).

Restates ``hermespy/channel/fading/fading.py``:

* ``MultipathFadingChannel.__init__``     :606-754  delay sorting (:706-711), LOS/NLOS
  gains ``sqrt(K/(1+K))`` / ``sqrt(1/((1+K) S))`` (:721-733)
* ``MultipathFadingRealization._sample``  :468-515  spatial response ``exp(2j pi U)``
  sliced to the antenna counts (:476-478), optional ``R_rx @ S @ R_tx`` (:480-489),
  angles/phases ``2 pi u`` and ``-pi + 2 pi u`` (:492-499)
* ``MultipathFadingSample.__path_impulse_generator`` :293-343  per-tap impulse
  ``sqrt(gain g_l) (nlos_l sum_n exp(j(f_D t/fs cos((2 pi n + theta)/S) + phi))
  + los_l exp(j(f_LOS t/fs cos(alpha) + psi)))``; delays ``rint(tau fs)``
* ``MultipathFadingSample._propagate``    :371-406  ``z[:, d:d+T] += x h_l``; ``y = S z``
* ``MultipathFadingSample.state``         :345-369  ``S (x) siso_csi`` impulse response
* ``Exponential`` power-delay profile (channel/fading/exponential.py:90-101)

The draw vector of one realization is laid out as
``[spatial Nrx*Ntx][LOS angle L][NLOS angles L*S][LOS phase L][NLOS phases L*S]``;
the engine reads the same positions from its Philox stream (``streams.fading_uniforms``).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import streams


@dataclass
class FadingConfig:
    delays: np.ndarray          # seconds, length L
    power_profile: np.ndarray   # linear, length L
    rice_factors: np.ndarray    # linear, length L (inf = pure LOS)
    num_sinusoids: int = 20
    doppler_frequency: float = 0.0
    los_doppler_frequency: float | None = None
    gain: float = 1.0
    rx_correlation: np.ndarray | None = None
    tx_correlation: np.ndarray | None = None

    def __post_init__(self) -> None:
        self.delays = np.asarray(self.delays, dtype=np.float64)
        self.power_profile = np.asarray(self.power_profile, dtype=np.float64)
        self.rice_factors = np.asarray(self.rice_factors, dtype=np.float64)
        if self.delays.ndim != 1 or self.power_profile.ndim != 1 or self.rice_factors.ndim != 1:
            raise ValueError("Delays, power profile and rice factors must be vectors")
        if self.delays.size < 1:
            raise ValueError("Configuration must contain at least one delay tap")
        if not (self.delays.size == self.power_profile.size == self.rice_factors.size):
            raise ValueError("Delays, power profile and rice factor vectors must be of equal length")
        if np.any(self.delays < 0):
            raise ValueError("Delays must be greater or equal to zero")
        if np.any(self.power_profile < 0):
            raise ValueError("Power profile factors must be greater or equal to zero")
        if np.any(self.rice_factors < 0):
            raise ValueError("Rice factors must be greater or equal to zero")
        order = np.argsort(self.delays, kind="stable")
        self.delays = self.delays[order]
        self.power_profile = self.power_profile[order]
        self.rice_factors = self.rice_factors[order]

    @property
    def num_taps(self) -> int:
        return int(self.delays.size)

    @property
    def los_doppler(self) -> float:
        return self.doppler_frequency if self.los_doppler_frequency is None else self.los_doppler_frequency

    def gains(self) -> tuple[np.ndarray, np.ndarray]:
        k = self.rice_factors
        inf = np.isposinf(k)
        los = np.ones_like(k)
        nlos = np.zeros_like(k)
        los[~inf] = np.sqrt(k[~inf] / (1 + k[~inf]))
        nlos[~inf] = np.sqrt(1 / ((1 + k[~inf]) * self.num_sinusoids))
        return los, nlos

    def delay_samples(self, fs: float) -> np.ndarray:
        return np.rint(self.delays * fs).astype(np.int64)

    def max_delay_samples(self, fs: float) -> int:
        return int(round(float(self.delays.max()) * fs))

    def num_draws(self, num_rx: int, num_tx: int) -> int:
        return num_rx * num_tx + 2 * self.num_taps * (1 + self.num_sinusoids)


def exponential_profile(tap_interval: float, rms_delay: float) -> tuple[np.ndarray, np.ndarray]:
    """``Exponential`` PDP (channel/fading/exponential.py:90-101): taps until power < 1e-5."""

    rms_norm = rms_delay / tap_interval
    alpha = -2 * np.log((-1 + np.sqrt(1 + 4 * rms_norm**2)) / (2 * rms_norm))
    max_delay_in_samples = int(-np.ceil(np.log(1e-5) / alpha))
    delays = np.arange(max_delay_in_samples + 1) * tap_interval
    power = np.exp(-alpha * np.arange(max_delay_in_samples + 1))
    return delays, power


@dataclass
class FadingSample:
    """The quantities of one ``MultipathFadingSample``."""

    config: FadingConfig
    spatial: np.ndarray         # (Nrx, Ntx) complex
    los_angles: np.ndarray      # (L,)
    nlos_angles: np.ndarray     # (L, S)
    los_phases: np.ndarray      # (L,)
    nlos_phases: np.ndarray     # (L, S)


def sample_from_uniforms(config: FadingConfig, u: np.ndarray, num_rx: int, num_tx: int) -> FadingSample:
    L, S = config.num_taps, config.num_sinusoids
    o = 0
    spatial = np.exp(2j * np.pi * u[o : o + num_rx * num_tx].reshape(num_rx, num_tx))
    o += num_rx * num_tx
    if config.rx_correlation is not None or config.tx_correlation is not None:
        rrx = np.eye(num_rx) if config.rx_correlation is None else config.rx_correlation[:num_rx, :num_rx]
        rtx = np.eye(num_tx) if config.tx_correlation is None else config.tx_correlation[:num_tx, :num_tx]
        spatial = rrx @ spatial @ rtx
    los_angles = 2 * np.pi * u[o : o + L]
    o += L
    nlos_angles = -np.pi + 2 * np.pi * u[o : o + L * S].reshape(L, S)
    o += L * S
    los_phases = -np.pi + 2 * np.pi * u[o : o + L]
    o += L
    nlos_phases = -np.pi + 2 * np.pi * u[o : o + L * S].reshape(L, S)
    return FadingSample(config, spatial, los_angles, nlos_angles, los_phases, nlos_phases)


def realize(config: FadingConfig, seed: int, drop: int, num_rx: int, num_tx: int) -> FadingSample:
    u = streams.fading_uniforms(seed, drop, config.num_draws(num_rx, num_tx))
    return sample_from_uniforms(config, u, num_rx, num_tx)


def path_impulses(sample: FadingSample, num_samples: int, fs: float) -> np.ndarray:
    """(L, T) complex tap coefficients (fading.py:293-343)."""

    c = sample.config
    S = c.num_sinusoids
    n = 1 + np.arange(S)
    t = np.arange(num_samples) / fs
    nlos_time = c.doppler_frequency * t
    los_time = c.los_doppler * t
    los_g, nlos_g = c.gains()
    out = np.empty((c.num_taps, num_samples), dtype=np.complex128)
    for l in range(c.num_taps):
        imp = nlos_g[l] * np.sum(
            np.exp(1j * (np.outer(nlos_time, np.cos((2 * np.pi * n + sample.nlos_angles[l]) / S))
                         + sample.nlos_phases[l][None, :])), axis=1)
        imp = imp + los_g[l] * np.exp(1j * (los_time * np.cos(sample.los_angles[l]) + sample.los_phases[l]))
        out[l] = imp * (c.gain * c.power_profile[l]) ** 0.5
    return out


def propagate(sample: FadingSample, x: np.ndarray, fs: float) -> np.ndarray:
    """(Ntx, T) -> (Nrx, T + D) (fading.py:371-406)."""

    x = np.atleast_2d(np.asarray(x, dtype=np.complex128))
    num_tx, T = x.shape
    if num_tx != sample.spatial.shape[1]:
        raise ValueError("Number of signal streams does not match the number of transmit antennas")
    D = sample.config.max_delay_samples(fs)
    z = np.zeros((num_tx, T + D), dtype=np.complex128)
    h = path_impulses(sample, T, fs)
    for l, d in enumerate(sample.config.delay_samples(fs)):
        z[:, d : d + T] += x * h[l][None, :]
    return sample.spatial @ z


def siso_state(sample: FadingSample, num_samples: int, fs: float, max_num_taps: int | None = None) -> np.ndarray:
    """(T, taps) impulse response shared by every antenna pair; ``state`` is its
    outer product with the spatial matrix (fading.py:345-369)."""

    max_num_taps = num_samples if max_num_taps is None else max_num_taps
    num_taps = min(1 + sample.config.max_delay_samples(fs), max_num_taps)
    siso = np.zeros((num_samples, num_taps), dtype=np.complex128)
    h = path_impulses(sample, num_samples, fs)
    for l, d in enumerate(sample.config.delay_samples(fs)):
        if d > num_taps:
            continue
        siso[:, d] += h[l]
    return siso


def state(sample: FadingSample, num_samples: int, fs: float, max_num_taps: int | None = None) -> np.ndarray:
    """(Nrx, Ntx, T, taps) impulse-response CSI (fading.py:345-369)."""

    max_num_taps = num_samples if max_num_taps is None else max_num_taps
    num_taps = min(1 + sample.config.max_delay_samples(fs), max_num_taps)
    siso = np.zeros((num_samples, num_taps), dtype=np.complex128)
    h = path_impulses(sample, num_samples, fs)
    for l, d in enumerate(sample.config.delay_samples(fs)):
        if d > num_taps:
            continue
        siso[:, d] += h[l]
    return np.einsum("ij,kl->ijkl", sample.spatial, siso)
