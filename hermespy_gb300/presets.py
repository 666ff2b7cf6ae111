"""Standard fading-channel presets of the drop-in API: 5G TDL, COST 259 and the
3GPP antenna correlations.

Mirrors ``hermespy/channel/fading/tdl.py`` (``TDL``, ``TDLType``, :22-443),
``hermespy/channel/fading/cost259.py`` (``Cost259``, ``Cost259Type``, :22-268) and
``hermespy/channel/fading/correlation.py`` (``StandardAntennaCorrelation``,
``CorrelationType``, ``DeviceType``, :13-116). Each preset only fixes the tap
delays, the power-delay profile and the Rice factors of a
``MultipathFadingChannel``; realization, propagation, channel state and the
batched engine are the same CUDA kernels as for any other profile (a Rice
factor of infinity is a pure line-of-sight tap, a finite one mixes a
line-of-sight sinusoid into the tap).

Reference behaviour kept:

* The TDL tables are the normalized delays and tap powers of ETSI TR 38.900
  Tables 7.7.2-1..5, scaled by ``rms_delay``; the powers are normalized to sum 1.
* TDL-D and TDL-E put the table's K-factor (13.3 and 22) as a *linear* Rice
  factor on the first tap and fix the line-of-sight Doppler frequency at 0.7 Hz;
  passing ``los_doppler_frequency`` to them is a ``ValueError``.
* COST 259 hilly terrain has a pure line-of-sight first tap (Rice factor
  infinity). Its ``los_angle = arccos(0.7)`` is stored but, as in the reference,
  does not enter the realization: line-of-sight angles are drawn per drop.
* Delays are sorted by ``MultipathFadingChannel`` (tables A, B, C, D and E list
  some out of order).
"""

from __future__ import annotations

import enum

import numpy as np

from .channel import AntennaCorrelation, MultipathFadingChannel


# --------------------------------------------------------------------------- TDL
class TDLType(enum.Enum):
    """5G TDL model types (the reference's enum values)."""

    A = 0
    B = 1
    C = 2
    D = 4
    E = 5


# (normalized delay, power in dB) per tap, in table order.
_TDL_TABLES: dict[TDLType, tuple[tuple[float, float], ...]] = {
    TDLType.A: (
        (0.0, -13.4), (0.3819, 0.0), (0.4025, -2.2), (0.5868, -4.0), (0.4610, -6.0), (0.5375, -8.2),
        (0.6708, -9.9), (0.5750, -10.5), (0.7618, -7.5), (1.5375, -15.9), (1.8978, -6.6), (2.2242, -16.7),
        (2.1717, -12.4), (2.4942, -15.2), (2.5119, -10.8), (3.0582, -11.3), (4.0810, -12.7), (4.4579, -16.2),
        (4.5695, -18.3), (4.7966, -18.9), (5.0066, -16.6), (5.3043, -19.9), (9.6586, -29.7),
    ),
    TDLType.B: (
        (0.0, 0.0), (0.1072, -2.2), (0.2155, -4.0), (0.2095, -3.2), (0.2870, -9.8), (0.2986, -3.2),
        (0.3752, -3.4), (0.5055, -5.2), (0.3681, -7.6), (0.3697, -3.0), (0.5700, -8.9), (0.5283, -9.0),
        (1.1021, -4.8), (1.2756, -5.7), (1.5474, -7.5), (1.7842, -1.9), (2.0169, -7.6), (2.8294, -12.2),
        (3.0219, -9.8), (3.6187, -11.4), (4.1067, -14.9), (4.2790, -9.2), (4.7834, -11.3),
    ),
    TDLType.C: (
        (0.0, -4.4), (0.2099, -1.2), (0.2219, -3.5), (0.2329, -5.2), (0.2176, -2.5), (0.6366, 0.0),
        (0.6448, -2.2), (0.6560, -3.9), (0.6584, -7.4), (0.7935, -7.1), (0.8213, -10.7), (0.9336, -11.1),
        (1.2285, -5.1), (1.3083, -6.8), (2.1704, -8.7), (2.7105, -13.2), (4.2589, -13.9), (4.6003, -13.9),
        (5.4902, -15.8), (5.6077, -17.1), (6.3065, -16.0), (6.6374, -15.7), (7.0427, -21.6), (8.6523, -22.8),
    ),
    TDLType.D: (
        (0.0, -13.5), (0.035, -18.8), (0.612, -21.0), (1.363, -22.8), (1.405, -17.9), (1.804, -20.1),
        (2.596, -21.9), (1.775, -22.9), (4.042, -27.8), (7.937, -23.6), (9.424, -24.8), (9.708, -30.0),
        (12.525, -27.7),
    ),
    TDLType.E: (
        (0.0, -22.03), (0.5133, -15.8), (0.5440, -18.1), (0.5630, -19.8), (0.5440, -22.9), (0.7112, -22.4),
        (1.9092, -18.6), (1.9293, -20.8), (1.9589, -22.6), (2.6426, -22.3), (3.7136, -25.6), (5.4524, -20.2),
        (12.0034, -29.8), (20.6519, -29.2),
    ),
}

# Line-of-sight first tap of the TDL-D / TDL-E models: (linear Rice factor, LOS Doppler [Hz]).
_TDL_LOS: dict[TDLType, tuple[float, float]] = {TDLType.D: (13.3, 0.7), TDLType.E: (22.0, 0.7)}


def _normalized_power(power_db) -> np.ndarray:
    p = 10.0 ** (np.asarray(power_db, dtype=np.float64) / 10.0)
    return p / np.sum(p)


class TDL(MultipathFadingChannel):
    """5G tapped-delay-line models A-E (tdl.py:32-443)."""

    def __init__(self, model_type: TDLType = TDLType.A, rms_delay: float = 0.0, *,
                 los_doppler_frequency: float | None = None, **kwargs) -> None:
        if rms_delay < 0.0:
            raise ValueError("Root-Mean-Squared delay must be greater or equal to zero")
        try:
            model_type = TDLType(model_type.value if isinstance(model_type, TDLType) else model_type)
        except ValueError:
            raise ValueError("Requested model type not supported") from None
        table = np.asarray(_TDL_TABLES[model_type], dtype=np.float64)
        rice = np.zeros(table.shape[0])
        if model_type in _TDL_LOS:
            if los_doppler_frequency is not None:
                raise ValueError(f"Model type {model_type.name} does not support line of sight doppler "
                                 "frequency configuration")
            rice[0], los_doppler_frequency = _TDL_LOS[model_type]
        self._model_type = model_type
        self._rms_delay = float(rms_delay)
        MultipathFadingChannel.__init__(self, rms_delay * table[:, 0], _normalized_power(table[:, 1]), rice,
                                        los_doppler_frequency=los_doppler_frequency, **kwargs)

    @property
    def model_type(self) -> TDLType:
        return self._model_type

    @property
    def rms_delay(self) -> float:
        return self._rms_delay


# ---------------------------------------------------------------------- COST 259
class Cost259Type(enum.Enum):
    """COST 259 environments (the reference's enum values)."""

    URBAN = 0
    RURAL = 1
    HILLY = 2


# (delay in microseconds, power in dB) per tap.
_COST259_TABLES: dict[Cost259Type, tuple[tuple[float, float], ...]] = {
    Cost259Type.URBAN: (
        (0.0, -5.7), (0.217, -7.6), (0.512, -10.1), (0.514, -10.2), (0.517, -10.2), (0.674, -11.5),
        (0.882, -13.4), (1.230, -16.3), (1.287, -16.9), (1.311, -17.1), (1.349, -17.4), (1.533, -19.0),
        (1.535, -19.0), (1.622, -19.8), (1.818, -21.5), (1.836, -21.6), (1.884, -22.1), (1.943, -22.6),
        (2.048, -23.5), (2.140, -24.3),
    ),
    Cost259Type.RURAL: (
        (0.0, -5.2), (0.042, -6.4), (0.101, -8.4), (0.129, -9.3), (0.149, -10.0), (0.245, -13.1),
        (0.312, -15.3), (0.410, -18.5), (0.469, -20.4), (0.528, -22.4),
    ),
    Cost259Type.HILLY: (
        (0.0, -3.6), (0.356, -8.9), (0.441, -10.2), (0.528, -11.5), (0.546, -11.8), (0.609, -12.7),
        (0.625, -13.0), (0.842, -16.2), (0.916, -17.3), (0.941, -17.7), (15.0, -17.6), (16.172, -22.7),
        (16.492, -24.1), (16.876, -25.8), (16.882, -25.8), (16.978, -26.2), (17.615, -29.0), (17.827, -29.9),
        (17.849, -30.0), (18.016, -30.7),
    ),
}


class Cost259(MultipathFadingChannel):
    """COST action 259 typical urban, rural area and hilly terrain models (cost259.py:35-268)."""

    def __init__(self, model_type: Cost259Type = Cost259Type.URBAN, *, los_angle: float | None = None,
                 **kwargs) -> None:
        try:
            model_type = Cost259Type(model_type.value if isinstance(model_type, Cost259Type) else model_type)
        except ValueError:
            raise ValueError("Requested model type not supported") from None
        table = np.asarray(_COST259_TABLES[model_type], dtype=np.float64)
        rice = np.zeros(table.shape[0])
        if model_type == Cost259Type.HILLY:
            rice[0] = np.inf
            los_angle = float(np.arccos(0.7))
        self._model_type = model_type
        MultipathFadingChannel.__init__(self, 1e-6 * table[:, 0], _normalized_power(table[:, 1]), rice,
                                        los_angle=los_angle, **kwargs)

    @property
    def model_type(self) -> Cost259Type:
        return self._model_type


# ------------------------------------------------------- 3GPP antenna correlation
class DeviceType(enum.Enum):
    """3GPP device type (correlation.py:13-20)."""

    BASE_STATION = 0
    TERMINAL = 1


class CorrelationType(enum.Enum):
    """3GPP correlation levels as (base station alpha, terminal beta) (correlation.py:23-36)."""

    LOW = (0.0, 0.0)
    MEDIUM = (0.3, 0.3)
    MEDIUM_A = (0.3, 0.3874)
    HIGH = (0.9, 0.9)


class StandardAntennaCorrelation(AntennaCorrelation):
    """3GPP TS 36.101/38.101 spatial correlation matrices for 1, 2 and 4 antennas
    (correlation.py:39-116).

    As in the reference, the transmitter is a base station (alpha) and the receiver a
    terminal (beta); the 4-antenna matrix has entries f^((|i-j|/3)^2).
    """

    def __init__(self, correlation: CorrelationType | str) -> None:
        self.correlation = correlation

    @property
    def correlation(self) -> CorrelationType:
        return self._correlation

    @correlation.setter
    def correlation(self, value: CorrelationType | str) -> None:
        self._correlation = CorrelationType[value] if isinstance(value, str) else CorrelationType(value)

    def sample_covariance(self, num_antennas: int, mode: str = "rx") -> np.ndarray:
        device = DeviceType.TERMINAL if mode == "rx" else DeviceType.BASE_STATION
        f = self._correlation.value[device.value]
        n = int(num_antennas)
        if n == 1:
            return np.ones((1, 1), dtype=np.complex128)
        if n == 2:
            return np.array([[1.0, f], [f, 1.0]], dtype=np.complex128)
        if n == 4:
            i = np.arange(4)
            return (f ** ((np.abs(i[:, None] - i[None, :]) / 3.0) ** 2)).astype(np.complex128)
        raise RuntimeError(f"3GPP standard antenna covariance is only defined for 1, 2 and 4 antennas, "
                           f"device has {n} antennas")
