"""Whole drops of the HermesPy reference fed the engine's random draws.

Test infrastructure for the fixture generators (``make_golden.py``,
``make_ber_curves.py``); never imported by the engine. Importing this module
imports the reference checkout named by ``$HERMESPY_REFERENCE`` (through
``refimport``), then builds ``SimulationScenario`` links whose random inputs are
the engine's Philox streams, routed through the reference's own extension points:

* bits:   a ``BitsSource`` subclass (modem/bits_source.py:34-63) returning the
          engine's per-stream bits of the current drop;
* noise:  an ``AWGN`` subclass whose realization adds the engine's Philox noise
          (simulation/rf/noise/model.py:143-178) at the power the reference's own
          noise level computes;
* fading: the channel's consistent generator (channel/consistent.py:410-459) is
          replaced by a static realization holding the normal quantiles of the
          engine's fading uniforms, so ``MultipathFadingRealization._sample``
          (channel/fading/fading.py:468-515) runs unchanged on them.

``SimulationScenario.drop()`` (simulation/scenario.py:772-804) and
``BitErrorEvaluator`` (modem/evaluators.py:239-258) then run as shipped.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
for p in (HERE, os.path.dirname(os.path.dirname(HERE))):
    if p not in sys.path:
        sys.path.insert(0, p)

import refimport  # noqa: E402

refimport.import_reference()

from scipy.stats import norm  # noqa: E402

from hermespy.channel import MultipathFadingChannel  # noqa: E402
from hermespy.channel.consistent import StaticConsistentRealization  # noqa: E402
from hermespy.modem import (  # noqa: E402
    BitErrorEvaluator,
    ElementType,
    GridElement,
    GridResource,
    OFDMWaveform,
    OrthogonalLeastSquaresChannelEstimation,
    OrthogonalZeroForcingChannelEqualization,
    SimplexLink,
    SymbolSection,
)
from hermespy.modem.bits_source import BitsSource  # noqa: E402
from hermespy.simulation import AWGN, OFDMIdealChannelEstimation, SimulationScenario  # noqa: E402
from hermespy.simulation import SimulatedIdealAntenna, SimulatedUniformArray  # noqa: E402
from hermespy.simulation.modem.noise import EBN0  # noqa: E402
from hermespy.simulation.rf.noise.level import SNR  # noqa: E402
from hermespy.simulation.rf.noise.model import AWGNRealization  # noqa: E402

from oracle import fading as ofad  # noqa: E402
from oracle import streams  # noqa: E402


def c1_waveform(order: int = 16) -> OFDMWaveform:
    """SISO 256-point frame: 200 used subcarriers, CP 18, 14 words, comb pilots
    on every 4th subcarrier of words 0 and 7."""

    N, U, CP = 256, 200, 18
    res = [
        GridResource(1, prefix_ratio=CP / N, elements=[GridElement(ElementType.DATA, U)]),
        GridResource(U // 4, prefix_ratio=CP / N,
                     elements=[GridElement(ElementType.REFERENCE, 1), GridElement(ElementType.DATA, 3)]),
    ]
    struct = [SymbolSection(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])]
    return OFDMWaveform(grid_resources=res, grid_structure=struct, num_subcarriers=N, modulation_order=order)


def c2_waveform(order: int = 64) -> OFDMWaveform:
    """1024-point frame: 600 used data subcarriers, CP 72, 14 words."""

    N, U, CP = 1024, 600, 72
    res = [GridResource(1, prefix_ratio=CP / N, elements=[GridElement(ElementType.DATA, U)])]
    struct = [SymbolSection(14, [0])]
    return OFDMWaveform(grid_resources=res, grid_structure=struct, num_subcarriers=N, modulation_order=order)


class InjectedBits(BitsSource):
    """Bits source returning the engine's Philox bits for the current drop."""

    def __init__(self, seed, num_streams):
        BitsSource.__init__(self)
        self.seed, self.num_streams, self.drop = seed, num_streams, 0

    def generate_bits(self, num_bits):
        per = num_bits // self.num_streams
        return np.concatenate([streams.data_bits(self.seed, self.drop, s, per) for s in range(self.num_streams)])

    def serialize(self, process):
        pass


class InjectedNoise(AWGN):
    """Noise model adding the engine's Philox AWGN for the current drop; remembers
    the power the reference's noise level asked for."""

    def __init__(self, seed):
        AWGN.__init__(self)
        self.inj_seed, self.drop, self.last_power = seed, 0, None

    def realize(self, power):
        model = self
        model.last_power = float(power)

        class _R(AWGNRealization):
            def add_to(self, signal):
                if self.power == 0.0:
                    return signal
                noisy = signal.copy()
                arr = noisy.view(np.ndarray)
                n = streams.awgn(model.inj_seed, model.drop, arr.shape[0], arr.shape[1], self.power)
                for block in noisy.blocks:
                    block += n
                noisy.noise_power = self.power
                return noisy

        return _R(power, 0)


class RefLink:
    """One simplex OFDM link of the reference over a ``MultipathFadingChannel``,
    driven drop by drop with the engine's random draws."""

    def __init__(self, wf, cfg: ofad.FadingConfig, fs: float, num_tx: int, num_rx: int, seed: int,
                 estimator: str = "ls") -> None:
        sc = SimulationScenario(seed=3)
        tx = sc.new_device(carrier_frequency=0.0, bandwidth=fs, oversampling_factor=1,
                           antennas=SimulatedUniformArray(SimulatedIdealAntenna, 0.01, [num_tx, 1, 1]))
        rx = sc.new_device(carrier_frequency=0.0, bandwidth=fs, oversampling_factor=1,
                           antennas=SimulatedUniformArray(SimulatedIdealAntenna, 0.01, [num_rx, 1, 1]))
        link = SimplexLink()
        tx.transmitters.add(link)
        rx.receivers.add(link)
        ch = MultipathFadingChannel(cfg.delays, cfg.power_profile, cfg.rice_factors,
                                    num_sinusoids=cfg.num_sinusoids, doppler_frequency=cfg.doppler_frequency)
        sc.set_channel(tx, rx, ch)
        if estimator == "ideal":
            wf.channel_estimation = OFDMIdealChannelEstimation(ch, tx, rx)
        else:
            wf.channel_estimation = OrthogonalLeastSquaresChannelEstimation()
        wf.channel_equalization = OrthogonalZeroForcingChannelEqualization()
        link.waveform = wf
        self.bits = InjectedBits(seed, num_tx)
        link.bits_source = self.bits
        self.noise = InjectedNoise(seed)
        rx.noise_model = self.noise
        tx.noise_model = InjectedNoise(seed + 1)
        self.ber = BitErrorEvaluator(link, link)
        self.sc, self.ch, self.link, self.tx, self.rx = sc, ch, link, tx, rx
        self.cfg, self.seed, self.num_tx, self.num_rx = cfg, seed, num_tx, num_rx

    def set_ebn0(self, ebn0_db: float) -> None:
        self.rx.noise_level = EBN0(self.link, 10 ** (ebn0_db / 10))

    def set_snr(self, snr_db: float) -> None:
        """``SNR`` relative to the link's power scaled by the channel's expected energy
        (simulation/rf/noise/level.py:200-259)."""

        self.rx.noise_level = SNR(10 ** (snr_db / 10), self.link, self.ch)

    def drop(self, drop: int):
        """Run drop ``drop``; returns (bit errors, the reference's drop object)."""

        self.bits.drop = self.noise.drop = drop
        inject_fading(self.ch, self.cfg, self.seed, drop, self.num_rx, self.num_tx)
        dr = self.sc.drop()
        return int(np.sum(self.ber.evaluate().evaluation)), dr


def inject_fading(ch, cfg, seed, drop, num_rx, num_tx):
    """Route the engine's fading uniforms through the reference's own variables."""

    L, S = cfg.num_taps, cfg.num_sinusoids
    u = streams.fading_uniforms(seed, drop, cfg.num_draws(num_rx, num_tx))
    ref_u = np.full(100 + 2 * L * (1 + S), 0.5)
    # SimulationScenario.propagate (simulation/scenario.py:575-609) samples the link
    # (device 1 -> device 0) and serves device 0 -> device 1 with its reciprocal, whose
    # spatial response is the transpose: entry [rx, tx] comes from variable entry [tx, rx].
    sp = np.full((10, 10), 0.5)
    sp[:num_tx, :num_rx] = u[: num_rx * num_tx].reshape(num_rx, num_tx).T
    ref_u[:100] = sp.reshape(-1)
    ref_u[100:] = u[num_rx * num_tx:]
    scalars = norm.ppf(ref_u)
    gen = ch._MultipathFadingChannel__rng
    gen.realize = lambda distance, *a, **k: StaticConsistentRealization(scalars)
