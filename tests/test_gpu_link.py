"""GPU: whole drops (batched engine and the per-drop drop-in API) against the oracle
on identical Philox draws, and BER curves inside the oracle's 95 % intervals."""

import numpy as np
import pytest
import torch

import hermespy_gb300 as hg
from oracle.link import LinkConfig, simulate_drop
from tests.configs import mimo_channel, mimo_frame, siso_channel, siso_frame

pytestmark = pytest.mark.gpu
SEED = 2024


def siso_waveform(order=16):
    N, U, CP = 256, 200, 18
    res = [hg.GridResource(1, prefix_ratio=CP / N, elements=[hg.GridElement(hg.ElementType.DATA, U)]),
           hg.GridResource(U // 4, prefix_ratio=CP / N, elements=[hg.GridElement(hg.ElementType.REFERENCE, 1),
                                                                    hg.GridElement(hg.ElementType.DATA, 3)])]
    return hg.OFDMWaveform(res, [hg.SymbolSection(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])],
                           num_subcarriers=N, modulation_order=order)


def mimo_waveform(order=64):
    N, U, CP = 1024, 600, 72
    res = [hg.GridResource(1, prefix_ratio=CP / N, elements=[hg.GridElement(hg.ElementType.DATA, U)])]
    return hg.OFDMWaveform(res, [hg.SymbolSection(14, [0])], num_subcarriers=N, modulation_order=order)


def engine_channel(cfg):
    return hg.MultipathFadingChannel(cfg.delays, cfg.power_profile, cfg.rice_factors,
                                     num_sinusoids=cfg.num_sinusoids, doppler_frequency=cfg.doppler_frequency,
                                     seed=SEED)


def close(a, b):
    return abs(a - b) <= max(3, 0.01 * max(a, b))


@pytest.mark.parametrize("ebn0", [5.0, 10.0, 20.0])
def test_siso_ls_zf_drops_match_oracle(ebn0):
    fs = 15.36e6
    eng = hg.LinkEngine(siso_waveform(), engine_channel(siso_channel(fs)), 1, 1, fs, "ls", "zf", "ebn0",
                        max_drops=16, seed=SEED)
    p = eng.noise_power([ebn0] * 6)
    errs = eng.simulate(p)
    cfg = LinkConfig(siso_frame(), siso_channel(fs), fs, 1, 1, "ls", "zf", "ebn0")
    for d in range(6):
        ref = simulate_drop(cfg, SEED, d, ebn0)["errors"]
        assert close(int(errs[d]), ref), (d, int(errs[d]), ref)


@pytest.mark.parametrize("equalizer", ["zf", "lmmse"])
def test_mimo_ideal_drops_match_oracle(equalizer):
    fs = 30.72e6
    ch = mimo_channel(fs)
    eng = hg.LinkEngine(mimo_waveform(), engine_channel(ch), 4, 4, fs, "ideal", equalizer, "snr", max_drops=4,
                        seed=SEED)
    levels = [15.0, 25.0]
    errs = eng.simulate(eng.noise_power(levels))
    cfg = LinkConfig(mimo_frame(), ch, fs, 4, 4, "ideal", equalizer, "snr")
    for d, lv in enumerate(levels):
        ref = simulate_drop(cfg, SEED, d, lv)["errors"]
        assert close(int(errs[d]), ref), (d, int(errs[d]), ref)


def test_siso_ber_curve_inside_oracle_interval():
    fs = 15.36e6
    eng = hg.LinkEngine(siso_waveform(), engine_channel(siso_channel(fs)), 1, 1, fs, "ls", "zf", "ebn0",
                        max_drops=512, seed=SEED)
    levels = [0.0, 6.0, 12.0, 18.0]
    per = 12
    pts = eng.ber_curve(levels, per)
    cfg = LinkConfig(siso_frame(), siso_channel(fs), fs, 1, 1, "ls", "zf", "ebn0")
    for i, pt in enumerate(pts):
        e = sum(simulate_drop(cfg, SEED, i * per + d, pt.level_db)["errors"] for d in range(per))
        lo, hi = hg.clopper_pearson(e, pt.bits)
        assert lo <= pt.ber <= hi, (pt.level_db, pt.ber, lo, hi)


def test_drop_in_scenario_matches_oracle():
    """SimulationScenario.drop() of the drop-in API simulates the oracle's drop."""

    fs = 15.36e6
    sc = hg.SimulationScenario(seed=SEED)
    tx = sc.new_device(bandwidth=fs, noise_model=hg.AWGN(SEED))
    rx = sc.new_device(bandwidth=fs, noise_model=hg.AWGN(SEED))
    wf = siso_waveform()
    wf.channel_estimation = hg.OrthogonalLeastSquaresChannelEstimation()
    wf.channel_equalization = hg.OrthogonalZeroForcingChannelEqualization()
    link = hg.SimplexLink(wf, seed=SEED)
    tx.transmitters.append(link)
    rx.receivers.append(link)
    sc.set_channel(tx, rx, engine_channel(siso_channel(fs)))
    rx.noise_level = hg.EBN0(link, 10.0)
    ber = hg.BitErrorEvaluator(link, link)
    cfg = LinkConfig(siso_frame(), siso_channel(fs), fs, 1, 1, "ls", "zf", "ebn0")
    for d in range(3):
        sc.drop()
        e = int(ber.evaluate().evaluation.sum())
        ref = simulate_drop(cfg, SEED, d, 10.0)["errors"]
        assert close(e, ref), (d, e, ref)


def test_drop_in_mimo_ideal_lmmse():
    fs = 30.72e6
    ch = engine_channel(mimo_channel(fs))
    sc = hg.SimulationScenario(seed=SEED)
    tx = sc.new_device(bandwidth=fs, antennas=4, noise_model=hg.AWGN(SEED))
    rx = sc.new_device(bandwidth=fs, antennas=4, noise_model=hg.AWGN(SEED))
    wf = mimo_waveform()
    wf.channel_estimation = hg.OFDMIdealChannelEstimation(ch, tx, rx)
    wf.channel_equalization = hg.LinearMinimumMeanSquareErrorChannelEqualization()
    link = hg.SimplexLink(wf, seed=SEED)
    tx.transmitters.append(link)
    rx.receivers.append(link)
    sc.set_channel(tx, rx, ch)
    rx.noise_level = hg.SNR(10 ** 2.0, link, ch)
    ber = hg.BitErrorEvaluator(link, link)
    out = sc.drop()
    e = int(ber.evaluate().evaluation.sum())
    cfg = LinkConfig(mimo_frame(), mimo_channel(fs), fs, 4, 4, "ideal", "lmmse", "snr")
    ref = simulate_drop(cfg, SEED, 0, 20.0)["errors"]
    assert close(e, ref), (e, ref)


def test_link_argument_errors():
    fs = 30.72e6
    with pytest.raises(NotImplementedError):
        hg.LinkEngine(mimo_waveform(), engine_channel(mimo_channel(fs)), 4, 4, fs, "ls", "zf", "snr", max_drops=2)
    eng = hg.LinkEngine(siso_waveform(), engine_channel(siso_channel(15.36e6)), 1, 1, 15.36e6, "ls", "zf", "ebn0",
                        max_drops=2)
    with pytest.raises(ValueError):
        eng.run(0, torch.zeros(3, device="cuda"))
