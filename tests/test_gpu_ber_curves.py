"""GPU: BER at the workloads' own shapes and drop counts against the reference's and
the oracle's drops (fixtures by tests/golden/make_ber_curves.py).

Every check runs the engine on the fixture's (seed, drop index, noise level), i.e. on
the very drops the fixture's CPU side simulated, and asks for two things:

* per-drop bit errors equal to the CPU drop's within max(3, 1 %) (FP32 against
  float64 symbols near decision boundaries; for the learned path max(3, 2 %), BF16
  network activations against the oracle's float64 accumulation);
* the engine's BER at each point inside the 95 % Clopper-Pearson interval of the CPU
  drops' BER (the acceptance rule for BER curves).

Config 1 and the ZF leg of config 2 compare with the reference's own
``SimulationScenario.drop()``; the LMMSE paths and the uneven batch, which the
reference does not have, with the oracle.
"""

import hashlib
import os

import numpy as np
import pytest
import torch

import hermespy_gb300 as hg
from hermespy_gb300.learned import WEIGHTS_DIR, CnnChannelEstimator
from hermespy_gb300.train_estimator import pilot_waveform, workload_channel
from hermespy_gb300.uneven import DropConfig, UnevenBatch
from tests.configs import siso_channel
from tests.test_gpu_link import engine_channel, mimo_waveform, siso_waveform

pytestmark = pytest.mark.gpu


def close(a, b, rel=0.01):
    return abs(int(a) - int(b)) <= max(3, rel * max(int(a), int(b)))


def check_drops(engine_errors, cpu_errors, rel=0.01, what=""):
    e = np.asarray(engine_errors, dtype=np.int64)
    c = np.asarray(cpu_errors, dtype=np.int64)
    bad = [i for i in range(e.size) if not close(e[i], c[i], rel)]
    assert not bad, f"{what}: drops {bad[:10]} differ, engine {e[bad[:10]].tolist()} vs {c[bad[:10]].tolist()}"


def check_interval(engine_errors, cpu_errors, bits, what=""):
    lo, hi = hg.clopper_pearson(int(np.sum(cpu_errors)), bits)
    ber = int(np.sum(engine_errors)) / bits
    assert lo <= ber <= hi, f"{what}: engine BER {ber:.6g} outside [{lo:.6g}, {hi:.6g}]"


def test_config1_siso_ber_curve_matches_reference(golden):
    """SISO 256/200, 16-QAM, LS + ZF, Eb/N0 0..20 dB, 1 000 drops per point."""

    z = golden("ber_siso.npz")
    fs = 15.36e6
    per = int(z["drops_per_level"])
    eng = hg.LinkEngine(siso_waveform(), engine_channel(siso_channel(fs)), 1, 1, fs, "ls", "zf", "ebn0",
                        max_drops=4096, seed=int(z["seed"]))
    assert np.allclose(eng.noise_power(z["levels_db"]), z["ref_noise_power"][::per], rtol=1e-12)
    pts = eng.ber_curve(z["levels_db"], per)
    errs = eng.simulate(np.repeat(eng.noise_power(z["levels_db"]), per))
    ref = z["ref_errors"]
    assert np.array_equal(ref, z["oracle_errors"])  # the oracle restates the reference drop exactly
    for i, pt in enumerate(pts):
        s = slice(i * per, (i + 1) * per)
        assert pt.errors == errs[s].sum()
        check_drops(errs[s], ref[s], what=f"Eb/N0 {pt.level_db} dB")
        check_interval(errs[s], ref[s], pt.bits, what=f"Eb/N0 {pt.level_db} dB")


@pytest.mark.parametrize("equalizer", ["zf", "lmmse"])
def test_config2_mimo_ideal_csi(golden, equalizer):
    """4x4 1024/600, 64-QAM, 23 taps, ideal CSI, SNR U[0, 30] dB, 256 drops: ZF against
    the reference's drops, LMMSE against the oracle's."""

    z = golden("ber_mimo.npz")
    fs = 30.72e6
    from tests.configs import mimo_channel

    eng = hg.LinkEngine(mimo_waveform(), engine_channel(mimo_channel(fs)), 4, 4, fs, "ideal", equalizer, "snr",
                        max_drops=256, seed=int(z["seed"]))
    p = eng.noise_power(z["snr_db"])
    assert np.allclose(p, z["ref_noise_power"], rtol=1e-12)
    errs = eng.simulate(p)
    cpu = z["ref_zf_errors"] if equalizer == "zf" else z["oracle_lmmse_errors"]
    if equalizer == "zf":
        assert np.array_equal(z["ref_zf_errors"], z["oracle_zf_errors"])
    check_drops(errs, cpu, what=equalizer)
    check_interval(errs, cpu, errs.size * int(z["bits_per_drop"]), what=equalizer)


@pytest.mark.parametrize("estimator", ["lmmse", "lmmse_robust", "ls", "learned"])
def test_headline_pilot_link_estimators(golden, estimator):
    """The learned-vs-LMMSE workload: 4x4 pilot-comb 1024/600, 64-QAM, SNR U[0, 30] dB,
    512 drops; tap-domain LMMSE with the channel's statistics and with the robust design
    statistics (both the fused tensor-core receiver), per-stream LS and LS + CNN, each
    with LMMSE detection, against the oracle's drops."""

    z = golden("ber_pilot.npz")
    wpath = os.path.join(WEIGHTS_DIR, "cnn_4x4_1024.npz")
    with open(wpath, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == str(z["weights_sha256"]), "fixture made with other weights"
    model = CnnChannelEstimator.load(wpath, max_batch=256) if estimator == "learned" else None
    eng = hg.LinkEngine(pilot_waveform(), workload_channel(), 4, 4, 30.72e6, estimator, "lmmse", "snr",
                        max_drops=512, seed=int(z["seed"]), model=model)
    p = eng.noise_power(z["snr_db"])
    assert np.allclose(p, z["noise_power"], rtol=1e-12)
    errs = eng.simulate(p)
    cpu = z[f"{estimator}_errors"]
    check_drops(errs, cpu, rel=0.02 if estimator == "learned" else 0.01, what=estimator)
    check_interval(errs, cpu, errs.size * int(z["bits_per_drop"]), what=estimator)


def test_config3_uneven_batch_matches_oracle(golden):
    """40 drops of the uneven distribution (incl. 8x8 / 2048-point / 256-QAM and 1x1 /
    128-point / 4-QAM) in one persistent launch: each drop against the oracle's drop,
    and against the homogeneous engine's count for that drop."""

    z = golden("uneven.npz")
    fields = ("num_rx", "num_tx", "fft_size", "num_words", "modulation_order", "num_taps", "tap_decay_db",
              "doppler_frequency", "snr_db")
    drops = [DropConfig(*[z[f][i].item() for f in fields]) for i in range(z["errors"].size)]
    assert np.allclose([d.noise_power() for d in drops], z["noise_power"], rtol=1e-12)
    batch = UnevenBatch(drops, 30e3, 50e-9, 20, max_slots=64)
    errs = hg._lib.drop_counts(batch.run(int(z["seed"]), int(z["drop0"])).cpu().numpy())
    check_drops(errs, z["errors"], what="uneven")
    bits = int(np.sum(batch.bits))
    check_interval(errs, z["errors"], bits, what="uneven")
    # and the homogeneous engine's counts for the same drops (see assert_same_counts)
    from tests.test_gpu_uneven import _homogeneous_errors, assert_same_counts

    p = batch.noise_power.cpu().numpy()
    pick = list(range(12))
    assert_same_counts(errs[pick], [_homogeneous_errors(drops[i], int(z["drop0"]) + i, float(p[i]), int(z["seed"]))
                                    for i in pick])
