"""GPU: the device-resident Monte Carlo campaign (per-level sums and the
confidence stopping rule on the GPU) against drop-by-drop runs of the same drops."""

import ctypes

import numpy as np
import pytest
from scipy.stats import norm

import hermespy_gb300 as hg
from hermespy_gb300 import _lib
from tests.configs import siso_channel
from tests.test_gpu_link import SEED, engine_channel, siso_waveform

pytestmark = pytest.mark.gpu


def _engine(max_drops):
    return hg.LinkEngine(siso_waveform(), engine_channel(siso_channel()), 1, 1, 15.36e6, "ls", "zf", "ebn0",
                         max_drops=max_drops, seed=SEED)


def test_campaign_matches_drop_by_drop():
    """accuracy 0 never satisfies the rule, so every level runs to its drop limit with
    drops dealt round-robin: the same drops as a plain batched run."""

    eng = _engine(48)
    levels = [0.0, 6.0, 12.0]
    pts = eng.ber_campaign(levels, accuracy=0.0, confidence=0.05, min_samples=8, max_drops_per_level=64, batch=48)
    assert [p.drops for p in pts] == [64, 64, 64]
    assert not any(p.confident for p in pts)
    powers = eng.noise_power(levels)
    per_drop = eng.simulate(np.array([powers[i % 3] for i in range(192)]), drop0=0)
    for k, p in enumerate(pts):
        assert p.errors == int(per_drop[k::3].sum())


def test_campaign_confidence_rule():
    """A noisy level stops early once the rule holds (re-checked here from the
    returned sums); an error-free level never does (std = 0) and runs to its limit."""

    eng = _engine(64)
    levels = [0.0, 40.0]
    power = np.ascontiguousarray(eng.noise_power(levels).astype(np.float32))
    h = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_campaign_create(2, power.ctypes.data_as(ctypes.c_void_p), 0.01, 0.05, 16, 1024, 64,
                                               float(eng.bits_per_drop), ctypes.byref(h)))
    done, active = ctypes.c_int64(), ctypes.c_int32()
    _lib.call("hpx_campaign_run", h, eng.link_handle, SEED, 0, 64, 1000, 1, ctypes.byref(done), ctypes.byref(active),
              _lib.stream_ptr())
    drops = np.zeros(2, dtype=np.int64)
    errs = np.zeros(2, dtype=np.int64)
    s = np.zeros(2)
    q = np.zeros(2)
    conf = np.zeros(2, dtype=np.int32)
    _lib.call("hpx_campaign_results", h, drops.ctypes.data_as(ctypes.c_void_p), errs.ctypes.data_as(ctypes.c_void_p),
              s.ctypes.data_as(ctypes.c_void_p), q.ctypes.data_as(ctypes.c_void_p), conf.ctypes.data_as(ctypes.c_void_p))
    _lib.load().hpx_campaign_destroy(h)
    assert active.value == 0
    assert conf[0] == 1 and drops[0] < 1024
    n = drops[0]
    sd = np.sqrt((q[0] - s[0] ** 2 / n) / (n - 1))
    assert 2 * (1 - norm.cdf(np.sqrt(n) * 0.01 / sd)) < 0.05
    assert abs(s[0] * eng.bits_per_drop - errs[0]) < 1e-6 * max(1, errs[0])
    if errs[1] == 0:
        assert conf[1] == 0 and drops[1] >= 1024


@pytest.mark.parametrize("estimator", ["lmmse", "learned"])
def test_staged_estimator_campaign_matches_plain_runs(estimator):
    """The campaign over the headline link's staged estimators (tap-domain LMMSE
    receiver, LS + CNN): with accuracy 0 every level runs to its limit, dealt
    round-robin, so the per-level errors equal a plain run of the same drops; with a
    real accuracy a noisy level stops early by the reference's rule."""

    from hermespy_gb300.learned import WEIGHTS_DIR, CnnChannelEstimator
    from hermespy_gb300.train_estimator import pilot_waveform, workload_channel

    model = CnnChannelEstimator.load(f"{WEIGHTS_DIR}/cnn_4x4_1024.npz", max_batch=48) if estimator == "learned" else None
    eng = hg.LinkEngine(pilot_waveform(), workload_channel(), 4, 4, 30.72e6, estimator, "lmmse", "snr",
                        max_drops=48, seed=SEED, model=model)
    levels = [5.0, 15.0, 25.0]
    # 48-drop batches deal 16 drops to each level: drop i of the campaign is at level i % 3
    pts = eng.ber_campaign(levels, accuracy=0.0, min_samples=8, max_drops_per_level=32, batch=48, check_every=2)
    assert [p.drops for p in pts] == [32, 32, 32]
    powers = eng.noise_power(levels)
    per_drop = eng.simulate(np.array([powers[i % 3] for i in range(96)]), drop0=0)
    for k, p in enumerate(pts):
        assert p.errors == int(per_drop[k::3].sum())
    pts = eng.ber_campaign([5.0], accuracy=0.01, confidence=0.05, min_samples=8, max_drops_per_level=4096, batch=48,
                           check_every=1)
    assert pts[0].confident and pts[0].drops < 4096
