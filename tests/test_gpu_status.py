"""GPU: device failures reach the caller as exceptions instead of entering BER sums.

The reference raises from the failing drop into its Monte Carlo actor
(core/pymonte/actors.py:444-452). The engine reports (a) bounded tensor-core / TMA
waits that ran out, through the handles' sticky status words and the per-drop
HPX_DROP_TIMEOUT flag, and (b) non-finite equalizer pivots through HPX_DROP_NUMERIC.
No test faults or stalls the GPU: a timeout is injected from the host by setting the
handle's status word (the kernels then take their skip path at once), and the numeric
failure comes from a NaN noise power.
"""

import ctypes
import math

import numpy as np
import pytest
import torch

import hermespy_gb300 as hg
from hermespy_gb300 import _lib
from hermespy_gb300.learned import WEIGHTS_DIR, CnnChannelEstimator
from hermespy_gb300.train_estimator import pilot_waveform, workload_channel

pytestmark = pytest.mark.gpu
SEED = 99


def pilot_engine(estimator, drops=4):
    model = None
    if estimator == "learned":
        model = CnnChannelEstimator.load(f"{WEIGHTS_DIR}/cnn_4x4_1024.npz", max_batch=drops)
    return hg.LinkEngine(pilot_waveform(), workload_channel(), 4, 4, 30.72e6, estimator, "lmmse", "snr",
                         max_drops=drops, seed=SEED, model=model)


def test_lmmse_timeout_raises_and_clears():
    eng = pilot_engine("lmmse")
    p = torch.from_numpy(eng.noise_power([10.0, 15.0, 20.0, 25.0]).astype(np.float32)).cuda()
    good = eng.counts(eng.run(0, p))
    assert good.sum() > 0
    _lib.call("hpx_lmmse_inject_timeout", eng._lmmse, _lib.stream_ptr())
    words = eng.run(0, p).cpu().numpy().astype(np.int64) & 0xFFFFFFFF
    assert np.all(words & _lib.DROP_TIMEOUT)  # every drop flagged, no count summed
    with pytest.raises(RuntimeError, match="tensor-core wait ran out"):
        eng.status()
    eng.status()  # cleared by the previous call
    assert np.array_equal(eng.counts(eng.run(0, p)), good)  # the handle works again, same drops


def test_lmmse_timeout_stops_simulate():
    eng = pilot_engine("lmmse")
    _lib.call("hpx_lmmse_inject_timeout", eng._lmmse, _lib.stream_ptr())
    with pytest.raises(RuntimeError, match="tensor-core wait ran out"):
        eng.simulate(eng.noise_power([12.0, 18.0]))
    assert eng.simulate(eng.noise_power([12.0, 18.0])).sum() > 0


def test_cnn_timeout_gives_nan_and_raises():
    eng = pilot_engine("learned")
    p = torch.from_numpy(eng.noise_power([10.0, 20.0]).astype(np.float32)).cuda()
    eng.receive(0, p)
    ref = eng.estimate(2, p).clone()
    assert torch.isfinite(ref).all()
    _lib.call("hpx_cnn_inject_timeout", eng.model.handle, _lib.stream_ptr())
    out = eng.estimate(2, p)
    assert torch.isnan(out).all()
    with pytest.raises(RuntimeError, match="wait ran out"):
        eng.model.status()
    # the learned path's drops now see NaN channels: the detector flags them numeric
    eng.receive(0, p)
    errors = torch.empty(2, dtype=torch.int32, device="cuda")
    _lib.call("hpx_cnn_inject_timeout", eng.model.handle, _lib.stream_ptr())
    eng.estimate(2, p)
    eng.detect(0, 2, p, errors)
    with pytest.raises(RuntimeError):
        eng.counts(errors)
    eng.status()
    eng.receive(0, p)
    assert torch.allclose(eng.estimate(2, p), ref)


@pytest.mark.parametrize("path", ["siso_ls", "ideal_4x4", "pilot_lmmse", "pilot_ls"])
def test_nan_noise_power_is_a_numeric_failure(path):
    if path == "siso_ls":
        from tests.test_gpu_link import engine_channel, siso_waveform
        from tests.configs import siso_channel

        eng = hg.LinkEngine(siso_waveform(), engine_channel(siso_channel(15.36e6)), 1, 1, 15.36e6, "ls", "zf",
                            "ebn0", max_drops=8, seed=SEED)
    elif path == "ideal_4x4":
        from tests.test_gpu_link import engine_channel, mimo_waveform
        from tests.configs import mimo_channel

        eng = hg.LinkEngine(mimo_waveform(), engine_channel(mimo_channel(30.72e6)), 4, 4, 30.72e6, "ideal",
                            "lmmse", "snr", max_drops=8, seed=SEED)
    else:
        eng = pilot_engine(path[6:])
    p = eng.noise_power([10.0, 10.0, 10.0])
    p[1] = math.nan
    words = eng.run(0, torch.from_numpy(p.astype(np.float32)).cuda()).cpu().numpy().astype(np.int64) & 0xFFFFFFFF
    assert words[1] & _lib.DROP_NUMERIC and not words[0] & _lib.DROP_NUMERIC and not words[2] & _lib.DROP_NUMERIC
    with pytest.raises(RuntimeError, match="drop 1: non-finite pivot"):
        eng.simulate(p)
    p[1] = p[0]
    eng.simulate(p)  # finite again: no exception


def test_campaign_stops_on_numeric_failure():
    from tests.test_gpu_link import engine_channel, siso_waveform
    from tests.configs import siso_channel

    eng = hg.LinkEngine(siso_waveform(), engine_channel(siso_channel(15.36e6)), 1, 1, 15.36e6, "ls", "zf", "ebn0",
                        max_drops=64, seed=SEED)
    with pytest.raises(RuntimeError, match="non-finite pivot"):
        eng.ber_campaign([10.0, float("nan")], min_samples=8, max_drops_per_level=64, batch=32, check_every=1)
    pts = eng.ber_campaign([10.0], min_samples=8, max_drops_per_level=64, batch=32, check_every=1)
    assert pts[0].drops > 0
