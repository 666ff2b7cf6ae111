"""GPU: the allocation-free batched drop loop (hpx_link_run_static).

Some callers cannot call cudaMalloc: hosts whose device memory is already
reserved by their own pool allocator, latency-critical loops that must not
allocate after start-up, and plugins that may not own device allocations.
hpx_link_run_static runs the same drop pipeline as hpx_link_run out of a fixed
64 MiB array in the library's device image. This file is collected last so that
a failure here never hides the results of the other GPU tests.
"""

import ctypes

import numpy as np
import pytest
import torch

import hermespy_gb300 as hg
from hermespy_gb300 import _lib
from tests.configs import mimo_channel, siso_channel

pytestmark = pytest.mark.gpu
SEED = 97


def _waveforms():
    siso = hg.OFDMWaveform(
        [hg.GridResource(1, prefix_ratio=18 / 256, elements=[hg.GridElement(hg.ElementType.DATA, 200)]),
         hg.GridResource(50, prefix_ratio=18 / 256, elements=[hg.GridElement(hg.ElementType.REFERENCE, 1),
                                                              hg.GridElement(hg.ElementType.DATA, 3)])],
        [hg.SymbolSection(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])], num_subcarriers=256, modulation_order=16)
    mimo = hg.OFDMWaveform(
        [hg.GridResource(1, prefix_ratio=72 / 1024, elements=[hg.GridElement(hg.ElementType.DATA, 600)])],
        [hg.SymbolSection(14, [0])], num_subcarriers=1024, modulation_order=64)
    return siso, mimo


def _channel(cfg):
    return hg.MultipathFadingChannel(cfg.delays, cfg.power_profile, cfg.rice_factors,
                                     num_sinusoids=cfg.num_sinusoids, doppler_frequency=cfg.doppler_frequency,
                                     seed=SEED)


def _run_static(eng, drop0, powers, ls=None):
    errors = torch.full((powers.numel(),), -1, dtype=torch.int32, device="cuda")
    _lib.call("hpx_link_run_static", eng._frame, eng._fading.handle, ls, eng._eq, SEED, drop0, powers.numel(),
              _lib.ptr(powers), _lib.ptr(errors), _lib.stream_ptr())
    torch.cuda.synchronize()
    return errors.cpu().numpy()


@pytest.mark.parametrize("case", ["mimo_ideal_lmmse", "siso_ls_zf"])
def test_static_scratch_matches_link_run(case):
    siso, mimo = _waveforms()
    if case == "mimo_ideal_lmmse":
        fs = 30.72e6
        eng = hg.LinkEngine(mimo, _channel(mimo_channel(fs)), 4, 4, fs, "ideal", "lmmse", "snr", max_drops=16,
                            seed=SEED)
        levels = np.linspace(0.0, 30.0, 16)
    else:
        fs = 15.36e6
        eng = hg.LinkEngine(siso, _channel(siso_channel(fs)), 1, 1, fs, "ls", "zf", "ebn0", max_drops=32, seed=SEED)
        levels = np.linspace(0.0, 20.0, 32)
    eng._eq = _lib.EQ_LMMSE if eng.equalizer == "lmmse" else _lib.EQ_ZF
    powers = torch.from_numpy(eng.noise_power(levels).astype(np.float32)).cuda()
    reference = eng.run(1000, powers).cpu().numpy()
    assert reference.sum() > 0
    # two calls in a row: the shared array keeps the first call's contents, which
    # the second call must not depend on
    first = _run_static(eng, 1000, powers, eng._ls)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    second = _run_static(eng, 1000, powers, eng._ls)
    free_after, _ = torch.cuda.mem_get_info()
    np.testing.assert_array_equal(first, reference)
    np.testing.assert_array_equal(second, reference)
    # the call the entry point exists for: no device memory taken or given back
    assert free_after == free_before, (free_before, free_after)


def test_static_setup_call_and_foreign_ls_table():
    """A zero-drop call performs the per-device set-up only (callers make it at
    start-up); an LS table of another frame layout is refused before any launch."""

    siso, _ = _waveforms()
    fs = 15.36e6
    eng = hg.LinkEngine(siso, _channel(siso_channel(fs)), 1, 1, fs, "ls", "zf", "ebn0", max_drops=2, seed=SEED)
    errors = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("hpx_link_run_static", eng._frame, eng._fading.handle, eng._ls, _lib.EQ_ZF, SEED, 0, 0, None,
              _lib.ptr(errors), _lib.stream_ptr())
    other = hg.OFDMWaveform(
        [hg.GridResource(1, prefix_ratio=18 / 256, elements=[hg.GridElement(hg.ElementType.DATA, 200)]),
         hg.GridResource(50, prefix_ratio=18 / 256, elements=[hg.GridElement(hg.ElementType.REFERENCE, 1),
                                                              hg.GridElement(hg.ElementType.DATA, 3)])],
        [hg.SymbolSection(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0])], num_subcarriers=256, modulation_order=16)
    powers = torch.ones(1, dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError, match="another frame layout"):
        _lib.call("hpx_link_run_static", other._frame(), eng._fading.handle, eng._ls, _lib.EQ_ZF, SEED, 0, 1,
                  _lib.ptr(powers), _lib.ptr(errors), _lib.stream_ptr())


def test_static_scratch_rejects_oversized_batches():
    _, mimo = _waveforms()
    fs = 30.72e6
    eng = hg.LinkEngine(mimo, _channel(mimo_channel(fs)), 4, 4, fs, "ideal", "lmmse", "snr", max_drops=1, seed=SEED)
    powers = torch.ones(4096, dtype=torch.float32, device="cuda")
    errors = torch.zeros(4096, dtype=torch.int32, device="cuda")
    with pytest.raises(ValueError, match="static array holds"):
        _lib.call("hpx_link_run_static", eng._frame, eng._fading.handle, None, _lib.EQ_LMMSE, SEED, 0, 4096,
                  _lib.ptr(powers), _lib.ptr(errors), _lib.stream_ptr())
