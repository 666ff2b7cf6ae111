"""GPU: pilot-comb transmit, per-stream LS, tap-domain LMMSE, the CSI-grid receiver
and the channel-estimate error sums against the oracle."""

import ctypes

import numpy as np
import pytest
import torch

from hermespy_gb300 import _lib
from hermespy_gb300.estimation import ls_stream_tables
from oracle import estimation, fading, mapping, ofdm, streams
from oracle.frame import FrameLayout
from tests.configs import mimo_channel, pilot_frame
from tests.gpu_util import cf, fading_handle, frame_handle, host, rel_rms, stream

pytestmark = pytest.mark.gpu
SEED = 91
FS = 30.72e6


def _chain(nd=2, level=10 ** (-2.0)):
    """Engine transmit + propagate + demodulate of the 4x4 pilot-comb frame."""

    lay = FrameLayout(pilot_frame())
    cfg = mimo_channel()
    fh = frame_handle(lay)
    h = fading_handle(cfg, 4, 4, FS)
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, SEED, 0, nd, _lib.ptr(st), stream())
    T, D = lay.samples_per_frame, h.max_delay
    x = torch.empty((nd, 4, T), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate_bits", fh, SEED, 0, nd, 4, _lib.ptr(x), stream())
    y = torch.empty((nd, 4, T + D), dtype=torch.complex64, device="cuda")
    p = torch.full((nd,), level, dtype=torch.float32, device="cuda")
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(x), T, _lib.ptr(y), _lib.ptr(p), SEED, 0,
              stream())
    C = lay.num_used
    grid = torch.empty((nd, 4, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_demodulate", fh, _lib.ptr(y), T + D, nd * 4, C, _lib.ptr(grid), stream())
    return lay, cfg, fh, h, st, x, grid, p


def _full(lay, g):
    """(..., W, C) -> (..., W, N) with zero columns past the used ones."""

    out = np.zeros(g.shape[:-1] + (lay.N,), dtype=np.complex128)
    out[..., : g.shape[-1]] = g
    return out


def test_comb_transmit_matches_oracle():
    lay, cfg, fh, h, st, x, grid, p = _chain()
    xs = host(x)
    for d in range(2):
        for s in range(4):
            bits = streams.data_bits(SEED, d, s, lay.bits_per_frame())
            ref = ofdm.modulate(lay, mapping.get_symbols(lay.order, bits), s)
            assert rel_rms(xs[d, s], ref) < 2e-6


def test_stream_ls_matches_oracle():
    lay, cfg, fh, h, st, x, grid, p = _chain()
    C = lay.num_used
    ip, ix, w = ls_stream_tables(lay.ref_mask[:, :C], 4, 4)
    ls = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_ls_create_streams(fh, C, 4, ip.ctypes.data_as(ctypes.c_void_p),
                                                 ix.ctypes.data_as(ctypes.c_void_p), w.ctypes.data_as(ctypes.c_void_p),
                                                 ctypes.byref(ls)))
    est = torch.empty((2, 4, 4, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ls_estimate_streams", ls, _lib.ptr(grid), C, 4, 2, _lib.ptr(est), stream())
    g = host(grid).astype(np.complex128)
    e = host(est)
    for d in range(2):
        ref = estimation.mimo_ls_estimate(lay, _full(lay, g[d]), 4)[..., :C]
        assert rel_rms(e[d], ref) < 1e-5
    _lib.call("hpx_ls_destroy", ls)


@pytest.mark.parametrize("level", [10 ** (-1.0), 10 ** (-2.5)])
def test_tap_lmmse_matches_oracle(level):
    lay, cfg, fh, h, st, x, grid, p = _chain(level=level)
    C = lay.num_used
    lm = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_lmmse_create(fh, h.handle, C, ctypes.byref(lm)))
    est = torch.empty((2, 4, 4, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_lmmse_estimate", lm, _lib.ptr(grid), C, 4, 2, _lib.ptr(p), _lib.ptr(est), stream())
    g = host(grid).astype(np.complex128)
    e = host(est)
    for d in range(2):
        ref = estimation.tap_lmmse_estimate(lay, _full(lay, g[d]), cfg, FS, level, 4)[..., :C]
        assert rel_rms(e[d], ref) < 1e-4
    _lib.call("hpx_lmmse_destroy", lm)


def test_csi_receiver_counts_exactly_and_error_sums():
    """hpx_detect_csi's count equals the reference demapper on hpx_equalize's symbols
    for the same CSI grid; hpx_csi_error equals the numpy sums."""

    lay, cfg, fh, h, st, x, grid, p = _chain(level=10 ** (-1.5))
    C, W, K = lay.num_used, lay.num_words, lay.num_data
    lm = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_lmmse_create(fh, h.handle, C, ctypes.byref(lm)))
    est = torch.empty((2, 4, 4, W, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_lmmse_estimate", lm, _lib.ptr(grid), C, 4, 2, _lib.ptr(p), _lib.ptr(est), stream())
    errs = torch.empty(2, dtype=torch.int32, device="cuda")
    _lib.call("hpx_detect_csi", fh, 4, 4, _lib.EQ_LMMSE, _lib.ptr(grid), C, _lib.ptr(est), C, _lib.ptr(p), SEED, 0, 2,
              _lib.ptr(errs), stream())
    yk = torch.empty((2 * 4, K), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_pick", fh, _lib.ptr(grid), C, 2 * 4, _lib.ptr(yk), stream())
    hk = torch.empty((2 * 16, K), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_pick", fh, _lib.ptr(est), C, 2 * 16, _lib.ptr(hk), stream())
    xe = torch.empty((2, 4, K), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_equalize", _lib.EQ_LMMSE, 4, 4, K, 2, _lib.ptr(hk), _lib.ptr(yk), _lib.ptr(p), _lib.ptr(xe), stream())
    xs, es = host(xe), host(errs)
    for d in range(2):
        tx = np.stack([streams.data_bits(SEED, d, s, lay.bits_per_frame()) for s in range(4)])
        rx = np.stack([mapping.detect_bits(lay.order, xs[d, s].astype(np.complex128)) for s in range(4)])
        assert int(np.sum(tx != rx)) == int(es[d])
        assert 0 < es[d] < tx.size // 4
    truth = torch.empty_like(est)
    _lib.call("hpx_fading_ideal_csi", h.handle, _lib.ptr(st), 2, fh, C, _lib.ptr(truth), stream())
    err = torch.empty(2, dtype=torch.float64, device="cuda")
    pw = torch.empty(2, dtype=torch.float64, device="cuda")
    _lib.call("hpx_csi_error", fh, _lib.ptr(est), _lib.ptr(truth), C, 16, 2, _lib.ptr(err), _lib.ptr(pw), stream())
    e, t_ = host(est).astype(np.complex128), host(truth).astype(np.complex128)
    m = lay.data_mask[:, :C]
    for d in range(2):
        ref_e = np.sum(np.abs(e[d][..., m] - t_[d][..., m]) ** 2)
        ref_p = np.sum(np.abs(t_[d][..., m]) ** 2)
        assert abs(host(err)[d] - ref_e) < 1e-4 * ref_e
        assert abs(host(pw)[d] - ref_p) < 1e-4 * ref_p
    _lib.call("hpx_lmmse_destroy", lm)


@pytest.mark.parametrize("est", ["ls", "lmmse"])
def test_engine_drops_match_oracle(est):
    """Whole drops of the staged engine against the oracle's drops (same draws)."""

    from oracle.link import LinkConfig, simulate_drop
    import hermespy_gb300 as hg

    spec = pilot_frame()
    wf = hg.OFDMWaveform([hg.GridResource(1, prefix_ratio=72 / 1024, elements=[hg.GridElement(hg.ElementType.DATA, 600)]),
                          hg.GridResource(1, prefix_ratio=72 / 1024,
                                          elements=[hg.GridElement(hg.ElementType.REFERENCE, 600)])],
                         [hg.SymbolSection(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])], num_subcarriers=1024,
                         modulation_order=64, pilot_comb=4)
    cfg = mimo_channel()
    ch = hg.MultipathFadingChannel(list(cfg.delays), list(cfg.power_profile), list(cfg.rice_factors),
                                   num_sinusoids=cfg.num_sinusoids, doppler_frequency=cfg.doppler_frequency)
    eng = hg.LinkEngine(wf, ch, 4, 4, FS, est, "lmmse", "snr", max_drops=4, seed=SEED)
    levels = np.array([15.0, 25.0])
    errs = eng.simulate(eng.noise_power(levels))
    lc = LinkConfig(spec, cfg, FS, 4, 4, est, "lmmse", "snr")
    for d, lv in enumerate(levels):
        ref = simulate_drop(lc, SEED, d, float(lv))
        assert abs(int(errs[d]) - ref["errors"]) <= max(3, 0.01 * ref["errors"])


def test_fused_lmmse_receiver_matches_staged():
    """hpx_detect_lmmse (estimate kept on chip) counts the same errors as
    hpx_lmmse_estimate + hpx_detect_csi on the same drops."""

    lay, cfg, fh, h, st, x, grid, p = _chain(nd=3, level=10 ** (-1.5))
    C, W = lay.num_used, lay.num_words
    lm = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_lmmse_create(fh, h.handle, C, ctypes.byref(lm)))
    p3 = torch.full((3,), 10 ** (-1.5), dtype=torch.float32, device="cuda")
    est = torch.empty((3, 4, 4, W, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_lmmse_estimate", lm, _lib.ptr(grid), C, 4, 3, _lib.ptr(p3), _lib.ptr(est), stream())
    e1 = torch.empty(3, dtype=torch.int32, device="cuda")
    _lib.call("hpx_detect_csi", fh, 4, 4, _lib.EQ_LMMSE, _lib.ptr(grid), C, _lib.ptr(est), C, _lib.ptr(p3), SEED, 0, 3,
              _lib.ptr(e1), stream())
    e2 = torch.empty(3, dtype=torch.int32, device="cuda")
    _lib.call("hpx_detect_lmmse", lm, 4, _lib.EQ_LMMSE, _lib.ptr(grid), C, _lib.ptr(p3), SEED, 0, 3, _lib.ptr(e2),
              stream())
    a, b = host(e1), host(e2)
    assert np.all(a > 0)
    assert np.all(np.abs(a.astype(np.int64) - b.astype(np.int64)) <= np.maximum(2, a // 1000)), (a, b)
    _lib.call("hpx_lmmse_destroy", lm)


def test_fused_robust_receiver_matches_staged():
    """hpx_detect_lmmse with design statistics (64 tap delays) counts the errors of
    hpx_lmmse_estimate + hpx_detect_csi on the same drops: the tensor-core receiver with
    the batched pilot LS at eight taps per thread (the genie estimator's 23 taps take
    three)."""

    import types

    from hermespy_gb300.estimation import robust_statistics

    lay = FrameLayout(pilot_frame(64, 4))
    cfg = mimo_channel()
    fh = frame_handle(lay)
    h = fading_handle(cfg, 4, 4, FS)
    nd = 3
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, SEED, 0, nd, _lib.ptr(st), stream())
    T, D = lay.samples_per_frame, h.max_delay
    x = torch.empty((nd, 4, T), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate_bits", fh, SEED, 0, nd, 4, _lib.ptr(x), stream())
    y = torch.empty((nd, 4, T + D), dtype=torch.complex64, device="cuda")
    p3 = torch.full((nd,), 10 ** (-1.5), dtype=torch.float32, device="cuda")
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(x), T, _lib.ptr(y), _lib.ptr(p3), SEED, 0,
              stream())
    C, W = lay.num_used, lay.num_words
    grid = torch.empty((nd, 4, W, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_demodulate", fh, _lib.ptr(y), T + D, nd * 4, C, _lib.ptr(grid), stream())
    design, ridge = robust_statistics(types.SimpleNamespace(gain=cfg.gain, power_profile=cfg.power_profile), FS)
    dh = design.handle(4, 4, FS)
    lm = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_lmmse_create_regularized(fh, dh.handle, C, float(ridge), ctypes.byref(lm)))
    est = torch.empty((nd, 4, 4, W, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_lmmse_estimate", lm, _lib.ptr(grid), C, 4, nd, _lib.ptr(p3), _lib.ptr(est), stream())
    e1 = torch.empty(nd, dtype=torch.int32, device="cuda")
    _lib.call("hpx_detect_csi", fh, 4, 4, _lib.EQ_LMMSE, _lib.ptr(grid), C, _lib.ptr(est), C, _lib.ptr(p3), SEED, 0, nd,
              _lib.ptr(e1), stream())
    e2 = torch.empty(nd, dtype=torch.int32, device="cuda")
    _lib.call("hpx_detect_lmmse", lm, 4, _lib.EQ_LMMSE, _lib.ptr(grid), C, _lib.ptr(p3), SEED, 0, nd, _lib.ptr(e2),
              stream())
    a, b = host(e1).astype(np.int64), host(e2).astype(np.int64)
    assert np.all(a > 0)
    assert np.all(np.abs(a - b) <= np.maximum(2, a // 1000)), (a, b)
    _lib.call("hpx_lmmse_destroy", lm)
