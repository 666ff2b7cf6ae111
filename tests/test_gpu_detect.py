"""GPU: LS estimation, ZF / LMMSE equalization and the fused receivers."""

import ctypes

import numpy as np
import pytest
import torch

from hermespy_gb300 import _lib
from hermespy_gb300.estimation import ls_interpolation_table
from oracle import estimation, fading, mapping, ofdm, streams
from oracle.frame import FrameLayout
from tests.configs import fading_case, mimo_frame, siso_frame
from tests.gpu_util import cf, fading_handle, frame_handle, host, rel_rms, stream

pytestmark = pytest.mark.gpu
SEED = 77


def _ls_handle(lay, fh, cols):
    ip, ix, w = ls_interpolation_table(lay.ref_mask[:, :cols])
    h = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_ls_create(fh, cols, ip.ctypes.data_as(ctypes.c_void_p), ix.ctypes.data_as(ctypes.c_void_p),
                                         w.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)))
    return h


def test_ls_estimate_golden(golden):
    g = golden("ls.npz")
    lay = FrameLayout(siso_frame())
    fh = frame_handle(lay)
    ls = _ls_handle(lay, fh, lay.N)
    grid = cf(g["grid"][None])
    out = torch.empty((1, lay.num_words, lay.N), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ls_estimate", ls, _lib.ptr(grid), lay.N, 1, _lib.ptr(out), stream())
    assert rel_rms(host(out)[0], g["estimate"]) < 1e-6


@pytest.mark.parametrize("name", ["siso", "mimo"])
def test_zf_golden(golden, name):
    g = golden("zf.npz")
    y, h = g[f"{name}_y"], g[f"{name}_h"]
    nrx, ntx, K = h.shape
    out_streams = 1 if nrx == 1 else ntx
    x = torch.empty((1, out_streams, K), dtype=torch.complex64, device="cuda")
    hd, yd = cf(h[None]), cf(y[None])  # keep the inputs alive until the kernel has run
    _lib.call("hpx_equalize", _lib.EQ_ZF, nrx, ntx, K, 1, _lib.ptr(hd), _lib.ptr(yd), None, _lib.ptr(x), stream())
    # random 4x4 matrices can be ill conditioned: float32 vs float64 pseudo-inverse
    assert rel_rms(host(x)[0], g[f"{name}_x"]) < 1e-4


@pytest.mark.parametrize("nrx,ntx", [(1, 1), (2, 2), (4, 4), (4, 2), (8, 4), (2, 4), (8, 8)])
def test_lmmse_matches_oracle(nrx, ntx):
    rng = np.random.default_rng(nrx * 10 + ntx)
    K = 4096
    h = (rng.standard_normal((nrx, ntx, K)) + 1j * rng.standard_normal((nrx, ntx, K))) / np.sqrt(2)
    y = rng.standard_normal((nrx, K)) + 1j * rng.standard_normal((nrx, K))
    s2 = 0.1
    x = torch.empty((1, ntx, K), dtype=torch.complex64, device="cuda")
    nv = torch.tensor([s2], dtype=torch.float32, device="cuda")
    h32, y32 = h.astype(np.complex64), y.astype(np.complex64)
    hd, yd = cf(h32[None]), cf(y32[None])
    _lib.call("hpx_equalize", _lib.EQ_LMMSE, nrx, ntx, K, 1, _lib.ptr(hd), _lib.ptr(yd), _lib.ptr(nv), _lib.ptr(x),
              stream())
    ref = estimation.lmmse_equalize(y32.astype(np.complex128), h32.astype(np.complex128), s2)
    assert rel_rms(host(x)[0], ref) < 1e-5


def _staged_equalized(lay, cfg, nrx, ntx, fs, mode, level):
    """Engine transmit + propagate + demodulate + ideal CSI + pick + equalize, staged."""

    fh = frame_handle(lay)
    h = fading_handle(cfg, nrx, ntx, fs)
    nd = 2
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, SEED, 0, nd, _lib.ptr(st), stream())
    T, D = lay.samples_per_frame, h.max_delay
    x = torch.empty((nd, ntx, T), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate_bits", fh, SEED, 0, nd, ntx, _lib.ptr(x), stream())
    y = torch.empty((nd, nrx, T + D), dtype=torch.complex64, device="cuda")
    p = torch.full((nd,), level, dtype=torch.float32, device="cuda")
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(x), T, _lib.ptr(y), _lib.ptr(p), SEED, 0,
              stream())
    C = lay.num_used
    grid = torch.empty((nd, nrx, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_demodulate", fh, _lib.ptr(y), T + D, nd * nrx, C, _lib.ptr(grid), stream())
    csi = torch.empty((nd, nrx, ntx, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_fading_ideal_csi", h.handle, _lib.ptr(st), nd, fh, C, _lib.ptr(csi), stream())
    K = lay.num_data
    yk = torch.empty((nd * nrx, K), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_pick", fh, _lib.ptr(grid), C, nd * nrx, _lib.ptr(yk), stream())
    hk = torch.empty((nd * nrx * ntx, K), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_pick", fh, _lib.ptr(csi), C, nd * nrx * ntx, _lib.ptr(hk), stream())
    out_streams = 1 if (mode == _lib.EQ_ZF and nrx == 1) else ntx
    xe = torch.empty((nd, out_streams, K), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_equalize", mode, nrx, ntx, K, nd, _lib.ptr(hk), _lib.ptr(yk), _lib.ptr(p), _lib.ptr(xe), stream())
    errs = torch.empty(nd, dtype=torch.int32, device="cuda")
    _lib.call("hpx_detect_ideal", h.handle, _lib.ptr(st), fh, mode, _lib.ptr(grid), C, _lib.ptr(p), SEED, 0, nd,
              _lib.ptr(errs), stream())
    return host(xe), host(errs), host(y), host(grid), host(csi)


@pytest.mark.parametrize("mode", [0, 1])
def test_fused_ideal_detection_counts_exactly(mode):
    """The fused receiver's error count equals the reference demapper applied to the
    staged engine's equalized symbols, against the oracle's Philox bits."""

    lay = FrameLayout(mimo_frame(64))
    cfg, _, _, _, fs = fading_case("c2")
    nrx = ntx = 4
    xe, errs, *_ = _staged_equalized(lay, cfg, nrx, ntx, fs, mode, 10 ** (-1.5))
    for d in range(2):
        tx = np.stack([streams.data_bits(SEED, d, s, lay.bits_per_frame()) for s in range(ntx)])
        rx = np.stack([mapping.detect_bits(64, xe[d, s].astype(np.complex128)) for s in range(ntx)])
        assert int(np.sum(tx != rx)) == int(errs[d])
        assert 0 < errs[d] < tx.size // 4


def test_staged_chain_matches_oracle():
    """Received grid and ideal CSI of the engine against the oracle's drop."""

    from oracle.link import LinkConfig, simulate_drop

    lay = FrameLayout(mimo_frame(64))
    cfg, _, _, _, fs = fading_case("c2")
    p = 10 ** (-2.0)
    _, _, y, grid, csi = _staged_equalized(lay, cfg, 4, 4, fs, 1, p)
    lc = LinkConfig(mimo_frame(64), cfg, fs, 4, 4, "ideal", "lmmse", "snr")
    for d in range(2):
        out = simulate_drop(lc, SEED, d, 0.0, keep=True)  # noise level replaced below
        smp = out["sample"]
        ref_y = fading.propagate(smp, out["x"], fs) + streams.awgn(SEED, d, 4, y.shape[2], p)
        assert rel_rms(y[d], ref_y) < 1e-5
        ref_grid = np.stack([ofdm.demodulate(lay, ref_y[r, : lay.samples_per_frame]) for r in range(4)])
        assert rel_rms(grid[d], ref_grid[:, :, : lay.num_used]) < 1e-5
        assert rel_rms(csi[d], estimation.ideal_csi(lay, smp, fs)[..., : lay.num_used]) < 1e-5


def test_fused_ls_detection_counts_exactly():
    lay = FrameLayout(siso_frame(16))
    cfg, _, _, _, fs = fading_case("c1")
    fh = frame_handle(lay)
    h = fading_handle(cfg, 1, 1, fs)
    nd = 4
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, SEED, 0, nd, _lib.ptr(st), stream())
    T, D = lay.samples_per_frame, h.max_delay
    x = torch.empty((nd, 1, T), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate_bits", fh, SEED, 0, nd, 1, _lib.ptr(x), stream())
    y = torch.empty((nd, 1, T + D), dtype=torch.complex64, device="cuda")
    p = torch.full((nd,), 0.25 / 10 ** 0.8, dtype=torch.float32, device="cuda")
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(x), T, _lib.ptr(y), _lib.ptr(p), SEED, 0,
              stream())
    C = lay.num_used
    grid = torch.empty((nd, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_demodulate", fh, _lib.ptr(y), T + D, nd, C, _lib.ptr(grid), stream())
    ls = _ls_handle(lay, fh, C)
    est = torch.empty((nd, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ls_estimate", ls, _lib.ptr(grid), C, nd, _lib.ptr(est), stream())
    errs = torch.empty(nd, dtype=torch.int32, device="cuda")
    _lib.call("hpx_detect_ls", ls, _lib.EQ_ZF, _lib.ptr(grid), C, _lib.ptr(p), SEED, 0, nd, _lib.ptr(errs), stream())
    g, e, ee = host(grid), host(est), host(errs)
    for d in range(nd):
        ref_est = estimation.ls_estimate(lay, np.pad(g[d], ((0, 0), (0, lay.N - C))).astype(np.complex128))
        assert rel_rms(e[d], ref_est[:, :C]) < 1e-5
        yk = ofdm.pick(lay, np.pad(g[d], ((0, 0), (0, lay.N - C))))
        hk = ofdm.pick(lay, np.pad(e[d], ((0, 0), (0, lay.N - C))))
        xe = (yk / hk).astype(np.complex64)
        rx = mapping.detect_bits(16, xe.astype(np.complex128))
        tx = streams.data_bits(SEED, d, 0, lay.bits_per_frame())
        assert abs(int(np.sum(tx != rx)) - int(ee[d])) <= 2  # float32 division order may flip a tie
