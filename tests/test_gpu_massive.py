"""GPU: the massive-MIMO receiver (BF16 split tensor-core Gram, FP32 Cholesky,
FP64 for ill-conditioned elements) against the float64 oracle."""

import numpy as np
import pytest
import torch

from hermespy_gb300 import _lib
from oracle import estimation, fading, mapping, streams
from oracle.frame import FrameLayout
from tests.configs import massive_channel, massive_frame
from tests.gpu_util import fading_handle, frame_handle, host, rel_rms, stream

pytestmark = pytest.mark.gpu
SEED = 404


def _run(lay, cfg, nrx, fs, mode, level, nd=2):
    fh = frame_handle(lay)
    h = fading_handle(cfg, nrx, 16, fs)
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, SEED, 0, nd, _lib.ptr(st), stream())
    T, D = lay.samples_per_frame, h.max_delay
    x = torch.empty((nd, 16, T), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate_bits", fh, SEED, 0, nd, 16, _lib.ptr(x), stream())
    y = torch.empty((nd, nrx, T + D), dtype=torch.complex64, device="cuda")
    p = torch.full((nd,), level, dtype=torch.float32, device="cuda")
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(x), T, _lib.ptr(y), _lib.ptr(p), SEED, 0,
              stream())
    C = lay.num_used
    grid = torch.empty((nd, nrx, lay.num_words, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_demodulate", fh, _lib.ptr(y), T + D, nd * nrx, C, _lib.ptr(grid), stream())
    errs = torch.empty(nd, dtype=torch.int32, device="cuda")
    n64 = torch.empty(nd, dtype=torch.int32, device="cuda")
    xe = torch.empty((nd, 16, lay.num_data), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_detect_massive", h.handle, _lib.ptr(st), fh, mode, _lib.ptr(grid), C, _lib.ptr(p), SEED, 0, nd,
              _lib.ptr(errs), _lib.ptr(n64), _lib.ptr(xe), stream())
    return host(grid), host(errs), host(n64), host(xe)


def _oracle_x(lay, cfg, nrx, fs, grid, d, mode, level):
    smp = fading.realize(cfg, SEED, d, nrx, 16)
    H = estimation.ideal_csi(lay, smp, fs)[..., : lay.num_used]
    m = lay.data_mask[:, : lay.num_used]
    yk = grid[d].astype(np.complex128)[:, m]
    hk = H[:, :, m]
    if mode == _lib.EQ_LMMSE:
        return estimation.lmmse_equalize(yk, hk, level)
    return estimation.lmmse_equalize(yk, hk, 0.0)


# The split BF16 Gram carries ~2^-16 relative error, so the solution error grows with
# the condition number of H^H H + s2 I: small for the tall 64x16 channel, larger for
# the square 16x16 one.
@pytest.mark.parametrize("nrx, tol", [(16, 5e-3), (64, 2e-4)])
def test_massive_lmmse_matches_fp64_oracle(nrx, tol):
    lay = FrameLayout(massive_frame(256, 200, 18))
    fs = 15.36e6
    cfg = massive_channel(nrx, 0.7, fs)
    level = 10 ** (-2.0)
    grid, errs, n64, xe = _run(lay, cfg, nrx, fs, _lib.EQ_LMMSE, level)
    for d in range(2):
        xr = _oracle_x(lay, cfg, nrx, fs, grid, d, _lib.EQ_LMMSE, level)
        err = rel_rms(xe[d], xr)
        assert err < tol, err
        # the fused count is the reference demapper on the kernel's own symbols
        tx = np.stack([streams.data_bits(SEED, d, s, lay.bits_per_frame()) for s in range(16)])
        rx = np.stack([mapping.detect_bits(lay.order, xe[d, s].astype(np.complex128)) for s in range(16)])
        assert int(np.sum(tx != rx)) == int(errs[d])
        rx_ref = np.stack([mapping.detect_bits(lay.order, xr[s]) for s in range(16)])
        ref = int(np.sum(tx != rx_ref))
        assert abs(int(errs[d]) - ref) <= max(3, 0.01 * ref)
        assert n64[d] == 0


def test_ill_conditioned_elements_take_fp64():
    """Strongly correlated receive antennas at high SNR make H^H H + s2 I
    ill-conditioned: those elements are re-solved in FP64 from their channel, stay
    finite and detect about as well as the oracle's float64 solve."""

    lay = FrameLayout(massive_frame(256, 200, 18))
    fs = 15.36e6
    cfg = massive_channel(16, 0.99, fs)
    level = 10 ** (-5.0)
    grid, errs, n64, xe = _run(lay, cfg, 16, fs, _lib.EQ_LMMSE, level)
    assert n64.sum() > 0
    assert np.all(np.isfinite(xe))
    for d in range(2):
        xr = _oracle_x(lay, cfg, 16, fs, grid, d, _lib.EQ_LMMSE, level)
        tx = np.stack([streams.data_bits(SEED, d, s, lay.bits_per_frame()) for s in range(16)])
        rx_ref = np.stack([mapping.detect_bits(lay.order, xr[s]) for s in range(16)])
        ref = int(np.sum(tx != rx_ref))
        assert int(errs[d]) <= 1.2 * ref + 20, (int(errs[d]), ref)


def test_config4_full_frame_matches_fp64():
    """Config 4 at its own size: 64 x 16, 4096-point FFT with 3300 used subcarriers,
    CP 288, 14 words, 16-QAM, 8 taps, rho = 0.7, 61.44 MHz; four drops at 15 dB against
    a float64 solve of the same systems (relative RMS of the equalized symbols)."""

    lay = FrameLayout(massive_frame())
    fs = 61.44e6
    cfg = massive_channel(64, 0.7, fs)
    level = 10 ** (-1.5)
    nd = 4
    grid, errs, n64, xe = _run(lay, cfg, 64, fs, _lib.EQ_LMMSE, level, nd=nd)
    worst = 0.0
    for d in range(nd):
        xr = _oracle_x(lay, cfg, 64, fs, grid, d, _lib.EQ_LMMSE, level)
        worst = max(worst, rel_rms(xe[d], xr))
        tx = np.stack([streams.data_bits(SEED, d, s, lay.bits_per_frame()) for s in range(16)])
        rx = np.stack([mapping.detect_bits(lay.order, xe[d, s].astype(np.complex128)) for s in range(16)])
        assert int(np.sum(tx != rx)) == int(errs[d])
        rx_ref = np.stack([mapping.detect_bits(lay.order, xr[s]) for s in range(16)])
        ref = int(np.sum(tx != rx_ref))
        assert abs(int(errs[d]) - ref) <= max(3, 0.01 * ref), (d, int(errs[d]), ref)
    assert worst < 1e-4, worst
