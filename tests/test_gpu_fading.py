"""GPU: fading realization, taps, propagation (+AWGN), channel state and ideal CSI
against the float64 oracle on identical Philox draws (relative RMS <= 1e-5)."""

import numpy as np
import pytest
import torch

from hermespy_gb300 import _lib
from oracle import estimation, fading, streams
from oracle.frame import FrameLayout
from tests.configs import FADING_CASES, fading_case, mimo_frame, siso_frame
from tests.gpu_util import cf, fading_handle, frame_handle, host, rel_rms, stream

pytestmark = pytest.mark.gpu
TOL = 1e-5
SEED = 0xC0FFEE


def _realize(h, nd, drop0=0):
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, SEED, drop0, nd, _lib.ptr(st), stream())
    return st


def test_draws_match_oracle():
    cfg, nrx, ntx, T, fs = fading_case("c2")
    h = fading_handle(cfg, nrx, ntx, fs)
    out = torch.empty((3, h.num_draws), dtype=torch.float64, device="cuda")
    _lib.call("hpx_fading_draws", h.handle, SEED, 4, 3, _lib.ptr(out), stream())
    got = host(out)
    for d in range(3):
        np.testing.assert_array_equal(got[d], streams.fading_uniforms(SEED, 4 + d, h.num_draws))


@pytest.mark.parametrize("doppler, expect_fp32", [(40.0, True), (400.0, False)])
def test_taps_either_rate_path_with_los(doppler, expect_fp32):
    """Realization takes FP32 rates while the largest rate is at most 2^-16 turns per
    sample (40 Hz and 20 Hz LOS at 1 MHz: 6.4e-6), FP64 above (400 Hz: 6.4e-5); both
    match the float64 oracle over 30 000 samples, LOS and NLOS taps alike."""

    from oracle import fading as ofad

    fs, T = 1e6, 30000
    cfg = ofad.FadingConfig(np.array([0.0, 2.0, 5.0]) / fs, np.array([1.0, 0.4, 0.2]), np.array([np.inf, 2.0, 0.0]),
                            9, doppler, doppler / 2, 1.0)
    assert (doppler / fs / (2 * np.pi) <= 2.0 ** -16) == expect_fp32
    h = fading_handle(cfg, 2, 2, fs)
    st = _realize(h, 2, 3)
    out = torch.empty((2, cfg.num_taps, T), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_fading_taps", h.handle, _lib.ptr(st), 2, T, _lib.ptr(out), stream())
    got = host(out)
    for d in range(2):
        smp = fading.realize(cfg, SEED, 3 + d, 2, 2)
        assert rel_rms(got[d], fading.path_impulses(smp, T, fs)) < TOL


@pytest.mark.parametrize("name", list(FADING_CASES))
def test_taps(name):
    cfg, nrx, ntx, T, fs = fading_case(name)
    h = fading_handle(cfg, nrx, ntx, fs)
    st = _realize(h, 2, 7)
    out = torch.empty((2, cfg.num_taps, T), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_fading_taps", h.handle, _lib.ptr(st), 2, T, _lib.ptr(out), stream())
    got = host(out)
    for d in range(2):
        smp = fading.realize(cfg, SEED, 7 + d, nrx, ntx)
        assert rel_rms(got[d], fading.path_impulses(smp, T, fs)) < TOL


@pytest.mark.parametrize("name", list(FADING_CASES))
@pytest.mark.parametrize("noisy", [False, True])
def test_propagate(name, noisy):
    cfg, nrx, ntx, T, fs = fading_case(name)
    h = fading_handle(cfg, nrx, ntx, fs)
    nd = 2
    st = _realize(h, nd, 3)
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((nd, ntx, T)) + 1j * rng.standard_normal((nd, ntx, T))) / np.sqrt(2)
    x = x.astype(np.complex64)
    xd = cf(x)
    D = h.max_delay
    y = torch.empty((nd, nrx, T + D), dtype=torch.complex64, device="cuda")
    p = np.array([0.3, 0.05], dtype=np.float32)
    pd = torch.from_numpy(p).cuda() if noisy else None
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(xd), T, _lib.ptr(y), _lib.ptr(pd), SEED, 3,
              stream())
    got = host(y)
    for d in range(nd):
        smp = fading.realize(cfg, SEED, 3 + d, nrx, ntx)
        ref = fading.propagate(smp, x[d].astype(np.complex128), fs)
        if noisy:
            ref = ref + streams.awgn(SEED, 3 + d, nrx, T + D, float(p[d]))
        assert got[d].shape == ref.shape
        assert rel_rms(got[d], ref) < TOL, rel_rms(got[d], ref)


def test_propagate_golden(golden):
    """The engine's sample built from explicit parameters reproduces the reference's propagation."""

    from hermespy_gb300 import LinkState, MultipathFadingSample

    g = golden("fading.npz")
    for name in FADING_CASES:
        cfg, nrx, ntx, T, fs = fading_case(name)
        smp = fading.realize(cfg, seed=1234, drop=3, num_rx=nrx, num_tx=ntx)
        los, nlos = cfg.gains()
        s = MultipathFadingSample(cfg.power_profile, cfg.delays, smp.los_angles, smp.nlos_angles, smp.los_phases,
                                  smp.nlos_phases, los, nlos, cfg.los_doppler, cfg.doppler_frequency, smp.spatial,
                                  cfg.gain, LinkState(ntx, nrx, fs))
        y = host(s.propagate_device(g[f"{name}_x"]))
        assert rel_rms(y, g[f"{name}_y"]) < TOL
        st = g[f"{name}_state"]
        Ts = st.shape[2]
        csi = host(s.state_device(Ts, Ts))[:2, :2]
        assert rel_rms(csi, st) < TOL


@pytest.mark.parametrize("name", ["c1", "c2", "los", "grp"])
def test_channel_state(name):
    cfg, nrx, ntx, T, fs = fading_case(name)
    h = fading_handle(cfg, nrx, ntx, fs)
    st = _realize(h, 1, 2)
    Ts = 300
    ntaps = min(1 + h.max_delay, Ts)
    out = torch.empty((1, nrx, ntx, Ts, ntaps), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_fading_csi", h.handle, _lib.ptr(st), 1, Ts, Ts, _lib.ptr(out), stream())
    smp = fading.realize(cfg, SEED, 2, nrx, ntx)
    assert rel_rms(host(out)[0], fading.state(smp, Ts, fs, Ts)) < TOL


@pytest.mark.parametrize("frame", ["siso", "mimo"])
def test_ideal_csi(frame):
    lay = FrameLayout(siso_frame() if frame == "siso" else mimo_frame())
    name = "c1" if frame == "siso" else "c2"
    cfg, nrx, ntx, T, fs = fading_case(name)
    nrx, ntx = (1, 1) if frame == "siso" else (2, 2)
    h = fading_handle(cfg, nrx, ntx, fs)
    fh = frame_handle(lay)
    st = _realize(h, 2, 9)
    out = torch.empty((2, nrx, ntx, lay.num_words, lay.N), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_fading_ideal_csi", h.handle, _lib.ptr(st), 2, fh, lay.N, _lib.ptr(out), stream())
    got = host(out)
    for d in range(2):
        smp = fading.realize(cfg, SEED, 9 + d, nrx, ntx)
        assert rel_rms(got[d], estimation.ideal_csi(lay, smp, fs)) < TOL


def test_ideal_csi_golden(golden):
    from hermespy_gb300 import LinkState, MultipathFadingSample

    g = golden("ideal.npz")
    cfg, _, _, _, fs = fading_case("c2")
    smp = fading.realize(cfg, seed=99, drop=7, num_rx=2, num_tx=2)
    los, nlos = cfg.gains()
    s = MultipathFadingSample(cfg.power_profile, cfg.delays, smp.los_angles, smp.nlos_angles, smp.los_phases,
                              smp.nlos_phases, los, nlos, cfg.los_doppler, cfg.doppler_frequency, smp.spatial,
                              cfg.gain, LinkState(2, 2, fs))
    lay = FrameLayout(mimo_frame())
    fh = frame_handle(lay)
    out = torch.empty((2, 2, lay.num_words, lay.N), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_fading_ideal_csi", s._handle.handle, _lib.ptr(s._state), 1, fh, lay.N, _lib.ptr(out), stream())
    assert rel_rms(host(out)[:, :, ::5, :], g["csi"]) < TOL


def test_correlated_massive_spatial():
    """64 x 16 spatial response with exponential correlation (rho = 0.7), beyond the
    reference's 10 x 10 limit: propagation against the oracle restatement."""

    i = np.arange(64)
    corr = (0.7 ** np.abs(i[:, None] - i[None, :])).astype(np.complex128)
    fs = 61.44e6
    cfg = fading.FadingConfig(np.arange(8) / fs, np.exp(-0.5 * np.arange(8)), np.zeros(8), 20, 50.0,
                              rx_correlation=corr, tx_correlation=corr[:16, :16])
    h = fading_handle(cfg, 64, 16, fs)
    st = _realize(h, 1, 1)
    T = 2000
    rng = np.random.default_rng(2)
    x = ((rng.standard_normal((16, T)) + 1j * rng.standard_normal((16, T))) / np.sqrt(2)).astype(np.complex64)
    y = torch.empty((1, 64, T + h.max_delay), dtype=torch.complex64, device="cuda")
    xd = cf(x)
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), 1, _lib.ptr(xd), T, _lib.ptr(y), None, 0, 0, stream())
    smp = fading.realize(cfg, SEED, 1, 64, 16)
    assert rel_rms(host(y)[0], fading.propagate(smp, x.astype(np.complex128), fs)) < TOL
