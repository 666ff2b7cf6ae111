"""GPU: OFDM modulate / demodulate / pick against the oracle and the reference's
golden frames (float32 engine vs float64 reference: relative RMS error bound)."""

import numpy as np
import pytest
import torch

from hermespy_gb300 import _lib
from oracle import mapping, ofdm, streams
from oracle.frame import DATA, REFERENCE, FrameLayout, FrameSpec, Resource, Section
from tests.configs import mimo_frame, siso_frame
from tests.gpu_util import cf, frame_handle, host, rel_rms, stream

pytestmark = pytest.mark.gpu
TOL = 1e-5  # relative RMS, float32 engine vs float64 oracle


def _modulate(h, lay, data):
    d = cf(np.atleast_2d(data))
    out = torch.empty((d.shape[0], lay.samples_per_frame), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate", h, _lib.ptr(d), d.shape[0], _lib.ptr(out), stream())
    return host(out)


def _demodulate(h, lay, x, cols):
    x = cf(np.atleast_2d(x))
    out = torch.empty((x.shape[0], lay.num_words, cols), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_demodulate", h, _lib.ptr(x), x.shape[1], x.shape[0], cols, _lib.ptr(out), stream())
    return host(out)


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("dc", [True, False])
def test_modulate_demodulate_golden(golden, name, dc):
    g = golden("ofdm.npz")
    spec = siso_frame() if name == "c1" else mimo_frame()
    spec.dc_suppression = dc
    lay = FrameLayout(spec)
    h = frame_handle(lay)
    x = _modulate(h, lay, g[f"{name}_data"])[0]
    ref_x = g[f"{name}_x" + ("" if dc else "_nodc")]
    assert rel_rms(x[: ref_x.size], ref_x) < TOL
    # demodulate the deterministic distortion of the reference transmit frame
    spec_dc = siso_frame() if name == "c1" else mimo_frame()
    rx_full = np.roll(ofdm.modulate(FrameLayout(spec_dc), g[f"{name}_data"]), 3)
    rx_full = rx_full + 0.5 * ofdm.modulate(FrameLayout(spec_dc), g[f"{name}_data"])
    grid = _demodulate(h, lay, rx_full, lay.N)[0]
    ref_g = g[f"{name}_grid" + ("" if dc else "_nodc")]
    assert rel_rms(grid[: ref_g.shape[0]], ref_g) < TOL


@pytest.mark.parametrize("N", [64, 128, 256, 512, 1024, 2048, 4096])
def test_fft_sizes(N):
    """Every supported FFT size, random full grids, zero-pad prefixes on odd words."""

    rng = np.random.default_rng(N)
    res = [Resource(1, 0.25, [(DATA, N)]), Resource(1, 0.125, [(DATA, N // 2), (REFERENCE, 1), (DATA, N // 2 - 1)],
                                                      "ZEROPAD")]
    spec = FrameSpec(N, res, [Section(2, [0, 1])], 64, True)
    lay = FrameLayout(spec)
    h = frame_handle(lay)
    data = (rng.standard_normal((3, lay.num_data)) + 1j * rng.standard_normal((3, lay.num_data))) / np.sqrt(2)
    x = _modulate(h, lay, data)
    for b in range(3):
        assert rel_rms(x[b], ofdm.modulate(lay, data[b])) < TOL
    y = x + 0.1 * (rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape))
    grid = _demodulate(h, lay, y, lay.N)
    for b in range(3):
        assert rel_rms(grid[b], ofdm.demodulate(lay, y[b].astype(np.complex64).astype(np.complex128))) < TOL


@pytest.mark.parametrize("name,order,streams_", [("c1", 16, 1), ("c2", 64, 4)])
def test_modulate_bits_matches_oracle(name, order, streams_):
    spec = siso_frame(order) if name == "c1" else mimo_frame(order)
    lay = FrameLayout(spec)
    h = frame_handle(lay)
    seed, drop0, nd = 99, 11, 2
    out = torch.empty((nd, streams_, lay.samples_per_frame), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate_bits", h, seed, drop0, nd, streams_, _lib.ptr(out), stream())
    got = host(out)
    for d in range(nd):
        for s in range(streams_):
            bits = streams.data_bits(seed, drop0 + d, s, lay.bits_per_frame())
            ref = ofdm.modulate(lay, mapping.get_symbols(order, bits))
            assert rel_rms(got[d, s], ref) < TOL


def test_modulate_grid_and_pick():
    lay = FrameLayout(siso_frame())
    h = frame_handle(lay)
    rng = np.random.default_rng(3)
    data = rng.standard_normal(lay.num_data) + 1j * rng.standard_normal(lay.num_data)
    grid = ofdm.place(lay, data)
    g = cf(grid[None])
    out = torch.empty((1, lay.samples_per_frame), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate_grid", h, _lib.ptr(g), lay.N, 1, _lib.ptr(out), stream())
    assert rel_rms(host(out)[0], ofdm.modulate(lay, data)) < TOL
    picked = torch.empty((1, lay.num_data), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_pick", h, _lib.ptr(g), lay.N, 1, _lib.ptr(picked), stream())
    np.testing.assert_array_equal(host(picked)[0], ofdm.pick(lay, grid).astype(np.complex64))


def test_frame_validation():
    spec = siso_frame()
    spec.num_subcarriers = 200
    with pytest.raises(NotImplementedError):
        frame_handle(FrameLayout(spec))
