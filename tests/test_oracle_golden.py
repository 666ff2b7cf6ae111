"""The oracle against outputs recorded from the HermesPy reference (tests/golden/*.npz)."""

import os

import numpy as np
import pytest

from oracle import estimation, fading, mapping, ofdm, streams
from oracle.frame import FrameLayout
from oracle.link import LinkConfig, simulate_drop
from tests.configs import fading_case, mimo_channel, mimo_frame, siso_channel, siso_frame

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("order", [2, 4, 16, 64, 256])
def test_qam_golden(golden, order):
    g = golden("qam.npz")
    np.testing.assert_array_equal(mapping.get_symbols(order, g[f"bits_{order}"]), g[f"symbols_{order}"])
    np.testing.assert_array_equal(mapping.get_mapping(order), g[f"mapping_{order}"])
    np.testing.assert_array_equal(mapping.detect_bits(order, g[f"detect_in_{order}"]), g[f"detect_out_{order}"])


def _rx_distortion(x):
    return np.roll(x, 3) + 0.5 * x


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("dc", [True, False])
def test_ofdm_golden(golden, name, dc):
    g = golden("ofdm.npz")
    spec = siso_frame() if name == "c1" else mimo_frame()
    spec.dc_suppression = dc
    lay = FrameLayout(spec)
    assert lay.samples_per_frame == int(g[f"{name}_samples_per_frame"])
    mask = g[f"{name}_mask"]
    np.testing.assert_array_equal(lay.ref_mask, mask[0])
    np.testing.assert_array_equal(lay.data_mask, mask[1])
    placed = ofdm.place(lay, g[f"{name}_data"])
    kw = g[f"{name}_placed"].shape[0]
    np.testing.assert_allclose(placed[:kw], g[f"{name}_placed"], rtol=0, atol=1e-15)
    x = ofdm.modulate(lay, g[f"{name}_data"])
    sfx = "" if dc else "_nodc"
    ref_x = g[f"{name}_x{sfx}"]
    np.testing.assert_allclose(x[: ref_x.size], ref_x, rtol=0, atol=1e-13)
    # the fixture's receive grid was demodulated with DC suppression on in both cases
    # only for "_grid"; "_grid_nodc" used the same received samples with it off
    grid = ofdm.demodulate(lay, _rx_distortion(ofdm.modulate(FrameLayout(_with_dc(spec, True)), g[f"{name}_data"])))
    ref_g = g[f"{name}_grid{sfx}"]
    np.testing.assert_allclose(grid[: ref_g.shape[0]], ref_g, rtol=0, atol=1e-12)


def _with_dc(spec, dc):
    import copy

    s = copy.copy(spec)
    s.dc_suppression = dc
    return s


@pytest.mark.parametrize("name", ["c1", "c2", "fast", "los", "grp", "grp_fast"])
def test_fading_golden(golden, name):
    g = golden("fading.npz")
    cfg, nrx, ntx, T, fs = fading_case(name)
    smp = fading.realize(cfg, seed=1234, drop=3, num_rx=nrx, num_tx=ntx)
    y = fading.propagate(smp, g[f"{name}_x"], fs)
    ref = g[f"{name}_y"]
    assert y.shape == ref.shape
    np.testing.assert_allclose(y, ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    st = g[f"{name}_state"]
    Ts = st.shape[2]
    mine = fading.state(smp, Ts, fs, Ts)[:2, :2]
    np.testing.assert_allclose(mine, st, rtol=0, atol=1e-9 * max(np.abs(st).max(), 1))


def test_ls_golden(golden):
    g = golden("ls.npz")
    lay = FrameLayout(siso_frame())
    est = estimation.ls_estimate(lay, g["grid"])
    np.testing.assert_allclose(est, g["estimate"], rtol=0, atol=1e-12)
    # the sparse weight table reproduces the same estimate
    indptr, indices, weights = estimation.ls_weight_table(lay)
    refs = g["grid"][lay.ref_mask] / lay.pilot_symbols()
    flat = np.array([np.dot(weights[indptr[i]:indptr[i + 1]], refs[indices[indptr[i]:indptr[i + 1]]])
                     for i in range(lay.num_words * lay.N)])
    np.testing.assert_allclose(flat.reshape(lay.num_words, lay.N), g["estimate"], rtol=0, atol=1e-12)


def test_ideal_csi_golden(golden):
    g = golden("ideal.npz")
    cfg, _, _, _, fs = fading_case("c2")
    smp = fading.realize(cfg, seed=99, drop=7, num_rx=2, num_tx=2)
    lay = FrameLayout(mimo_frame())
    csi = estimation.ideal_csi(lay, smp, fs)[:, :, ::5, :]
    np.testing.assert_allclose(csi, g["csi"], rtol=0, atol=1e-10 * np.abs(g["csi"]).max())


@pytest.mark.parametrize("name", ["siso", "mimo"])
def test_zf_golden(golden, name):
    g = golden("zf.npz")
    x = estimation.zf_equalize(g[f"{name}_y"], g[f"{name}_h"])
    np.testing.assert_allclose(x, g[f"{name}_x"], rtol=1e-10, atol=1e-12)


def test_ber_golden(golden):
    g = golden("ber.npz")
    for i in range(3):
        a, b = g[f"tx_{i}"].astype(np.int8), g[f"rx_{i}"].astype(np.int8)
        n = max(a.size, b.size)
        err = np.abs(np.pad(a, (0, n - a.size)) - np.pad(b, (0, n - b.size)))
        np.testing.assert_array_equal(err, g[f"errors_{i}"])
        assert err.mean() == pytest.approx(float(g[f"ber_{i}"]))


@pytest.mark.parametrize("i", [0, 1, 2])
def test_siso_drop_golden(golden, i):
    """A whole SISO LS+ZF drop of the reference, fed the engine's draws, matches the oracle bit for bit."""

    g = golden("drops.npz")
    seed = int(g["seed"])
    cfg = LinkConfig(siso_frame(), siso_channel(), 15.36e6, 1, 1, "ls", "zf", "ebn0")
    out = simulate_drop(cfg, seed, int(g[f"c1_{i}_drop"]), float(g[f"c1_{i}_ebn0_db"]), keep=True)
    assert out["errors"] == int(g[f"c1_{i}_errors"])
    np.testing.assert_array_equal(np.packbits(out["rx_bits"].reshape(-1)), g[f"c1_{i}_rx_bits"])


def test_mimo_ideal_drop_golden(golden):
    """A 2x2 ideal-CSI + ZF drop of the reference (23 taps, 1024/600 frame, 16-QAM) matches the oracle."""

    g = golden("drops.npz")
    seed = int(g["seed"])
    ch = mimo_channel()
    ch.delays = np.rint(ch.delays * 30.72e6) / 30.72e6
    cfg = LinkConfig(mimo_frame(16), ch, 30.72e6, 2, 2, "ideal", "zf", "ebn0")
    out = simulate_drop(cfg, seed, 5, 15.0, keep=True)
    assert out["errors"] == int(g["c2_errors"])
    np.testing.assert_array_equal(np.packbits(out["rx_bits"].reshape(-1)), g["c2_rx_bits"])


def test_philox_known_answers():
    from oracle.philox import philox4x32

    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, expect in kat:
        out = philox4x32(np.array([ctr], dtype=np.uint32), key)[0]
        assert tuple(int(v) for v in out) == expect


def test_stream_statistics():
    bits = streams.data_bits(1, 2, 0, 200_000)
    assert abs(bits.mean() - 0.5) < 0.005
    n = streams.noise_normals(1, 2, 0, 100_000)
    assert abs(np.var(n.real) - 1) < 0.02 and abs(np.var(n.imag) - 1) < 0.02
    u = streams.fading_uniforms(1, 2, 100_000)
    assert 0 < u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.005


def test_ber_fixtures_reference_equals_oracle(golden):
    """The oracle's drops reproduce the reference's own SimulationScenario.drop() bit
    errors exactly on every fixture drop (11 000 SISO LS + ZF drops over Eb/N0 0..20 dB,
    256 4x4 ideal-CSI + ZF drops over SNR U[0, 30] dB), at the same noise powers."""

    z = golden("ber_siso.npz")
    assert z["ref_errors"].size == 11 * 1000
    assert np.array_equal(z["ref_errors"], z["oracle_errors"])
    assert np.array_equal(z["ref_noise_power"], z["oracle_noise_power"])
    m = golden("ber_mimo.npz")
    assert m["ref_zf_errors"].size == 256
    assert np.array_equal(m["ref_zf_errors"], m["oracle_zf_errors"])
    assert np.allclose(m["ref_noise_power"], m["oracle_noise_power"], rtol=1e-14, atol=0)
    # LMMSE detection beats ZF on the same drops (what the engine's LMMSE path adds)
    assert m["oracle_lmmse_errors"].astype(np.int64).sum() < m["oracle_zf_errors"].astype(np.int64).sum()


def test_ber_fixtures_match_their_inputs(golden):
    """Fixture bookkeeping: the shipped CNN weights are the ones the learned-path
    fixture was made with, and the uneven fixture's noise powers are the engine's."""

    import hashlib

    from hermespy_gb300.uneven import DropConfig

    p = golden("ber_pilot.npz")
    with open(os.path.join(ROOT, "hermespy_gb300", "weights", "cnn_4x4_1024.npz"), "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == str(p["weights_sha256"])
    n = 512 * 172800
    ber = {k: p[f"{k}_errors"].astype(np.int64).sum() / n for k in ("lmmse", "lmmse_robust", "ls", "learned")}
    assert ber["lmmse"] < ber["learned"] < ber["ls"]
    assert ber["lmmse"] < ber["lmmse_robust"] < ber["ls"]  # design statistics cost accuracy, still beat LS
    u = golden("uneven.npz")
    fields = ("num_rx", "num_tx", "fft_size", "num_words", "modulation_order", "num_taps", "tap_decay_db",
              "doppler_frequency", "snr_db")
    for i in range(u["errors"].size):
        d = DropConfig(*[u[f][i].item() for f in fields])
        assert abs(d.noise_power() / u["noise_power"][i] - 1) < 1e-12
