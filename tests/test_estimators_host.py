"""CPU: per-stream LS tables and the tap-domain LMMSE estimator of the oracle."""

import numpy as np

from hermespy_gb300.estimation import ls_stream_tables
from oracle import estimation
from oracle.frame import FrameLayout
from oracle.link import LinkConfig, simulate_drop
from tests.configs import mimo_channel, pilot_frame


def test_stream_tables_match_oracle():
    """The host table builder (the reference's griddata calls per stream) equals the
    oracle's unit-probe tables of each stream, on the used columns."""

    lay = FrameLayout(pilot_frame())
    C = lay.num_used
    ip, ix, w = ls_stream_tables(lay.ref_mask[:, :C], 4, 4)
    rows = lay.num_words * C
    assert ip.size == 4 * rows + 1
    for s in range(4):
        oip, oix, ow = estimation.ls_weight_table(lay, s)
        for row in range(0, rows, 97):
            wd, c = divmod(row, C)
            orow = wd * lay.N + c
            a = slice(ip[s * rows + row], ip[s * rows + row + 1])
            b = slice(oip[orow], oip[orow + 1])
            da = dict(zip(ix[a].tolist(), w[a].tolist()))
            db = dict(zip(oix[b].tolist(), ow[b].tolist()))
            assert da.keys() == db.keys()
            assert all(abs(da[k] - db[k]) < 1e-6 for k in da)
            # every index is a reference element the stream transmits
            keep = lay.stream_ref_mask(s)[lay.ref_mask]
            assert all(keep[k] for k in da)


def test_stream_pilots_are_disjoint():
    lay = FrameLayout(pilot_frame())
    masks = [lay.stream_ref_mask(s) for s in range(4)]
    assert sum(int(m.sum()) for m in masks) == lay.num_refs
    for s in range(4):
        p = lay.stream_pilot_symbols(s)
        assert np.count_nonzero(p) == lay.num_refs // 4


def test_tap_lmmse_beats_ls():
    """LMMSE with the channel's statistics estimates the 4x4 channel several dB
    better than per-stream LS + interpolation at 20 dB SNR, and its BER is closer to
    ideal CSI."""

    lay = FrameLayout(pilot_frame())
    res = {}
    for est in ("ls", "lmmse", "ideal"):
        lc = LinkConfig(pilot_frame(), mimo_channel(), 30.72e6, 4, 4, est, "lmmse", "snr")
        res[est] = simulate_drop(lc, 5, 3, 20.0, keep=True)
    H = res["ideal"]["H"]
    n_ls = estimation.nmse_db(res["ls"]["H"], H, lay.data_mask)
    n_lm = estimation.nmse_db(res["lmmse"]["H"], H, lay.data_mask)
    assert n_lm < n_ls - 5.0
    assert res["ideal"]["errors"] <= res["lmmse"]["errors"] < res["ls"]["errors"]


def test_cnn_oracle_matches_torch_conv():
    """The oracle's CNN (im2col over (word, column), taps 3 dy + dx, BF16 rounding
    points) equals the same network written with torch's float64 conv2d."""

    import torch

    from oracle import cnn

    rng = np.random.default_rng(5)
    params = rng.normal(0, 0.05, cnn.LAYERS * 32 * 9 * 32 + cnn.LAYERS * 32).astype(np.float32)
    ls = rng.normal(size=(4, 4, 5, 37)) + 1j * rng.normal(size=(4, 4, 5, 37))
    out = cnn.refine(params, ls)
    w, b = cnn.split(params)
    z = ls.reshape(16, 5, 37)
    s = np.sqrt(np.mean(np.abs(z) ** 2))
    x = np.empty((32, 5, 37))
    x[0::2], x[1::2] = z.real, z.imag
    h = torch.from_numpy(cnn.bf16(x / s).astype(np.float64))[None]
    for layer in range(cnn.LAYERS):
        # [out][tap][in] with tap = 3 dy + dx -> conv2d's [out][in][dy][dx]
        wt = torch.from_numpy(w[layer].reshape(32, 3, 3, 32).transpose(0, 3, 1, 2).copy())
        h = torch.nn.functional.conv2d(h, wt, torch.from_numpy(b[layer]), padding=1)
        if layer < cnn.LAYERS - 1:
            h = torch.from_numpy(cnn.bf16(torch.relu(h).numpy()).astype(np.float64))
    d = h[0].numpy() * s
    ref = (z + d[0::2] + 1j * d[1::2]).reshape(ls.shape)
    assert np.max(np.abs(out - ref)) < 1e-9
    # the round trip through bf16 is round-to-nearest-even
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5e-3], dtype=np.float32)
    assert cnn.bf16(v).tolist() == [1.0, 1.0, 1.0 + 2 ** -6, np.float32(-0.0025024414)]


def test_robust_lmmse_oracle_needs_only_design_statistics():
    """The robust tap-domain LMMSE (uniform profile over 64 delays, 1000 Hz, tap
    estimates regularized at a 20 dB design SNR) comes within ~2 dB NMSE of the genie
    estimator and beats per-stream LS by more than 5 dB on the 4x4 pilot link; without
    the regularization its dense-delay LS diverges."""

    from tests.configs import robust_design

    fs = 30.72e6
    ch = mimo_channel(fs)
    lay = FrameLayout(pilot_frame())
    U = lay.num_used
    design, ridge = robust_design(ch, fs)
    nmse = {}
    for name, kw in {"genie": {}, "robust": dict(estimation_channel=design, estimation_ridge=ridge),
                     "unregularized": dict(estimation_channel=design)}.items():
        cfg = LinkConfig(pilot_frame(), ch, fs, 4, 4, "lmmse", "lmmse", "snr", **kw)
        r = simulate_drop(cfg, 5, 3, 15.0, keep=True)
        nmse[name] = estimation.nmse_db(r["H"][..., :U], estimation.ideal_csi(lay, r["sample"], fs)[..., :U])
    ls = simulate_drop(LinkConfig(pilot_frame(), ch, fs, 4, 4, "ls", "lmmse", "snr"), 5, 3, 15.0, keep=True)
    nmse["ls"] = estimation.nmse_db(ls["H"][..., :U], estimation.ideal_csi(lay, ls["sample"], fs)[..., :U])
    assert nmse["robust"] < nmse["genie"] + 2.5
    assert nmse["robust"] < nmse["ls"] - 5.0
    assert nmse["unregularized"] > 0.0
