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
