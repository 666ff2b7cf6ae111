"""Train and validate the learned channel estimator of the 4x4 pilot-comb link.

    python -m hermespy_gb300.train_estimator --pairs 2000000 --out hermespy_gb300/weights/cnn_4x4_1024.npz

Frame: 1024-point OFDM, 600 used subcarriers, CP 72, 14 words, 64-QAM, reference
elements on all used subcarriers of words 0 and 7 with pilot comb 4 (stream s
sends on columns c % 4 == s). Training channels: 4-23 taps spaced 50 ns with an
exponential power-delay profile (0.2-3 dB per tap), Doppler U[0, 1000] Hz, SNR
U[-5, 30] dB, 30.72 MHz sampling. Validation reports the NMSE of per-stream LS,
tap-domain LMMSE and the network over held-out channels and over the 4x4
workload channel (23 taps, -0.4 dB per tap, 500 Hz).
"""

from __future__ import annotations

import argparse
import json
import os

import numpy as np
import torch

from . import _lib
from .learned import CnnChannelEstimator, PairSource, csi_error, nmse_db, random_channels, train

FS = 30.72e6


def pilot_waveform():
    from .waveform import ElementType, GridElement, GridResource, OFDMWaveform, SymbolSection

    data = GridResource(1, prefix_ratio=72 / 1024, elements=[GridElement(ElementType.DATA, 600)])
    refs = GridResource(1, prefix_ratio=72 / 1024, elements=[GridElement(ElementType.REFERENCE, 600)])
    return OFDMWaveform([data, refs], [SymbolSection(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])],
                        num_subcarriers=1024, modulation_order=64, pilot_comb=4)


def workload_channel():
    from .channel import MultipathFadingChannel

    k = np.arange(23)
    return MultipathFadingChannel(list(k * 50e-9), list(10 ** (-0.04 * k)), [0.0] * 23, doppler_frequency=500.0)


def evaluate(model: CnnChannelEstimator | None, engines, snr_db, drops: int, seed: int) -> dict:
    """NMSE (dB) of LS, LMMSE and the network over `drops` drops of every engine."""

    rng = np.random.default_rng(seed)
    sums = {k: [0.0, 0.0] for k in ("ls", "lmmse", "learned")}
    for eng_ls, eng_lm in engines:
        n = eng_ls.max_drops
        for d0 in range(0, drops, n):
            snr = rng.uniform(snr_db[0], snr_db[1], n)
            p = torch.from_numpy(eng_ls.noise_power(snr).astype(np.float32)).cuda()
            eng_ls.receive(d0, p)
            truth = torch.empty_like(eng_ls._csi)
            _lib.call("hpx_fading_ideal_csi", eng_ls._fading.handle, _lib.ptr(eng_ls._state), n, eng_ls._frame,
                      eng_ls.num_columns, _lib.ptr(truth), _lib.stream_ptr())
            ls = eng_ls.estimate(n, p, estimator="ls")
            e, w = csi_error(eng_ls._frame, ls, truth)
            sums["ls"][0] += e
            sums["ls"][1] += w
            if model is not None:
                est = model.refine(ls.clone())
                e, w = csi_error(eng_ls._frame, est, truth)
                sums["learned"][0] += e
                sums["learned"][1] += w
            # the LMMSE engine sees the same received grid
            eng_lm._grid.copy_(eng_ls._grid)
            lm = eng_lm.estimate(n, p, estimator="lmmse")
            e, w = csi_error(eng_ls._frame, lm, truth)
            sums["lmmse"][0] += e
            sums["lmmse"][1] += w
    return {k: nmse_db(*v) for k, v in sums.items() if v[1] > 0}


def engines_for(waveform, channels, batch: int, seed: int):
    from .engine import LinkEngine

    out = []
    for i, ch in enumerate(channels):
        a = LinkEngine(waveform, ch, 4, 4, FS, "ls", "lmmse", "snr", max_drops=batch, seed=seed + i)
        b = LinkEngine(waveform, ch, 4, 4, FS, "lmmse", "lmmse", "snr", max_drops=batch, seed=seed + i)
        out.append((a, b))
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=2_000_000, help="training pairs (drops)")
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--channels", type=int, default=64, help="random channel draws in the training pool")
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--val-drops", type=int, default=256)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "weights", "cnn_4x4_1024.npz"))
    ap.add_argument("--init", default=None, help="start from these parameters")
    args = ap.parse_args(argv)

    from .channel import MultipathFadingChannel

    wf = pilot_waveform()
    W, C = wf.words_per_frame, wf._layout()["num_columns"]
    params = np.load(args.init)["params"] if args.init else None
    model = CnnChannelEstimator(W, C, max_batch=max(args.batch, 64), params=params, seed=args.seed)
    source = PairSource(wf, FS, random_channels(args.channels, args.seed), args.batch, args.seed)
    info = train(model, source, args.pairs, lr=args.lr)

    held = []
    for cd in random_channels(8, args.seed + 999):
        d, p = cd.profile(50e-9)
        held.append(MultipathFadingChannel(list(d), list(p), [0.0] * cd.num_taps, doppler_frequency=cd.doppler))
    val_random = evaluate(model, engines_for(wf, held, 64, 10_000), (-5.0, 30.0), args.val_drops, 1)
    val_work = evaluate(model, engines_for(wf, [workload_channel()], 64, 20_000), (0.0, 30.0), args.val_drops, 2)
    report = {"train": {k: v for k, v in info.items() if k != "history"}, "history": info["history"],
              "nmse_db_random_channels": val_random, "nmse_db_workload_channel": val_work}
    print(json.dumps(report))
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    model.save(args.out, report=json.dumps(report))


if __name__ == "__main__":
    main()
