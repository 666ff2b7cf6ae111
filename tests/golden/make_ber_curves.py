"""Generate the BER-curve fixtures: per-drop bit-error counts of whole simulated
drops at the workloads' own shapes, for the GPU tests' 95 % interval checks.

Usage:  python tests/golden/make_ber_curves.py <path-to-hermespy-checkout> [fixture ...]
        (or with HERMESPY_REFERENCE=<path> set and the path argument omitted)

Fixtures (``tests/golden/``), each holding the seed, drop indices, noise levels
and per-drop error counts:

ber_siso.npz    SISO 256/200 comb-pilot frame, 16-QAM, 6-tap Rayleigh (100 Hz,
                15.36 MHz), LS + ZF, Eb/N0 0..20 dB in steps of 2, 1 000 drops per
                point: the reference's own ``SimulationScenario.drop()`` +
                ``BitErrorEvaluator`` fed the engine's Philox draws, and the oracle's
                drop on the same draws.
ber_mimo.npz    4x4 1024/600 data-only frame, 64-QAM, 23-tap Rayleigh (500 Hz, 30.72
                MHz), ideal CSI, SNR U[0, 30] dB, 256 drops: the reference's drop with
                ZF (its nearest equalizer) and the oracle's with ZF and with LMMSE.
ber_pilot.npz   4x4 1024/600 pilot-comb frame (words 0 and 7, comb 4), 64-QAM, same
                channel, SNR U[0, 30] dB, 512 drops, LMMSE detection after the four
                estimators of the learned-vs-LMMSE comparison: tap-domain LMMSE with the
                channel's statistics, the same with the robust design statistics
                (uniform profile over 64 delays, 1000 Hz, tap estimates regularized at a
                20 dB design SNR), per-stream LS, and LS refined
                by the shipped CNN weights (oracle drops; the reference has none of
                them). Records the weights' SHA-256.
uneven.npz      40 drops of the uneven-batch distribution (antennas {1,2,4,8}^2,
                FFT 128..2048, 4/7/14 words, 4..256-QAM, 1-23 taps), including the
                8x8 / 2048-point / 256-QAM and 1x1 / 128-point / 4-QAM corners, ideal
                CSI + LMMSE: oracle drops.

The reference runs in worker processes (spawned, one per core); every worker
imports the same checkout through ``refimport``.
"""

from __future__ import annotations

import hashlib
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (HERE, os.path.dirname(HERE), ROOT):  # the workloads' frames and channels: tests/configs.py
    if p not in sys.path:
        sys.path.insert(0, p)

SISO_SEED, SISO_LEVELS, SISO_DROPS = 20261204, np.arange(0.0, 20.1, 2.0), 1000
MIMO_SEED, MIMO_DROPS = 20261205, 256
PILOT_SEED, PILOT_DROPS = 20261203, 512
UNEVEN_SEED, UNEVEN_DROP0 = 7171, 100
WEIGHTS = os.path.join(ROOT, "hermespy_gb300", "weights", "cnn_4x4_1024.npz")
CHUNK = 50


def snr_draws(seed: int, n: int) -> np.ndarray:
    """Per-drop SNRs in dB, uniform over [0, 30]."""

    return np.random.default_rng(seed).uniform(0.0, 30.0, n)


def uneven_shapes():
    """Drop shapes of the uneven fixture: fixed corners first, then random draws."""

    from hermespy_gb300.uneven import DropConfig, random_drops

    fixed = [DropConfig(8, 8, 2048, 14, 256, 23, 1.5, 900.0, 25.0), DropConfig(1, 1, 128, 4, 4, 1, 3.0, 0.0, 5.0),
             DropConfig(8, 1, 2048, 7, 4, 12, 2.5, 10.0, -5.0), DropConfig(1, 8, 128, 14, 256, 23, 1.0, 1000.0, 30.0),
             DropConfig(2, 4, 512, 7, 16, 9, 2.0, 300.0, 12.0), DropConfig(4, 1, 256, 14, 64, 17, 1.0, 1000.0, 30.0),
             DropConfig(4, 4, 1024, 14, 64, 23, 0.4, 500.0, 20.0), DropConfig(8, 8, 256, 4, 64, 5, 3.0, 50.0, 18.0)]
    return fixed + random_drops(32, 2026)


# ------------------------------------------------------------------ workers
def _siso_cfg():
    from oracle.link import LinkConfig
    from configs import siso_channel, siso_frame

    fs = 15.36e6
    return LinkConfig(siso_frame(), siso_channel(fs), fs, 1, 1, "ls", "zf", "ebn0"), fs


def _mimo_cfg(equalizer):
    from oracle.link import LinkConfig
    from configs import mimo_channel, mimo_frame

    fs = 30.72e6
    return LinkConfig(mimo_frame(), mimo_channel(fs), fs, 4, 4, "ideal", equalizer, "snr"), fs


def work(task):
    """One chunk of drops: ('ref'|'oracle'|..., fixture, drops, levels)."""

    kind, name, drops, levels = task
    out = []
    if kind == "ref":
        import refdrops

        if name == "siso":
            cfg, fs = _siso_cfg()
            link = refdrops.RefLink(refdrops.c1_waveform(), cfg.channel, fs, 1, 1, SISO_SEED, "ls")
            for d, lv in zip(drops, levels):
                link.set_ebn0(lv)
                out.append((link.drop(int(d))[0], link.noise.last_power))
        else:
            cfg, fs = _mimo_cfg("zf")
            link = refdrops.RefLink(refdrops.c2_waveform(), cfg.channel, fs, 4, 4, MIMO_SEED, "ideal")
            for d, lv in zip(drops, levels):
                link.set_snr(lv)
                out.append((link.drop(int(d))[0], link.noise.last_power))
        return out
    from oracle.link import LinkConfig, simulate_drop

    if name == "siso":
        cfg, _ = _siso_cfg()
        seed = SISO_SEED
    elif name.startswith("mimo_"):
        cfg, _ = _mimo_cfg(name[5:])
        seed = MIMO_SEED
    elif name.startswith("pilot_"):
        from configs import mimo_channel, pilot_frame, robust_design

        est = name[6:]
        params = np.load(WEIGHTS)["params"] if est == "learned" else None
        design, ridge = robust_design(mimo_channel(30.72e6), 30.72e6) if est == "lmmse_robust" else (None, 0.0)
        cfg = LinkConfig(pilot_frame(), mimo_channel(30.72e6), 30.72e6, 4, 4, "lmmse" if design else est, "lmmse",
                         "snr", cnn_params=params, estimation_channel=design, estimation_ridge=ridge)
        seed = PILOT_SEED
    else:  # uneven
        from oracle.fading import FadingConfig
        from oracle.frame import DATA, FrameSpec, Resource, Section

        shapes = uneven_shapes()
        for d in drops:
            s = shapes[int(d) - UNEVEN_DROP0]
            N = s.fft_size
            C, cp = int(np.floor(0.586 * N)), N * 72 // 1024
            spec = FrameSpec(N, [Resource(1, cp / N, [(DATA, C)])], [Section(s.num_words, [0])], s.modulation_order,
                             True)
            k = np.arange(s.num_taps)
            ch = FadingConfig(k * 50e-9, s.power_profile(), np.zeros(s.num_taps), 20, s.doppler_frequency)
            cfg = LinkConfig(spec, ch, N * 30e3, s.num_tx, s.num_rx, "ideal", "lmmse", "snr")
            r = simulate_drop(cfg, UNEVEN_SEED, int(d), s.snr_db)
            out.append((r["errors"], r["noise_power"]))
        return out
    for d, lv in zip(drops, levels):
        r = simulate_drop(cfg, seed, int(d), float(lv))
        out.append((r["errors"], r["noise_power"]))
    return out


def run(pool, kind, name, drops, levels, chunk=CHUNK):
    tasks = [(kind, name, drops[i:i + chunk], levels[i:i + chunk]) for i in range(0, len(drops), chunk)]
    t0 = time.time()
    res = [r for part in pool.map(work, tasks, chunksize=1) for r in part]
    print(f"  {kind:6s} {name:14s} {len(drops):6d} drops in {time.time() - t0:6.1f} s", flush=True)
    return np.array([r[0] for r in res], dtype=np.int64), np.array([r[1] for r in res], dtype=np.float64)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({os.path.getsize(path) // 1024} KiB)", flush=True)


def make_siso(pool):
    drops = np.arange(SISO_LEVELS.size * SISO_DROPS)
    levels = np.repeat(SISO_LEVELS, SISO_DROPS)
    ref, ref_p = run(pool, "ref", "siso", drops, levels, 100)
    orc, orc_p = run(pool, "oracle", "siso", drops, levels, 250)
    save("ber_siso.npz", seed=SISO_SEED, levels_db=SISO_LEVELS, drops_per_level=SISO_DROPS, bits_per_drop=10800,
         ref_errors=ref.astype(np.uint32), oracle_errors=orc.astype(np.uint32), ref_noise_power=ref_p,
         oracle_noise_power=orc_p)


def make_mimo(pool):
    drops = np.arange(MIMO_DROPS)
    snr = snr_draws(MIMO_SEED, MIMO_DROPS)
    ref, ref_p = run(pool, "ref", "mimo", drops, snr, 4)
    zf, zf_p = run(pool, "oracle", "mimo_zf", drops, snr, 8)
    mm, _ = run(pool, "oracle", "mimo_lmmse", drops, snr, 8)
    save("ber_mimo.npz", seed=MIMO_SEED, snr_db=snr, bits_per_drop=201600, ref_zf_errors=ref.astype(np.uint32),
         oracle_zf_errors=zf.astype(np.uint32), oracle_lmmse_errors=mm.astype(np.uint32), ref_noise_power=ref_p,
         oracle_noise_power=zf_p)


def make_pilot(pool):
    drops = np.arange(PILOT_DROPS)
    snr = snr_draws(PILOT_SEED + 1, PILOT_DROPS)
    out = {}
    for est in ("lmmse", "lmmse_robust", "ls", "learned"):
        e, pw = run(pool, "oracle", "pilot_" + est, drops, snr, 8)
        out[f"{est}_errors"] = e.astype(np.uint32)
    with open(WEIGHTS, "rb") as f:
        sha = hashlib.sha256(f.read()).hexdigest()
    save("ber_pilot.npz", seed=PILOT_SEED, snr_db=snr, bits_per_drop=172800, noise_power=pw, weights_sha256=sha,
         **out)


def make_uneven(pool):
    shapes = uneven_shapes()
    drops = UNEVEN_DROP0 + np.arange(len(shapes))
    e, pw = run(pool, "oracle", "uneven", drops, np.zeros(len(shapes)), 1)
    fields = ("num_rx", "num_tx", "fft_size", "num_words", "modulation_order", "num_taps", "tap_decay_db",
              "doppler_frequency", "snr_db")
    cols = {f: np.array([getattr(s, f) for s in shapes]) for f in fields}
    save("uneven.npz", seed=UNEVEN_SEED, drop0=UNEVEN_DROP0, errors=e.astype(np.uint32), noise_power=pw, **cols)


MAKERS = {"siso": make_siso, "mimo": make_mimo, "pilot": make_pilot, "uneven": make_uneven}

if __name__ == "__main__":
    import refimport

    refimport.import_reference(sys.argv[1] if len(sys.argv) > 1 else None)  # checks the path, exports it
    only = set(sys.argv[2:])
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        for name, fn in MAKERS.items():
            if not only or name in only:
                fn(pool)
