"""GPU: the uneven batch (one persistent launch over drops of different shapes)
against the homogeneous engine drop by drop (equal counts), and its CUDA-graph
replay. The comparison with the oracle's drops is in test_gpu_ber_curves.py."""

import numpy as np
import pytest
import torch

import hermespy_gb300 as hg
from hermespy_gb300.uneven import DropConfig, UnevenBatch, random_drops

pytestmark = pytest.mark.gpu
SEED = 7171
SCS, TAP = 30e3, 50e-9


def _homogeneous_errors(d: DropConfig, drop: int, noise_power: float, seed: int = SEED) -> int:
    N = d.fft_size
    C, cp = int(np.floor(0.586 * N)), N * 72 // 1024
    wf = hg.OFDMWaveform([hg.GridResource(1, prefix_ratio=cp / N, elements=[hg.GridElement(hg.ElementType.DATA, C)])],
                         [hg.SymbolSection(d.num_words, [0])], num_subcarriers=N, modulation_order=d.modulation_order)
    k = np.arange(d.num_taps)
    ch = hg.MultipathFadingChannel(list(k * TAP), list(d.power_profile()), [0.0] * d.num_taps, num_sinusoids=20,
                                   doppler_frequency=d.doppler_frequency)
    eng = hg.LinkEngine(wf, ch, d.num_tx, d.num_rx, N * SCS, "ideal", "lmmse", "snr", max_drops=1, seed=seed)
    p = torch.tensor([noise_power], dtype=torch.float32, device="cuda")
    return int(eng.run(drop, p).cpu()[0])


def assert_same_counts(errs, refs):
    """The persistent kernel runs the homogeneous kernels' arithmetic (same FMA order
    in the source, noise streams and solver), but the two are separate kernels whose
    FMA contraction the compiler chooses per kernel: a near-singular system (one
    receive antenna, eight streams, 256-QAM) can flip a single bit. Counts must be equal
    for most drops and within max(2, count / 5000) for every drop."""

    errs, refs = np.asarray(errs, dtype=np.int64), np.asarray(refs, dtype=np.int64)
    assert np.all(np.abs(errs - refs) <= np.maximum(2, refs // 5000)), (errs.tolist(), refs.tolist())
    assert np.mean(errs == refs) >= 0.75, (errs.tolist(), refs.tolist())


def _mixed():
    fixed = [DropConfig(8, 8, 2048, 14, 256, 23, 1.5, 900.0, 25.0), DropConfig(1, 1, 128, 4, 4, 1, 3.0, 0.0, 5.0),
             DropConfig(2, 4, 512, 7, 16, 9, 2.0, 300.0, 12.0), DropConfig(4, 1, 256, 14, 64, 17, 1.0, 1000.0, 30.0),
             DropConfig(4, 4, 1024, 14, 64, 23, 0.4, 500.0, 20.0)]
    return fixed + random_drops(7, 11)


def test_uneven_drops_equal_homogeneous_engine():
    drops = _mixed()
    batch = UnevenBatch(drops, SCS, TAP, 20, max_slots=64)
    errs = batch.run(SEED, 100).cpu().numpy()
    p = batch.noise_power.cpu().numpy()
    assert_same_counts(errs, [_homogeneous_errors(d, 100 + i, float(p[i])) for i, d in enumerate(drops)])
    # the 8x8 drop at 25 dB and the 1x1 drop at 5 dB are neither error-free nor all wrong
    assert 0 < errs[0] < batch.bits[0] // 2 and 0 < errs[1] < batch.bits[1] // 2


def test_uneven_tune_graph_and_bits():
    drops = random_drops(40, 5)
    batch = UnevenBatch(drops, SCS, TAP, 20, max_slots=152)
    for i, d in enumerate(drops):
        C = int(np.floor(0.586 * d.fft_size))
        assert batch.bits[i] == d.num_words * C * int(np.log2(d.modulation_order)) * d.num_tx
    first = batch.run(SEED, 0).clone()
    best = batch.tune(SEED, 0, repeats=1)
    assert best["threads"] in (128, 256) and best["ms"] > 0
    assert torch.equal(batch.run(SEED, 0), first)  # the launch shape does not change results
    batch.capture(SEED, 0)
    batch.errors.zero_()
    batch.replay()
    assert torch.equal(batch.errors, first)
    assert batch.config()["variant"] in (0, 1, 2)
    with pytest.raises(ValueError):
        batch.set_config(96, 1)


def test_three_cta_variant_for_small_antenna_batches():
    """Batches whose drops have at most 4 antennas a side also run the 80-register
    instantiation at three CTAs of 256 threads per SM, with the same counts; a batch
    with 8-antenna drops cannot select it."""

    small = [DropConfig(4, 4, 1024, 14, 64, 23, 0.4, 500.0, 20.0), DropConfig(2, 4, 512, 7, 16, 9, 2.0, 300.0, 12.0),
             DropConfig(4, 1, 256, 14, 64, 17, 1.0, 1000.0, 30.0), DropConfig(1, 1, 128, 4, 4, 1, 3.0, 0.0, 5.0)] * 3
    batch = UnevenBatch(small, SCS, TAP, 20, max_slots=4 * 152)
    batch.set_config(256, 2, 1)
    ref = batch.run(SEED, 0).clone()
    assert batch.fit(256, 2) >= 3
    batch.set_config(256, 3, 2)
    assert torch.equal(batch.run(SEED, 0), ref)
    big = UnevenBatch([DropConfig(8, 8, 1024, 14, 64, 23, 0.4, 500.0, 20.0)], SCS, TAP, 20, max_slots=152)
    assert big.fit(256, 2) == 0
    with pytest.raises(NotImplementedError):
        big.set_config(256, 1, 2)
