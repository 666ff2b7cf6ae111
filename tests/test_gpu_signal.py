"""GPU: the block signal model (dense / sparse signals, offsets, DLPack exchange)
and its propagation and noise paths.

Follows the reference's signal_model.py rules (Create :866-911, offsets
:2490-2574, to_dense :1734-1741, energy / power :1717-1724) and the per-block
propagation of channel.py:370-379 with fading.py:371-406 (each block from time
zero of the realization, offset kept), checked against the float64 oracle."""

import numpy as np
import pytest
import torch

from hermespy_gb300 import (
    AWGN,
    DenseSignal,
    MultipathFadingChannel,
    Signal,
    SignalBlock,
    SparseSignal,
)
from oracle import fading, streams
from tests.gpu_util import rel_rms

pytestmark = pytest.mark.gpu
FS = 1e6


def _rand(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def test_create_dense_and_sparse():
    a, b = _rand((2, 50), 1), _rand((2, 30), 2)
    dense = Signal.Create(a, FS)
    assert isinstance(dense, DenseSignal) and dense.shape == (2, 50) and dense.num_blocks == 1
    np.testing.assert_allclose(dense.samples, a)
    one = Signal.Create([a], FS, offsets=[7])
    assert isinstance(one, DenseSignal) and one.delay == pytest.approx(7 / FS)
    sparse = Signal.Create([a, b], FS, offsets=[10, 100])
    assert isinstance(sparse, SparseSignal)
    assert sparse.block_offsets == [10, 100] and sparse.num_samples == 130 and sparse.num_blocks == 2
    d = sparse.to_dense().samples
    assert np.all(d[:, :10] == 0) and np.all(d[:, 60:100] == 0)
    np.testing.assert_allclose(d[:, 10:60], a)
    np.testing.assert_allclose(d[:, 100:130], b)
    follow = Signal.Create([a, b], FS)  # arrays without offsets follow each other
    assert follow.block_offsets == [0, 50]
    energies = [np.sum(np.abs(x.astype(np.complex128)) ** 2, axis=1) for x in (a, b)]
    assert sparse.energy == pytest.approx(np.sum(energies), rel=1e-5)
    np.testing.assert_allclose(sparse.power, np.mean([energies[0] / 50, energies[1] / 30], axis=0), rtol=1e-5)
    np.testing.assert_allclose(dense.energy, energies[0], rtol=1e-5)


def test_offset_validation():
    a = _rand((1, 20), 3)
    with pytest.raises(ValueError):
        Signal.Create([a, a], FS, offsets=[0, 10])  # overlap
    with pytest.raises(ValueError):
        Signal.Create([a, a], FS, offsets=[0])
    with pytest.raises(ValueError):
        Signal.Create([a, _rand((2, 5), 4)], FS)  # stream count
    with pytest.raises(ValueError):
        SignalBlock(a, -1)


def test_dlpack_zero_copy():
    t = torch.randn(3, 64, dtype=torch.complex64, device="cuda")
    s = Signal.from_dlpack(t, FS)
    assert s.device_samples.data_ptr() == t.data_ptr()
    back = torch.from_dlpack(s)
    assert back.data_ptr() == t.data_ptr()
    block = SignalBlock(t, 5)
    assert torch.from_dlpack(block).data_ptr() == t.data_ptr()


def test_superimpose():
    a, b = _rand((2, 40), 5), _rand((2, 25), 6)
    sa, sb = Signal.Create(a, FS, noise_power=0.1), Signal.Create([b], FS, offsets=[0])
    out = sa.superimpose(Signal.Create([b, b], FS, offsets=[0, 30]))
    ref = a.astype(np.complex128).copy()
    ref[:, :25] += b
    ext = np.zeros((2, 55), np.complex128)
    ext[:, :40] = ref
    ext[:, 30:55] += b
    np.testing.assert_allclose(out.samples, ext, rtol=1e-5, atol=1e-6)
    assert sa.superimpose(sb).noise_power == pytest.approx(0.1)


def test_sparse_propagation_matches_oracle():
    ch = MultipathFadingChannel([0.0, 3e-6, 7e-6], [1.0, 0.4, 0.1], [0.0, 0.0, 0.0], doppler_frequency=2e3,
                                seed=77)
    sample = ch.realize().sample(2, 2, sampling_rate=FS)
    a, b = _rand((2, 60), 7), _rand((2, 45), 8)
    sig = Signal.Create([a, b], FS, offsets=[5, 200])
    out = sample.propagate(sig)
    assert isinstance(out, SparseSignal) and out.block_offsets == [5, 200]
    cfg = fading.FadingConfig(ch.delays, ch.power_profile, ch.rice_factors, ch.num_sinusoids, ch.doppler_frequency,
                              ch.los_doppler_frequency, ch.gain)
    smp = fading.realize(cfg, ch.seed, 0, 2, 2)
    for blk, x in zip(out.blocks, (a, b)):
        ref = fading.propagate(smp, x.astype(np.complex128), FS)
        assert blk.shape == ref.shape
        assert rel_rms(blk.samples, ref) < 1e-5


def test_sparse_noise_follows_dense_stream():
    a, b = _rand((2, 40), 9), _rand((2, 20), 10)
    sig = Signal.Create([a, b], FS, offsets=[3, 90])
    noise = AWGN(seed=123)
    out = noise.realize(0.5).add_to(sig)
    n = streams.awgn(123, 0, 2, sig.num_samples, 0.5)
    np.testing.assert_allclose(out.blocks[0].samples, a + n[:, 3:43], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(out.blocks[1].samples, b + n[:, 90:110], rtol=1e-5, atol=1e-5)
    assert out.noise_power == 0.5 and sig.noise_power == 0.0
