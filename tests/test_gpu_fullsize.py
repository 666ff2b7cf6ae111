"""GPU: properties that hold at any size, checked at the headline workload's full size
(8 192 drops of the 4x4 pilot-comb link, 1024-point frames, 23 taps), where the
float64 oracle cannot follow drop by drop:

* propagation is linear in the transmit samples (noise off);
* OFDM demodulation inverts modulation on the used subcarriers;
* a drop depends on its index only: the same drops in one batch or in two halves give
  bit-identical realizations and equal error counts (what makes drop sharding across
  GPUs exact);
* realization and the whole link are deterministic for a given seed.
"""

import numpy as np
import pytest
import torch

import hermespy_gb300 as hg
from hermespy_gb300 import _lib
from hermespy_gb300.train_estimator import pilot_waveform, workload_channel

pytestmark = pytest.mark.gpu
B = 8192
SEED = 3141


def rel(a, b):
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


@pytest.fixture(scope="module")
def engine():
    return hg.LinkEngine(pilot_waveform(), workload_channel(), 4, 4, 30.72e6, "lmmse", "lmmse", "snr", max_drops=B,
                         seed=SEED)


def test_realization_depends_on_drop_index_only(engine):
    fh = engine._fading.handle
    # zeroed first: the per-drop records have alignment padding that realization does not write
    st_all, st_a, st_b = (engine._fading.new_state(n).zero_() for n in (B, B // 2, B // 2))
    _lib.call("hpx_fading_realize", fh, SEED, 0, B, _lib.ptr(st_all), _lib.stream_ptr())
    _lib.call("hpx_fading_realize", fh, SEED, 0, B // 2, _lib.ptr(st_a), _lib.stream_ptr())
    _lib.call("hpx_fading_realize", fh, SEED, B // 2, B // 2, _lib.ptr(st_b), _lib.stream_ptr())
    half = st_all.numel() // 2
    assert torch.equal(st_all.view(-1)[:half], st_a.view(-1)) and torch.equal(st_all.view(-1)[half:], st_b.view(-1))


def test_propagation_is_linear_at_full_size(engine):
    fh, T, D = engine._fading.handle, engine._T, engine._D
    st = engine._fading.new_state(B)
    _lib.call("hpx_fading_realize", fh, SEED, 0, B, _lib.ptr(st), _lib.stream_ptr())
    g = torch.Generator(device="cuda").manual_seed(7)
    x1 = torch.randn((B, 4, T), dtype=torch.complex64, device="cuda", generator=g)
    x2 = torch.randn((B, 4, T), dtype=torch.complex64, device="cuda", generator=g)

    def prop(x):
        y = torch.empty((B, 4, T + D), dtype=torch.complex64, device="cuda")
        _lib.call("hpx_fading_propagate", fh, _lib.ptr(st), B, _lib.ptr(x), T, _lib.ptr(y), None, SEED, 0,
                  _lib.stream_ptr())
        return y

    y1, y2 = prop(x1), prop(x2)
    y3 = prop((x1 + 2j * x2).contiguous())
    assert rel(y3, y1 + 2j * y2) < 1e-5
    del x1, x2, y1, y2, y3


def test_ofdm_round_trip_at_full_size(engine):
    wf = engine.waveform
    fd, C = engine._frame, engine.num_columns
    n = B * 4
    g = torch.Generator(device="cuda").manual_seed(11)
    data = torch.randn((n, wf.num_data_symbols), dtype=torch.complex64, device="cuda", generator=g)
    x = torch.empty((n, wf.samples_per_frame()), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_modulate", fd, _lib.ptr(data), n, _lib.ptr(x), _lib.stream_ptr())
    grid = torch.empty((n, wf.words_per_frame, C), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_ofdm_demodulate", fd, _lib.ptr(x), x.shape[1], n, C, _lib.ptr(grid), _lib.stream_ptr())
    picked = torch.empty_like(data)
    _lib.call("hpx_ofdm_pick", fd, _lib.ptr(grid), C, n, _lib.ptr(picked), _lib.stream_ptr())
    assert rel(picked, data) < 1e-5


def test_link_counts_depend_on_drop_index_only(engine):
    p = torch.from_numpy(engine.noise_power(np.random.default_rng(5).uniform(0, 30, B)).astype(np.float32)).cuda()
    whole = engine.counts(engine.run(0, p))
    first = engine.counts(engine.run(0, p[: B // 2].contiguous()))
    second = engine.counts(engine.run(B // 2, p[B // 2:].contiguous()))
    assert np.array_equal(whole, np.concatenate([first, second]))
    assert np.array_equal(whole, engine.counts(engine.run(0, p)))  # deterministic
    assert 0.15 < whole.sum() / (B * engine.bits_per_drop) < 0.2
