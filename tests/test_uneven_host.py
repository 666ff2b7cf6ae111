"""CPU: the uneven workload's drop distribution and noise levels."""

import numpy as np

from hermespy_gb300.uneven import DropConfig, random_drops


def test_random_drops_cover_the_distribution():
    drops = random_drops(4000, 3)
    assert {d.num_rx for d in drops} == {1, 2, 4, 8} and {d.num_tx for d in drops} == {1, 2, 4, 8}
    assert {d.fft_size for d in drops} == {128, 256, 512, 1024, 2048}
    assert {d.num_words for d in drops} == {4, 7, 14} and {d.modulation_order for d in drops} == {4, 16, 64, 256}
    taps = np.array([d.num_taps for d in drops])
    assert taps.min() == 1 and taps.max() == 23
    dop = np.array([d.doppler_frequency for d in drops])
    snr = np.array([d.snr_db for d in drops])
    assert 0 <= dop.min() and dop.max() <= 1000 and -5 <= snr.min() and snr.max() <= 30
    # deterministic in the seed
    assert random_drops(5, 9) == random_drops(5, 9)


def test_noise_power_is_snr_relative_to_channel_energy():
    d = DropConfig(2, 2, 256, 7, 16, 3, 3.0, 100.0, 10.0)
    energy = 1 + 10 ** -0.3 + 10 ** -0.6
    assert abs(d.noise_power() - energy / 10.0) < 1e-12
