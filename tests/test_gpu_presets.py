"""GPU: the channel presets (5G TDL A-E, COST 259 urban / rural / hilly) through the
engine's realization and propagation kernels, against the float64 oracle on the
same Philox draws, and the reference's expected-energy check
(tests/unit_tests/channel/test_fading.py:714-731, 799-816): 1 000 drops of a
unit-energy signal keep their energy within 0.1 of the expected scale."""

import numpy as np
import pytest
import torch

from hermespy_gb300 import TDL, CorrelationType, Cost259, Cost259Type, StandardAntennaCorrelation, TDLType, _lib
from oracle import fading, streams
from tests.gpu_util import cf, host, rel_rms, stream

pytestmark = pytest.mark.gpu
TOL = 1e-5
SEED = 0x7D1
FS = 10e6  # 5 MHz bandwidth, oversampling 2 (the reference's preset tests)

PRESETS = {
    **{f"tdl_{t.name}": (lambda t=t: TDL(t, 300e-9, doppler_frequency=100.0, seed=SEED)) for t in TDLType},
    **{f"cost259_{t.name}": (lambda t=t: Cost259(t, doppler_frequency=100.0, seed=SEED)) for t in Cost259Type},
}


def _oracle_config(ch, nrx, ntx):
    rx = tx = None
    if ch.antenna_correlation is not None:
        rx = ch.antenna_correlation.sample_covariance(nrx, "rx")
        tx = ch.antenna_correlation.sample_covariance(ntx, "tx")
    return fading.FadingConfig(ch.delays, ch.power_profile, ch.rice_factors, ch.num_sinusoids, ch.doppler_frequency,
                               ch.los_doppler_frequency, ch.gain, rx, tx)


@pytest.mark.parametrize("name", list(PRESETS))
def test_preset_propagate_matches_oracle(name):
    ch = PRESETS[name]()
    ch.antenna_correlation = StandardAntennaCorrelation(CorrelationType.MEDIUM_A)
    nrx, ntx, T, nd, drop0 = 2, 2, 1500, 2, 11
    h = ch.handle(nrx, ntx, FS)
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, ch.seed, drop0, nd, _lib.ptr(st), stream())
    rng = np.random.default_rng(5)
    x = ((rng.standard_normal((nd, ntx, T)) + 1j * rng.standard_normal((nd, ntx, T))) / np.sqrt(2)).astype(np.complex64)
    D = h.max_delay
    y = torch.empty((nd, nrx, T + D), dtype=torch.complex64, device="cuda")
    p = torch.tensor([0.2, 0.01], dtype=torch.float32, device="cuda")
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(cf(x)), T, _lib.ptr(y), _lib.ptr(p),
              ch.seed, drop0, stream())
    got = host(y)
    cfg = _oracle_config(ch, nrx, ntx)
    for d in range(nd):
        smp = fading.realize(cfg, ch.seed, drop0 + d, nrx, ntx)
        ref = fading.propagate(smp, x[d].astype(np.complex128), FS)
        ref = ref + streams.awgn(ch.seed, drop0 + d, nrx, T + D, float(p[d]))
        assert rel_rms(got[d], ref) < TOL, (name, rel_rms(got[d], ref))


@pytest.mark.parametrize("name", ["cost259_HILLY", "tdl_E"])
def test_preset_expected_energy(name):
    ch = (Cost259(Cost259Type.HILLY, doppler_frequency=10.0, seed=42) if name == "cost259_HILLY"
          else TDL(TDLType.E, doppler_frequency=10.0, seed=42))
    nd, T = 1000, 100
    h = ch.handle(1, 1, FS)
    st = h.new_state(nd)
    _lib.call("hpx_fading_realize", h.handle, ch.seed, 0, nd, _lib.ptr(st), stream())
    x = torch.full((nd, 1, T), 0.1, dtype=torch.complex64, device="cuda")  # unit energy
    y = torch.empty((nd, 1, T + h.max_delay), dtype=torch.complex64, device="cuda")
    _lib.call("hpx_fading_propagate", h.handle, _lib.ptr(st), nd, _lib.ptr(x), T, _lib.ptr(y), None, 0, 0, stream())
    energy = host((y.abs() ** 2).sum(dim=(1, 2)).double())
    scale = ch.gain * float(np.sum(ch.power_profile))
    assert abs(energy.mean() - scale ** 2) < 0.1, (energy.mean(), scale)
