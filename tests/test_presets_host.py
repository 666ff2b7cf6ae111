"""CPU: channel presets (TDL A-E, COST 259, Exponential) and the 3GPP antenna
correlations against the reference's own values (tests/golden/presets.npz), and
the constructors' validation errors (tdl.py:91-96, 286-300; cost259.py:235;
correlation.py:112-116)."""

import numpy as np
import pytest

from hermespy_gb300 import (
    TDL,
    CorrelationType,
    Cost259,
    Cost259Type,
    Exponential,
    StandardAntennaCorrelation,
    TDLType,
)


@pytest.mark.parametrize("model_type", list(TDLType))
@pytest.mark.parametrize("tag,rms", [("0", 0.0), ("300ns", 300e-9)])
def test_tdl_matches_reference(golden, model_type, tag, rms):
    g = golden("presets.npz")
    ch = TDL(model_type, rms, doppler_frequency=10.0, seed=1)
    key = f"tdl_{model_type.name}_{tag}"
    np.testing.assert_allclose(ch.delays, g[key + "_delays"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(ch.power_profile, g[key + "_power"], rtol=1e-14)
    np.testing.assert_array_equal(ch.rice_factors, g[key + "_rice"])
    assert ch.los_doppler_frequency == float(g[key + "_los_doppler"])
    assert ch.model_type is model_type and ch.rms_delay == rms


@pytest.mark.parametrize("model_type", list(Cost259Type))
def test_cost259_matches_reference(golden, model_type):
    g = golden("presets.npz")
    ch = Cost259(model_type, doppler_frequency=10.0, seed=1)
    key = f"cost259_{model_type.name}"
    np.testing.assert_allclose(ch.delays, g[key + "_delays"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(ch.power_profile, g[key + "_power"], rtol=1e-14)
    np.testing.assert_array_equal(ch.rice_factors, g[key + "_rice"])
    assert ch.los_doppler_frequency == float(g[key + "_los_doppler"])
    assert ch.model_type is model_type


@pytest.mark.parametrize("interval,rms", [(1e-7, 3e-7), (5e-8, 1e-6)])
def test_exponential_matches_reference(golden, interval, rms):
    g = golden("presets.npz")
    ch = Exponential(interval, rms, seed=1)
    key = f"exponential_{interval:g}_{rms:g}"
    np.testing.assert_allclose(ch.delays, g[key + "_delays"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(ch.power_profile, g[key + "_power"], rtol=1e-14)


@pytest.mark.parametrize("corr", list(CorrelationType))
@pytest.mark.parametrize("n", [1, 2, 4])
def test_standard_correlation_matches_reference(golden, corr, n):
    g = golden("presets.npz")
    model = StandardAntennaCorrelation(corr)
    for mode in ("rx", "tx"):
        cov = model.sample_covariance(n, mode)
        np.testing.assert_allclose(cov, g[f"corr_{corr.name}_{n}_{mode}"], rtol=1e-15, atol=0)
        assert np.allclose(cov, cov.T.conj())


def test_preset_validation():
    with pytest.raises(ValueError):
        TDL(model_type=100000)
    with pytest.raises(ValueError):
        TDL(rms_delay=-1.0)
    for t in (TDLType.D, TDLType.E):
        with pytest.raises(ValueError):
            TDL(model_type=t, los_doppler_frequency=0.0)
    with pytest.raises(ValueError):
        Cost259(100000)
    with pytest.raises(RuntimeError):
        StandardAntennaCorrelation(CorrelationType.LOW).sample_covariance(5)
    assert StandardAntennaCorrelation("HIGH").correlation is CorrelationType.HIGH


def test_preset_gains():
    """Line-of-sight taps: TDL-E's first tap is Rician (K = 22), COST 259 hilly's is
    pure line of sight (K = inf: LOS gain 1, scattered gain 0)."""

    los, nlos = TDL(TDLType.E, 100e-9).gains()
    assert los[0] == pytest.approx(np.sqrt(22 / 23)) and nlos[0] == pytest.approx(np.sqrt(1 / (23 * 20)))
    los, nlos = Cost259(Cost259Type.HILLY).gains()
    assert los[0] == 1.0 and nlos[0] == 0.0 and np.all(los[1:] == 0.0)
