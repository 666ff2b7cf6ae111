"""CPU: the GPU subclasses of the reference's own classes plug into the reference's
unchanged SimulationScenario (hermespy_gb300/plugin.py).

Needs a HermesPy checkout named by HERMESPY_REFERENCE (skipped otherwise). There is
no GPU here, so the checks are about wiring: the subclasses are the reference's
classes, the reference's scenario accepts them, its realization hands out the GPU
sample carrying the reference's own draw, and its drop() reaches the engine, which
refuses to run without a CUDA device (no CPU fallback). The array cores behind the
subclasses are checked against the reference's recorded outputs on the GPU
(tests/test_gpu_plugin.py)."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

REF = os.environ.get("HERMESPY_REFERENCE")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF or "", "hermespy")),
                                reason="set HERMESPY_REFERENCE to a HermesPy source checkout")


@pytest.fixture(scope="module")
def hp():
    import refimport

    return refimport.import_reference(REF)


def _scenario(hp, channel, waveform, fs, nant=1):
    from hermespy.modem import BitErrorEvaluator, SimplexLink
    from hermespy.simulation import SimulatedIdealAntenna, SimulatedUniformArray, SimulationScenario

    sc = SimulationScenario(seed=3)
    tx = sc.new_device(carrier_frequency=0.0, bandwidth=fs, oversampling_factor=1,
                       antennas=SimulatedUniformArray(SimulatedIdealAntenna, 0.01, [nant, 1, 1]))
    rx = sc.new_device(carrier_frequency=0.0, bandwidth=fs, oversampling_factor=1,
                       antennas=SimulatedUniformArray(SimulatedIdealAntenna, 0.01, [nant, 1, 1]))
    link = SimplexLink()
    tx.transmitters.add(link)
    rx.receivers.add(link)
    link.waveform = waveform
    sc.set_channel(tx, rx, channel)
    return sc, BitErrorEvaluator(link, link)


def test_plugins_are_the_reference_classes(hp):
    from hermespy.channel.fading.fading import (MultipathFadingChannel, MultipathFadingRealization,
                                                MultipathFadingSample)
    from hermespy.modem import OFDMWaveform

    from hermespy_gb300.plugin import make_plugins

    p = make_plugins(hp)
    assert issubclass(p.GpuMultipathFadingChannel, MultipathFadingChannel)
    assert issubclass(p.GpuMultipathFadingRealization, MultipathFadingRealization)
    assert issubclass(p.GpuMultipathFadingSample, MultipathFadingSample)
    assert issubclass(p.GpuOFDMWaveform, OFDMWaveform)
    # only the hot methods are overridden
    assert set(vars(p.GpuMultipathFadingSample)) >= {"_propagate", "state"}
    assert "_sample" in vars(p.GpuMultipathFadingRealization) and "_realize" in vars(p.GpuMultipathFadingChannel)


def test_reference_scenario_routes_the_drop_into_the_engine(hp):
    """The reference's SimulationScenario.drop() with the GPU channel: its realization
    samples the reference's own angles and phases into a GPU sample, and propagation
    runs through the engine (which needs a GPU; none is here)."""

    from hermespy.modem import ElementType, GridElement, GridResource, OFDMWaveform, SymbolSection
    from hermespy.simulation.simulated_device import SimulatedDevice  # noqa: F401 (import check)

    from hermespy_gb300.plugin import make_plugins, sample_parameters

    p = make_plugins(hp)
    fs = 15.36e6
    ch = p.GpuMultipathFadingChannel(np.arange(6) / fs, 10 ** (-0.3 * np.arange(6)), np.zeros(6), num_sinusoids=20,
                                     doppler_frequency=100.0)
    res = [GridResource(1, prefix_ratio=18 / 256, elements=[GridElement(ElementType.DATA, 200)])]
    wf = OFDMWaveform(grid_resources=res, grid_structure=[SymbolSection(14, [0])], num_subcarriers=256,
                      modulation_order=16)
    sc, _ = _scenario(hp, ch, wf, fs)
    sample = ch.realize().sample(sc.devices[0], sc.devices[1])
    assert isinstance(sample, p.GpuMultipathFadingSample)
    prm = sample_parameters(sample)  # the reference's own draw, as the engine's sample takes it
    assert np.array_equal(prm["nlos_angles"], sample.nlos_angles) and prm["spatial_response"].shape == (1, 1)
    assert prm["state"].sampling_rate == fs
    with pytest.raises(RuntimeError, match="CUDA device"):
        sc.drop()


def test_reference_scenario_modulates_through_the_engine(hp):
    """The reference's drop with the GPU OFDM waveform reaches the engine's modulator."""

    from hermespy.channel import MultipathFadingChannel
    from hermespy.modem import ElementType, GridElement, GridResource, SymbolSection

    from hermespy_gb300.plugin import engine_waveform, make_plugins

    p = make_plugins(hp)
    fs = 30.72e6
    res = [GridResource(1, prefix_ratio=72 / 1024, elements=[GridElement(ElementType.DATA, 600)])]
    wf = p.GpuOFDMWaveform(grid_resources=res, grid_structure=[SymbolSection(14, [0])], num_subcarriers=1024,
                           modulation_order=64)
    eng = engine_waveform(wf)  # the engine's frame of the same grid
    assert eng.samples_per_frame() == wf.samples_per_frame(fs, 1)
    assert eng.num_data_symbols == wf.num_data_symbols and eng.words_per_frame == wf.words_per_frame
    assert np.array_equal(eng.resource_mask[:, :, :600], wf.resource_mask[:, :, :600])
    ch = MultipathFadingChannel([0.0], [1.0], [0.0], doppler_frequency=10.0)
    sc, _ = _scenario(hp, ch, wf, fs)
    with pytest.raises(RuntimeError, match="CUDA device"):
        sc.drop()
