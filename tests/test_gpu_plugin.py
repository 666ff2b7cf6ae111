"""GPU: the array cores behind the GPU subclasses of the reference's own classes
(hermespy_gb300/plugin.py) reproduce the reference's recorded outputs.

The subclasses themselves need an importable HermesPy (tests/test_plugin_host.py
checks their wiring into the reference's SimulationScenario where it is); the cores
take any object with the reference's public properties, so here they get stand-ins
carrying the values the fixtures were recorded with: the reference's
MultipathFadingSample._propagate / state outputs (fading.npz) and OFDMWaveform
modulate / demodulate outputs (ofdm.npz)."""

from types import SimpleNamespace as NS

import numpy as np
import pytest

from hermespy_gb300 import plugin
from oracle import fading, ofdm
from oracle.frame import FrameLayout
from tests.configs import FADING_CASES, fading_case, siso_frame
from tests.gpu_util import rel_rms

pytestmark = pytest.mark.gpu
TOL = 1e-5


def reference_sample(name):
    """An object with the public properties of the reference's MultipathFadingSample
    (fading.py:153-299) holding the realization the fixture was recorded with."""

    cfg, nrx, ntx, T, fs = fading_case(name)
    smp = fading.realize(cfg, seed=1234, drop=3, num_rx=nrx, num_tx=ntx)
    los, nlos = cfg.gains()
    return NS(power_profile=cfg.power_profile, delay_profile=cfg.delays, los_angles=smp.los_angles,
              nlos_angles=smp.nlos_angles, los_phases=smp.los_phases, nlos_phases=smp.nlos_phases, los_gains=los,
              nlos_gains=nlos, los_doppler=cfg.los_doppler, nlos_doppler=cfg.doppler_frequency,
              spatial_response=smp.spatial, gain=cfg.gain, bandwidth=fs, num_transmit_antennas=ntx,
              num_receive_antennas=nrx)


@pytest.mark.parametrize("name", list(FADING_CASES))
def test_plugin_propagate_and_state_match_reference(golden, name):
    g = golden("fading.npz")
    s = reference_sample(name)
    y = plugin.propagate_block(s, g[f"{name}_x"])
    assert y.dtype == np.complex128 and y.shape == g[f"{name}_y"].shape
    assert rel_rms(y, g[f"{name}_y"]) < TOL
    st = g[f"{name}_state"]
    csi = plugin.channel_state(s, st.shape[2], st.shape[2])[:2, :2]
    assert rel_rms(csi, st) < TOL


def reference_waveform(dc):
    """An object with the reference OFDMWaveform's grid attributes for the SISO
    256/200 comb-pilot frame (waveform.py:102-175, 463-520, ofdm.py:33-95)."""

    spec = siso_frame()
    kinds = {0: "REFERENCE", 1: "DATA", 2: "NULL"}
    res = [NS(repetitions=r.repetitions, prefix_ratio=r.prefix_ratio, prefix_type=NS(name=r.prefix_type),
              elements=[NS(type=NS(name=kinds[k]), repetitions=n) for k, n in r.elements]) for r in spec.resources]
    sec = [NS(num_repetitions=s.num_repetitions, pattern=list(s.pattern), sample_offset=0) for s in spec.sections]
    return NS(grid_resources=res, grid_structure=sec, num_subcarriers=spec.num_subcarriers,
              modulation_order=spec.modulation_order, dc_suppression=dc)


@pytest.mark.parametrize("dc", [True, False])
def test_plugin_modulate_demodulate_match_reference(golden, dc):
    g = golden("ofdm.npz")
    eng = plugin.engine_waveform(reference_waveform(dc))
    x = plugin.modulate_grid(eng, g["c1_placed"])
    ref_x = g["c1_x" if dc else "c1_x_nodc"]
    assert x.dtype == np.complex128 and rel_rms(x[: ref_x.size], ref_x) < TOL
    lay = FrameLayout(siso_frame())
    tx = ofdm.modulate(lay, g["c1_data"])
    grid = plugin.demodulate_frame(eng, np.roll(tx, 3) + 0.5 * tx)
    ref_g = g["c1_grid" if dc else "c1_grid_nodc"]
    assert rel_rms(grid[: ref_g.shape[0]], ref_g) < TOL
