"""GPU: preambles and frame synchronization through the hpx_sync_* kernels against
the reference's outputs (tests/golden/sync.npz) and the float64 oracle."""

import numpy as np
import pytest
import torch

from hermespy_gb300 import (
    ElementType,
    GridElement,
    GridResource,
    OFDMCorrelationSynchronization,
    OFDMWaveform,
    PilotSection,
    SchmidlCoxPilotSection,
    SchmidlCoxSynchronization,
    Symbols,
    SymbolSection,
    Synchronization,
    _lib,
)
from oracle import sync
from tests.gpu_util import cf, host, rel_rms, stream

pytestmark = pytest.mark.gpu
N, CP, WORDS, ORDER = 128, 10, 4, 16
SPF = WORDS * (N + CP) + N


def _waveform(dc=True, pilot=None):
    res = [GridResource(1, prefix_ratio=CP / N, elements=[GridElement(ElementType.DATA, 100)])]
    return OFDMWaveform(res, [SymbolSection(WORDS, [0])], num_subcarriers=N, modulation_order=ORDER,
                        dc_suppression=dc, pilot_section=pilot)


@pytest.mark.parametrize("dc", [True, False])
def test_preambles_match_reference(golden, dc):
    g = golden("sync.npz")
    for cls, key in ((SchmidlCoxPilotSection, "schmidl_cox_pilot"), (PilotSection, "plain_pilot")):
        wf = _waveform(dc, cls())
        got = wf.pilot_section.generate(1)
        assert rel_rms(got, g[f"{key}_dc{int(dc)}"].reshape(-1)) < 1e-6
        assert wf.samples_per_frame() == SPF


def test_frame_with_preamble_round_trip():
    wf = _waveform(True, SchmidlCoxPilotSection())
    rng = np.random.default_rng(3)
    data = (rng.standard_normal(wf.num_data_symbols) + 1j * rng.standard_normal(wf.num_data_symbols)) / np.sqrt(2)
    placed = wf.place(Symbols(data[None, :, None]))
    frame = wf.modulate(placed)
    assert frame.shape == (SPF,)
    assert rel_rms(frame[:N], wf.pilot_section.generate(1)) < 1e-12
    back = wf.demodulate(frame).raw[0]
    assert rel_rms(back[:, :100], placed.raw[0][:, :100]) < 1e-5


@pytest.mark.parametrize("case", ["sc", "sc3"])
def test_schmidl_cox_matches_reference(golden, case):
    g = golden("sync.npz")
    wf = _waveform(True, SchmidlCoxPilotSection())
    sc = SchmidlCoxSynchronization()
    wf.synchronization = sc
    x = g[f"{case}_signal"]
    metric = host(sc.metric_device(x))
    ref = sync.schmidl_cox_metric(x.astype(np.complex64), N)
    assert metric.shape == ref.shape
    assert np.max(np.abs(metric - ref)) <= 1e-5 * np.max(ref)
    assert sc.synchronize(x) == g[f"{case}_indices"].tolist()


@pytest.mark.parametrize("case", ["corr", "corr3"])
def test_correlation_matches_reference(golden, case):
    g = golden("sync.npz")
    wf = _waveform(True, PilotSection())
    cs = OFDMCorrelationSynchronization()
    cs.waveform = wf
    x = g[f"{case}_signal"]
    prof = host(cs.correlation_device(x))
    ref = sync.correlation_profile(x.astype(np.complex64), wf.pilot_section.generate(1))
    assert np.max(np.abs(prof - ref)) <= 1e-5 * np.max(ref)
    assert cs.synchronize(x) == g[f"{case}_indices"].tolist()


def test_batched_metrics(golden):
    """Several signals per launch give each signal's own metric."""

    g = golden("sync.npz")
    a, b = g["sc_signal"], g["sc3_signal"][:, : g["sc_signal"].shape[1]]
    x = cf(np.stack([a, b]))
    n = x.shape[-1]
    out = torch.empty((2, n - N + 2), dtype=torch.float64, device="cuda")
    _lib.call("hpx_sync_schmidl_cox", _lib.ptr(x), 2, 2, n, N, _lib.ptr(out), stream())
    got = host(out)
    for i, sig in enumerate((a, b)):
        ref = sync.schmidl_cox_metric(sig.astype(np.complex64), N)
        assert np.max(np.abs(got[i] - ref)) <= 1e-5 * np.max(ref)
    pilot = cf(sync.preamble(ORDER, N, True, False))
    out = torch.empty((2, n + N - 1), dtype=torch.float64, device="cuda")
    _lib.call("hpx_sync_correlation", _lib.ptr(x), 2, 2, n, _lib.ptr(pilot), N, _lib.ptr(out), stream())
    got = host(out)
    for i, sig in enumerate((a, b)):
        ref = sync.correlation_profile(sig.astype(np.complex64), host(pilot))
        assert np.max(np.abs(got[i] - ref)) <= 1e-5 * np.max(ref)


def test_default_and_floating_synchronization():
    wf = _waveform(True, None)
    s = Synchronization(wf)
    assert s.synchronize(np.zeros((1, 2 * wf.samples_per_frame() + 5), np.complex64)) == [0, wf.samples_per_frame()]
    assert s.synchronize(np.zeros((1, 10), np.complex64)) == []
    with pytest.raises(RuntimeError):
        Synchronization().synchronize(np.zeros((1, 10), np.complex64))
    with pytest.raises(RuntimeError):
        OFDMCorrelationSynchronization(waveform=wf).synchronize(np.ones((1, 300), np.complex64))
    with pytest.raises(ValueError):
        OFDMCorrelationSynchronization(threshold=1.5)


@pytest.mark.parametrize("normalize", [False, True])
def test_device_peaks_match_find_peaks(normalize):
    """hpx_sync_peaks against scipy.signal.find_peaks on metrics with plateaus
    (runs of equal samples) and several frames. Distinct peaks have distinct
    heights: for exact ties numpy's argsort order is platform dependent."""

    from scipy.signal import find_peaks

    rng = np.random.default_rng(21)
    height = 0.9 if normalize else 0.75
    rows = []
    t = np.arange(3000)
    for _ in range(6):
        x = np.zeros(3000)
        for c in rng.choice(np.arange(200, 2800), 3, replace=False):
            x += np.maximum(0.0, 1.0 - np.abs(t - c) / 200.0) * rng.uniform(0.8, 1.0)
        x = x + 0.05 * rng.standard_normal(3000)
        for i in rng.choice(np.arange(1, 2990), 60, replace=False):  # plateaus of 2-5 equal samples
            x[i:i + rng.integers(2, 6)] = x[i]
        x[1500:1504] = x.max() * 1.01  # a flat top
        rows.append(x)
    metric = torch.from_numpy(np.stack(rows)).cuda()
    from hermespy_gb300.synchronization import _peaks

    for distance in (1, 7, 400):
        got = _peaks(metric, normalize, height, distance, -1, max_frames=512)
        for b, x in enumerate(rows):
            h = x / x.max() if normalize else x
            ref, _ = find_peaks(h, height=height if normalize else height * x.max(), distance=distance)
            assert got[b] == (ref - 1).tolist(), (b, distance)


def test_batched_synchronize_matches_single(golden):
    g = golden("sync.npz")
    wf = _waveform(True, SchmidlCoxPilotSection())
    sc = SchmidlCoxSynchronization(wf)
    a, b = g["sc_signal"], g["sc3_signal"][:, : g["sc_signal"].shape[1]]
    assert sc.synchronize_batch(np.stack([a, b])) == [sc.synchronize(a), sc.synchronize(b)]
