"""Generate the golden fixtures of the HermesPy reference (run where its source is available).

Usage:  python tests/golden/make_golden.py <path-to-hermespy-checkout> [fixture ...]
        (or with HERMESPY_REFERENCE=<path> set and the path argument omitted)

With fixture names (``qam``, ``ofdm``, ``fading``, ``ls``, ``ideal``, ``zf``, ``ber``,
``drops``, ``presets``) only those are regenerated.

Every fixture is an output of the reference's own code, fed inputs that the
oracle can reproduce (seeded numpy draws or the engine's Philox streams):

qam.npz      ``PskQamMapping.get_symbols`` / ``get_mapping`` / ``detect_bits`` for
             BPSK, QPSK, 16-, 64-, 256-QAM, including decision-boundary ties.
ofdm.npz     ``OFDMWaveform.place`` + ``modulate`` and ``demodulate`` for the SISO
             256/200 comb-pilot frame and the 1024/600 data-only frame.
fading.npz   ``MultipathFadingSample.propagate`` and ``.state`` for samples built
             from explicit angles/phases (low Doppler, high Doppler, 2x3 MIMO, LOS).
ls.npz       ``OrthogonalLeastSquaresChannelEstimation.estimate_channel`` on the
             comb-pilot frame.
ideal.npz    ``OFDMIdealChannelEstimation.estimate_channel`` for a 2x2 sample.
zf.npz       ``ZeroForcingChannelEqualization.equalize_channel``, SISO and 4x4.
ber.npz      ``BitErrorEvaluator.evaluate`` including unequal-length padding.
sync.npz     ``PilotSection`` / ``SchmidlCoxPilotSection`` preambles (128 subcarriers,
             with and without DC suppression) and the frame starts that
             ``SchmidlCoxSynchronization`` and ``OFDMCorrelationSynchronization``
             find in noisy two-stream signals holding two or three frames.
ldpc.npz     Edges of the parity-check matrix the reference ships for its 5G NR OFDM
             modem (``modem/resources/ofdm_ldpc.alist``, read as data; the aff3ct
             decoder that the reference wraps is not part of the checkout).
presets.npz  Tap delays, power profiles, Rice factors and line-of-sight Doppler of
             the ``TDL`` (A-E), ``Cost259`` (urban, rural, hilly) and
             ``Exponential`` presets, and ``StandardAntennaCorrelation``
             covariances for 1, 2 and 4 antennas per correlation type and side.
drops.npz    Whole ``SimulationScenario.drop()`` runs (SISO LS+ZF at three Eb/N0,
             2x2 ideal CSI + ZF) with bits, fading draws and noise injected from
             the engine's Philox streams.
"""

from __future__ import annotations

import os
import sys
from types import SimpleNamespace
from unittest.mock import patch

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import refimport  # noqa: E402

REF = refimport.reference_path(sys.argv[1] if len(sys.argv) > 1 else None)
ONLY = set(sys.argv[2:])
refimport.import_reference(REF)

from scipy.stats import norm  # noqa: E402

from hermespy.channel import MultipathFadingChannel  # noqa: E402
from hermespy.channel.channel import LinkState  # noqa: E402
from hermespy.channel.consistent import StaticConsistentRealization  # noqa: E402
from hermespy.channel.fading.fading import MultipathFadingSample  # noqa: E402
from hermespy.core import Signal  # noqa: E402
from hermespy.modem import (  # noqa: E402
    BitErrorEvaluator,
    ElementType,
    GridElement,
    GridResource,
    OFDMWaveform,
    OrthogonalLeastSquaresChannelEstimation,
    OrthogonalZeroForcingChannelEqualization,
    PskQamMapping,
    SimplexLink,
    StatedSymbols,
    Symbols,
    SymbolSection,
)
from hermespy.modem.bits_source import BitsSource  # noqa: E402
from hermespy.modem.waveform import ZeroForcingChannelEqualization  # noqa: E402
from hermespy.simulation import AWGN, OFDMIdealChannelEstimation, SimulationScenario  # noqa: E402
from hermespy.simulation.modem.noise import EBN0  # noqa: E402
from hermespy.simulation.rf.noise.model import AWGNRealization  # noqa: E402
from hermespy.simulation import SimulatedUniformArray, SimulatedIdealAntenna  # noqa: E402

from oracle import fading as ofad  # noqa: E402
from oracle import streams  # noqa: E402
from refdrops import RefLink, c1_waveform, c2_waveform  # noqa: E402

OUT = HERE


def save(name: str, **arrays) -> None:
    path = os.path.join(OUT, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({os.path.getsize(path) // 1024} KiB)")


# ----------------------------------------------------------------------------- frames
# ----------------------------------------------------------------------------- QAM
def make_qam() -> None:
    rng = np.random.default_rng(7)
    out = {}
    for M in (2, 4, 16, 64, 256):
        m = PskQamMapping(M)
        k = int(np.log2(M))
        idx = np.arange(M)
        bits = ((idx[:, None] >> (k - 1 - np.arange(k))[None, :]) & 1).astype(np.uint8).reshape(-1)
        out[f"bits_{M}"] = bits
        out[f"symbols_{M}"] = m.get_symbols(bits)
        out[f"mapping_{M}"] = m.get_mapping()
        pam_scale = {2: 1.0, 4: 1.0, 16: np.sqrt(5), 64: np.sqrt(21), 256: np.sqrt(85)}[M]
        ties = np.arange(-18, 19) / np.sqrt(2) / pam_scale
        pts = np.concatenate([
            (rng.standard_normal(1000) + 1j * rng.standard_normal(1000)) * 0.9,
            ties + 1j * ties[::-1],
            np.nextafter(ties, np.inf) + 1j * np.nextafter(ties, -np.inf),
            np.array([0.0, np.nan, np.inf, -np.inf, 1e-300]) + 0j,
        ])
        with np.errstate(invalid="ignore"):
            out[f"detect_in_{M}"] = pts
            out[f"detect_out_{M}"] = m.detect_bits(pts).astype(np.uint8)
    save("qam.npz", **out)


# ----------------------------------------------------------------------------- OFDM
def ofdm_rx_distortion(x: np.ndarray) -> np.ndarray:
    """Deterministic stand-in for a channel so that the fixture needs no received samples."""

    return np.roll(x, 3) + 0.5 * x


def make_ofdm() -> None:
    rng = np.random.default_rng(11)
    out = {}
    for name, wf in (("c1", c1_waveform()), ("c2", c2_waveform())):
        data = ((rng.standard_normal(wf.num_data_symbols) + 1j * rng.standard_normal(wf.num_data_symbols))
                / np.sqrt(2)).astype(np.complex64).astype(np.complex128)
        placed = wf.place(Symbols(data[None, :, None]))
        x = wf.modulate(placed, 1.0, 1)
        rx = ofdm_rx_distortion(x)
        grid = wf.demodulate(rx, 1.0, 1).raw[0]
        # The 1024-point frame repeats one resource per word, so its first words pin it;
        # keep the fixture small by storing those only.
        keep_words = 14 if name == "c1" else 3
        keep_samples = keep_words * wf.samples_per_frame(1.0, 1) // wf.words_per_frame
        out[f"{name}_data"] = data
        out[f"{name}_placed"] = placed.raw[0][:keep_words]
        out[f"{name}_x"] = x[:keep_samples]
        out[f"{name}_grid"] = grid[:keep_words]
        out[f"{name}_mask"] = wf.resource_mask
        out[f"{name}_samples_per_frame"] = wf.samples_per_frame(1.0, 1)
        # DC suppression off
        wf.dc_suppression = False
        out[f"{name}_x_nodc"] = wf.modulate(placed, 1.0, 1)[:keep_samples]
        out[f"{name}_grid_nodc"] = wf.demodulate(rx, 1.0, 1).raw[0][:keep_words]
    save("ofdm.npz", **out)


# ----------------------------------------------------------------------------- fading
def _state(num_tx: int, num_rx: int, fs: float):
    sc = SimulationScenario(seed=1)
    tx = sc.new_device(carrier_frequency=0.0, bandwidth=fs, oversampling_factor=1,
                       antennas=SimulatedUniformArray(SimulatedIdealAntenna, 0.01, [num_tx, 1, 1]))
    rx = sc.new_device(carrier_frequency=0.0, bandwidth=fs, oversampling_factor=1,
                       antennas=SimulatedUniformArray(SimulatedIdealAntenna, 0.01, [num_rx, 1, 1]))
    return LinkState(tx.state(0.0), rx.state(0.0), 0.0, fs, 0.0)


def ref_sample(cfg: ofad.FadingConfig, smp: ofad.FadingSample, fs: float) -> MultipathFadingSample:
    los_g, nlos_g = cfg.gains()
    num_rx, num_tx = smp.spatial.shape
    return MultipathFadingSample(
        cfg.power_profile, cfg.delays, smp.los_angles, smp.nlos_angles, smp.los_phases, smp.nlos_phases,
        los_g, nlos_g, cfg.los_doppler, cfg.doppler_frequency, smp.spatial, cfg.gain,
        _state(num_tx, num_rx, fs))


from configs import FADING_CASES  # noqa: E402  (shared with the tests)


def make_fading() -> None:
    out = {}
    rng = np.random.default_rng(5)
    for name, (d, p, k, S, fd, flos, g, nrx, ntx, T, fs) in FADING_CASES.items():
        cfg = ofad.FadingConfig(np.asarray(d, float) / fs, p, k, S, fd, flos, g)
        smp = ofad.realize(cfg, seed=1234, drop=3, num_rx=nrx, num_tx=ntx)
        ref = ref_sample(cfg, smp, fs)
        x = ((rng.standard_normal((ntx, T)) + 1j * rng.standard_normal((ntx, T))) / np.sqrt(2)
             ).astype(np.complex64).astype(np.complex128)
        sig = Signal.Create(x, fs, 0.0)
        y = np.array(ref.propagate(sig).view(np.ndarray))
        out[f"{name}_x"] = x
        out[f"{name}_y"] = y
        Ts = min(T, 96)
        out[f"{name}_state"] = ref.state(Ts, Ts).dense_state()[:2, :2]
    save("fading.npz", **out)


# ----------------------------------------------------------------------------- LS
def make_ls() -> None:
    wf = c1_waveform()
    wf.channel_estimation = OrthogonalLeastSquaresChannelEstimation()
    rng = np.random.default_rng(13)
    grid = rng.standard_normal((14, 256)) + 1j * rng.standard_normal((14, 256))
    est = wf.channel_estimation.estimate_channel(Symbols(grid[None]), 1.0, 1)
    save("ls.npz", grid=grid, estimate=np.asarray(est.dense_states())[0, 0])


# ----------------------------------------------------------------------------- ideal CSI
def make_ideal() -> None:
    fs = 30.72e6
    d, p, k, S, fd, flos, g, nrx, ntx, T, _ = FADING_CASES["c2"]
    cfg = ofad.FadingConfig(np.asarray(d, float) / fs, p, k, S, fd, flos, g)
    smp = ofad.realize(cfg, seed=99, drop=7, num_rx=2, num_tx=2)
    ref = ref_sample(cfg, smp, fs)
    wf = c2_waveform()
    est = OFDMIdealChannelEstimation.__new__(OFDMIdealChannelEstimation)
    est.reference_position = None
    est._IdealChannelEstimation__cached_sample = ref
    with patch.object(type(est), "waveform", new=wf):
        syms = Symbols(np.zeros((2, 14, 1024), complex))
        out = est.estimate_channel(syms, fs, 1)
    # words 0, 5, 10 of the (2, 2, 14, 1024) state keep the fixture small
    save("ideal.npz", csi=np.asarray(out.dense_states())[:, :, ::5, :])


# ----------------------------------------------------------------------------- ZF
def make_zf() -> None:
    rng = np.random.default_rng(17)
    eq = ZeroForcingChannelEqualization()
    out = {}
    for nrx, ntx, name in ((1, 1, "siso"), (4, 4, "mimo")):
        y = rng.standard_normal((nrx, 50, 1)) + 1j * rng.standard_normal((nrx, 50, 1))
        h = rng.standard_normal((nrx, ntx, 50, 1)) + 1j * rng.standard_normal((nrx, ntx, 50, 1))
        res = eq.equalize_channel(StatedSymbols(y, h))
        out[f"{name}_y"], out[f"{name}_h"], out[f"{name}_x"] = y[..., 0], h[..., 0], res.raw[..., 0]
    save("zf.npz", **out)


# ----------------------------------------------------------------------------- BER
def make_ber() -> None:
    rng = np.random.default_rng(19)
    ev = BitErrorEvaluator.__new__(BitErrorEvaluator)
    out = {}
    for i, (nt, nr) in enumerate(((500, 500), (480, 500), (500, 470))):
        a = rng.integers(0, 2, nt).astype(np.uint8)
        b = rng.integers(0, 2, nr).astype(np.uint8)
        b[: min(nt, nr) // 2] = a[: min(nt, nr) // 2]
        with patch.object(BitErrorEvaluator, "_fetch_dsp_results",
                          return_value=(SimpleNamespace(bits=a), SimpleNamespace(bits=b))):
            e = ev.evaluate()
        out[f"tx_{i}"], out[f"rx_{i}"] = a, b
        out[f"errors_{i}"] = np.asarray(e.evaluation)
        out[f"ber_{i}"] = e.artifact().to_scalar()
    save("ber.npz", **out)


# ----------------------------------------------------------------------------- full drops
def make_drops() -> None:
    out = {}
    seed = 20240611
    fs = 15.36e6
    cfg = ofad.FadingConfig(np.arange(6) / fs, 10 ** (-0.3 * np.arange(6)), np.zeros(6), 20, 100.0)
    for i, (drop, ebn0_db) in enumerate(((0, 0.0), (1, 10.0), (2, 20.0))):
        link = RefLink(c1_waveform(), cfg, fs, 1, 1, seed, "ls")
        link.set_ebn0(ebn0_db)
        errors, dr = link.drop(drop)
        out[f"c1_{i}_drop"], out[f"c1_{i}_ebn0_db"] = drop, ebn0_db
        out[f"c1_{i}_errors"] = errors
        out[f"c1_{i}_rx_bits"] = np.packbits(dr.device_receptions[1].operator_receptions[0].bits)
    # 2x2 ideal CSI + ZF on the 1024/600 frame with 23 taps
    fs2 = 30.72e6
    d, p, k, S, fd, flos, g, _, _, _, _ = FADING_CASES["c2"]
    cfg2 = ofad.FadingConfig(np.asarray(d, float) / fs2, p, k, S, fd, flos, g)
    link = RefLink(c2_waveform(16), cfg2, fs2, 2, 2, seed, "ideal")
    link.set_ebn0(15.0)
    errors, dr = link.drop(5)
    out["c2_errors"] = errors
    out["c2_rx_bits"] = np.packbits(dr.device_receptions[1].operator_receptions[0].bits)
    out["seed"] = seed
    save("drops.npz", **out)


def make_presets() -> None:
    from hermespy.channel import TDL, Cost259, Cost259Type, Exponential, TDLType
    from hermespy.channel.fading.correlation import CorrelationType, StandardAntennaCorrelation
    from hermespy.core import AntennaMode

    out = {}
    for t in TDLType:
        for tag, rms in (("0", 0.0), ("300ns", 300e-9)):
            ch = TDL(model_type=t, rms_delay=rms, doppler_frequency=10.0, seed=1)
            key = f"tdl_{t.name}_{tag}"
            out[key + "_delays"] = np.asarray(ch.delays, dtype=np.float64)
            out[key + "_power"] = np.asarray(ch.power_profile, dtype=np.float64)
            out[key + "_rice"] = np.asarray(ch.rice_factors, dtype=np.float64)
            out[key + "_los_doppler"] = np.float64(ch.los_doppler_frequency)
    for t in Cost259Type:
        ch = Cost259(model_type=t, doppler_frequency=10.0, seed=1)
        key = f"cost259_{t.name}"
        out[key + "_delays"] = np.asarray(ch.delays, dtype=np.float64)
        out[key + "_power"] = np.asarray(ch.power_profile, dtype=np.float64)
        out[key + "_rice"] = np.asarray(ch.rice_factors, dtype=np.float64)
        out[key + "_los_doppler"] = np.float64(ch.los_doppler_frequency)
    for interval, rms in ((1e-7, 3e-7), (5e-8, 1e-6)):
        ch = Exponential(interval, rms, seed=1)
        key = f"exponential_{interval:g}_{rms:g}"
        out[key + "_delays"] = np.asarray(ch.delays, dtype=np.float64)
        out[key + "_power"] = np.asarray(ch.power_profile, dtype=np.float64)
    for c in CorrelationType:
        model = StandardAntennaCorrelation(c)
        for n in (1, 2, 4):
            arr = SimpleNamespace(num_receive_antennas=n, num_transmit_antennas=n)
            out[f"corr_{c.name}_{n}_rx"] = model.sample_covariance(arr, AntennaMode.RX)
            out[f"corr_{c.name}_{n}_tx"] = model.sample_covariance(arr, AntennaMode.TX)
    save("presets.npz", **out)


def sync_waveform(dc: bool, pilot):
    """128-point frame with a preamble: 100 used data subcarriers, CP 10, 4 words."""

    N, U, CP = 128, 100, 10
    res = [GridResource(1, prefix_ratio=CP / N, elements=[GridElement(ElementType.DATA, U)])]
    struct = [SymbolSection(4, [0])]
    return OFDMWaveform(grid_resources=res, grid_structure=struct, num_subcarriers=N, modulation_order=16,
                        dc_suppression=dc, pilot_section=pilot)


def make_sync() -> None:
    from hermespy.modem.waveforms.orthogonal.ofdm import (
        OFDMCorrelationSynchronization,
        SchmidlCoxPilotSection,
        SchmidlCoxSynchronization,
    )
    from hermespy.modem.waveforms.orthogonal.waveform import PilotSection

    out = {}
    for dc in (True, False):
        out[f"schmidl_cox_pilot_dc{int(dc)}"] = sync_waveform(dc, SchmidlCoxPilotSection()).pilot_section.generate(1)
        out[f"plain_pilot_dc{int(dc)}"] = sync_waveform(dc, PilotSection()).pilot_section.generate(1)
    rng = np.random.default_rng(11)
    cases = (("sc", SchmidlCoxPilotSection, SchmidlCoxSynchronization, (37, 700), 0.05),
             ("sc3", SchmidlCoxPilotSection, SchmidlCoxSynchronization, (0, 650, 1400), 0.2),
             ("corr", PilotSection, OFDMCorrelationSynchronization, (53, 760), 0.05),
             ("corr3", PilotSection, OFDMCorrelationSynchronization, (5, 640, 1290), 0.2))
    for name, section, routine, starts, noise in cases:
        wf = sync_waveform(True, section())
        spf = wf.samples_per_frame(1.0, 1)
        n = starts[-1] + spf + 80
        signal = np.zeros((2, n), dtype=np.complex128)
        for s0 in starts:
            bits = rng.integers(0, 2, wf.bits_per_frame(), dtype=np.uint8)
            frame = wf.modulate(wf.place(wf.map(bits)), 1.0, 1)
            signal[0, s0:s0 + spf] += frame
            signal[1, s0:s0 + spf] += 0.6j * frame
        signal += noise * (rng.standard_normal(signal.shape) + 1j * rng.standard_normal(signal.shape))
        signal = signal.astype(np.complex64).astype(np.complex128)  # representable in the engine's complex64
        sync = routine()
        sync.waveform = wf
        out[f"{name}_signal"] = signal
        out[f"{name}_starts"] = np.asarray(starts)
        out[f"{name}_indices"] = np.asarray(sync.synchronize(signal, 1.0, 1), dtype=np.int64)
    save("sync.npz", **out)


def make_ldpc() -> None:
    from oracle import ldpc as oldpc

    N, M, ev, ec = oldpc.read_alist(os.path.join(REF, "hermespy", "modem", "resources", "ofdm_ldpc.alist"))
    save("ldpc.npz", N=np.int64(N), M=np.int64(M), edge_var=ev, edge_chk=ec)


MAKERS = {"qam": make_qam, "ofdm": make_ofdm, "fading": make_fading, "ls": make_ls, "ideal": make_ideal,
          "zf": make_zf, "ber": make_ber, "drops": make_drops, "presets": make_presets,
          "sync": make_sync, "ldpc": make_ldpc}

if __name__ == "__main__":
    for name, maker in MAKERS.items():
        if not ONLY or name in ONLY:
            maker()
