"""The engine behind HermesPy's own classes: GPU subclasses for an installed reference.

``make_plugins(hermespy)`` takes the user's HermesPy package and returns
subclasses of its own classes whose hot methods run on this library, so that an
unchanged HermesPy script (``SimulationScenario.set_channel``, ``SimplexLink``,
``Simulation.run``) simulates its drops on the GPU:

* ``GpuMultipathFadingChannel(MultipathFadingChannel)`` overrides ``_realize``
  (channel/fading/fading.py:893-910) to hand out ``GpuMultipathFadingRealization``
  objects, whose ``_sample`` (fading.py:468-515) keeps the reference's own draw of
  angles, phases and spatial response and returns a ``GpuMultipathFadingSample``;
* ``GpuMultipathFadingSample(MultipathFadingSample)`` overrides ``_propagate``
  (fading.py:371-406) and ``state`` (fading.py:345-369) with
  ``hpx_fading_load`` + ``hpx_fading_propagate`` / ``hpx_fading_csi``;
* ``GpuOFDMWaveform(OFDMWaveform)`` overrides ``modulate`` and ``demodulate``
  (modem/waveforms/orthogonal/waveform.py:1292-1364, ofdm.py:98-161) with
  ``hpx_ofdm_modulate_grid`` / ``hpx_ofdm_demodulate``.

The realization and sampling logic stays the reference's; only the arithmetic on
samples moves to the GPU. The subclasses convert at the numpy boundary the
reference's methods define (complex128 in and out); the array-level cores below
(``propagate_block``, ``channel_state``, ``modulate_grid``, ``demodulate_frame``)
do the work and take any object that exposes the reference's public properties.
"""

from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import torch

from . import _lib
from .channel import LinkState, MultipathFadingSample
from .waveform import ElementType, GridElement, GridResource, OFDMWaveform, PrefixType, SymbolSection


# ------------------------------------------------------------------ array cores
def sample_parameters(sample) -> dict:
    """Constructor arguments of the engine's fading sample from an object with the
    public properties of the reference's ``MultipathFadingSample`` (fading.py:153-299)."""

    ntx = int(sample.num_transmit_antennas)
    nrx = int(sample.num_receive_antennas)
    spatial = np.asarray(sample.spatial_response, dtype=np.complex128)[:nrx, :ntx]
    return dict(power_profile=np.asarray(sample.power_profile, dtype=np.float64),
                delay_profile=np.asarray(sample.delay_profile, dtype=np.float64),
                los_angles=np.asarray(sample.los_angles, dtype=np.float64),
                nlos_angles=np.asarray(sample.nlos_angles, dtype=np.float64),
                los_phases=np.asarray(sample.los_phases, dtype=np.float64),
                nlos_phases=np.asarray(sample.nlos_phases, dtype=np.float64),
                los_gains=np.asarray(sample.los_gains, dtype=np.float64),
                nlos_gains=np.asarray(sample.nlos_gains, dtype=np.float64),
                los_doppler=float(sample.los_doppler), nlos_doppler=float(sample.nlos_doppler),
                spatial_response=np.ascontiguousarray(spatial), gain=float(sample.gain),
                state=LinkState(ntx, nrx, float(sample.bandwidth)))


def engine_sample(sample) -> MultipathFadingSample:
    """The engine's device-resident fading sample holding the same realization."""

    return MultipathFadingSample(**sample_parameters(sample))


def propagate_block(sample, samples: np.ndarray) -> np.ndarray:
    """``MultipathFadingSample._propagate`` on the GPU: (Ntx, T) complex samples ->
    (Nrx, T + D) complex128, D the largest tap delay in samples (fading.py:371-406)."""

    _lib.require_cuda()
    x = torch.from_numpy(np.ascontiguousarray(np.asarray(samples).reshape(int(sample.num_transmit_antennas), -1),
                                              dtype=np.complex64))
    return engine_sample(sample).propagate_device(x).cpu().numpy().astype(np.complex128)


def channel_state(sample, num_samples: int, max_num_taps: int) -> np.ndarray:
    """``MultipathFadingSample.state`` as a dense (Nrx, Ntx, num_samples, taps) array."""

    _lib.require_cuda()
    st = engine_sample(sample).state_device(int(num_samples), int(max_num_taps))
    return st.cpu().numpy().astype(np.complex128)


def engine_waveform(waveform) -> OFDMWaveform:
    """The engine's OFDM waveform with the grid of a reference ``OFDMWaveform``
    (the same resources, sections, FFT size, modulation order and DC suppression)."""

    resources = [GridResource(r.repetitions, prefix_type=PrefixType[r.prefix_type.name], prefix_ratio=r.prefix_ratio,
                              elements=[GridElement(ElementType[e.type.name], e.repetitions) for e in r.elements])
                 for r in waveform.grid_resources]
    sections = [SymbolSection(s.num_repetitions, list(s.pattern), getattr(s, "sample_offset", 0))
                for s in waveform.grid_structure]
    return OFDMWaveform(resources, sections, num_subcarriers=int(waveform.num_subcarriers),
                        modulation_order=int(waveform.modulation_order), dc_suppression=bool(waveform.dc_suppression))


def modulate_grid(engine: OFDMWaveform, grid: np.ndarray) -> np.ndarray:
    """Placed (words, N) grid -> complex128 frame samples (waveform.py:1292-1323)."""

    _lib.require_cuda()
    g = torch.from_numpy(np.ascontiguousarray(np.asarray(grid).reshape(1, engine.words_per_frame, -1),
                                              dtype=np.complex64)).cuda()
    return engine.modulate_device(g)[0].cpu().numpy().astype(np.complex128)


def demodulate_frame(engine: OFDMWaveform, samples: np.ndarray) -> np.ndarray:
    """Frame samples -> complex128 (words, N) grid (waveform.py:1325-1364)."""

    _lib.require_cuda()
    s = torch.from_numpy(np.ascontiguousarray(np.asarray(samples).reshape(1, -1), dtype=np.complex64)).cuda()
    T = engine.samples_per_frame()
    if s.shape[1] < T:
        s = torch.nn.functional.pad(s, (0, T - s.shape[1]))
    return engine.demodulate_device(s)[0].cpu().numpy().astype(np.complex128)


# ------------------------------------------------------------ reference classes
def make_plugins(hermespy=None) -> SimpleNamespace:
    """GPU subclasses of the reference's own channel, realization, sample and OFDM
    waveform classes (``hermespy`` defaults to the importable package)."""

    if hermespy is None:
        import hermespy  # noqa: F401  (the user's installation)
    from hermespy.core import ChannelStateFormat, ChannelStateInformation
    from hermespy.channel.fading.fading import (MultipathFadingChannel, MultipathFadingRealization,
                                                MultipathFadingSample as RefSample)
    from hermespy.core import SignalBlock
    from hermespy.modem import OFDMWaveform as RefOFDMWaveform
    from hermespy.modem.symbols import Symbols
    from sparse import GCXS

    class GpuMultipathFadingSample(RefSample):
        """The reference's sample; propagation and channel state run on the GPU."""

        def _propagate(self, signal, interpolation):
            y = propagate_block(self, np.asarray(signal))
            return SignalBlock(y.shape[0], y.shape[1], signal.offset, y.tobytes())

        def state(self, num_samples, max_num_taps, interpolation_mode=None):
            dense = channel_state(self, num_samples, max_num_taps)
            return ChannelStateInformation(ChannelStateFormat.IMPULSE_RESPONSE,
                                           GCXS.from_numpy(dense, compressed_axes=(0, 1, 2)),
                                           num_delay_taps=dense.shape[3])

    class GpuMultipathFadingRealization(MultipathFadingRealization):
        """The reference's realization; its samples are GPU samples."""

        def _sample(self, state):
            sample = MultipathFadingRealization._sample(self, state)
            sample.__class__ = GpuMultipathFadingSample  # same attributes, GPU methods
            return sample

    class GpuMultipathFadingChannel(MultipathFadingChannel):
        """The reference's statistical multipath fading channel on the GPU."""

        def _realize(self):
            realization = MultipathFadingChannel._realize(self)
            realization.__class__ = GpuMultipathFadingRealization
            return realization

    class GpuOFDMWaveform(RefOFDMWaveform):
        """The reference's OFDM waveform; modulation and demodulation run on the GPU."""

        def _engine(self) -> OFDMWaveform:
            key = (tuple((r.repetitions, r.prefix_ratio, r.prefix_type.name,
                          tuple((e.type.name, e.repetitions) for e in r.elements)) for r in self.grid_resources),
                   tuple((s.num_repetitions, tuple(s.pattern)) for s in self.grid_structure),
                   self.num_subcarriers, self.modulation_order, self.dc_suppression)
            if getattr(self, "_hpx_key", None) != key:
                self._hpx_engine, self._hpx_key = engine_waveform(self), key
            return self._hpx_engine

        def modulate(self, data_symbols, bandwidth, oversampling_factor):
            if oversampling_factor != 1:
                return RefOFDMWaveform.modulate(self, data_symbols, bandwidth, oversampling_factor)
            return modulate_grid(self._engine(), data_symbols.raw[0])

        def demodulate(self, signal, bandwidth, oversampling_factor):
            if oversampling_factor != 1:
                return RefOFDMWaveform.demodulate(self, signal, bandwidth, oversampling_factor)
            return Symbols(demodulate_frame(self._engine(), signal)[None])

    return SimpleNamespace(GpuMultipathFadingChannel=GpuMultipathFadingChannel,
                           GpuMultipathFadingRealization=GpuMultipathFadingRealization,
                           GpuMultipathFadingSample=GpuMultipathFadingSample, GpuOFDMWaveform=GpuOFDMWaveform)
