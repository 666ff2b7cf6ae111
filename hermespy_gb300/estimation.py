"""Channel estimation and equalization of the drop-in API.

Mirrors the reference's plugin classes and their contracts:

* ``ChannelEstimation`` / ``ChannelEqualization`` (modem/waveform.py:111-223):
  unit states / no equalization by default.
* ``OrthogonalLeastSquaresChannelEstimation``
  (modem/waveforms/orthogonal/channel.py:25-66): LS at the reference elements,
  linear ``griddata`` interpolation, nearest-neighbour fill; SISO only
  (``NotImplementedError`` otherwise, as the reference). The interpolator is a
  fixed sparse linear map of the pilot LS values for a given frame; it is
  recorded once per frame with the very ``griddata`` calls the reference makes
  and applied on the GPU.
* ``OFDMIdealChannelEstimation`` (simulation/modem/channel_estimation.py:182-295):
  the channel sample's impulse response averaged over each word's FFT window,
  transformed to the grid's bins, computed in closed form on the GPU.
* ``ZeroForcingChannelEqualization`` (modem/waveform.py:235-250) and
  ``OrthogonalZeroForcingChannelEqualization`` (orthogonal/channel.py:83-86).
* ``LinearMinimumMeanSquareErrorChannelEqualization`` (no counterpart in the
  reference): ``(H^H H + s2 I)^-1 H^H y`` per resource element by Cholesky, with
  ``s2`` the noise power per subcarrier.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch
from scipy.interpolate import griddata

from . import _lib
from .containers import StatedSymbols, Symbols


class ChannelEstimation:
    def __init__(self, waveform=None) -> None:
        self.waveform = waveform

    def estimate_channel(self, symbols: Symbols, bandwidth: float = 1.0, oversampling_factor: int = 1,
                         delay: float = 0.0) -> StatedSymbols:
        raw = symbols.device_raw
        return StatedSymbols(raw, torch.ones((raw.shape[0], 1) + tuple(raw.shape[1:]), dtype=torch.complex64,
                                             device=raw.device))


def ls_interpolation_table(ref_mask: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """CSR map (indptr, indices, weights) from pilot LS values to the (W, C) grid.

    Makes the reference's two ``griddata`` calls (orthogonal/channel.py:49-64)
    once, on the identity matrix of pilot values, so that every row holds the
    interpolation weights of one resource element.
    """

    W, C = ref_mask.shape
    num_refs = int(ref_mask.sum())
    eye = np.eye(num_refs)
    est = np.zeros((1, 1, W, C, num_refs))
    est[0, 0, ref_mask] = eye
    holes = np.where(np.invert(ref_mask))
    if holes[0].size != 0:
        stems = np.where(ref_mask)
        est[0, 0, holes[0], holes[1]] = griddata(stems, eye, holes, method="linear")
    nan_rows = np.isnan(est[..., 0])
    if nan_rows.any():
        nan_idx = np.where(nan_rows)
        stem_idx = np.where(np.invert(nan_rows))
        est[nan_idx] = griddata(stem_idx, est[stem_idx], nan_idx, method="nearest")
    dense = est.reshape(W * C, num_refs)
    indptr = np.zeros(W * C + 1, dtype=np.int32)
    indices, weights = [], []
    for r in range(W * C):
        nz = np.nonzero(dense[r])[0]
        indices.append(nz)
        weights.append(dense[r, nz])
        indptr[r + 1] = indptr[r] + nz.size
    return indptr, np.concatenate(indices).astype(np.int32), np.concatenate(weights).astype(np.float32)


def ls_stream_tables(ref_mask: np.ndarray, comb: int, num_streams: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Stacked CSR tables of ``num_streams`` streams under a pilot comb.

    Stream ``s`` owns the reference elements of grid columns ``c % comb == s % comb``;
    its table is ``ls_interpolation_table`` of that sub-mask with the indices mapped
    back to the frame's reference numbering (row-major over the grid).
    """

    W, C = ref_mask.shape
    if num_streams > 1 and comb < num_streams:
        raise NotImplementedError("Least-Squares channel estimation of several streams needs a pilot comb")
    ptrs, idxs, wts = [np.zeros(1, dtype=np.int64)], [], []
    base = 0
    for s in range(num_streams):
        sub = ref_mask & (np.arange(C)[None, :] % comb == s % comb) if comb > 1 else ref_mask
        gidx = np.nonzero(sub[ref_mask])[0]
        indptr, indices, weights = ls_interpolation_table(sub)
        ptrs.append(indptr[1:].astype(np.int64) + base)
        idxs.append(gidx[indices])
        wts.append(weights)
        base += int(indptr[-1])
    return (np.concatenate(ptrs).astype(np.int32), np.concatenate(idxs).astype(np.int32),
            np.concatenate(wts).astype(np.float32))


def robust_statistics(channel, sampling_rate: float, num_delays: int = 64, doppler_frequency: float = 1000.0,
                      design_snr_db: float = 20.0):
    """Design statistics of the robust tap-domain LMMSE estimator: a channel that
    knows nothing of the true one but its expected energy, and the prior noise
    variance that regularizes its tap estimates.

    The robust LMMSE of Li, Cimini and Sollenberger (IEEE Trans. Commun. 46(7), 1998)
    replaces the channel's power-delay profile and Doppler by a uniform profile over
    an assumed delay window and a design Doppler bound. Here the window is
    ``num_delays`` sample delays (64 at 30.72 MHz: 2.1 us, beyond the 4x4 workload's
    1.1 us and within its 2.3 us cyclic prefix), the bound ``doppler_frequency``, the
    uniform profile carries the channel's expected energy (gain times the sum of its
    powers, which the receiver can measure as received power), and the prior noise is
    that of ``design_snr_db`` (20 dB gave the lowest NMSE over 5-25 dB). Returns
    (design channel, ridge noise variance) for ``hpx_lmmse_create_regularized``. No
    counterpart in the reference."""

    from .channel import MultipathFadingChannel

    energy = float(channel.gain) * float(np.sum(channel.power_profile))
    delays = np.arange(int(num_delays)) / float(sampling_rate)
    design = MultipathFadingChannel(list(delays), [energy / num_delays] * int(num_delays), [0.0] * int(num_delays),
                                    doppler_frequency=float(doppler_frequency))
    return design, energy * 10.0 ** (-design_snr_db / 10.0)


class OrthogonalLeastSquaresChannelEstimation(ChannelEstimation):
    """Least-squares estimation with linear interpolation (SISO)."""

    def __init__(self, waveform=None) -> None:
        ChannelEstimation.__init__(self, waveform)
        self._ls = None
        self._ls_key = None

    def _handle(self):
        wf = self.waveform
        frame = wf._frame()
        key = (id(frame), wf._key)
        if self._ls is None or self._ls_key != key:
            mask = wf.resource_mask[0]  # REFERENCE elements over (W, N)
            indptr, indices, weights = ls_interpolation_table(mask)
            h = ctypes.c_void_p()
            _lib.check(_lib.load().hpx_ls_create(
                frame, mask.shape[1], indptr.ctypes.data_as(ctypes.c_void_p), indices.ctypes.data_as(ctypes.c_void_p),
                weights.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)))
            self._ls = h
            self._ls_key = key
            self._tables = (indptr, indices, weights)
        return self._ls

    def __del__(self):
        try:
            if self._ls is not None and _lib._lib is not None:
                _lib._lib.hpx_ls_destroy(self._ls)
        except Exception:
            pass

    def estimate_device(self, grids: torch.Tensor) -> torch.Tensor:
        """(batch, W, G) received grids -> (batch, W, N) estimates."""

        h = self._handle()
        grids = grids.contiguous()
        W, N = self.waveform.words_per_frame, self.waveform.num_subcarriers
        out = torch.empty((grids.shape[0], W, N), dtype=torch.complex64, device=grids.device)
        _lib.call("hpx_ls_estimate", h, _lib.ptr(grids), grids.shape[-1], grids.shape[0], _lib.ptr(out),
                  _lib.stream_ptr())
        return out

    def estimate_channel(self, symbols: Symbols, bandwidth: float = 1.0, oversampling_factor: int = 1,
                         delay: float = 0.0) -> StatedSymbols:
        if symbols.num_streams != 1:
            raise NotImplementedError("Least-Squares channel estimation is only implemented for SISO links")
        est = self.estimate_device(symbols.device_raw)
        return StatedSymbols(symbols.device_raw, est[:, None])


class OFDMIdealChannelEstimation(ChannelEstimation):
    """Ideal channel state of the cached channel sample of a (transmitter, receiver) link."""

    def __init__(self, channel, transmitter, receiver, waveform=None) -> None:
        ChannelEstimation.__init__(self, waveform)
        self._sample = None
        channel.add_sample_hook(self._cache, transmitter, receiver)

    def _cache(self, sample) -> None:
        self._sample = sample

    def estimate_channel(self, symbols: Symbols, bandwidth: float = 1.0, oversampling_factor: int = 1,
                         delay: float = 0.0) -> StatedSymbols:
        if self.waveform is None:
            raise RuntimeError("Ideal channel state estimation routine floating")
        if self._sample is None:
            raise RuntimeError("No channel sample available from which to estimate the ideal channel state information")
        smp = self._sample
        wf = self.waveform
        W, N = wf.words_per_frame, wf.num_subcarriers
        h = smp._handle
        out = torch.empty((h.nrx, h.ntx, W, N), dtype=torch.complex64, device=smp._state.device)
        _lib.call("hpx_fading_ideal_csi", h.handle, _lib.ptr(smp._state), 1, wf._frame(), N, _lib.ptr(out),
                  _lib.stream_ptr())
        return StatedSymbols(symbols.device_raw, out[: symbols.num_streams])


class ChannelEqualization:
    def __init__(self, waveform=None) -> None:
        self.waveform = waveform

    def equalize_channel(self, stated_symbols: StatedSymbols) -> Symbols:
        return stated_symbols


def _equalize(mode: int, stated: StatedSymbols, noise_variance: float) -> Symbols:
    raw = stated.device_raw          # (Nrx, B, S)
    st = stated.device_states        # (Nrx, Ntx, B, S)
    nrx, ntx = st.shape[0], st.shape[1]
    k = raw.shape[1] * raw.shape[2]
    y = raw.reshape(nrx, k).contiguous()
    h = st.reshape(nrx, ntx, k).contiguous()
    out_streams = 1 if (mode == _lib.EQ_ZF and nrx == 1) else ntx
    x = torch.empty((out_streams, k), dtype=torch.complex64, device=raw.device)
    nv = torch.tensor([noise_variance], dtype=torch.float32, device=raw.device)
    _lib.call("hpx_equalize", mode, nrx, ntx, k, 1, _lib.ptr(h), _lib.ptr(y), _lib.ptr(nv), _lib.ptr(x),
              _lib.stream_ptr())
    return Symbols(x.reshape((out_streams,) + tuple(raw.shape[1:])))


class ZeroForcingChannelEqualization(ChannelEqualization):
    def equalize_channel(self, stated_symbols: StatedSymbols) -> Symbols:
        return _equalize(_lib.EQ_ZF, stated_symbols, 0.0)


class OrthogonalZeroForcingChannelEqualization(ZeroForcingChannelEqualization):
    pass


class LinearMinimumMeanSquareErrorChannelEqualization(ChannelEqualization):
    """LMMSE detection; the noise variance comes from the stated symbols (the received
    signal's noise power) unless given here."""

    def __init__(self, waveform=None, noise_variance: float | None = None) -> None:
        ChannelEqualization.__init__(self, waveform)
        self.noise_variance = noise_variance

    def equalize_channel(self, stated_symbols: StatedSymbols) -> Symbols:
        nv = stated_symbols.noise_variance if self.noise_variance is None else self.noise_variance
        return _equalize(_lib.EQ_LMMSE, stated_symbols, nv)


OrthogonalLinearMinimumMeanSquareErrorChannelEqualization = LinearMinimumMeanSquareErrorChannelEqualization
