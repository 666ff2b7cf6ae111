"""Channel estimation and equalization (oracle side, float64).

* ``ls_estimate``   restates ``OrthogonalLeastSquaresChannelEstimation.estimate_channel``
  (modem/waveforms/orthogonal/channel.py:29-66): LS at the reference elements,
  ``griddata(method="linear")`` over (word, subcarrier) for the holes, then
  ``griddata(method="nearest")`` for the NaNs left outside the convex hull.
* ``ideal_csi``     restates ``OFDMIdealChannelEstimation.estimate_channel`` and
  ``__extract_channel`` (simulation/modem/channel_estimation.py:215-295): the impulse
  response of ``MultipathFadingSample.state`` is averaged over each word's FFT window
  and transformed with ``_backward_transformation(normalize=False)``.
* ``zf_equalize``   restates ``ZeroForcingChannelEqualization.equalize_channel``
  (modem/waveform.py:235-250): ``y / sum_tx h`` for one receive stream, per-element
  ``pinv(H) y`` otherwise.
* ``lmmse_equalize`` has no counterpart in the reference (its only "MMSE" class,
  modem/waveform_single_carrier.py:586-630, falls back to a pseudo-inverse). It is the
  engine's definition: ``x = (H^H H + s2 I)^-1 H^H y`` per resource element, ``s2`` the
  noise variance per subcarrier.
"""

from __future__ import annotations

import numpy as np
from scipy.interpolate import griddata

from . import fading
from .frame import FrameLayout


def ls_estimate(layout: FrameLayout, grid: np.ndarray) -> np.ndarray:
    """(words, N) received grid -> (words, N) LS channel estimate (SISO)."""

    ref = layout.ref_mask
    refs = grid[ref] / layout.pilot_symbols()
    est = np.zeros((layout.num_words, layout.N), dtype=complex)
    est[ref] = refs
    holes = np.where(~ref)
    if holes[0].size:
        stems = np.where(ref)
        est[holes[0], holes[1]] = griddata(stems, refs, holes, method="linear")
    nan = np.where(np.isnan(est))
    if nan[0].size:
        good = np.where(~np.isnan(est))
        est[nan] = griddata(good, est[good], nan, method="nearest")
    return est


def ls_weight_table(layout: FrameLayout) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """The LS interpolator as a sparse linear map of the pilot LS values.

    Returns (indptr, indices, weights) in CSR form over the (words * N) grid.
    Linear and nearest-neighbour ``griddata`` are linear in the data for a fixed
    geometry, so probing with unit vectors recovers the map exactly.
    """

    num_refs = layout.num_refs
    cols = []
    for k in range(num_refs):
        e = np.zeros(num_refs, dtype=complex)
        e[k] = 1.0
        grid = np.zeros((layout.num_words, layout.N), dtype=complex)
        grid[layout.ref_mask] = e * layout.pilot_symbols()
        cols.append(ls_estimate(layout, grid).reshape(-1).real)
    dense = np.stack(cols, axis=1)  # (words*N, refs)
    indptr = [0]
    indices, weights = [], []
    for row in dense:
        nz = np.nonzero(np.abs(row) > 1e-14)[0]
        indices += nz.tolist()
        weights += row[nz].tolist()
        indptr.append(len(indices))
    return np.asarray(indptr), np.asarray(indices), np.asarray(weights)


def ideal_csi(layout: FrameLayout, sample: fading.FadingSample, fs: float) -> np.ndarray:
    """(Nrx, Ntx, words, N) frequency-domain channel state."""

    T = layout.samples_per_frame
    csi = fading.state(sample, T, fs, T)  # (Nrx, Ntx, T, taps)
    n = layout.N
    num_taps = csi.shape[3]
    out = np.empty(csi.shape[:2] + (layout.num_words, n), dtype=np.complex128)
    bins = layout.bins()
    for w in range(layout.num_words):
        s = int(layout.window_start[w])
        avg = csi[:, :, s : s + n, :].mean(axis=2)  # (Nrx, Ntx, taps)
        padded = np.zeros(csi.shape[:2] + (n,), dtype=np.complex128)
        padded[..., : min(num_taps, n)] = avg[..., :n]
        spec = np.fft.fft(padded, axis=-1)
        out[:, :, w, :] = spec[..., bins]
    return out


def zf_equalize(y: np.ndarray, h: np.ndarray) -> np.ndarray:
    """y: (Nrx, K), h: (Nrx, Ntx, K) -> (Ntx, K)."""

    if y.shape[0] < 2:
        with np.errstate(divide="ignore", invalid="ignore"):
            return y / np.sum(h, axis=1)
    hk = np.moveaxis(h, 2, 0)  # (K, Nrx, Ntx)
    pinv = np.linalg.pinv(hk)  # (K, Ntx, Nrx)
    return np.einsum("kij,jk->ik", pinv, y)


def lmmse_equalize(y: np.ndarray, h: np.ndarray, noise_variance) -> np.ndarray:
    """y: (Nrx, K), h: (Nrx, Ntx, K), noise variance scalar or (K,) -> (Ntx, K)."""

    hk = np.moveaxis(h, 2, 0)  # (K, Nrx, Ntx)
    ntx = hk.shape[2]
    s2 = np.broadcast_to(np.asarray(noise_variance, dtype=np.float64), (hk.shape[0],))
    gram = np.conj(np.swapaxes(hk, 1, 2)) @ hk + s2[:, None, None] * np.eye(ntx)[None]
    mf = np.einsum("kji,jk->ki", np.conj(hk), y)
    return np.linalg.solve(gram, mf[..., None])[..., 0].T
