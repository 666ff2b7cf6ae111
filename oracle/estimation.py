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
* ``mimo_ls_estimate`` and ``tap_lmmse_estimate`` have no counterpart in the
  reference either (its LS estimator stops at one stream, channel.py:32-35). With a
  pilot comb (``FrameSpec.pilot_comb``) every stream has pilots of its own:
  ``mimo_ls_estimate`` runs the reference's LS + griddata procedure per stream on
  that stream's pilots; ``tap_lmmse_estimate`` is the engine's LMMSE estimator
  with the channel's statistics (delays, powers, Doppler) known: weighted LS of
  the tap gains per pilot word, per-tap LMMSE interpolation over words with the
  Jakes correlation J0(w_D dt) of the sum-of-sinusoids model, then the tap DFT
  on every subcarrier.
* ``lmmse_equalize`` has no counterpart in the reference (its only "MMSE" class,
  modem/waveform_single_carrier.py:586-630, falls back to a pseudo-inverse). It is the
  engine's definition: ``x = (H^H H + s2 I)^-1 H^H y`` per resource element, ``s2`` the
  noise variance per subcarrier.
"""

from __future__ import annotations

import numpy as np
from scipy.interpolate import griddata
from scipy.special import j0

from . import fading
from .frame import FrameLayout


def _stream_refs(layout: FrameLayout, stream: int | None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(grid mask, pilot symbols, global reference indices) of one stream's pilots."""

    if stream is None:
        return layout.ref_mask, layout.pilot_symbols(), np.arange(layout.num_refs)
    keep = layout.stream_ref_mask(stream)[layout.ref_mask]
    return layout.stream_ref_mask(stream), layout.pilot_symbols()[keep], np.nonzero(keep)[0]


def ls_estimate(layout: FrameLayout, grid: np.ndarray, stream: int | None = None) -> np.ndarray:
    """(words, N) received grid -> (words, N) LS channel estimate (SISO, or the
    pilots of one stream under a pilot comb)."""

    ref, pilots, _ = _stream_refs(layout, stream)
    refs = grid[ref] / pilots
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


def ls_weight_table(layout: FrameLayout, stream: int | None = None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """The LS interpolator as a sparse linear map of the pilot LS values.

    Returns (indptr, indices, weights) in CSR form over the (words * N) grid, the
    indices numbering the frame's reference elements. Linear and
    nearest-neighbour ``griddata`` are linear in the data for a fixed geometry, so
    probing with unit vectors recovers the map exactly.
    """

    ref, pilots, gidx = _stream_refs(layout, stream)
    n = pilots.size
    cols = []
    for k in range(n):
        e = np.zeros(n, dtype=complex)
        e[k] = 1.0
        grid = np.zeros((layout.num_words, layout.N), dtype=complex)
        grid[ref] = e * pilots
        cols.append(ls_estimate(layout, grid, stream).reshape(-1).real)
    dense = np.stack(cols, axis=1)  # (words*N, stream refs)
    indptr = [0]
    indices, weights = [], []
    for row in dense:
        nz = np.nonzero(np.abs(row) > 1e-14)[0]
        indices += gidx[nz].tolist()
        weights += row[nz].tolist()
        indptr.append(len(indices))
    return np.asarray(indptr), np.asarray(indices), np.asarray(weights)


def mimo_ls_estimate(layout: FrameLayout, grids: np.ndarray, num_tx: int) -> np.ndarray:
    """(Nrx, words, N) received grids -> (Nrx, Ntx, words, N) per-stream LS estimates."""

    if num_tx > 1 and layout.spec.pilot_comb < num_tx:
        raise NotImplementedError("Least-Squares channel estimation of several streams needs a pilot comb")
    streams = [None] if num_tx == 1 and layout.spec.pilot_comb <= 1 else list(range(num_tx))
    return np.stack([np.stack([ls_estimate(layout, g, s) for s in streams]) for g in grids])


def tap_statistics(config: fading.FadingConfig, fs: float, N: int) -> tuple[np.ndarray, np.ndarray, callable]:
    """Distinct tap delays (samples, < N), their powers E|g|^2 and a function
    rho(u, dt) giving each delay's time correlation at lag dt samples."""

    d = config.delay_samples(fs)
    los_g, nlos_g = config.gains()
    power = config.gain * config.power_profile
    w_n = config.doppler_frequency / fs  # rad/sample: the model has no 2 pi (fading.py:307-343)
    w_l = config.los_doppler / fs
    S = config.num_sinusoids
    delays = np.unique(d[d < N])
    P = np.array([power[d == u].sum() for u in delays])

    def rho(ui: int, dt: np.ndarray) -> np.ndarray:
        sel = d == delays[ui]
        num = sum(power[l] * (S * nlos_g[l] ** 2 * j0(w_n * dt) + los_g[l] ** 2 * j0(w_l * dt))
                  for l in np.nonzero(sel)[0])
        return num / P[ui] if P[ui] > 0 else np.zeros_like(dt, dtype=float)

    return delays, P, rho


def tap_lmmse_estimate(layout: FrameLayout, grids: np.ndarray, config: fading.FadingConfig, fs: float,
                       noise_variance: float, num_tx: int, ridge_noise: float = 0.0) -> np.ndarray:
    """(Nrx, words, N) received grids -> (Nrx, Ntx, words, N) LMMSE channel estimate.

    ``ridge_noise`` > 0 regularizes each pilot word's tap estimate with the profile of
    ``config`` as prior, (A^H A + ridge_noise diag(1 / P_u))^-1 A^H y, and takes the
    per-tap noise variance of that estimate as noise_variance diag(M^-1 A^H A M^-1):
    the robust (design-statistics) estimator, whose dense delay grid makes A^H A
    ill-conditioned on a partly occupied band."""

    N = layout.N
    delays, P, rho = tap_statistics(config, fs, N)
    U = delays.size
    bins = layout.bins()
    W = layout.num_words
    centres = layout.window_start.astype(float)
    streams = [None] if num_tx == 1 and layout.spec.pilot_comb <= 1 else list(range(num_tx))
    out = np.zeros((grids.shape[0], len(streams), W, N), dtype=np.complex128)
    F_all = np.exp(-2j * np.pi * np.outer(bins, delays) / N)  # (N columns, U)
    for ti, s in enumerate(streams):
        ref, pilots, _ = _stream_refs(layout, s)
        rw, rc = np.nonzero(ref)  # frame order
        words = np.unique(rw)
        g_ls = np.zeros((grids.shape[0], words.size, U), dtype=np.complex128)
        e = np.zeros((words.size, U))
        for pi, w in enumerate(words):
            sel = rw == w
            A = pilots[sel][:, None] * F_all[rc[sel]]  # (n_p, U)
            AhA = A.conj().T @ A
            if ridge_noise > 0:
                inv = np.linalg.inv(AhA + np.diag(ridge_noise / np.maximum(P, 1e-300)))
                e[pi] = noise_variance * np.real(np.diag(inv @ AhA @ inv))
            else:
                inv = np.linalg.inv(AhA)
                e[pi] = noise_variance * np.real(np.diag(inv))
            G = inv @ A.conj().T  # (regularized) weighted LS of the tap gains
            for r in range(grids.shape[0]):
                g_ls[r, pi] = G @ grids[r, w, rc[sel]]
        taps = np.zeros((grids.shape[0], W, U), dtype=np.complex128)
        for u in range(U):
            dt_pp = centres[words][:, None] - centres[words][None, :]
            R = P[u] * rho(u, dt_pp) + np.diag(e[:, u])
            r = P[u] * rho(u, centres[:, None] - centres[words][None, :])  # (W, pilots words)
            C = np.linalg.solve(R.T, r.T).T if P[u] > 0 else np.zeros_like(r)
            taps[:, :, u] = g_ls[:, :, u] @ C.T
        out[:, ti] = taps @ F_all.T
    return out


def nmse_db(est: np.ndarray, truth: np.ndarray, mask: np.ndarray | None = None) -> float:
    """10 log10(sum |est - truth|^2 / sum |truth|^2) over the masked grid elements."""

    if mask is not None:
        est, truth = est[..., mask], truth[..., mask]
    return 10 * np.log10(np.sum(np.abs(est - truth) ** 2) / np.sum(np.abs(truth) ** 2))


def ideal_csi(layout: FrameLayout, sample: fading.FadingSample, fs: float) -> np.ndarray:
    """(Nrx, Ntx, words, N) frequency-domain channel state."""

    T = layout.samples_per_frame
    # state(...) = spatial (x) siso: average and transform the shared SISO response,
    # then scale by every pair's spatial coefficient (same values, no Nrx*Ntx*T*taps array)
    siso = fading.siso_state(sample, T, fs, T)  # (T, taps)
    n = layout.N
    num_taps = siso.shape[1]
    out = np.empty(sample.spatial.shape + (layout.num_words, n), dtype=np.complex128)
    bins = layout.bins()
    for w in range(layout.num_words):
        s = int(layout.window_start[w])
        avg = siso[s : s + n, :].mean(axis=0)  # (taps,)
        padded = np.zeros(n, dtype=np.complex128)
        padded[: min(num_taps, n)] = avg[:n]
        spec = np.fft.fft(padded)
        out[:, :, w, :] = sample.spatial[:, :, None] * spec[bins][None, None, :]
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
