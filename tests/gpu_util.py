"""Helpers for the GPU parity tests: C-ABI calls on torch tensors and error metrics."""

import ctypes

import numpy as np
import torch

from hermespy_gb300 import _lib

DEV = "cuda"


def t(a, dtype=None):
    a = np.ascontiguousarray(a)
    if dtype is not None:
        a = a.astype(dtype)
    return torch.from_numpy(a).to(DEV)


def cf(a):
    return t(np.asarray(a).astype(np.complex64))


def host(x):
    torch.cuda.synchronize()
    return x.cpu().numpy()


def rel_rms(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.sqrt(np.sum(np.abs(a - b) ** 2) / max(np.sum(np.abs(b) ** 2), 1e-300)))


def frame_handle(layout):
    """hpx_frame for an oracle FrameLayout."""

    kind = np.ascontiguousarray(layout.kind[:, : layout.num_used].astype(np.int8))
    prefix = np.ascontiguousarray(layout.prefix.astype(np.int32))
    zero = np.ascontiguousarray(layout.zero_prefix.astype(np.int32))
    desc = _lib.FrameDesc(layout.N, layout.num_words, layout.num_used, layout.order, int(layout.spec.dc_suppression),
                          prefix.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                          zero.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                          kind.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), int(layout.spec.pilot_comb))
    h = ctypes.c_void_p()
    _lib.check(_lib.load().hpx_frame_create(ctypes.byref(desc), ctypes.byref(h)))
    return h


def fading_handle(cfg, nrx, ntx, fs):
    """hpx_fading (wrapped) for an oracle FadingConfig."""

    from hermespy_gb300.channel import _FadingHandle

    rx = None if cfg.rx_correlation is None else cfg.rx_correlation[:nrx, :nrx]
    tx = None if cfg.tx_correlation is None else cfg.tx_correlation[:ntx, :ntx]
    return _FadingHandle(cfg.delays, cfg.power_profile, cfg.rice_factors, cfg.num_sinusoids, cfg.doppler_frequency,
                         cfg.los_doppler, cfg.gain, nrx, ntx, fs, rx, tx)


def stream():
    return _lib.stream_ptr()
