"""ctypes binding of the engine's C ABI (include/hpx.h).

The CUDA library is loaded from the package directory (``libhpx.so``, built by
``hermespy_gb300.build``). There is no CPU fallback: if the library or a CUDA
device is missing, every engine call raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhpx.so")

HPX_OK, HPX_ERR_ARG, HPX_ERR_SHAPE, HPX_ERR_UNSUPPORTED, HPX_ERR_CUDA, HPX_ERR_NUMERIC, HPX_ERR_TIMEOUT = range(7)
RE_REFERENCE, RE_DATA, RE_NULL = 0, 1, 2
EQ_ZF, EQ_LMMSE = 0, 1
EST_IDEAL, EST_LS = 0, 1
# flag bits of the per-drop error words (a flagged drop holds no valid count)
DROP_TIMEOUT, DROP_NUMERIC, DROP_COUNT = 0x80000000, 0x40000000, 0x3FFFFFFF

c_void_p = ctypes.c_void_p
c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_uint64 = ctypes.c_uint64
c_double = ctypes.c_double


class FrameDesc(ctypes.Structure):
    _fields_ = [
        ("num_subcarriers", c_int32),
        ("num_words", c_int32),
        ("num_columns", c_int32),
        ("modulation_order", c_int32),
        ("dc_suppression", c_int32),
        ("prefix", ctypes.POINTER(c_int32)),
        ("zero_prefix", ctypes.POINTER(c_int32)),
        ("kind", ctypes.POINTER(ctypes.c_int8)),
        ("pilot_comb", c_int32),
    ]


class FrameInfo(ctypes.Structure):
    _fields_ = [
        ("num_subcarriers", c_int32),
        ("num_words", c_int32),
        ("num_columns", c_int32),
        ("modulation_order", c_int32),
        ("bits_per_symbol", c_int32),
        ("num_data", c_int32),
        ("num_refs", c_int32),
        ("samples_per_frame", c_int32),
    ]


class FadingDesc(ctypes.Structure):
    _fields_ = [
        ("num_taps", c_int32),
        ("num_sinusoids", c_int32),
        ("num_rx", c_int32),
        ("num_tx", c_int32),
        ("sampling_rate", c_double),
        ("doppler_frequency", c_double),
        ("los_doppler_frequency", c_double),
        ("gain", c_double),
        ("delays", ctypes.POINTER(c_double)),
        ("power_profile", ctypes.POINTER(c_double)),
        ("rice_factors", ctypes.POINTER(c_double)),
        ("rx_correlation", ctypes.POINTER(c_double)),
        ("tx_correlation", ctypes.POINTER(c_double)),
        ("los_gains", ctypes.POINTER(c_double)),
        ("nlos_gains", ctypes.POINTER(c_double)),
    ]


# name: argument types (all return int32 status)
_SIGNATURES = {
    "hpx_frame_create": [ctypes.POINTER(FrameDesc), ctypes.POINTER(c_void_p)],
    "hpx_frame_destroy": [c_void_p],
    "hpx_frame_get_info": [c_void_p, ctypes.POINTER(FrameInfo)],
    "hpx_bits_generate": [c_uint64, c_int64, c_int32, c_int32, c_int64, c_void_p, c_void_p],
    "hpx_qam_map": [c_int32, c_void_p, c_int64, c_void_p, c_void_p],
    "hpx_qam_demap": [c_int32, c_void_p, c_int64, c_void_p, c_void_p],
    "hpx_count_errors": [c_void_p, c_int64, c_void_p, c_int64, c_int32, c_void_p, c_void_p],
    "hpx_ofdm_modulate": [c_void_p, c_void_p, c_int32, c_void_p, c_void_p],
    "hpx_ofdm_modulate_grid": [c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_ofdm_modulate_bits": [c_void_p, c_uint64, c_int64, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_ofdm_demodulate": [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_ofdm_pick": [c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_fading_create": [ctypes.POINTER(FadingDesc), ctypes.POINTER(c_void_p)],
    "hpx_fading_destroy": [c_void_p],
    "hpx_fading_state_bytes": [c_void_p, c_int32, ctypes.POINTER(c_int64)],
    "hpx_fading_max_delay": [c_void_p, ctypes.POINTER(c_int32)],
    "hpx_fading_realize": [c_void_p, c_uint64, c_int64, c_int32, c_void_p, c_void_p],
    "hpx_fading_load": [c_void_p, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "hpx_fading_draws": [c_void_p, c_uint64, c_int64, c_int32, c_void_p, c_void_p],
    "hpx_fading_taps": [c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_fading_csi": [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_fading_propagate": [c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_void_p, c_void_p, c_uint64, c_int64,
                             c_void_p],
    "hpx_fading_ideal_csi": [c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_void_p, c_void_p],
    "hpx_ls_create": [c_void_p, c_int32, c_void_p, c_void_p, c_void_p, ctypes.POINTER(c_void_p)],
    "hpx_ls_destroy": [c_void_p],
    "hpx_ls_estimate": [c_void_p, c_void_p, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_equalize": [c_int32, c_int32, c_int32, c_int64, c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "hpx_detect_ideal": [c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_void_p, c_uint64, c_int64,
                         c_int32, c_void_p, c_void_p],
    "hpx_awgn_add": [c_void_p, c_int32, c_int32, c_int64, c_void_p, c_uint64, c_int64, c_void_p],
    "hpx_sync_schmidl_cox": [c_void_p, c_int32, c_int32, c_int64, c_int32, c_void_p, c_void_p],
    "hpx_sync_correlation": [c_void_p, c_int32, c_int32, c_int64, c_void_p, c_int32, c_void_p, c_void_p],
    "hpx_ldpc_create": [c_int32, c_int32, c_int32, c_void_p, c_void_p, ctypes.POINTER(c_void_p)],
    "hpx_ldpc_destroy": [c_void_p],
    "hpx_ldpc_info": [c_void_p, ctypes.POINTER(c_int32), ctypes.POINTER(c_int32), c_void_p],
    "hpx_ldpc_encode": [c_void_p, c_void_p, c_int32, c_void_p, c_void_p],
    "hpx_ldpc_decode": [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "hpx_sync_peaks": [c_void_p, c_int32, c_int64, c_int32, ctypes.c_double, c_int64, c_int64, c_int32, c_int64,
                       c_int64, c_int32, c_void_p, c_void_p, c_void_p],
    "hpx_link_workspace_bytes": [c_void_p, c_void_p, c_int32, ctypes.POINTER(c_int64)],
    "hpx_link_create": [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, ctypes.POINTER(c_void_p)],
    "hpx_link_destroy": [c_void_p],
    "hpx_link_run": [c_void_p, c_uint64, c_int64, c_int32, c_void_p, c_void_p, c_void_p],
    "hpx_link_run_static": [c_void_p, c_void_p, c_void_p, c_int32, c_uint64, c_int64, c_int32, c_void_p, c_void_p,
                            c_void_p],
    "hpx_detect_ls": [c_void_p, c_int32, c_void_p, c_int32, c_void_p, c_uint64, c_int64, c_int32, c_void_p, c_void_p],
    "hpx_ls_create_streams": [c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p],
    "hpx_ls_estimate_streams": [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p],
    "hpx_lmmse_create": [c_void_p, c_void_p, c_int32, c_void_p],
    "hpx_lmmse_create_regularized": [c_void_p, c_void_p, c_int32, c_double, c_void_p],
    "hpx_lmmse_destroy": [c_void_p],
    "hpx_lmmse_estimate": [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "hpx_csi_error": [c_void_p, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p],
    "hpx_cnn_num_params": [],
    "hpx_cnn_create": [c_int32, c_int32, c_int32, c_void_p, c_uint64, c_void_p],
    "hpx_cnn_destroy": [c_void_p],
    "hpx_cnn_get_params": [c_void_p, c_void_p],
    "hpx_cnn_get_grads": [c_void_p, c_void_p],
    "hpx_cnn_refine": [c_void_p, c_void_p, c_int32, c_int32, c_void_p],
    "hpx_cnn_train_step": [c_void_p, c_void_p, c_void_p, c_int32, c_int32, ctypes.c_float, c_void_p, c_void_p],
    "hpx_detect_massive": [c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_void_p, c_uint64, c_int64,
                           c_int32, c_void_p, c_void_p, c_void_p, c_void_p],
    "hpx_campaign_create": [c_int32, c_void_p, c_double, c_double, c_int32, c_int64, c_int32, c_double, c_void_p],
    "hpx_campaign_destroy": [c_void_p],
    "hpx_campaign_reset": [c_void_p],
    "hpx_campaign_run": [c_void_p, c_void_p, c_uint64, c_int64, c_int32, c_int32, c_int32, c_void_p, c_void_p,
                         c_void_p],
    "hpx_campaign_results": [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "hpx_detect_lmmse": [c_void_p, c_int32, c_int32, c_void_p, c_int32, c_void_p, c_uint64, c_int64, c_int32, c_void_p,
                         c_void_p],
    "hpx_uneven_create": [c_void_p, c_int32, c_double, c_double, c_int32, c_int32, c_void_p],
    "hpx_uneven_destroy": [c_void_p],
    "hpx_uneven_bits": [c_void_p, c_void_p],
    "hpx_uneven_config": [c_void_p, c_int32, c_int32, c_int32],
    "hpx_uneven_get_config": [c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p],
    "hpx_uneven_run": [c_void_p, c_uint64, c_int64, c_void_p, c_void_p, c_void_p],
    "hpx_uneven_capture": [c_void_p, c_uint64, c_int64, c_void_p, c_void_p],
    "hpx_uneven_replay": [c_void_p, c_void_p],
    "hpx_detect_csi": [c_void_p, c_int32, c_int32, c_int32, c_void_p, c_int32, c_void_p, c_int32, c_void_p, c_uint64,
                       c_int64, c_int32, c_void_p, c_void_p],
    "hpx_drop_status": [c_void_p, c_int64],
    "hpx_campaign_assign": [c_void_p, c_int32, c_void_p, c_void_p],
    "hpx_campaign_accumulate": [c_void_p, c_int32, c_void_p, c_void_p],
    "hpx_campaign_poll": [c_void_p, ctypes.POINTER(c_int32), c_void_p],
    "hpx_lmmse_status": [c_void_p, c_int32, c_void_p],
    "hpx_lmmse_inject_timeout": [c_void_p, c_void_p],
    "hpx_cnn_status": [c_void_p, c_int32, c_void_p],
    "hpx_cnn_inject_timeout": [c_void_p, c_void_p],
}

_lock = threading.Lock()
_lib = None


def exported_symbols() -> list[str]:
    """Every entry point the header declares (used by the ABI tests)."""

    return ["hpx_version", "hpx_last_error", *_SIGNATURES.keys()]


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load (once) and return the engine library. Raises if it was not built."""

    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"engine library {path} is missing; build it with `python -m hermespy_gb300.build` "
                "(the engine has no CPU fallback)"
            )
        lib = ctypes.CDLL(path)
        lib.hpx_version.restype = ctypes.c_int
        lib.hpx_version.argtypes = []
        lib.hpx_last_error.restype = ctypes.c_char_p
        lib.hpx_last_error.argtypes = []
        for name, args in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = c_int32
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int) -> None:
    """Map a status code to the reference's exception types."""

    if status == HPX_OK:
        return
    msg = _lib.hpx_last_error().decode() if _lib is not None else f"status {status}"
    if status in (HPX_ERR_ARG, HPX_ERR_SHAPE):
        raise ValueError(msg)
    if status == HPX_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)


def drop_counts(errors) -> "np.ndarray":
    """Host per-drop error words (any integer array of the device's uint32 words) ->
    int64 bit-error counts. Raises RuntimeError (through hpx_drop_status) if a drop
    carries a failure flag: a bounded device wait ran out (HPX_DROP_TIMEOUT) or its
    equalizer met a non-finite pivot (HPX_DROP_NUMERIC); such a drop has no count,
    so nothing may be summed."""

    import numpy as np

    words = np.ascontiguousarray(np.asarray(errors).astype(np.int64) & 0xFFFFFFFF, dtype=np.uint32)
    check(load().hpx_drop_status(words.ctypes.data_as(c_void_p), words.size))
    return words.astype(np.int64)


def call(name: str, *args) -> None:
    lib = load()
    check(getattr(lib, name)(*args))


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("the engine needs a CUDA device (GB300); no CPU fallback exists")
    load()
    return torch.device("cuda", torch.cuda.current_device())


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("engine buffers must be CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("engine buffers must be contiguous")
    return t.data_ptr()


def stream_ptr(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
