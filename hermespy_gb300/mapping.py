"""Gray PSK/QAM mapping on the GPU.

``PskQamMapping`` mirrors the reference class (modem/tools/psk_qam_mapping.py:20-538)
for the default complex constellations (BPSK, QPSK, 16-, 64-, 256-QAM):
``get_symbols`` maps MSB-first bit groups with the 3GPP amplitudes;
``detect_bits`` returns hard decisions that equal the reference's ``llr > 0``
evaluated in float64 on the same float32 symbols (ties and NaN give 0).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .containers import to_device, to_numpy


class PskQamMapping:
    mapping_available = [2, 4, 16, 64, 256]

    def __init__(self, modulation_order: int, mapping: np.ndarray | None = None, soft_output: bool = False,
                 is_complex: bool = True) -> None:
        if modulation_order <= 0 or (modulation_order & (modulation_order - 1)) != 0:
            raise ValueError("modulation_order must be a power of two")
        if mapping is not None or not is_complex:
            raise NotImplementedError("only the default complex 3GPP constellations run on the engine")
        if soft_output:
            raise NotImplementedError("soft-output demapping is not part of the engine's hot path")
        if modulation_order not in self.mapping_available:
            raise ValueError("constellation must be provided for this modulation order")
        self.modulation_order = int(modulation_order)
        self.bits_per_symbol = int(np.log2(modulation_order))
        self.is_complex = True
        self.soft_output = False
        self.mapping = None

    def get_symbols_device(self, bits: torch.Tensor) -> torch.Tensor:
        bits = to_device(bits, torch.uint8).reshape(-1)
        n = bits.numel() // self.bits_per_symbol
        out = torch.empty(n, dtype=torch.complex64, device=bits.device)
        _lib.call("hpx_qam_map", self.modulation_order, _lib.ptr(bits), n, _lib.ptr(out), _lib.stream_ptr())
        return out

    def get_symbols(self, bits) -> np.ndarray:
        return to_numpy(self.get_symbols_device(bits))

    def detect_bits_device(self, symbols) -> torch.Tensor:
        s = to_device(symbols).reshape(-1)
        out = torch.empty(s.numel() * self.bits_per_symbol, dtype=torch.uint8, device=s.device)
        _lib.call("hpx_qam_demap", self.modulation_order, _lib.ptr(s), s.numel(), _lib.ptr(out), _lib.stream_ptr())
        return out

    def detect_bits(self, rx_symbols, noise_variance=1.0) -> np.ndarray:
        return to_numpy(self.detect_bits_device(rx_symbols))

    def get_mapping(self) -> np.ndarray:
        m = self.bits_per_symbol
        idx = np.arange(self.modulation_order)
        bits = ((idx[:, None] >> (m - 1 - np.arange(m))[None, :]) & 1).astype(np.uint8).reshape(-1)
        return self.get_symbols(bits)
