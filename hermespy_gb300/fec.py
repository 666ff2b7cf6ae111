"""Forward error correction of the drop-in API: the coding pipeline and LDPC codes.

Mirrors ``hermespy/fec/coding.py`` (``Encoder`` :22-155, ``EncoderManager`` :158-480)
and the aff3ct LDPC wrapper (``fec/aff3ct/ldpc.cpp``, ``fec/aff3ct_wrappers.py``
``LDPCCoding``): ``LDPCCoding(num_iterations, h_source_path, g_save_path,
enable_syndrome_checking, min_num_iterations)`` reads the parity-check matrix from an
alist file; ``encode`` / ``decode`` take one block of bits as the reference does, and
``encode_device`` / ``decode_device`` run batches of blocks on the GPU
(``hpx_ldpc_encode`` / ``hpx_ldpc_decode``). The encoder is systematic (data bits at
the non-pivot columns of H's reduced row-echelon form); the decoder is flooding
belief propagation with the sum-product check update; hard input (the wrapper's
hard-in / hard-out decode) becomes channel LLRs +-4. aff3ct's own sources are not
available, so codewords, the hard-input LLR magnitude and iteration details follow the
published algorithms rather than aff3ct bit for bit.
"""

from __future__ import annotations

import ctypes
import os
from math import ceil

import numpy as np
import torch

from . import _lib
from .containers import to_device, to_numpy


class Encoder:
    """One coding step of a pipeline (coding.py:22-155)."""

    def __init__(self, manager: "EncoderManager | None" = None) -> None:
        self._manager = None
        self.enabled = True
        if manager is not None:
            self.manager = manager

    @property
    def manager(self) -> "EncoderManager | None":
        return self._manager

    @manager.setter
    def manager(self, value: "EncoderManager | None") -> None:
        self._manager = value

    def encode(self, bits: np.ndarray) -> np.ndarray:  # pragma: no cover - interface
        raise NotImplementedError

    def decode(self, encoded_bits: np.ndarray) -> np.ndarray:  # pragma: no cover - interface
        raise NotImplementedError

    @property
    def bit_block_size(self) -> int:  # pragma: no cover - interface
        raise NotImplementedError

    @property
    def code_block_size(self) -> int:  # pragma: no cover - interface
        raise NotImplementedError

    @property
    def rate(self) -> float:
        return self.bit_block_size / self.code_block_size


def read_alist(path: str) -> tuple[int, int, np.ndarray, np.ndarray]:
    """(N, M, edge variables, edge checks) of the parity-check matrix in an alist file
    (N M, maximum degrees, column and row degrees, then one line per column with its
    1-based check indices, zero entries padding it to the maximum degree)."""

    with open(path) as f:
        lines = [ln.split() for ln in f.read().splitlines() if ln.strip()]
    if len(lines) < 4 or len(lines[0]) < 2:
        raise ValueError(f"{path} is not an alist file")
    N, M = int(lines[0][0]), int(lines[0][1])
    if len(lines) < 4 + N:
        raise ValueError(f"{path} lists fewer than {N} columns")
    ev, ec = [], []
    for v in range(N):  # one line per column, zero entries pad to the maximum degree
        for t in lines[4 + v]:
            if int(t) > 0:
                ev.append(v)
                ec.append(int(t) - 1)
    return N, M, np.asarray(ev, np.int32), np.asarray(ec, np.int32)


class LDPCCoding(Encoder):
    """LDPC block code decoded by belief propagation (fec/aff3ct/ldpc.cpp:20-126)."""

    def __init__(self, num_iterations: int, h_source_path: str, g_save_path: str = "",
                 enable_syndrome_checking: bool = True, min_num_iterations: int = 10) -> None:
        Encoder.__init__(self)
        if num_iterations < 1:
            raise ValueError("Number of decoding iterations must be greater than zero")
        self._num_iterations = int(num_iterations)
        self.h_source_path = h_source_path
        self.g_save_path = g_save_path
        self.enable_syndrome_checking = bool(enable_syndrome_checking)
        self.min_num_iterations = int(min_num_iterations)
        N, M, ev, ec = read_alist(h_source_path)
        self._create(N, M, ev, ec)
        if g_save_path:
            self._save_generator(g_save_path)

    @classmethod
    def from_edges(cls, N: int, M: int, edge_var, edge_chk, num_iterations: int = 100,
                   enable_syndrome_checking: bool = True, min_num_iterations: int = 10) -> "LDPCCoding":
        """A code from the edges of its parity-check matrix (no alist file)."""

        obj = cls.__new__(cls)
        Encoder.__init__(obj)
        if num_iterations < 1:
            raise ValueError("Number of decoding iterations must be greater than zero")
        obj._num_iterations = int(num_iterations)
        obj.h_source_path, obj.g_save_path = "", ""
        obj.enable_syndrome_checking = bool(enable_syndrome_checking)
        obj.min_num_iterations = int(min_num_iterations)
        obj._create(int(N), int(M), np.asarray(edge_var, np.int32), np.asarray(edge_chk, np.int32))
        return obj

    @classmethod
    def ofdm_code(cls, num_iterations: int = 100, enable_syndrome_checking: bool = True,
                  min_num_iterations: int = 10) -> "LDPCCoding":
        """The (128, 64) code of the reference's 5G NR OFDM modem resources
        (modem/resources/ofdm_ldpc.alist), shipped as the edges of its parity-check
        matrix in ``codes/ofdm_ldpc.npz``."""

        z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "codes", "ofdm_ldpc.npz"))
        return cls.from_edges(int(z["N"]), int(z["M"]), z["edge_var"], z["edge_chk"], num_iterations,
                              enable_syndrome_checking, min_num_iterations)

    def _create(self, N: int, M: int, ev: np.ndarray, ec: np.ndarray) -> None:
        lib = _lib.load()
        self.device = _lib.require_cuda()
        ev = np.ascontiguousarray(ev, np.int32)
        ec = np.ascontiguousarray(ec, np.int32)
        h = ctypes.c_void_p()
        _lib.check(lib.hpx_ldpc_create(N, M, len(ev), ev.ctypes.data_as(ctypes.c_void_p),
                                       ec.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)))
        self.handle = h
        k, n = ctypes.c_int32(), ctypes.c_int32()
        _lib.call("hpx_ldpc_info", h, ctypes.byref(k), ctypes.byref(n), None)
        self._K, self._N = int(k.value), int(n.value)
        info = np.empty(self._K, np.int32)
        _lib.call("hpx_ldpc_info", h, None, None, info.ctypes.data_as(ctypes.c_void_p))
        self.info_positions = info
        self._edges = (N, M, ev, ec)

    def _save_generator(self, path: str) -> None:
        """The systematic generator matrix (K x N, rows = unit data vectors encoded) in alist format."""

        eye = np.eye(self._K, dtype=np.uint8)
        g = self.encode_device(torch.from_numpy(eye)).cpu().numpy()
        rows = [np.nonzero(g[i])[0] + 1 for i in range(self._K)]
        cols = [np.nonzero(g[:, j])[0] + 1 for j in range(self._N)]
        with open(path, "w") as f:
            f.write(f"{self._N} {self._K}\n{max(len(c) for c in cols)} {max(len(r) for r in rows)}\n")
            f.write(" ".join(str(len(c)) for c in cols) + "\n")
            f.write(" ".join(str(len(r)) for r in rows) + "\n")
            for c in cols:
                f.write(" ".join(map(str, c)) + "\n")
            for r in rows:
                f.write(" ".join(map(str, r)) + "\n")

    def __del__(self):
        try:
            if _lib._lib is not None and getattr(self, "handle", None) is not None:
                _lib._lib.hpx_ldpc_destroy(self.handle)
        except Exception:
            pass

    def __getstate__(self):
        return (self._num_iterations, self._edges, self.enable_syndrome_checking, self.min_num_iterations)

    def __setstate__(self, state):
        it, (N, M, ev, ec), syn, mn = state
        Encoder.__init__(self)
        self._num_iterations, self.enable_syndrome_checking, self.min_num_iterations = it, syn, mn
        self.h_source_path, self.g_save_path = "", ""
        self._create(N, M, ev, ec)

    @property
    def num_iterations(self) -> int:
        return self._num_iterations

    @num_iterations.setter
    def num_iterations(self, value: int) -> None:
        if value < 1:
            raise ValueError("Number of decoding iterations must be greater than zero")
        self._num_iterations = int(value)

    @property
    def bit_block_size(self) -> int:
        return self._K

    @property
    def code_block_size(self) -> int:
        return self._N

    @property
    def rate(self) -> float:
        return self._K / self._N

    # ----------------------------------------------------------------- batches
    def encode_device(self, data: torch.Tensor) -> torch.Tensor:
        """(B, K) bits -> (B, N) code bits, uint8 on the GPU."""

        d = to_device(data, torch.uint8).reshape(-1, self._K).contiguous()
        out = torch.empty((d.shape[0], self._N), dtype=torch.uint8, device=d.device)
        for b0 in range(0, d.shape[0], 65535):
            n = min(65535, d.shape[0] - b0)
            _lib.call("hpx_ldpc_encode", self.handle, _lib.ptr(d[b0:]), n, _lib.ptr(out[b0:]), _lib.stream_ptr())
        return out

    def decode_device(self, code: torch.Tensor | None = None, llr: torch.Tensor | None = None,
                      iterations_used: bool = False):
        """(B, N) hard code bits or channel LLRs -> (B, K) data bits (and the iterations run)."""

        if (code is None) == (llr is None):
            raise ValueError("decode needs either hard code bits or channel LLRs")
        if llr is not None:
            x = to_device(llr, torch.float32).reshape(-1, self._N).contiguous()
        else:
            x = to_device(code, torch.uint8).reshape(-1, self._N).contiguous()
        B = x.shape[0]
        out = torch.empty((B, self._K), dtype=torch.uint8, device=x.device)
        used = torch.empty(B, dtype=torch.int32, device=x.device) if iterations_used else None
        _lib.call("hpx_ldpc_decode", self.handle, None if llr is not None else _lib.ptr(x),
                  _lib.ptr(x) if llr is not None else None, B, self._num_iterations,
                  int(self.enable_syndrome_checking), self.min_num_iterations, _lib.ptr(out), _lib.ptr(used),
                  _lib.stream_ptr())
        return (out, used) if iterations_used else out

    # ------------------------------------------------------------ single block
    def encode(self, bits: np.ndarray) -> np.ndarray:
        bits = np.asarray(bits)
        if bits.size != self._K:
            raise ValueError(f"LDPC encoding expects blocks of {self._K} bits ({bits.size} given)")
        return to_numpy(self.encode_device(bits.astype(np.uint8).reshape(1, -1)))[0].astype(bits.dtype)

    def decode(self, encoded_bits: np.ndarray) -> np.ndarray:
        encoded_bits = np.asarray(encoded_bits)
        if encoded_bits.size != self._N:
            raise ValueError(f"LDPC decoding expects blocks of {self._N} bits ({encoded_bits.size} given)")
        out = self.decode_device(code=(encoded_bits != 0).astype(np.uint8).reshape(1, -1))
        return to_numpy(out)[0].astype(encoded_bits.dtype)


class EncoderManager:
    """Coding pipeline of encoders sorted by block size (coding.py:158-480)."""

    def __init__(self, allow_padding: bool = True, allow_truncating: bool = True, seed: int | None = None) -> None:
        self._encoders: list[Encoder] = []
        self.allow_padding = allow_padding
        self.allow_truncating = allow_truncating
        self._rng = np.random.default_rng(seed)

    def add_encoder(self, encoder: Encoder) -> None:
        encoder.manager = self
        self._encoders.append(encoder)
        self._encoders = sorted(self._encoders, key=lambda e: e.bit_block_size)

    @property
    def encoders(self) -> list[Encoder]:
        return self._encoders

    def encode(self, data_bits: np.ndarray, num_code_bits: int | None = None) -> np.ndarray:
        code_state = np.asarray(data_bits).copy()
        for encoder in self._encoders:
            if not encoder.enabled:
                continue
            k, n = encoder.bit_block_size, encoder.code_block_size
            num_blocks = ceil(len(code_state) / k)
            data_state = code_state
            if len(data_state) < num_blocks * k:
                if not self.allow_padding:
                    raise RuntimeError("Encoding would require padding, but padding is not allowed")
                data_state = np.append(data_state, self._rng.integers(0, 2, num_blocks * k - len(data_state),
                                                                      dtype=bool))
            if isinstance(encoder, LDPCCoding):  # every block in one launch
                code_state = to_numpy(encoder.encode_device(
                    data_state.astype(np.uint8).reshape(num_blocks, k))).reshape(-1).astype(bool)
            else:
                code_state = np.concatenate([encoder.encode(data_state[i * k:(i + 1) * k])
                                             for i in range(num_blocks)]).astype(bool)
        if num_code_bits and len(code_state) > num_code_bits:
            raise RuntimeError("Too many input bits provided for encoding, truncating would destroy information")
        if num_code_bits and len(code_state) < num_code_bits:
            if not self.allow_padding:
                raise RuntimeError("Encoding would require padding, but padding is not allowed")
            pad = num_code_bits - len(code_state)
            if pad >= self.code_block_size:
                raise ValueError("Insufficient number of input blocks provided for encoding")
            code_state = np.append(code_state, self._rng.integers(0, 2, pad, dtype=bool))
        return code_state

    def decode(self, encoded_bits: np.ndarray, num_data_bits: int | None = None) -> np.ndarray:
        encoded_bits = np.asarray(encoded_bits)
        num_blocks = int(encoded_bits.shape[0] / self.code_block_size)
        if num_data_bits is not None:
            full = num_blocks * self.bit_block_size
            if num_data_bits > full:
                raise RuntimeError("The requested number of data bits is larger than number of bits recovered "
                                   "by decoding")
            if not self.allow_truncating and num_data_bits != full:
                raise RuntimeError("Data truncating is required but not allowed")
        else:
            num_data_bits = num_blocks * self.bit_block_size
        data_state = encoded_bits.copy()
        for encoder in reversed(self._encoders):
            if not encoder.enabled:
                continue
            n, k = encoder.code_block_size, encoder.bit_block_size
            nb = int(len(data_state) / n)
            code_state = data_state[: nb * n]
            if isinstance(encoder, LDPCCoding):
                data_state = to_numpy(encoder.decode_device(
                    code=(code_state != 0).astype(np.uint8).reshape(nb, n))).reshape(-1).astype(bool)
            else:
                data_state = np.concatenate([encoder.decode(code_state[i * n:(i + 1) * n])
                                             for i in range(nb)]).astype(bool)
        return data_state[:num_data_bits]

    @property
    def bit_block_size(self) -> int:
        if not self._encoders:
            return 1
        idx, block, nbits = 0, 1, 1
        for idx, enc in enumerate(self._encoders):
            if enc.enabled:
                block, nbits = enc.bit_block_size, enc.code_block_size
                break
        for enc in self._encoders[idx + 1:]:
            if not enc.enabled:
                continue
            reps = int(enc.bit_block_size / nbits)
            block *= reps
            nbits *= int(reps / enc.rate)
        return block

    @property
    def code_block_size(self) -> int:
        for enc in reversed(self._encoders):
            if enc.enabled:
                return enc.code_block_size
        return 1

    @property
    def rate(self) -> float:
        r = 1.0
        for enc in self._encoders:
            if enc.enabled:
                r *= enc.rate
        return r

    def required_num_data_bits(self, num_code_bits: int) -> int:
        return self.bit_block_size * int(num_code_bits / self.code_block_size)

    def __getitem__(self, item: int) -> Encoder:
        return self._encoders[item]
