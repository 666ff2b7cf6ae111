"""GPU: Philox bits, QAM mapping and hard demapping against the oracle and the
reference's golden vectors (bit-exact)."""

import numpy as np
import pytest
import torch

from hermespy_gb300 import _lib
from oracle import mapping, streams
from tests.gpu_util import cf, host, stream, t

pytestmark = pytest.mark.gpu


def test_bits_match_oracle_stream():
    seed, drop0, nd, ns, nb = 0x1234_5678_9ABC_DEF0, 5, 3, 4, 10_001
    out = torch.empty((nd, ns, nb), dtype=torch.uint8, device="cuda")
    _lib.call("hpx_bits_generate", seed, drop0, nd, ns, nb, _lib.ptr(out), stream())
    got = host(out)
    for d in range(nd):
        for s in range(ns):
            np.testing.assert_array_equal(got[d, s], streams.data_bits(seed, drop0 + d, s, nb))


@pytest.mark.parametrize("order", [2, 4, 16, 64, 256])
def test_map_golden(golden, order):
    g = golden("qam.npz")
    bits = t(g[f"bits_{order}"], np.uint8)
    n = bits.numel() // int(np.log2(order))
    out = torch.empty(n, dtype=torch.complex64, device="cuda")
    _lib.call("hpx_qam_map", order, _lib.ptr(bits), n, _lib.ptr(out), stream())
    np.testing.assert_allclose(host(out), g[f"symbols_{order}"], rtol=0, atol=2e-7)


def _demap(order, sym):
    s = cf(sym)
    m = int(np.log2(order))
    out = torch.empty(s.numel() * m, dtype=torch.uint8, device="cuda")
    _lib.call("hpx_qam_demap", order, _lib.ptr(s), s.numel(), _lib.ptr(out), stream())
    return host(out)


@pytest.mark.parametrize("order", [2, 4, 16, 64, 256])
def test_demap_bit_exact(golden, order):
    """Hard decisions equal the reference's float64 llr > 0 on the same float32 symbols,
    including values within one ulp of every decision boundary, zeros, NaN and inf."""

    g = golden("qam.npz")
    pts = g[f"detect_in_{order}"].astype(np.complex64)
    scale = {2: 1.0, 4: np.sqrt(2), 16: np.sqrt(2) * np.sqrt(5), 64: np.sqrt(2) * np.sqrt(21),
             256: np.sqrt(2) * np.sqrt(85)}[order]
    edges = np.arange(-16, 17, dtype=np.float64) / scale
    e32 = edges.astype(np.float32)
    near = np.concatenate([e32, np.nextafter(e32, np.float32(np.inf)), np.nextafter(e32, np.float32(-np.inf))])
    extra = (near + 1j * near[::-1]).astype(np.complex64)
    special = np.array([np.nan + 0j, np.inf + 1j, -np.inf - 1j, complex(1.0, np.nan), 0j], dtype=np.complex64)
    allpts = np.concatenate([pts, extra, special])
    expect = mapping.detect_bits(order, allpts.astype(np.complex128))
    np.testing.assert_array_equal(_demap(order, allpts), expect)
    # the golden decisions on float64 inputs agree wherever float32 rounding cannot flip them
    ref = g[f"detect_out_{order}"]
    same = pts.astype(np.complex128) == g[f"detect_in_{order}"]
    m = int(np.log2(order))
    np.testing.assert_array_equal(_demap(order, pts).reshape(-1, m)[same], ref.reshape(-1, m)[same])


@pytest.mark.parametrize("order", [4, 16, 64, 256])
def test_map_demap_round_trip(order):
    m = int(np.log2(order))
    bits = np.random.default_rng(order).integers(0, 2, m * 5000).astype(np.uint8)
    b = t(bits)
    sym = torch.empty(5000, dtype=torch.complex64, device="cuda")
    _lib.call("hpx_qam_map", order, _lib.ptr(b), 5000, _lib.ptr(sym), stream())
    np.testing.assert_array_equal(_demap(order, host(sym)), bits)


def test_count_errors(golden):
    g = golden("ber.npz")
    for i in range(3):
        a, b = t(g[f"tx_{i}"], np.uint8), t(g[f"rx_{i}"], np.uint8)
        out = torch.empty(1, dtype=torch.int64, device="cuda")
        _lib.call("hpx_count_errors", _lib.ptr(a), a.numel(), _lib.ptr(b), b.numel(), 1, _lib.ptr(out), stream())
        assert int(host(out)[0]) == int(g[f"errors_{i}"].sum())


def test_empty_inputs_are_noops():
    _lib.call("hpx_qam_map", 16, None, 0, None, stream())
    _lib.call("hpx_bits_generate", 1, 0, 0, 1, 8, None, stream())
    out = torch.full((2,), 7, dtype=torch.int64, device="cuda")
    _lib.call("hpx_count_errors", None, 0, None, 0, 2, _lib.ptr(out), stream())
    assert host(out).tolist() == [0, 0]
