"""GPU: batched LDPC encoding and belief-propagation decoding (hpx_ldpc_*) against the
oracle on the parity-check matrix the reference ships (tests/golden/ldpc.npz), plus the
reference's own LDPC checks (tests/unit_tests/fec/test_ldpc.py: encode / flip / decode,
pickling, iteration validation) and the coding pipeline (fec/coding.py)."""

import pickle

import numpy as np
import pytest
import torch

from hermespy_gb300 import EncoderManager, LDPCCoding
from oracle import ldpc
from tests.gpu_util import host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def code(golden):
    g = golden("ldpc.npz")
    return LDPCCoding.from_edges(int(g["N"]), int(g["M"]), g["edge_var"], g["edge_chk"], 100, True, 10)


@pytest.fixture(scope="module")
def h(golden):
    g = golden("ldpc.npz")
    return ldpc.dense_h(int(g["N"]), int(g["M"]), g["edge_var"], g["edge_chk"])


def test_systematic_layout(code, h):
    info, _, _ = ldpc.systematic(h)
    assert (code.bit_block_size, code.code_block_size) == (64, 128) and code.rate == 0.5
    np.testing.assert_array_equal(code.info_positions, info)


@pytest.mark.parametrize("B", [1, 9, 1000])
def test_encode_bit_exact(code, h, B):
    rng = np.random.default_rng(B)
    data = rng.integers(0, 2, (B, 64)).astype(np.uint8)
    got = host(code.encode_device(torch.from_numpy(data)))
    np.testing.assert_array_equal(got, ldpc.encode(h, data))


def test_hard_decode_matches_oracle(code, h):
    rng = np.random.default_rng(7)
    B = 40
    data = rng.integers(0, 2, (B, 64)).astype(np.uint8)
    cw = ldpc.encode(h, data)
    rx = cw.copy()
    for b in range(B):
        rx[b, rng.choice(128, 1 + b % 4, replace=False)] ^= 1
    out, used = code.decode_device(code=torch.from_numpy(rx), iterations_used=True)
    out, used = host(out), host(used)
    info, _, _ = ldpc.systematic(h)
    for b in range(B):
        hard, it = ldpc.decode(h, ldpc.hard_llr(rx[b]), 100, True, 10)
        np.testing.assert_array_equal(out[b], hard[info])
        assert used[b] == it


def test_soft_decode_matches_oracle(code, h):
    """BPSK over AWGN at 1-4 dB: wherever the float64 oracle converges to a codeword the
    FP32 decoder returns the same data bits (a slowly converging block may need a few
    iterations more or less; blocks that never satisfy the checks follow chaotic message
    trajectories and are only counted)."""

    rng = np.random.default_rng(11)
    B = 80
    data = rng.integers(0, 2, (B, 64)).astype(np.uint8)
    cw = ldpc.encode(h, data)
    info, _, _ = ldpc.systematic(h)
    snr = 10 ** (rng.uniform(1.0, 4.0, (B, 1)) / 10)
    sigma2 = 1.0 / snr
    y = (1.0 - 2.0 * cw) + np.sqrt(sigma2) * rng.standard_normal(cw.shape)
    llr = (2.0 * y / sigma2).astype(np.float32)
    out, used = code.decode_device(llr=torch.from_numpy(llr), iterations_used=True)
    out, used = host(out), host(used)
    converged = 0
    for b in range(B):
        hard, it = ldpc.decode(h, llr[b].astype(np.float64), 100, True, 10)
        if np.any((h.astype(np.int64) @ hard) % 2):
            continue
        converged += 1
        np.testing.assert_array_equal(out[b], hard[info])
        assert used[b] < 100
    assert converged >= B // 2


def test_reference_encode_flip_decode(code):
    """tests/unit_tests/fec/test_ldpc.py:50-70 on the shipped code: 20 blocks, one bit
    flipped each, no residual error."""

    rng = np.random.default_rng(42)
    errors = 0
    for _ in range(20):
        block = rng.integers(0, 2, code.bit_block_size, dtype=np.int32)
        flip = rng.integers(0, code.bit_block_size, dtype=np.int32)
        cw = code.encode(block)
        cw[flip] = not bool(cw[flip])
        errors += np.sum(block != code.decode(cw))
    assert errors < 1


def test_pickle_and_validation(code):
    again = pickle.loads(pickle.dumps(code))
    assert again.num_iterations == 100 and again.bit_block_size == 64
    block = np.random.default_rng(1).integers(0, 2, 64, dtype=np.int32)
    np.testing.assert_array_equal(again.decode(again.encode(block)), block)
    with pytest.raises(ValueError):
        code.num_iterations = 0
    with pytest.raises(ValueError):
        code.encode(np.zeros(10))


def test_encoder_manager_pads_and_truncates(code):
    m = EncoderManager(seed=5)
    m.add_encoder(code)
    assert m.bit_block_size == 64 and m.code_block_size == 128 and m.rate == 0.5
    bits = np.random.default_rng(2).integers(0, 2, 150).astype(bool)
    coded = m.encode(bits, 3 * 128)
    assert coded.size == 384
    np.testing.assert_array_equal(m.decode(coded, 150), bits)
    assert m.required_num_data_bits(400) == 192
