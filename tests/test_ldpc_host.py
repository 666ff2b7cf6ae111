"""CPU: the oracle's LDPC code on the parity-check matrix the reference ships
(tests/golden/ldpc.npz from modem/resources/ofdm_ldpc.alist): systematic encoding
satisfies every check, and belief propagation corrects the single bit errors the
reference's own LDPC test flips (tests/unit_tests/fec/test_ldpc.py:50-70), and more."""

import numpy as np
import pytest

from hermespy_gb300.fec import read_alist
from oracle import ldpc


def _h(golden):
    g = golden("ldpc.npz")
    return ldpc.dense_h(int(g["N"]), int(g["M"]), g["edge_var"], g["edge_chk"])


def test_shipped_code_shape(golden):
    h = _h(golden)
    assert h.shape == (64, 128)
    assert set(h.sum(0)) == {3, 5} and set(h.sum(1)) == {8}
    info, piv, rows = ldpc.systematic(h)
    assert len(info) == 64 and len(piv) == 64


def test_encode_satisfies_checks(golden):
    h = _h(golden)
    rng = np.random.default_rng(3)
    data = rng.integers(0, 2, (50, 64))
    code = ldpc.encode(h, data)
    assert not np.any((h.astype(np.int64) @ code.T) % 2)
    info, _, _ = ldpc.systematic(h)
    np.testing.assert_array_equal(code[:, info], data)


@pytest.mark.parametrize("flips", [1, 2, 3])
def test_decode_corrects_flips(golden, flips):
    h = _h(golden)
    info, _, _ = ldpc.systematic(h)
    rng = np.random.default_rng(40 + flips)
    for _ in range(10):
        d = rng.integers(0, 2, 64)
        c = ldpc.encode(h, d)[0]
        y = c.copy()
        y[rng.choice(128, flips, replace=False)] ^= 1
        hard, it = ldpc.decode(h, ldpc.hard_llr(y), 100, True, 10)
        np.testing.assert_array_equal(hard[info], d)
        assert it == 10  # the syndrome holds at the first allowed check


def test_alist_reader_matches_oracle(golden, tmp_path):
    """The package's alist reader (zero-padded columns) gives the oracle's edges."""

    h = _h(golden)
    path = tmp_path / "code.alist"
    cols = [np.nonzero(h[:, v])[0] + 1 for v in range(h.shape[1])]
    rows = [np.nonzero(h[c])[0] + 1 for c in range(h.shape[0])]
    dc, dr = max(map(len, cols)), max(map(len, rows))
    with open(path, "w") as f:
        f.write(f"{h.shape[1]} {h.shape[0]}\n{dc} {dr}\n")
        f.write(" ".join(str(len(c)) for c in cols) + "\n" + " ".join(str(len(r)) for r in rows) + "\n")
        for c in cols:
            f.write(" ".join(map(str, list(c) + [0] * (dc - len(c)))) + "\n")
        for r in rows:
            f.write(" ".join(map(str, list(r) + [0] * (dr - len(r)))) + "\n")
    N, M, ev, ec = read_alist(str(path))
    assert (N, M) == (128, 64)
    np.testing.assert_array_equal(ldpc.dense_h(N, M, ev, ec), h)


def test_shipped_code_is_the_reference_matrix(golden):
    """The package's copy of the OFDM modem's parity-check edges (used by the benchmark)
    is the fixture recorded from the reference's alist file."""

    import os

    import hermespy_gb300

    g = golden("ldpc.npz")
    z = np.load(os.path.join(os.path.dirname(hermespy_gb300.__file__), "codes", "ofdm_ldpc.npz"))
    for k in ("N", "M", "edge_var", "edge_chk"):
        assert np.array_equal(z[k], g[k])
