"""CPU: the oracle's preambles and frame synchronization against the reference's
outputs (tests/golden/sync.npz: PilotSection / SchmidlCoxPilotSection.generate,
SchmidlCoxSynchronization and OFDMCorrelationSynchronization on noisy signals)."""

import numpy as np
import pytest

from oracle import sync

N, CP, WORDS, ORDER = 128, 10, 4, 16
SPF = WORDS * (N + CP) + N


@pytest.mark.parametrize("dc", [True, False])
def test_preambles_match_reference(golden, dc):
    g = golden("sync.npz")
    np.testing.assert_allclose(sync.preamble(ORDER, N, dc, True), g[f"schmidl_cox_pilot_dc{int(dc)}"].reshape(-1),
                               rtol=0, atol=1e-12)
    np.testing.assert_allclose(sync.preamble(ORDER, N, dc, False), g[f"plain_pilot_dc{int(dc)}"].reshape(-1),
                               rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", ["sc", "sc3"])
def test_schmidl_cox_matches_reference(golden, case):
    g = golden("sync.npz")
    assert sync.schmidl_cox_synchronize(g[f"{case}_signal"], N, SPF) == g[f"{case}_indices"].tolist()


@pytest.mark.parametrize("case", ["corr", "corr3"])
def test_correlation_matches_reference(golden, case):
    g = golden("sync.npz")
    pilot = sync.preamble(ORDER, N, True, False)
    assert sync.correlation_synchronize(g[f"{case}_signal"], pilot, SPF) == g[f"{case}_indices"].tolist()


def test_short_signal_has_no_frame():
    assert sync.schmidl_cox_synchronize(np.zeros((1, N - 1), complex), N, SPF) == []
