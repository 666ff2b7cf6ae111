"""Same-core timing of the oracle port against the reference's own drop.

Usage:  python oracle/calibrate.py <path-to-hermespy-checkout> [drops]

TEST INFRASTRUCTURE. The benchmark's CPU baseline runs the oracle (``oracle.link``),
because the reference cannot be installed where the GPU runs. This script states
how the two relate: on one core of the machine that runs it, it times the
reference's ``SimulationScenario.drop()`` + ``BitErrorEvaluator`` (simulation/
scenario.py:772-804, modem/evaluators.py:239-258; random inputs injected from the
engine's Philox streams through ``tests/golden/refdrops.py``) and the oracle's drop
on the same drops, for config 1 (SISO LS + ZF) and config 2 (4x4 ideal CSI + ZF),
checks that both count the same bit errors, and prints seconds per drop and their
ratio as one JSON line. BLAS threads are pinned to one.
"""

from __future__ import annotations

import json
import os
import sys
import time

for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ[v] = "1"

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (os.path.join(ROOT, "tests", "golden"), os.path.join(ROOT, "tests"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402


def main() -> None:
    import refimport

    refimport.import_reference(sys.argv[1] if len(sys.argv) > 1 else None)
    n = int(sys.argv[2]) if len(sys.argv) > 2 else 20
    import platform

    import refdrops
    from configs import mimo_channel, mimo_frame, siso_channel, siso_frame

    from oracle.link import LinkConfig, simulate_drop

    seed = 31337
    out = {"host": platform.processor() or platform.machine(), "cores": 1, "drops": n}
    cases = {
        "config1_siso_ls_zf": (refdrops.c1_waveform(), siso_channel(15.36e6), 15.36e6, 1, "ls",
                               LinkConfig(siso_frame(), siso_channel(15.36e6), 15.36e6, 1, 1, "ls", "zf", "ebn0"),
                               10800),
        "config2_4x4_ideal_zf": (refdrops.c2_waveform(), mimo_channel(30.72e6), 30.72e6, 4, "ideal",
                                 LinkConfig(mimo_frame(), mimo_channel(30.72e6), 30.72e6, 4, 4, "ideal", "zf",
                                            "ebn0"), 201600),
    }
    for name, (wf, ch, fs, nant, est, cfg, bits) in cases.items():
        link = refdrops.RefLink(wf, ch, fs, nant, nant, seed, est)
        link.set_ebn0(10.0)
        link.drop(10_000)  # warm-up (imports, caches)
        simulate_drop(cfg, seed, 10_000, 10.0)
        t0 = time.perf_counter()
        ref = [link.drop(d)[0] for d in range(n)]
        t_ref = (time.perf_counter() - t0) / n
        t0 = time.perf_counter()
        orc = [simulate_drop(cfg, seed, d, 10.0)["errors"] for d in range(n)]
        t_orc = (time.perf_counter() - t0) / n
        assert ref == orc, (name, ref, orc)
        out[name] = {"reference_s_per_drop": round(t_ref, 5), "oracle_s_per_drop": round(t_orc, 5),
                     "reference_over_oracle": round(t_ref / t_orc, 3), "bits_per_drop": bits,
                     "same_errors": True}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
