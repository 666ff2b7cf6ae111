"""CPU oracle for the HermesPy OFDM fading-link drop loop.

TEST INFRASTRUCTURE ONLY. This package restates, in float64 numpy, the
reference's algorithm for every stage of the hot path so that the CUDA engine
can be checked against it on identical random draws. It is imported only by
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py``; the engine package never imports it and has no CPU fallback.

Each function cites the reference file and line range (paths relative to the
HermesPy source tree) whose behaviour it restates. The restatement is pinned
against outputs of the reference itself, recorded as fixtures under
``tests/golden/`` by ``tests/golden/make_golden.py``.

Modules
-------
philox      Philox4x32-10 counter-based generator (bit-exact with the engine).
streams     The engine's random-stream layout (bits, fading draws, noise).
mapping     3GPP Gray PSK/QAM mapping and hard demapping.
frame       OFDM resource grid description (resources, sections, masks).
ofdm        OFDM place / modulate / demodulate.
fading      Sum-of-sinusoids multipath fading: realization, taps, propagation,
            channel state.
estimation  LS (interpolated) and ideal channel estimation, ZF and LMMSE
            equalization.
link        One full drop, bits to bit errors.
"""
