"""CPU tests: the C-ABI library loads and exports every declared entry point, and the
host-side logic (frame tables, LS interpolation map, noise levels, validation)
matches the oracle. No CUDA device is touched."""

import ctypes
import os
import re

import numpy as np
import pytest

from hermespy_gb300 import _lib
from hermespy_gb300.build import LIB, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "hpx.h")).read()
    return sorted(set(re.findall(r"^(?:hpx_status|int|int32_t|const char\*)\s+(hpx_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    build()
    return ctypes.CDLL(LIB)


def test_library_exports_header(lib):
    names = header_symbols()
    assert len(names) > 25
    for name in names:
        assert hasattr(lib, name), name


def test_binding_covers_header():
    assert sorted(set(_lib.exported_symbols())) == header_symbols()


def test_version_and_error_state(lib):
    lib.hpx_version.restype = ctypes.c_int
    assert lib.hpx_version() >= 10000
    lib.hpx_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.hpx_last_error(), bytes)


def test_argument_errors_without_device(lib):
    """Argument validation runs before any device work and maps to ValueError."""

    _lib.load()
    with pytest.raises(ValueError):
        _lib.call("hpx_qam_map", 3, None, 4, None, None)
    with pytest.raises(ValueError, match="Unsupported modulation order"):
        _lib.call("hpx_qam_demap", 32, None, 1, None, None)
    desc = _lib.FadingDesc()
    desc.num_taps = 0
    h = ctypes.c_void_p()
    with pytest.raises(ValueError, match="at least one delay tap"):
        _lib.check(_lib.load().hpx_fading_create(ctypes.byref(desc), ctypes.byref(h)))


def test_frame_tables_match_oracle():
    from hermespy_gb300.waveform import ElementType, GridElement, GridResource, OFDMWaveform, SymbolSection
    from oracle.frame import FrameLayout
    from tests.configs import siso_frame

    res = [GridResource(1, prefix_ratio=18 / 256, elements=[GridElement(ElementType.DATA, 200)]),
           GridResource(50, prefix_ratio=18 / 256,
                        elements=[GridElement(ElementType.REFERENCE, 1), GridElement(ElementType.DATA, 3)])]
    wf = OFDMWaveform(res, [SymbolSection(1, [1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0])], num_subcarriers=256,
                      modulation_order=16)
    lay = FrameLayout(siso_frame())
    assert wf.samples_per_frame() == lay.samples_per_frame
    assert wf.num_data_symbols == lay.num_data and wf.references_per_frame == lay.num_refs
    mask = wf.resource_mask
    np.testing.assert_array_equal(mask[0], lay.ref_mask)
    np.testing.assert_array_equal(mask[1], lay.data_mask)
    np.testing.assert_array_equal(wf._layout()["prefix"], lay.prefix)


def test_ls_table_matches_oracle():
    from hermespy_gb300.estimation import ls_interpolation_table
    from oracle import estimation
    from oracle.frame import FrameLayout
    from tests.configs import siso_frame

    lay = FrameLayout(siso_frame())
    ip, ix, w = ls_interpolation_table(lay.ref_mask)
    ip2, ix2, w2 = estimation.ls_weight_table(lay)
    rng = np.random.default_rng(0)
    refs = rng.standard_normal(lay.num_refs) + 1j * rng.standard_normal(lay.num_refs)
    a = np.array([np.dot(w[ip[i]:ip[i + 1]], refs[ix[ip[i]:ip[i + 1]]]) for i in range(len(ip) - 1)])
    b = np.array([np.dot(w2[ip2[i]:ip2[i + 1]], refs[ix2[ip2[i]:ip2[i + 1]]]) for i in range(len(ip2) - 1)])
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-6)
    # rows are convex combinations (linear interpolation / nearest fill)
    sums = np.add.reduceat(w.astype(np.float64), ip[:-1])
    np.testing.assert_allclose(sums, 1.0, atol=1e-6)


def test_ls_table_on_golden(golden):
    from hermespy_gb300.estimation import ls_interpolation_table
    from oracle.frame import FrameLayout
    from tests.configs import siso_frame

    g = golden("ls.npz")
    lay = FrameLayout(siso_frame())
    ip, ix, w = ls_interpolation_table(lay.ref_mask)
    refs = g["grid"][lay.ref_mask] / lay.pilot_symbols()
    est = np.array([np.dot(w[ip[i]:ip[i + 1]], refs[ix[ip[i]:ip[i + 1]]]) for i in range(len(ip) - 1)])
    np.testing.assert_allclose(est.reshape(lay.num_words, lay.N), g["estimate"], rtol=0, atol=1e-5)


def test_channel_validation():
    from hermespy_gb300 import MultipathFadingChannel

    with pytest.raises(ValueError, match="equal length"):
        MultipathFadingChannel([0, 1e-6], [1.0], [0, 0])
    with pytest.raises(ValueError, match="greater or equal to zero"):
        MultipathFadingChannel([-1e-6], [1.0], [0])
    with pytest.raises(ValueError, match="Power profile"):
        MultipathFadingChannel([0.0], [-1.0], [0])
    with pytest.raises(ValueError, match="Rice"):
        MultipathFadingChannel([0.0], [1.0], [-1])
    ch = MultipathFadingChannel([2e-6, 0.0], [0.5, 1.0], [0, 1.0], num_sinusoids=4)
    np.testing.assert_array_equal(ch.delays, [0.0, 2e-6])
    los, nlos = ch.gains()
    np.testing.assert_allclose(los, [np.sqrt(0.5), 0.0])
    np.testing.assert_allclose(nlos, [np.sqrt(1 / 8), np.sqrt(1 / 4)])


def test_noise_levels():
    from hermespy_gb300 import EBN0, SNR, MultipathFadingChannel
    from hermespy_gb300.waveform import ElementType, GridElement, GridResource, OFDMWaveform, SymbolSection

    wf = OFDMWaveform([GridResource(1, elements=[GridElement(ElementType.DATA, 8)])], [SymbolSection(1, [0])],
                      num_subcarriers=64, modulation_order=64)
    assert EBN0(wf, 10.0).get_power() == pytest.approx(1 / 6 / 10)
    ch = MultipathFadingChannel([0.0, 1e-7], [1.0, 0.5], [0, 0], gain=0.5)
    assert SNR(4.0, wf, ch).get_power() == pytest.approx(0.25 * 0.5 * 1.5)
    with pytest.raises(ValueError):
        EBN0(wf, 0.0)


def test_clopper_pearson():
    from hermespy_gb300 import clopper_pearson

    lo, hi = clopper_pearson(0, 100)
    assert lo == 0.0 and hi == pytest.approx(0.0362, abs=1e-3)
    lo, hi = clopper_pearson(50, 100)
    assert lo == pytest.approx(0.3983, abs=1e-3) and hi == pytest.approx(0.6017, abs=1e-3)


def test_drop_status_flags_without_device():
    """Per-drop failure flags of a host copy of error words raise instead of being counted."""

    assert _lib.drop_counts(np.array([0, 7, 123456], dtype=np.uint32)).tolist() == [0, 7, 123456]
    with pytest.raises(RuntimeError, match="drop 2: non-finite pivot"):
        _lib.drop_counts(np.array([0, 5, _lib.DROP_NUMERIC | 3], dtype=np.uint32))
    with pytest.raises(RuntimeError, match="drop 1: a bounded tensor-core wait ran out"):
        _lib.drop_counts(np.array([_lib.DROP_NUMERIC, _lib.DROP_TIMEOUT], dtype=np.uint32))
    # int32 views of the device words (torch has no uint32 arithmetic) carry the same flags
    with pytest.raises(RuntimeError, match="wait ran out"):
        _lib.drop_counts(np.array([-2147483648], dtype=np.int32))
    with pytest.raises(ValueError):
        _lib.check(_lib.load().hpx_drop_status(None, 3))
