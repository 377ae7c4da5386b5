"""Pins of the CPU oracle: the reference's table-free known-answer tests
(test/unit/test-stdfunctions.cpp, test-xilltab.cpp, tests-execmodel.cpp),
restated here, and the golden outputs of the compiled reference
(tests/golden/golden_small.npz, made by tests/golden/make_golden.py)."""
import ctypes
import os

import numpy as np
import pytest

import oracle_lib
from cases import CASES, CONV_MODELS, conv_input, grid

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_small.npz")
LIMIT_PREC = 1e-6  # test/unit (LIMIT_PREC of the reference's unit tests)


def test_rebin_spectrum_known_answer(oracle):
    # test-stdfunctions.cpp:129-152
    ener0 = np.array([1, 3, 4, 5, 6, 7, 9], dtype=float)
    val0 = np.array([1, 1, 1, 2, 1, 1], dtype=float)
    ener = np.array([0.5, 2, 4, 5.5, 7.5, 8], dtype=float)
    val = np.zeros(5)
    oracle.relxo_rebin_spectrum(oracle_lib.p(ener), val.ctypes.data_as(oracle_lib._dp), 5, oracle_lib.p(ener0),
                                oracle_lib.p(val0), 6)
    np.testing.assert_allclose(val, [0.5, 1.5, 2.0, 2.25, 0.25], atol=LIMIT_PREC)


def test_interpolation_known_answers(oracle):
    # test-stdfunctions.cpp:184-211
    oracle.relxo_interp_lin_1d.restype = ctypes.c_double
    oracle.relxo_interp_lin_1d.argtypes = [ctypes.c_double] * 3
    assert abs(oracle.relxo_interp_lin_1d(0.2, 1.0, 2.0) - 1.2) < LIMIT_PREC
    oracle.relxo_interp_lin_2d.restype = ctypes.c_double
    oracle.relxo_interp_lin_2d.argtypes = [ctypes.c_double] * 6
    assert abs(oracle.relxo_interp_lin_2d(0.4, 0.8, 1.0, 2.0, 2.0, 4.0) - 2.52) < LIMIT_PREC
    oracle.relxo_interp_lin_2d_float.restype = ctypes.c_double
    oracle.relxo_interp_lin_2d_float.argtypes = [ctypes.c_double] * 2 + [ctypes.c_float] * 4
    assert abs(oracle.relxo_interp_lin_2d_float(0.4, 0.8, 1.0, 2.0, 2.0, 4.0) - 2.52) < LIMIT_PREC


def test_primary_continuum_normalisation(oracle):
    # test-xilltab.cpp:244-286: normalised primary has 1e15/4pi in 0.1-1000 keV
    e = np.exp(np.linspace(np.log(0.1), np.log(1000.0), 501))
    for gam, ect in [(2.0, 300.0), (1.4, 50.0), (3.0, 800.0)]:
        nf = oracle.relxo_primary_norm_factor(ect, gam)
        em = 0.5 * (e[1:] + e[:-1])
        pl = np.exp(1 / ect) * em ** -gam * np.exp(-em / ect) * np.diff(e) * nf
        s = (pl * em).sum() * 1e20 * 1.602177e-09
        assert abs(s / (1e15 / 4 / np.pi) - 1) < 1e-6


def test_normalisation_change_direction(oracle):
    # test-xilltab.cpp:288-324: Ecut shifted down raises the normalisation, up lowers it
    assert oracle.relxo_norm_change(0.5, 40.0, 2.0) > 1.0
    assert oracle.relxo_norm_change(2.0, 40.0, 2.0) < 1.0
    assert oracle.relxo_norm_change(1.0, 40.0, 2.0) == 1.0


def test_fft_convolution_keeps_normalisation(oracle, small_tables):
    # test-stdfunctions.cpp:253-297
    cg = oracle_lib.conv_grid()
    st, prof = oracle_lib.evaluate("relline", [1.0, 3, 3, 15, 0.998, 30, -1, 400, 0, 0], cg)
    assert st == 0 and abs(prof.sum() - 1) < 1e-8
    em = 0.5 * (cg[1:] + cg[:-1])
    xill = em ** -1.0 * np.diff(cg) * np.exp(-em / 300)
    band = (cg[:-1] >= 0.01) & (cg[1:] <= 1000)
    out = np.zeros(4096)
    oracle.relxo_conv_spectrum_normalized(oracle_lib.p(cg), oracle_lib.p(xill), oracle_lib.p(prof),
                                          out.ctypes.data_as(oracle_lib._dp), 4096)
    assert abs(xill[band].sum() - out[band].sum()) < 1e-8 * xill[band].sum() * 10
    prof2 = prof.copy()
    prof2[1000] = 1000.0
    oracle.relxo_conv_spectrum_normalized(oracle_lib.p(cg), oracle_lib.p(xill), oracle_lib.p(prof2),
                                          out.ctypes.data_as(oracle_lib._dp), 4096)
    assert abs(xill[band].sum() - out[band].sum()) > 1e-8


def test_relconv_outside_range_is_zero(oracle, small_tables):
    # tests-execmodel.cpp:211-235
    e = np.exp(np.linspace(np.log(1200.0), np.log(3000.0), 51))
    st, f = oracle_lib.evaluate("relconv", [3, 3, 15, 0.9, 45, -1, 400, 0], e, np.ones(50))
    assert st == 0 and not f.any()


def test_all_models_execute(oracle, small_tables):
    # tests-execmodel.cpp:87-105
    for name, model, params, gspec, igt, igi in CASES[:10]:
        e = grid(gspec)
        st, f = oracle_lib.evaluate(model, params, e, conv_input(e) if model in CONV_MODELS else None)
        assert st == 0 and f.sum() > 0, name


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_equals_compiled_reference(oracle, small_tables, monkeypatch, case):
    """The golden outputs come from the reference's own sources (oracle/build_ref.sh)."""
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")
    name, model, params, gspec, igt, igi = case
    e = grid(gspec)
    st, f = oracle_lib.evaluate(model, params, e, conv_input(e) if model in CONV_MODELS else None, igt, igi)
    ref = np.load(GOLDEN)[name]
    assert st == 0
    m = ref > 1e-12 * ref.max()
    rel = np.abs(f[m] - ref[m]) / ref[m]
    assert rel.max() < 1e-12, f"{name}: {rel.max():.3e}"


def test_oracle_bit_exact_against_reference_library(small_tables, monkeypatch):
    """When the compiled reference is present (built here from the reference
    sources), the oracle matches it exactly on fresh random parameters."""
    if not os.path.exists(oracle_lib.REF_SO):
        pytest.skip("compiled reference not built (reference sources absent)")
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")
    ref = ctypes.CDLL(oracle_lib.REF_SO)
    rng = np.random.default_rng(5)
    e = np.exp(np.linspace(np.log(0.2), np.log(300.0), 801))
    for _ in range(6):
        p = np.array([rng.uniform(3, 100), 0.0, rng.uniform(0, 0.998), rng.uniform(5, 85), -1, 400, 0,
                      rng.uniform(1.4, 2.8), rng.uniform(0, 4.5), 1.0, 300, 1.0, 0, 0])
        f1 = np.zeros(800)
        ref.ref_reset_xillver_cache()
        assert ref.ref_eval(3, oracle_lib.p(p), oracle_lib.p(e), 800, f1.ctypes.data_as(oracle_lib._dp)) == 0
        st, f2 = oracle_lib.evaluate("relxilllp", p, e)
        assert st == 0
        np.testing.assert_array_equal(f1, f2)
