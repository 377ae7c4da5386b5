"""GPU parity: the CUDA path against the CPU oracle (run here) and against the
reference's own outputs (tests/golden, made by the compiled reference)."""
import os

import numpy as np
import pytest

import oracle_lib
from cases import CASES, CONV_MODELS, conv_input, grid
from tolerance import assert_close, compare

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_small.npz")


@pytest.fixture(autouse=True)
def _zones_env(monkeypatch):
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")


def _gpu_eval(R, model, params, e, igt=0, igi=0.0):
    fin = [conv_input(e)] if model in CONV_MODELS else None
    out, st = R.eval_batch(model, np.asarray(params)[None], [e], flux_in=fin,
                           ion_grad_type=[igt] if igt else None, iongrad_index=[igi] if igt else None)
    assert st[0] == 0, (model, st[0], R.last_error())
    return out[0]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_case_vs_oracle_and_reference(gpu, oracle, case):
    name, model, params, gspec, igt, igi = case
    e = grid(gspec)
    got = _gpu_eval(gpu, model, params, e, igt, igi)
    st, orc = oracle_lib.evaluate(model, params, e, conv_input(e) if model in CONV_MODELS else None, igt, igi)
    assert st == 0
    assert_close(got, orc, f"{name} vs oracle")
    ref = np.load(GOLDEN)[name]
    assert_close(got, ref, f"{name} vs reference")


def test_lmod_entry_points_match_batch(gpu):
    e = grid(CASES[0][3])
    a = gpu.relline(e, CASES[0][2])
    b = _gpu_eval(gpu, "relline", CASES[0][2], e)
    np.testing.assert_array_equal(a, b)
    e2 = grid(CASES[7][3])
    np.testing.assert_array_equal(gpu.relxilllp(e2, CASES[7][2]), _gpu_eval(gpu, "relxilllp", CASES[7][2], e2))


def _random_lp_sets(n, seed):
    rng = np.random.default_rng(seed)
    sets, grids = [], []
    for _ in range(n):
        h = rng.uniform(3, 100)
        a = rng.uniform(0, 0.998)
        inc = rng.uniform(5, 85)
        gam = rng.uniform(1.4, 2.8)
        lxi = rng.uniform(0, 4.5)
        sets.append([h, 0.0, a, inc, -1, 400, 0, gam, lxi, 1.0, 300, 1.0, 0, 0])
        nb = int(rng.integers(300, 1200))
        grids.append(np.exp(np.linspace(np.log(0.3), np.log(80), nb + 1)))
    return np.array(sets), grids


def test_batched_relxilllp_random_sets(gpu, oracle):
    params, grids = _random_lp_sets(12, 2026)
    out, st = gpu.eval_batch("relxilllp", params, grids)
    assert not st.any()
    worst = 0.0
    for i in range(len(grids)):
        s, orc = oracle_lib.evaluate("relxilllp", params[i], grids[i])
        assert s == 0
        r, t = compare(out[i], orc)
        worst = max(worst, r)
        assert_close(out[i], orc, f"set {i}")
    print("worst per-bin relative error", worst)


def test_deterministic_alone_and_in_batch(gpu):
    params, grids = _random_lp_sets(8, 7)
    a, _ = gpu.eval_batch("relxilllp", params, grids)
    b, _ = gpu.eval_batch("relxilllp", params, grids)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    for i in (0, 3, 7):
        one, _ = gpu.eval_batch("relxilllp", params[i:i + 1], grids[i:i + 1])
        np.testing.assert_array_equal(one[0], a[i])


def test_parameter_errors(gpu):
    e = grid(CASES[7][3])
    bad = list(CASES[7][2])
    bad[2] = 0.999  # a > 0.9982 (ModelDefinition.cpp:191-195)
    out, st = gpu.eval_batch("relxilllp", np.array([bad, CASES[7][2]]), [e, e], check=False)
    assert st[0] == 1 and st[1] == 0
    assert not out[0].any() and out[1].sum() > 0
    rr = list(CASES[7][2])
    rr[12] = 3  # $switch_returnrad takes 0, 1, -1 or 2 (Rellp.cpp:497-506)
    out, st = gpu.eval_batch("relxilllp", np.array([rr]), [e], check=False)
    assert st[0] == 1 and not out[0].any()
    inc = list(CASES[5][2])
    inc[4] = 89.0  # inclination outside 3-87 degrees
    out, st = gpu.eval_batch("relxill", np.array([inc]), [e], check=False)
    assert st[0] == 1


def test_relconv_rejects_empty_input(gpu):
    e = grid(CASES[4][3])
    out, st = gpu.eval_batch("relconv", np.array([CASES[4][2]]), [e], flux_in=[np.zeros(len(e) - 1)], check=False)
    assert st[0] == 5 and not out[0].any()


def test_relline_grid_without_line_and_single_bin(gpu, oracle):
    p = CASES[0][2]
    e = np.array([50.0, 60.0, 70.0])  # far above the line: all zero in the reference
    st, orc = oracle_lib.evaluate("relline", p, e)
    out, s = gpu.eval_batch("relline", np.array([p]), [e], check=False)
    assert st == s[0]
    if st == 0:  # the reference renormalises an empty profile to NaN (0 * 1/0)
        np.testing.assert_allclose(out[0], orc, rtol=1e-4, atol=0, equal_nan=True)
    e1 = np.array([5.0, 7.0])  # one bin holding the whole line
    st, orc = oracle_lib.evaluate("relline", p, e1)
    out, s = gpu.eval_batch("relline", np.array([p]), [e1])
    assert s[0] == 0
    np.testing.assert_allclose(out[0], orc, rtol=1e-6)


def test_relline_normalised_to_one(gpu):
    e = grid(CASES[0][3])
    f = gpu.relline(e, CASES[0][2])
    assert abs(f.sum() - 1.0) < 1e-6


def test_bounded_wait_reports_timeout_and_context_survives(gpu):
    """The TMA pipeline's bounded mbarrier wait gives up after its limit with status 8, without
    a fault; evaluations work afterwards."""
    import ctypes
    import time

    L = gpu.lib()
    L.relx_selftest_wait_timeout.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
    st = ctypes.c_int(-1)
    t0 = time.time()
    assert L.relx_selftest_wait_timeout(5.0, ctypes.byref(st)) == 0
    assert st.value == 8
    assert time.time() - t0 < 10.0
    e = grid(CASES[7][3])
    _gpu_eval(gpu, "relxilllp", CASES[7][2], e)
