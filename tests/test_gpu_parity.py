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


def test_same_numbers_in_small_and_large_batches(gpu):
    """Few sets run the line profile and histograms with a CTA per zone and the finalize with 512
    threads; many sets with one CTA per tile and 128.  A set gives the same numbers either way, for
    relxilllp (lamp post) and relxill (broken power law)."""
    params, grids = _random_lp_sets(320, 11)
    big, st = gpu.eval_batch("relxilllp", params, grids)
    assert not st.any()
    for i in (0, 157, 319):
        one, _ = gpu.eval_batch("relxilllp", params[i:i + 1], grids[i:i + 1])
        np.testing.assert_array_equal(one[0], big[i])
    rng = np.random.default_rng(12)
    n = 320
    q = np.column_stack([rng.uniform(2, 4, n), rng.uniform(2, 4, n), rng.uniform(5, 30, n), rng.uniform(0, 0.998, n),
                         rng.uniform(10, 80, n), -np.ones(n), np.full(n, 400.0), np.zeros(n), rng.uniform(1.5, 2.8, n),
                         rng.uniform(0, 4, n), np.ones(n), np.full(n, 300.0), np.ones(n)])
    big, st = gpu.eval_batch("relxill", q, grids)
    assert not st.any()
    for i in (0, 158, 319):
        one, _ = gpu.eval_batch("relxill", q[i:i + 1], grids[i:i + 1])
        np.testing.assert_array_equal(one[0], big[i])


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


def test_relline_profile_edges_on_conv_grid(gpu, oracle):
    """Line profiles on the 4096-bin convolution grid, where the blue and red
    edges of single radii fall on bin edges in every possible position: a
    geometry whose gmax at one radius lies a hair below a bin edge (the edge
    term of that radius must stay in the bin below), and random geometries."""
    cg = oracle_lib.conv_grid()
    rng = np.random.default_rng(71)
    rows = [[1.0, 2.3746189592624702, 2.633860796331297, 6.812861314634864, -0.4762755685025275,
             50.195840694470434, -1.0, 131.52308866238963, 0.0, 0.0]]
    for _ in range(47):
        rows.append([rng.uniform(0.3, 30.0), rng.uniform(1.0, 5.0), rng.uniform(1.0, 5.0), rng.uniform(3.0, 30.0),
                     rng.uniform(-0.998, 0.998), rng.uniform(5.0, 85.0), -1.0, rng.uniform(20.0, 1000.0), 0.0,
                     float(rng.integers(0, 3))])
    p = np.array(rows)
    out, st = gpu.eval_batch("relline", p, [cg] * len(p))
    assert not st.any()
    for i in range(len(p)):
        s, orc = oracle_lib.evaluate("relline", p[i], cg)
        assert s == 0
        assert_close(out[i], orc, f"relline geometry {i}")


def test_mixed_zone_counts_in_one_batch(gpu, oracle, monkeypatch):
    """One batch whose sets need different zone counts: relxill sets without an ionisation
    gradient (1 zone) beside power-law and alpha-disc gradients (25 zones), and relxilllp sets
    with 10 zones beside 25; every set against the oracle with its own switch."""
    monkeypatch.delenv("RELXILL_NUM_RZONES", raising=False)  # the default zone counts differ per switch
    rng = np.random.default_rng(73)
    e = [np.exp(np.linspace(np.log(0.3), np.log(80.0), int(k) + 1)) for k in rng.integers(200, 900, 6)]
    igt = np.array([0, 1, 0, 2, 0, 1], dtype=np.int32)
    igi = np.where(igt == 1, 1.5, 0.0)
    p = np.column_stack([rng.uniform(2.5, 4, 6), rng.uniform(2.5, 4, 6), rng.uniform(8, 30, 6),
                         rng.uniform(0, 0.998, 6), rng.uniform(10, 80, 6), -np.ones(6), np.full(6, 400.0),
                         np.zeros(6), rng.uniform(1.5, 2.8, 6), rng.uniform(1, 4, 6), np.ones(6),
                         np.full(6, 300.0), np.ones(6)])
    out, st = gpu.eval_batch("relxill", p, e, ion_grad_type=igt, iongrad_index=igi)
    assert not st.any()
    for i in range(6):
        s, orc = oracle_lib.evaluate("relxill", p[i], e[i], None, int(igt[i]), float(igi[i]))
        assert s == 0
        assert_close(out[i], orc, f"relxill set {i} (ion_grad_type {igt[i]})")
    q = np.column_stack([rng.uniform(3, 30, 6), np.zeros(6), rng.uniform(0, 0.998, 6), rng.uniform(10, 80, 6),
                         -np.ones(6), np.full(6, 400.0), np.zeros(6), rng.uniform(1.5, 2.8, 6),
                         rng.uniform(1, 4, 6), np.ones(6), np.full(6, 300.0), np.ones(6), np.zeros(6), np.zeros(6)])
    out, st = gpu.eval_batch("relxilllp", q, e, ion_grad_type=igt, iongrad_index=igi)
    assert not st.any()
    for i in range(6):
        s, orc = oracle_lib.evaluate("relxilllp", q[i], e[i], None, int(igt[i]), float(igi[i]))
        assert s == 0
        assert_close(out[i], orc, f"relxilllp set {i} (ion_grad_type {igt[i]})")


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
