"""relline_lp, relconv_lp and the xillver model on the GPU: random batches
against the CPU oracle, the local-model entry points against the batched
call, the line-profile cache keeping the models apart, and the serving
engine with xillver requests in the mix."""
import time

import numpy as np
import pytest

import oracle_lib
from cases import conv_input, log_grid
from tolerance import assert_close

pytestmark = pytest.mark.gpu


def _rng_grids(rng, n, lo, hi, nmin, nmax):
    return [log_grid(lo, hi, int(rng.integers(nmin, nmax))) for _ in range(n)]


def _check_batch(R, model, params, grids, fin=None):
    out, st = R.eval_batch(model, params, grids, flux_in=fin)
    assert not st.any(), (st, R.last_error())
    for i in range(len(grids)):
        s, orc = oracle_lib.evaluate(model, params[i], grids[i], None if fin is None else fin[i])
        assert s == 0
        assert_close(out[i], orc, f"{model} set {i}")
    return out


def test_relline_lp_random_sets(gpu, oracle):
    rng = np.random.default_rng(41)
    n = 10
    p = np.column_stack([rng.uniform(1, 8, n), rng.uniform(3, 100, n), rng.uniform(-0.9, 0.998, n),
                         rng.uniform(5, 85, n), -rng.uniform(1, 3, n), rng.uniform(50, 1000, n),
                         rng.uniform(0, 0.5, n), rng.integers(0, 3, n), rng.uniform(1.2, 3.2, n), np.zeros(n)])
    _check_batch(gpu, "relline_lp", p, _rng_grids(rng, n, 0.05, 15.0, 200, 3000))


def test_relconv_lp_random_sets(gpu, oracle):
    rng = np.random.default_rng(42)
    n = 8
    p = np.column_stack([rng.uniform(3, 100, n), rng.uniform(0, 0.9, n), rng.uniform(-0.9, 0.998, n),
                         rng.uniform(5, 85, n), -rng.uniform(1, 3, n), rng.uniform(50, 1000, n),
                         rng.integers(0, 3, n), rng.uniform(1.2, 3.2, n), np.zeros(n)])
    grids = _rng_grids(rng, n, 0.2, 100.0, 200, 1500)
    _check_batch(gpu, "relconv_lp", p, grids, [conv_input(e) for e in grids])


def test_xillver_random_sets(gpu, oracle):
    rng = np.random.default_rng(43)
    n = 24
    p = np.column_stack([rng.uniform(1.0, 3.4, n), rng.uniform(0.5, 10, n), rng.uniform(5, 1000, n),
                         rng.uniform(0, 4.7, n), rng.choice([0.0, 0.02, 0.3], n), rng.uniform(3, 87, n),
                         rng.choice([-1.0, -0.3, 0.0, 0.5, 3.0], n)])
    grids = _rng_grids(rng, n, 0.05, 500.0, 50, 4000)
    grids[0] = log_grid(0.5, 0.6, 3)             # a few bins inside one or two table bins
    grids[1] = log_grid(0.001, 0.05, 40)         # below the table: primary only
    grids[2] = np.array([0.1, 1000.0])           # one bin over the whole table
    _check_batch(gpu, "xillver", p, grids)


def test_local_model_entry_points_match_batch(gpu):
    e = log_grid(0.1, 20.0, 600)
    pl = [6.4, 6, 0.998, 30, -1, 400, 0, 0, 2, 0]
    out, _ = gpu.eval_batch("relline_lp", np.array([pl]), [e])
    np.testing.assert_array_equal(gpu.relline_lp(e, pl), out[0])
    pc = [6, 0, 0.998, 30, -1, 400, 0, 2, 0]
    f = conv_input(e)
    out, _ = gpu.eval_batch("relconv_lp", np.array([pc]), [e], flux_in=[f])
    np.testing.assert_array_equal(gpu.relconv_lp(e, pc, f), out[0])
    px = [2, 1, 300, 3.1, 0, 30, -1]
    w = log_grid(0.1, 1000.0, 900)
    out, _ = gpu.eval_batch("xillver", np.array([px]), [w])
    np.testing.assert_array_equal(gpu.xillver(w, px), out[0])


def test_returning_radiation_switch_values(gpu, oracle):
    """$switch_returnrad 1 adds the returning radiation, -1 and 2 keep only it, other values fail
    (add_returnrad_emis, Rellp.cpp:483-509)."""
    e = log_grid(0.1, 20.0, 600)
    base = [6.4, 6, 0.998, 30, -1, 400, 0, 0, 2, 0]
    for sw in (1, -1, 2):
        p = list(base)
        p[9] = sw
        out, st = gpu.eval_batch("relline_lp", np.array([p]), [e])
        s, orc = oracle_lib.evaluate("relline_lp", p, e)
        assert st[0] == 0 and s == 0
        assert_close(out[0], orc, f"switch {sw}")
    p = list(base)
    p[9] = 3
    out, st = gpu.eval_batch("relline_lp", np.array([p]), [e], check=False)
    assert st[0] == 1 and not out[0].any()


def test_returning_radiation_random_relxilllp(gpu, oracle):
    """Random lamp-post sets with returning radiation over both spin signs (corrections only for
    a > 0) and heights, against the oracle."""
    rng = np.random.default_rng(45)
    n = 10
    p = np.column_stack([rng.uniform(3, 60, n), np.zeros(n), rng.uniform(-0.9, 0.998, n), rng.uniform(5, 85, n),
                         -np.ones(n), rng.uniform(100, 1000, n), np.zeros(n), rng.uniform(1.4, 2.8, n),
                         rng.uniform(0, 4.5, n), rng.uniform(0.5, 5, n), rng.uniform(20, 500, n), np.ones(n),
                         np.ones(n), np.zeros(n)])
    grids = _rng_grids(rng, n, 0.3, 80.0, 300, 2000)
    _check_batch(gpu, "relxilllp", p, grids)


def test_returning_radiation_outer_zone_total(gpu, oracle, monkeypatch):
    """A relxilllp set whose xillver-corrected returning emissivity stays high out to Rout, so that
    a handful of outer radii dominate some bins.  In one such bin the reference's Romberg test of
    a radius near Rout gives obtprec 0.0200002, which an FP32 test puts on the other side of 0.02
    (one Romberg level less, 3e-4 off in that bin, 1.6e-6 in the total): the kernel integrates
    such bins again in FP64.  Both returning-radiation switches, at the project's bar."""
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")
    p = [7.819159105467463, 0.06318223691180253, 0.7520664936838367, 20.839453254507205, -1, 242.08828763042303,
         0.0, 1.2155558003015097, 1.2222305853986382, 9.569424921641735, 210.91094357446238, 5.727814656047778,
         1.0, 0.0]
    e = log_grid(0.5722, 177.1, 1114)
    for sw in (1.0, -1.0):
        q = list(p)
        q[12] = sw
        out, st = gpu.eval_batch("relxilllp", np.array([q]), [e])
        s, orc = oracle_lib.evaluate("relxilllp", q, e)
        assert st[0] == 0 and s == 0
        assert_close(out[0], orc, f"relxilllp returning radiation switch {sw}")


def test_romberg_threshold_bins_of_outer_radii(gpu, oracle, monkeypatch):
    """relline_lp and relline on the 4096-bin convolution grid with the physical normalisation and
    emissivities that weight the outer radii, where single radii dominate bins: the bins whose
    Romberg test sits at 0.02 within FP32 rounding match the oracle (1e-4 to 3e-4 off with an FP32
    decision)."""
    monkeypatch.setenv("RELLINE_PHYSICAL_NORM", "1")
    e = oracle_lib.conv_grid()
    a, inc, rout = 0.7520664936838367, 20.839453254507205, 242.08828763042303
    cases = [("relline_lp", [1.0, 7.819159105467463, a, inc, -1.0, rout, 0.0, 0.0, 1.2155558003015097, sw])
             for sw in (-1.0, 1.0, 0.0)]
    cases += [("relline", [1.0, q, q, 15.0, a, inc, -1.0, rout, 0.0, 0.0]) for q in (-2.0, 0.0, 3.0)]
    cases += [("relline", [1.0, -2.0, -2.0, 15.0, a, inc, 100.0, rout, 0.0, 0.0])]
    for model, p in cases:
        out, st = gpu.eval_batch(model, np.array([p]), [e])
        s, orc = oracle_lib.evaluate(model, p, e)
        assert st[0] == 0 and s == 0
        assert_close(out[0], orc, f"{model} {p}")


def test_cache_separates_models(gpu):
    """relconv (limb 1) and relxill (z 1) with the same leading eight numbers, and a relconv_lp
    set, through the line-profile cache: every result equals the uncached one, and the second
    pass hits for all three (the key carries the caller's model)."""
    e = log_grid(0.3, 80.0, 500)
    w = log_grid(0.1, 1000.0, 800)
    f = conv_input(e)
    p_bkn = np.array([[3, 3, 15, 0.9, 45, -1, 400, 1]], dtype=float)
    p_x = np.array([[3, 3, 15, 0.9, 45, -1, 400, 1, 2.0, 3.1, 1, 300, 3]], dtype=float)
    p_lp = np.array([[6, 0.3, 0.9, 45, -1, 400, 1, 2.0, 0]], dtype=float)

    def run():
        a, sa = gpu.eval_batch("relconv", p_bkn, [e], flux_in=[f])
        b, sb = gpu.eval_batch("relxill", p_x, [w])
        c, sc = gpu.eval_batch("relconv_lp", p_lp, [e], flux_in=[f])
        assert not (sa.any() or sb.any() or sc.any())
        return a[0], b[0], c[0]

    gpu.cache_config(0)
    want = run()
    gpu.cache_config(64)
    try:
        for _ in range(2):
            for got, ref in zip(run(), want):
                np.testing.assert_array_equal(got, ref)
        st = gpu.cache_stats()
        assert st["lookups"] == 6 and st["hits"] == 3, st
    finally:
        gpu.cache_config(0)


def test_serve_mixes_xillver_with_relxilllp(gpu):
    rng = np.random.default_rng(44)
    lp = [[rng.uniform(3, 50), 0, rng.uniform(0, 0.99), rng.uniform(10, 80), -1, 400, 0, rng.uniform(1.5, 2.5),
           rng.uniform(0, 4), 1, 300, 1, 0, 0] for _ in range(8)]
    xi = [[rng.uniform(1.2, 3.0), rng.uniform(0.5, 5), rng.uniform(20, 500), rng.uniform(0, 4.5), 0,
           rng.uniform(10, 80), -1] for _ in range(8)]
    grids = [log_grid(0.3, 80.0, int(rng.integers(200, 900))) for _ in range(16)]
    want = [gpu.eval_batch("relxilllp", np.array([lp[i]]), [grids[i]])[0][0] for i in range(8)]
    want += [gpu.eval_batch("xillver", np.array([xi[i]]), [grids[8 + i]])[0][0] for i in range(8)]
    with gpu.Server(hbm_budget_bytes=2 << 30, max_batch=8, cache_slots=0) as srv:
        outs = []
        for i in range(16):
            k = i // 2 if i % 2 == 0 else 8 + i // 2  # interleave the two models
            model, p = ("relxilllp", lp[k]) if k < 8 else ("xillver", xi[k - 8])
            out = np.empty(len(grids[k]) - 1)
            srv.submit(model, np.array(p), grids[k], out)
            outs.append((k, out))
        done, t0 = 0, time.time()
        while done < 16 and time.time() - t0 < 60:
            for _, st, _ in srv.poll():
                assert st == 0
                done += 1
            time.sleep(0.001)
        assert done == 16
    for k, out in outs:
        np.testing.assert_array_equal(out, want[k])
