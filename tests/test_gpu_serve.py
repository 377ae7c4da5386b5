"""Line-profile cache and serving engine: results are the same numbers as the
plain batched path, alone and in any mix of requests."""
import time

import numpy as np
import pytest

from cases import conv_input, log_grid

pytestmark = pytest.mark.gpu


def _lp_sets(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        out.append([rng.uniform(3, 100), 0.0, rng.uniform(0, 0.998), rng.uniform(5, 85), -1, 400, 0,
                    rng.uniform(1.4, 2.8), rng.uniform(0, 4.5), 1.0, 300, 1.0, 0, 0])
    return np.array(out)


def _bkn_sets(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        out.append([rng.uniform(2, 4), 3, 15, rng.uniform(0, 0.998), rng.uniform(5, 85), -1, 400, 0,
                    rng.uniform(1.4, 2.8), rng.uniform(0, 4.5), 1.0, 300, 2.0])
    return np.array(out)


def _grids(n, seed):
    rng = np.random.default_rng(seed)
    return [log_grid(0.3, 80.0, int(rng.integers(300, 1200))) for _ in range(n)]


def _batch(R, model, params, grids, flux_in=None):
    out, st = R.eval_batch(model, params, grids, flux_in=flux_in)
    assert not np.any(st), R.last_error()
    return out


@pytest.fixture
def cache(gpu):
    gpu.cache_config(256)
    try:
        yield gpu
    finally:
        gpu.cache_config(0)


def test_cache_hits_return_the_uncached_numbers(gpu):
    lp, bkn = _lp_sets(12, 5), _bkn_sets(6, 6)
    g_lp, g_bkn = _grids(12, 7), _grids(6, 8)
    want_lp = _batch(gpu, "relxilllp", lp, g_lp)
    want_bkn = _batch(gpu, "relxill", bkn, g_bkn)
    gpu.cache_config(256)
    try:
        for _ in range(2):  # misses, then hits
            got = _batch(gpu, "relxilllp", lp, g_lp)
            for a, b in zip(got, want_lp):
                np.testing.assert_array_equal(a, b)
            got = _batch(gpu, "relxill", bkn, g_bkn)
            for a, b in zip(got, want_bkn):
                np.testing.assert_array_equal(a, b)
        st = gpu.cache_stats()
        # direct mapped: a set whose slot another set of its batch claimed is not stored
        assert st["lookups"] == 36 and st["hits"] >= 15, st
    finally:
        gpu.cache_config(0)


def test_cache_xillver_only_change_and_duplicates(cache):
    R = cache
    base = _bkn_sets(1, 11)[0]
    sets = []
    for lxi in (0.5, 1.5, 2.5, 3.5):  # same relativistic parameters, other xillver parameters
        p = base.copy()
        p[9] = lxi
        sets.append(p)
    sets = np.array(sets + [sets[0], sets[0]])  # duplicates inside one batch
    grids = _grids(len(sets), 12)
    R.cache_config(0)
    want = _batch(R, "relxill", sets, grids)
    R.cache_config(256)
    got1 = _batch(R, "relxill", sets, grids)
    got2 = _batch(R, "relxill", sets, grids)
    for a, b, c in zip(got1, got2, want):
        np.testing.assert_array_equal(a, c)
        np.testing.assert_array_equal(b, c)
    assert R.cache_stats()["hits"] >= len(sets)


def test_relconv_through_cache(cache):
    R = cache
    p = np.array([[3, 3, 15, 0.9, 45, -1, 400, 0], [4, 3, 10, 0.5, 30, -1, 300, 1]], dtype=float)
    e = [log_grid(0.3, 80.0, 500), log_grid(0.5, 50.0, 700)]
    fin = [conv_input(x) for x in e]
    a = _batch(R, "relconv", p, e, fin)
    b = _batch(R, "relconv", p, e, fin)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_serve_results_match_batch_alone(gpu):
    lp, bkn = _lp_sets(40, 21), _bkn_sets(24, 22)
    g_lp, g_bkn = _grids(40, 23), _grids(24, 24)
    want_lp = [_batch(gpu, "relxilllp", lp[i:i + 1], [g_lp[i]])[0] for i in range(len(lp))]
    want_bkn = [_batch(gpu, "relxill", bkn[i:i + 1], [g_bkn[i]])[0] for i in range(len(bkn))]
    with gpu.Server(hbm_budget_bytes=4 << 30, max_batch=16, cache_slots=64) as srv:
        outs = {}
        order = [("relxilllp", i) for i in range(len(lp))] + [("relxill", i) for i in range(len(bkn))]
        rng = np.random.default_rng(3)
        rng.shuffle(order)
        for rep in range(2):  # the second round hits the cache
            for model, i in order:
                p, g = (lp[i], g_lp[i]) if model == "relxilllp" else (bkn[i], g_bkn[i])
                out = np.empty(len(g) - 1)
                rid = srv.submit(model, p, g, out)
                outs[rid] = (model, i, out)
            done = 0
            t0 = time.time()
            while done < len(order) and time.time() - t0 < 60:
                for rid, st, lat in srv.poll():
                    assert st == 0
                    assert lat >= 0.0
                    done += 1
                time.sleep(0.001)
            assert done == len(order)
        for rid, (model, i, out) in outs.items():
            want = want_lp[i] if model == "relxilllp" else want_bkn[i]
            np.testing.assert_array_equal(out, want)
        s = srv.stats()
        assert s["completed"] == 2 * len(order)
        assert s["p99_ms"] >= s["p50_ms"] > 0.0
        assert s["batches"] >= 2
    gpu.cache_config(0)


def test_chunks_and_graphs_give_the_same_numbers(gpu, monkeypatch):
    """Pipelined chunks and CUDA-graph replay change nothing."""
    lp = _lp_sets(9, 31)
    g = _grids(9, 32)
    gpu.tuning_config(autotune=False, graphs=False)
    try:
        want = _batch(gpu, "relxilllp", lp, g)
        monkeypatch.setenv("RELX_CHUNK_SETS", "2")
        for a, b in zip(_batch(gpu, "relxilllp", lp, g), want):
            np.testing.assert_array_equal(a, b)
        monkeypatch.delenv("RELX_CHUNK_SETS")
        gpu.tuning_config(autotune=True, graphs=True)
        for _ in range(3):  # tuning trials, a direct launch, then a captured graph and its replay
            for a, b in zip(_batch(gpu, "relxilllp", lp, g), want):
                np.testing.assert_array_equal(a, b)
        assert any(t["model"] == 3 for t in gpu.tuning_report())
    finally:
        gpu.tuning_config(autotune=True, graphs=True)


def test_serve_allocates_nothing_and_refuses_request_beyond_slot(gpu):
    """Each slot carves its batches from the half of the budget it allocated at creation: device
    memory does not change while serving, and a request that alone needs more than a slot completes
    with RELX_ERR_NOMEM (7) while the requests around it complete normally.  With a 600 KB budget a
    relline set of 200 bins (about 100 KB of workspace) fits a slot and one of 16000 bins (about
    600 KB: 32 bytes per energy edge) does not."""
    torch = pytest.importorskip("torch")
    p = np.array([6.4, 3, 3, 15, 0.9, 30, -1, 400, 0, 0], dtype=float)
    small = [log_grid(1.0, 10.0, 200 + 7 * k) for k in range(5)]
    big = log_grid(1.0, 10.0, 16000)
    want = [_batch(gpu, "relline", p[None], [g])[0] for g in small]
    with gpu.Server(hbm_budget_bytes=600 << 10, max_batch=8) as srv:
        o = np.empty(len(small[0]) - 1)  # first batch: the streams the slots launch on are set up
        srv.submit("relline", p, small[0], o)
        t0 = time.time()
        while not srv.poll() and time.time() - t0 < 60:
            time.sleep(0.001)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        outs, ids = [], []
        for k, g in enumerate(small[:3] + [big] + small[3:]):
            o = np.empty(len(g) - 1)
            outs.append(o)
            ids.append(srv.submit("relline", p, g, o))
        st = {}
        t0 = time.time()
        while len(st) < len(ids) and time.time() - t0 < 60:
            for rid, s, _ in srv.poll():
                st[rid] = s
            time.sleep(0.001)
        assert len(st) == len(ids)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
    assert st[ids[3]] == 7
    got = [outs[k] for k in (0, 1, 2, 4, 5)]
    for k, (a, b) in enumerate(zip(got, want)):
        assert st[ids[k if k < 3 else k + 1]] == 0
        np.testing.assert_array_equal(a, b)
