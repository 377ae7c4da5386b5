"""The output cache of the local-model calls, the counterpart of the reference's RelxillCache
(Relcache.h:182-251, Relxill.cpp:295-400): a relxill-family call repeated with parameters within
1e-8 (the reference's CACHE_LIMIT) on the same grid returns the first call's flux without
evaluating; any other change evaluates."""
import numpy as np
import pytest

import oracle_lib
from tolerance import assert_close

pytestmark = pytest.mark.gpu

P = np.array([6.0, 0.0, 0.9, 30.0, -1.0, 400.0, 0.0, 2.0, 3.1, 1.0, 300.0, 1.0, 0.0, 0.0])


def _grid(n=700, lo=0.3, hi=80.0):
    return np.exp(np.linspace(np.log(lo), np.log(hi), n + 1))


def _delta(gpu, before):
    s = gpu.output_cache_stats()
    return s["lookups"] - before["lookups"], s["hits"] - before["hits"]


def test_repeated_call_is_served_from_the_cache(gpu, oracle, monkeypatch):
    gpu.output_cache_config(50)
    try:
        e = _grid()
        s0 = gpu.output_cache_stats()
        first = gpu.relxilllp(e, P)
        again = gpu.relxilllp(e, P)
        assert _delta(gpu, s0) == (2, 1)
        np.testing.assert_array_equal(first, again)
        st, ref = oracle_lib.evaluate("relxilllp", P, e)
        assert st == 0
        assert_close(first, ref, "relxilllp, first call")

        # within the reference's 1e-8: the same entry
        q = P.copy()
        q[2] += 5e-9
        s1 = gpu.output_cache_stats()
        np.testing.assert_array_equal(gpu.relxilllp(e, q), first)
        assert _delta(gpu, s1) == (1, 1)

        # a parameter beyond 1e-8, another grid, another zone count: evaluated
        q[2] = P[2] + 1e-3
        s2 = gpu.output_cache_stats()
        moved = gpu.relxilllp(e, q)
        other = gpu.relxilllp(_grid(701), P)
        monkeypatch.setenv("RELXILL_NUM_RZONES", "7")
        zones = gpu.relxilllp(e, P)
        monkeypatch.delenv("RELXILL_NUM_RZONES")
        assert _delta(gpu, s2) == (3, 0)
        assert not np.array_equal(moved, first) and len(other) == 701 and not np.array_equal(zones, first)
        st, ref = oracle_lib.evaluate("relxilllp", q, e)
        assert_close(moved, ref, "relxilllp, spin moved by 1e-3")

        # relline is not cached (the reference's relline_kernel has no output cache)
        s3 = gpu.output_cache_stats()
        line = np.array([6.4, 3.0, 3.0, 15.0, 0.9, 30.0, -1.0, 400.0, 0.0, 0.0])
        gpu.relline(_grid(300, 3.0, 8.0), line)
        gpu.relline(_grid(300, 3.0, 8.0), line)
        assert _delta(gpu, s3) == (0, 0)
    finally:
        gpu.output_cache_config(50)


def test_cache_off_and_bounded(gpu):
    e = _grid(400)
    gpu.output_cache_config(0)
    try:
        s0 = gpu.output_cache_stats()
        a = gpu.relxilllp(e, P)
        b = gpu.relxilllp(e, P)
        assert _delta(gpu, s0) == (0, 0) and gpu.output_cache_stats()["entries"] == 0
        np.testing.assert_array_equal(a, b)  # the evaluation itself is deterministic
        gpu.output_cache_config(2)
        for k in range(4):
            q = P.copy()
            q[3] = 20.0 + k
            gpu.relxilllp(e, q)
        assert gpu.output_cache_stats()["entries"] == 2
        s1 = gpu.output_cache_stats()
        q = P.copy()
        q[3] = 20.0  # the oldest of the four, dropped
        gpu.relxilllp(e, q)
        q[3] = 23.0  # the newest, kept
        gpu.relxilllp(e, q)
        assert _delta(gpu, s1) == (2, 1)
    finally:
        gpu.output_cache_config(50)


def test_cache_emptied_when_tables_are_loaded_again(gpu, small_tables):
    """relx_init with another table path reloads the tables and drops every cached flux (an entry
    belongs to the tables it was computed with)."""
    import os

    gpu.output_cache_config(50)
    e = _grid(350)
    gpu.relxilllp(e, P)
    assert gpu.output_cache_stats()["entries"] >= 1
    try:
        gpu.init(small_tables.rstrip("/") + os.sep)  # the same files under another path string
        assert gpu.output_cache_stats()["entries"] == 0
        s0 = gpu.output_cache_stats()
        gpu.relxilllp(e, P)
        assert _delta(gpu, s0) == (1, 0)
    finally:
        gpu.init(small_tables)
