"""Parity over many parameter sets, per bin and in the total flux.

* The batched relxilllp workload of the throughput measurement on the full-size tables: 128 of
  its 4096 sets, and 32 sets each of its ionisation-gradient, returning-radiation and
  relxilllpCp variants, taken from a 4096-set batch evaluated on the GPU in one call.
* A random sweep of 100 sets per model over the ranges of the public model list
  (lmodel_relxill_public.dat), each set on its own random grid, on the small tables.

The oracle runs in spawned processes (it keeps the first tables it loads)."""
import os

import numpy as np
import pytest

import oracle_lib
from cases import CONV_MODELS, conv_input
from tolerance import compare, REL_BIN, REL_TOTAL

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ZONES_ENV = {"RELXILL_NUM_RZONES": "10"}


def _check(name, got, ref, gst, ost, failures, worst):
    if (gst != 0) != (ost != 0):
        failures.append(f"{name}: status GPU {gst} oracle {ost}")
        return
    if ost != 0:
        return
    r, t = compare(got, ref)
    worst[0] = max(worst[0], r)
    worst[1] = max(worst[1], t)
    if r > REL_BIN or t > REL_TOTAL:
        failures.append(f"{name}: per-bin {r:.3e}, total {t:.3e}")


def _report(failures, worst, what):
    print(f"{what}: worst per-bin {worst[0]:.3e}, worst total {worst[1]:.3e}")
    per = {}
    for f in failures:
        per[f.split(" set ")[0]] = per.get(f.split(" set ")[0], 0) + 1
    assert not failures, f"{len(failures)} sets off the bar {per}; first: " + "; ".join(failures[:8])


# ---------------------------------------------------------------------------
# the throughput workload on the full-size tables
# ---------------------------------------------------------------------------
@pytest.fixture()
def full_tables(gpu, small_tables):
    from relxill_gb300 import synth_tables

    d = os.path.join(ROOT, "_tables", "full")
    synth_tables.ensure_tables(d, xill="full")
    gpu.init(d)
    yield d
    gpu.init(small_tables)  # the other modules compare against the oracle on the small tables


def _bench():
    import importlib
    import sys

    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    return importlib.import_module("bench")


def test_throughput_workload_full_tables(gpu, full_tables, monkeypatch):
    bench = _bench()
    n = bench.N_SETS
    legs = [  # (name, model, params, grids, ion_grad_type, stride)
        ("relxilllp", "relxilllp", *bench.workload(n), 0, 32),
        ("iongrad", "relxilllp", *bench.iongrad_workload(n), 2, 128),
        ("rrad", "relxilllp", *bench.rrad_workload(n), 0, 128),
        ("cp", "relxilllpCp", *bench.cp_workload(n), 0, 128),
    ]
    failures, worst = [], [0.0, 0.0]
    pl = oracle_lib.pool(full_tables, env=ZONES_ENV)
    try:
        for name, model, params, grids, igt, stride in legs:
            if igt:
                monkeypatch.setenv("RELXILL_NUM_RZONES", "10")
            else:
                monkeypatch.delenv("RELXILL_NUM_RZONES", raising=False)
            out, st = gpu.eval_batch(model, params, grids, ion_grad_type=[igt] * n if igt else None,
                                     iongrad_index=[0.0] * n if igt else None, check=False)
            idx = list(range(0, n, stride))
            res = oracle_lib.evaluate_many(pl, [(model, params[i], grids[i], None, igt, 0.0) for i in idx])
            for i, (ost, ref) in zip(idx, res):
                _check(f"{name} set {i}", out[i], ref, int(st[i]), ost, failures, worst)
    finally:
        pl.close()
        pl.join()
    _report(failures, worst, "throughput workload, full-size tables")


# ---------------------------------------------------------------------------
# random sweep, every model, small tables
# ---------------------------------------------------------------------------
def _rin(rng):
    u = rng.uniform()
    if u < 0.7:
        return -1.0
    if u < 0.85:
        return -rng.uniform(1.0, 3.0)  # in units of the ISCO
    return rng.uniform(2.0, 20.0)


def _geom(rng):
    return dict(a=rng.uniform(-0.998, 0.998), incl=rng.uniform(5.0, 85.0), rin=_rin(rng),
                rout=float(np.exp(rng.uniform(np.log(50.0), np.log(1000.0)))),
                z=0.0 if rng.uniform() < 0.7 else rng.uniform(0.0, 0.3))


def _xill(rng, cp):
    d = dict(gam=rng.uniform(1.4, 3.2), lxi=rng.uniform(0.0, 4.7), afe=rng.uniform(0.5, 10.0),
             rf=rng.uniform(0.1, 10.0) if rng.uniform() < 0.8 else -rng.uniform(0.1, 3.0))
    if cp:
        d.update(kte=float(np.exp(rng.uniform(np.log(5.0), np.log(400.0)))), logn=rng.uniform(15.0, 20.0))
    else:
        d.update(ecut=float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0)))))
    return d


def _random_set(model, rng):
    """(params, ion_grad_type, iongrad_index) of one set; parameter order of lmodel_relxill_public.dat."""
    g = _geom(rng)
    i1, i2, rbr = rng.uniform(-1.0, 8.0), rng.uniform(-1.0, 6.0), rng.uniform(3.0, 100.0)
    limb = int(rng.integers(0, 3))
    h, beta = rng.uniform(3.0, 100.0), (0.0 if rng.uniform() < 0.7 else rng.uniform(0.0, 0.6))
    rr = int(rng.choice([0, 1, -1]))
    boost = int(rng.integers(0, 2))
    line_e = rng.uniform(1.0, 10.0)
    igt, igi = 0, 0.0
    if model == "relline":
        p = [line_e, i1, i2, rbr, g["a"], g["incl"], g["rin"], g["rout"], g["z"], limb]
    elif model == "relconv":
        p = [i1, i2, rbr, g["a"], g["incl"], g["rin"], g["rout"], limb]
    elif model == "relline_lp":
        p = [line_e, h, g["a"], g["incl"], g["rin"], g["rout"], g["z"], limb, rng.uniform(1.4, 3.4), rr]
    elif model == "relconv_lp":
        p = [h, beta, g["a"], g["incl"], g["rin"], g["rout"], limb, rng.uniform(1.4, 3.4), rr]
    elif model == "relxill":
        x = _xill(rng, False)
        p = [i1, i2, rbr, g["a"], g["incl"], g["rin"], g["rout"], g["z"], x["gam"], x["lxi"], x["afe"], x["ecut"],
             x["rf"]]
    elif model == "relxilllp":
        x = _xill(rng, False)
        p = [h, beta, g["a"], g["incl"], g["rin"], g["rout"], g["z"], x["gam"], x["lxi"], x["afe"], x["ecut"],
             x["rf"], rr, boost]
        u = rng.uniform()
        if u < 0.2:
            igt, igi = 1, rng.uniform(0.0, 3.0)
        elif u < 0.4:
            igt = 2
    elif model == "xillver":
        x = _xill(rng, False)
        p = [x["gam"], x["afe"], x["ecut"], x["lxi"], g["z"], g["incl"], x["rf"]]
    elif model == "xillverCp":
        x = _xill(rng, True)
        p = [x["gam"], x["afe"], x["kte"], x["lxi"], x["logn"], g["z"], g["incl"], x["rf"]]
    elif model == "relxillCp":
        x = _xill(rng, True)
        p = [g["incl"], g["a"], g["rin"], g["rout"], rbr, i1, i2, g["z"], x["gam"], x["lxi"], x["logn"], x["afe"],
             x["kte"], x["rf"]]
    elif model == "relxilllpCp":
        x = _xill(rng, True)
        u = rng.uniform()
        pig, pgt = (rng.uniform(0.0, 3.0), 1) if u < 0.2 else ((0.0, 2) if u < 0.4 else (0.0, 0))
        p = [g["incl"], g["a"], g["rin"], g["rout"], h, beta, x["gam"], x["lxi"], x["logn"], x["afe"], x["kte"],
             x["rf"], g["z"], pig, pgt, rr, boost]
    else:
        raise ValueError(model)
    return np.array(p, dtype=np.float64), igt, igi


def _random_grid(model, params, rng):
    nb = int(rng.integers(200, 2001))
    if model in ("relline", "relline_lp"):
        e0 = params[0]
        lo, hi = e0 * rng.uniform(0.05, 0.4), e0 * rng.uniform(1.3, 2.0)
    elif model in CONV_MODELS:
        lo, hi = rng.uniform(0.1, 0.5), rng.uniform(50.0, 200.0)
    else:
        lo, hi = rng.uniform(0.1, 1.0), rng.uniform(20.0, 500.0)
    return np.exp(np.linspace(np.log(lo), np.log(hi), nb + 1))


SWEEP_MODELS = ("relline", "relconv", "relline_lp", "relconv_lp", "relxill", "relxilllp", "xillver", "xillverCp",
                "relxillCp", "relxilllpCp")


def test_random_sweep_every_model(gpu, small_tables, monkeypatch):
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")
    n = 100
    failures, worst = [], [0.0, 0.0]
    pl = oracle_lib.pool(small_tables, env=ZONES_ENV)
    try:
        for k, model in enumerate(SWEEP_MODELS):
            rng = np.random.default_rng(5000 + k)
            sets = [_random_set(model, rng) for _ in range(n)]
            params = [s[0] for s in sets]
            grids = [_random_grid(model, p, rng) for p in params]
            fin = [conv_input(e) for e in grids] if model in CONV_MODELS else None
            igt = [s[1] for s in sets]
            igi = [s[2] for s in sets]
            out, st = gpu.eval_batch(model, np.array(params), grids, flux_in=fin,
                                     ion_grad_type=igt if any(igt) else None,
                                     iongrad_index=igi if any(igt) else None, check=False)
            jobs = [(model, params[i], grids[i], fin[i] if fin else None, igt[i], igi[i]) for i in range(n)]
            for i, (ost, ref) in enumerate(oracle_lib.evaluate_many(pl, jobs)):
                _check(f"{model} set {i} {np.array2string(params[i], precision=4)} igt {igt[i]}", out[i], ref,
                       int(st[i]), ost, failures, worst)
    finally:
        pl.close()
        pl.join()
    _report(failures, worst, "random sweep, small tables")
