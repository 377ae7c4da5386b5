#!/usr/bin/env python3
"""Benchmark: batched relxilllp spectra per second on GB300.

Workload (one step): 4096 relxilllp parameter sets, h ~ U[3,100] rg,
a ~ U[0,0.998], incl ~ U[5,85] deg, Gamma ~ U[1.4,2.8], logxi ~ U[0,4.5],
A_Fe = 1, Ecut = 300 keV, beta = 0, Rin = ISCO, Rout = 400 rg, refl_frac = 1,
returning radiation off; each set has its own energy grid of U{300..5000}
log-spaced bins over 0.3-80 keV; 10 radial zones.  Tables are the seeded
synthetic tables in the reference FITS layouts at full size (relline
25x30x100x40, lamp post 20x250x100, xillver 13x4x16x10x10 x 2999 bins,
1 GB), written to _tables/full on first use.

value: spectra/s with inputs resident in HBM (device-pointer C ABI).
e2e:   the same through the host-buffer C ABI (relx_eval_batch), copies
       of parameters, grids and fluxes included.
--impl reference: the CPU oracle (C restatement of the reference) on all
       host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "relxilllp spectra/s batched vs plain GPU at ≤1e-4 rel err; serve p50/p99 ms"
N_SETS = 4096
# DRAM bytes (read + write) of one step's line-profile launches over the 4096-set workload (ncu, one-pass
# capture): the per-set interpolated table (line_table_kernel) and the line profile (relline_kernel)
LINE_DRAM_BYTES_4096 = (33.64e6 + 205.33e6) + (391.13e6 + 561.29e6)
WORKLOAD = ("relxilllp batched, 4096 sets per GPU, per-set grids 300-5000 log bins 0.3-80 keV, "
            "10 radial zones")
N_PROF = 9  # kernel kinds of the per-kernel event profiler (relx_profile_name)
FLOPS_PER_EVAL = 25  # FP32 operations of one integrand evaluation (relb_func, Relprofile.cpp:489-521)


def workload(n: int, seed_params: int = 2026, seed_grids: int = 7):
    """Parameter sets and energy grids of the batched relxilllp workload."""
    rng = np.random.default_rng(seed_params)
    h = rng.uniform(3, 100, n)
    a = rng.uniform(0, 0.998, n)
    inc = rng.uniform(5, 85, n)
    gam = rng.uniform(1.4, 2.8, n)
    lxi = rng.uniform(0, 4.5, n)
    p = np.zeros((n, 14))
    p[:, 0], p[:, 2], p[:, 3], p[:, 7], p[:, 8] = h, a, inc, gam, lxi
    p[:, 1] = 0.0      # beta
    p[:, 4] = -1.0     # Rin = ISCO
    p[:, 5] = 400.0    # Rout
    p[:, 9] = 1.0      # A_Fe
    p[:, 10] = 300.0   # Ecut
    p[:, 11] = 1.0     # refl_frac
    rg = np.random.default_rng(seed_grids)
    nb = rg.integers(300, 5001, n)
    grids = [np.exp(np.linspace(np.log(0.3), np.log(80.0), int(k) + 1)) for k in nb]
    return p, grids


def iongrad_workload(n: int):
    """The relxilllp draws of the ionisation-gradient leg (ALPHA gradient, 10 zones; the gradient type
    travels beside the parameters)."""
    return workload(n, seed_params=2027, seed_grids=8)


def rrad_workload(n: int):
    """The relxilllp draws with returning radiation on ($switch_returnrad = 1)."""
    params, grids = workload(n, seed_params=2028, seed_grids=9)
    params = params.copy()
    params[:, 12] = 1.0
    return params, grids


def cp_workload(n: int):
    """relxilllpCp sets from the same draws: logN 15-19, kTe 20-300 keV (lmodel_relxill_public.dat:112-129)."""
    base, grids = workload(n, seed_params=2029, seed_grids=10)
    rng = np.random.default_rng(2030)
    p = np.zeros((n, 17))
    p[:, 0], p[:, 1], p[:, 2], p[:, 3] = base[:, 3], base[:, 2], -1.0, 400.0   # Incl, a, Rin, Rout
    p[:, 4], p[:, 5], p[:, 6], p[:, 7] = base[:, 0], 0.0, base[:, 7], base[:, 8]  # h, beta, gamma, logxi
    p[:, 8] = rng.uniform(15.0, 19.0, n)                                         # logN
    p[:, 9], p[:, 10], p[:, 11] = 1.0, rng.uniform(20.0, 300.0, n), 1.0          # Afe, kTe, refl_frac
    return p, grids


# ----------------------------------------------------------------------------
# serving workload: walkers of a sampler, Poisson arrivals
# ----------------------------------------------------------------------------
# relxilllp: h, a, incl move on full steps; Gamma, logxi, A_Fe, Ecut, refl_frac on every step
LP_SPEC = {"rel": {0: (1.0, 3.0, 100.0), 2: (0.01, 0.0, 0.998), 3: (1.0, 5.0, 85.0)},
           "xill": {7: (0.02, 1.4, 2.8), 8: (0.05, 0.0, 4.5), 9: (0.05, 0.5, 10.0), 10: (5.0, 20.0, 1000.0),
                    11: (0.05, 0.1, 10.0)}}
# relxill: Index1, a, incl on full steps; Gamma, logxi, A_Fe, Ecut, refl_frac on every step
BKN_SPEC = {"rel": {0: (0.05, 1.5, 5.0), 3: (0.01, 0.0, 0.998), 4: (1.0, 5.0, 85.0)},
            "xill": {8: (0.02, 1.4, 2.8), 9: (0.05, 0.0, 4.5), 10: (0.05, 0.5, 10.0), 11: (5.0, 20.0, 1000.0),
                     12: (0.05, 0.1, 10.0)}}


def serve_walkers(n_walkers: int, seed: int = 42):
    """Walkers: half relxilllp, half relxill, each with a fixed grid of U{300..5000} bins over 0.3-80 keV."""
    rng = np.random.default_rng(seed)
    lp, _ = workload(n_walkers, seed_params=seed + 1, seed_grids=seed + 2)
    models, params, grids = [], [], []
    for w in range(n_walkers):
        nb = int(rng.integers(300, 5001))
        grids.append(np.exp(np.linspace(np.log(0.3), np.log(80.0), nb + 1)))
        if w % 2 == 0:
            models.append("relxilllp")
            params.append(lp[w].copy())
        else:
            models.append("relxill")
            params.append(np.array([rng.uniform(2, 4), 3.0, 15.0, rng.uniform(0, 0.998), rng.uniform(5, 85), -1.0,
                                    400.0, 0.0, rng.uniform(1.4, 2.8), rng.uniform(0, 4.5), 1.0, 300.0, 2.0]))
    return models, params, grids


def run_serve(R, seconds: float, rate: float, n_walkers: int, budget_gb: float, seed: int = 42):
    """Open-loop Poisson arrivals from sampler walkers through the serving engine (relx_serve_*).

    Each request moves its walker: with probability 0.7 only the xillver parameters change
    (Gamma, logxi, A_Fe, Ecut, refl_frac), otherwise the relativistic ones too.  Latency is
    submit to result in the client's buffer."""
    L = R.lib()
    models, params, grids = serve_walkers(n_walkers, seed)
    rng = np.random.default_rng(seed + 3)
    n_req = int(seconds * rate)
    t_arr = np.cumsum(rng.exponential(1.0 / rate, n_req))
    who = rng.integers(0, n_walkers, n_req)
    full = rng.random(n_req) >= 0.7
    noise = rng.standard_normal((n_req, 14))
    ring = 16
    outs = [[np.zeros(len(g) - 1) for _ in range(ring)] for g in grids]
    count = np.zeros(n_walkers, dtype=np.int64)
    dp = ctypes.POINTER(ctypes.c_double)
    mid = {"relline": 0, "relconv": 1, "relxill": 2, "relxilllp": 3}
    keep = {}  # sampled requests for the parity check: id -> (model, params, walker, ring slot, walker's request no.)
    srv = R.Server(hbm_budget_bytes=int(budget_gb * (1 << 30)), max_batch=2048, cache_slots=4096)
    try:
        # warm-up: one request per walker
        for w in range(n_walkers):
            srv.submit(models[w], params[w], grids[w], outs[w][0])
        t0 = time.perf_counter()
        while srv.stats()["completed"] < n_walkers and time.perf_counter() - t0 < 60:
            srv.poll()
            time.sleep(0.001)
        srv.poll()
        srv.stats(reset=True)
        c0 = R.cache_stats()
        done = 0
        start = time.perf_counter()
        for k in range(n_req):
            w = int(who[k])
            spec = LP_SPEC if models[w] == "relxilllp" else BKN_SPEC
            p = params[w]
            for i, (sd, lo, hi) in spec["xill"].items():
                p[i] = min(max(p[i] + sd * noise[k, i], lo), hi)
            if full[k]:
                for i, (sd, lo, hi) in spec["rel"].items():
                    p[i] = min(max(p[i] + sd * noise[k, i], lo), hi)
            slot = int(count[w] % ring)
            count[w] += 1
            out = outs[w][slot]
            while time.perf_counter() - start < t_arr[k]:
                pass
            rid = L.relx_serve_submit(srv._h, mid[models[w]], p.ctypes.data_as(dp), grids[w].ctypes.data_as(dp),
                                      len(grids[w]) - 1, None, out.ctypes.data_as(dp), 0, 0.0)
            if rid < 0:
                raise RuntimeError(f"relx_serve_submit: {-rid}")
            if k >= n_req - 4096 and k % 61 == 0:
                keep[int(rid)] = (models[w], p.copy(), w, slot, int(count[w] - 1))
            if k % 64 == 0:
                done += len(srv.poll())
        t_sub = time.perf_counter() - start
        while done < n_req and time.perf_counter() - start < t_sub + 60:
            done += len(srv.poll())
            time.sleep(0.0005)
        elapsed = time.perf_counter() - start
        st = srv.stats()
        c1 = R.cache_stats()
        # the sampled results against the same sets evaluated alone (ring slots are not reused for
        # 16 requests of the walker, so check only requests that are still in place)
        same = True
        checked = 0
        for rid, (model, pp, w, slot, nw) in keep.items():
            if count[w] - 1 - nw >= ring:  # the ring slot has been reused since
                continue
            alone, sts = R.eval_batch(model, pp[None], [grids[w]])
            same = same and bool(np.array_equal(alone[0], outs[w][slot]))
            checked += 1
    finally:
        srv.close()
        R.cache_config(0)
    lookups = c1["lookups"] - c0["lookups"]
    return {"walkers": n_walkers, "models": "relxilllp and relxill (half each)", "offered_rate": rate,
            "achieved_submit_rate": n_req / t_sub, "requests": n_req, "seconds": round(elapsed, 3),
            "spectra_s": done / elapsed, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
            "batches": int(st["batches"]), "mean_batch": st["mean_batch"], "hbm_budget_gb": budget_gb,
            "cache_hit_rate": (c1["hits"] - c0["hits"]) / lookups if lookups else None,
            "xillver_only_steps": 0.7, "identical_to_alone": same, "checked": checked}


def _time_device_variant(R, L, torch, dev, steps: int, warmup: int, params, grids, igt_value: int, n_check: int = 2,
                         model: str = "relxilllp", profile_steps: int = 0):
    """A batched model through the device API on its own stream (CUDA events on that stream):
    spectra/s, ms per step and the largest per-bin error of n_check sets against the oracle;
    with profile_steps, per-kernel times of that many further steps (outside the timed region)."""
    mid = R.MODELS[model]
    n = len(grids)
    edges, offs = R.pack_grids(grids)
    nflux = int(offs[-1]) - n
    igt = np.full(n, igt_value, dtype=np.int32)
    d_params = torch.from_numpy(params).to(dev)
    d_e = torch.from_numpy(edges).to(dev)
    d_off = torch.from_numpy(offs).to(dev)
    d_igt = torch.from_numpy(igt).to(dev)
    d_igi = torch.zeros(n, dtype=torch.float64, device=dev)
    d_flux = torch.empty(nflux, dtype=torch.float64, device=dev)
    d_status = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    offs_ptr = offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    igt_ptr = igt.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    use_igt = igt_value != 0

    def step():
        st = L.relx_eval_batch_device(mid, n, d_params.data_ptr(), d_e.data_ptr(), d_off.data_ptr(), offs_ptr, None,
                                      d_flux.data_ptr(), d_status.data_ptr(), d_igt.data_ptr() if use_igt else None,
                                      igt_ptr if use_igt else None, d_igi.data_ptr() if use_igt else None,
                                      stream.cuda_stream)
        if st:
            raise RuntimeError(f"relx_eval_batch_device: {st} {R.last_error()}")

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    assert int((d_status != 0).sum()) == 0
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        ev0.record()
    for _ in range(steps):
        step()
    with torch.cuda.stream(stream):
        ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    out = d_flux.cpu().numpy()
    kernels = None
    if profile_steps > 0:
        L.relx_profile_enable(1)
        for _ in range(profile_steps):
            step()
        torch.cuda.synchronize()
        ms_k = (ctypes.c_double * N_PROF)()
        n_k = (ctypes.c_int64 * N_PROF)()
        L.relx_profile_read(ms_k, n_k, N_PROF)
        L.relx_profile_enable(0)
        kernels = {L.relx_profile_name(k).decode(): round(ms_k[k] / profile_steps, 4)
                   for k in range(N_PROF) if n_k[k] > 0}
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib

    max_err = 0.0
    for i in range(min(n_check, n)):
        st, ref = oracle_lib.evaluate(model, params[i], grids[i], None, igt_value, 0.0)
        got = out[offs[i] - i: offs[i + 1] - i - 1]
        m = ref > 1e-6 * ref.max()
        max_err = max(max_err, float(np.max(np.abs(got[m] / ref[m] - 1))))
    r = {"value": n * steps / (ms / 1e3), "unit": "spectra/s", "sets": n, "steps": steps,
         "ms_per_step": ms / steps, "max_rel_err_vs_oracle": max_err}
    if kernels is not None:
        r["kernel_ms_per_step"] = kernels
    return r


def run_iongrad(R, L, torch, dev, steps: int, warmup: int, n: int = 2048):
    """Batched relxilllp with the ALPHA ionisation gradient (IonGradient.cpp:128-171) over 10 zones:
    2048 sets of the same draws, device buffers, CUDA events on the launching stream."""
    os.environ["RELXILL_NUM_RZONES"] = "10"
    try:
        params, grids = iongrad_workload(n)
        r = _time_device_variant(R, L, torch, dev, steps, warmup, params, grids, 2)
        r.update({"zones": 10, "mode": "ALPHA ionisation gradient (IonGradient.cpp:128-171)"})
        return r
    finally:
        os.environ.pop("RELXILL_NUM_RZONES", None)


def run_rrad(R, L, torch, dev, steps: int, warmup: int, n: int = N_SETS):
    """The 4096-set relxilllp workload with returning radiation switched on ($switch_returnrad = 1,
    the reference's default): the return-table emissivity, the zones' xillver flux corrections for
    a > 0 and the emissivity recomputed with them (Relxill.cpp:336-344)."""
    params, grids = rrad_workload(n)
    r = _time_device_variant(R, L, torch, dev, steps, warmup, params, grids, 0, profile_steps=2)
    r.update({"zones": 10, "mode": "returning radiation on (Relreturn_Corona.cpp, Relreturn_Table.cpp)"})
    return r


def run_cp(R, L, torch, dev, steps: int, warmup: int, n: int = N_SETS):
    """The 4096-set workload as relxilllpCp: nthcomp continua for the source and the 10 zones
    (donthcomp.c), 6-parameter xillverCp brackets (32 corners per zone), logN 15-19, kTe 20-300 keV."""
    p, grids = cp_workload(n)
    r = _time_device_variant(R, L, torch, dev, steps, warmup, p, grids, 0, model="relxilllpCp", profile_steps=2)
    r.update({"zones": 10, "mode": "relxilllpCp: nthcomp primary and zone normalisations, 6-parameter xillverCp table "
                                   "(synthetic, 4x3x4x4x3 grid x 10 inclinations)"})
    return r


def tables(kind: str = "full") -> str:
    from relxill_gb300 import synth_tables

    d = os.path.join(ROOT, "_tables", kind)
    synth_tables.ensure_tables(d, xill=kind)
    return d


# ----------------------------------------------------------------------------
# CPU oracle (reference algorithm restated in C), multi-process
# ----------------------------------------------------------------------------
_oracle = None


def _oracle_init(tdir: str):
    global _oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib

    _oracle = oracle_lib
    oracle_lib.lib(tdir)


def _oracle_eval(args):
    """One oracle evaluation: its status and the integrand evaluations it made."""
    p, e = args
    lib = _oracle.lib()
    lib.relxo_relb_calls.restype = ctypes.c_longlong
    lib.relxo_relb_calls(1)
    st, f = _oracle.evaluate("relxilllp", p, e)
    return st, int(lib.relxo_relb_calls(1))


def cpu_pool(tdir: str, procs: int):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib

    oracle_lib.build()
    ctx = mp.get_context("spawn")
    return ctx.Pool(procs, initializer=_oracle_init, initargs=(tdir,))


def cpu_rate(pool, params, grids, idx):
    """Spectra per second of the oracle over the sets idx, the seconds taken, and the integrand
    evaluations per set (the line profile's algorithmic work, counted by the oracle)."""
    t0 = time.perf_counter()
    res = pool.map(_oracle_eval, [(params[i], grids[i]) for i in idx], chunksize=1)
    dt = time.perf_counter() - t0
    assert not any(st for st, _ in res)
    return len(idx) / dt, dt, sum(n for _, n in res) / max(len(res), 1)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    tdir = tables("full")
    procs = os.cpu_count() or 1
    params, grids = workload(N_SETS)
    pool = cpu_pool(tdir, procs)
    per_step = max(procs * 2, 32)
    rng = np.random.default_rng(11)
    # warm-up (table loads)
    for _ in range(args.warmup):
        cpu_rate(pool, params, grids, rng.choice(N_SETS, per_step, replace=False))
    times = []
    for _ in range(args.steps):
        r, dt, _ = cpu_rate(pool, params, grids, rng.choice(N_SETS, per_step, replace=False))
        times.append(dt)
    pool.close()
    total = per_step * args.steps / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": total, "unit": "spectra/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sets_per_gpu": N_SETS, "parallelism": "CPU processes",
                   "tables": "synthetic full-size (xillver 1 GB)",
                   "sample": f"{per_step} sets per step drawn from the 4096-set workload"},
        "cpu_baseline": {"value": total, "unit": "spectra/s", "cores": procs, "kind": "port",
                         "sample": f"{per_step} sets per step x {args.steps} steps on {procs} processes"},
        "e2e": {"value": total, "unit": "spectra/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        out = os.environ.get("RELX_CLOCK_LOG_DIR")  # keep the raw samples there (default: the temp folder)
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv", dir=out if out and os.path.isdir(out) else None)
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def run_gpu(args):
    import torch

    import relxill_gb300 as R

    from relxill_gb300 import replicas

    rank, world, local = replicas.rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    tdir = tables("full")
    # CPU baseline pool first (spawned processes, before the GPU context exists in them)
    pool = None
    procs = os.cpu_count() or 1
    if rank == 0 and not args.no_cpu_baseline:
        pool = cpu_pool(tdir, procs)
    L = R.lib()
    torch.zeros(1, device=f"cuda:{local}")  # the CUDA context first: the load time below is the tables'
    t_load = time.perf_counter()
    R.init(tdir)
    table_load_s = time.perf_counter() - t_load
    L.relx_profile_enable.argtypes = [ctypes.c_int]
    L.relx_profile_read.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64), ctypes.c_int]
    L.relx_profile_name.restype = ctypes.c_char_p
    L.relx_launch_count.restype = ctypes.c_int64
    L.relx_batch_stats.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
    tb = ctypes.c_int64(0)
    L.relx_table_bytes(ctypes.byref(tb))

    S = args.sets
    seed_p, seed_g = replicas.rank_seeds(rank)
    params, grids = workload(S, seed_params=seed_p, seed_grids=seed_g)
    edges, offs = R.pack_grids(grids)
    nflux = int(offs[-1]) - S
    dev = torch.device("cuda", local)
    d_params = torch.from_numpy(params).to(dev)
    d_e = torch.from_numpy(edges).to(dev)
    d_off = torch.from_numpy(offs).to(dev)
    d_flux = torch.empty(nflux, dtype=torch.float64, device=dev)
    d_status = torch.empty(S, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    offs_ptr = offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))

    def step():
        st = L.relx_eval_batch_device(3, S, d_params.data_ptr(), d_e.data_ptr(), d_off.data_ptr(), offs_ptr, None,
                                      d_flux.data_ptr(), d_status.data_ptr(), None, None, None, stream.cuda_stream)
        if st:
            raise RuntimeError(f"relx_eval_batch_device: {st} {R.last_error()}")

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    assert int((d_status != 0).sum()) == 0, "sets failed"
    st6 = (ctypes.c_int64 * 5)()
    L.relx_batch_stats(S, st6)

    # timed region: the production path (autotuned tiles, the step replayed as a CUDA graph)
    clocks = Clocks(local)
    clocks.start()
    l0 = L.relx_launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        ev0.record()
    for _ in range(args.steps):
        step()
    with torch.cuda.stream(stream):
        ev1.record()
    torch.cuda.synchronize()
    barrier()
    launches = L.relx_launch_count() - l0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    # second timed region of the same steps with every kernel bracketed by CUDA events on its
    # stream (no graph replay while profiling): per-kernel times and the roofline
    # (one range per batch: with pipelined chunks the kernels of two streams overlap in time)
    os.environ["RELX_CHUNK_SETS"] = "0"
    L.relx_profile_enable(1)
    torch.cuda.synchronize()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    os.environ.pop("RELX_CHUNK_SETS", None)
    ms_k = (ctypes.c_double * N_PROF)()
    n_k = (ctypes.c_int64 * N_PROF)()
    L.relx_profile_read(ms_k, n_k, N_PROF)
    L.relx_profile_enable(0)
    ms = replicas.max_over_ranks(ms, dist, dev)
    value = replicas.job_throughput(S, args.steps, world, ms / 1e3)

    # end-to-end through the host-buffer C ABI (copies in the timed region)
    e2e = None
    if not args.no_e2e:
        flux = np.zeros(nflux)
        status = np.zeros(S, dtype=np.int32)
        pp = params.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        ep = edges.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        fp = flux.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        sp = status.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        for _ in range(args.warmup):  # untimed: the group shapes' graphs are captured here
            L.relx_eval_batch(3, S, pp, ep, offs_ptr, None, fp, sp, None, None)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rc = L.relx_eval_batch(3, S, pp, ep, offs_ptr, None, fp, sp, None, None)
            assert rc == 0
        t1 = time.perf_counter()
        dt = replicas.max_over_ranks(t1 - t0, dist, dev)
        e2e = {"value": replicas.job_throughput(S, args.steps, world, dt), "unit": "spectra/s",
               "h2d_bytes_per_step": int(params.nbytes + edges.nbytes + offs.nbytes),
               "d2h_bytes_per_step": int(flux.nbytes + status.nbytes)}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # plain path: one synchronous c_lmodrelxilllp call per spectrum, every call evaluated (the output
    # cache of the local-model calls would serve the warm-up sets again)
    plain = None
    if not args.no_plain:
        n_plain = min(64, S)
        R.output_cache_config(0)
        for i in range(min(4, S)):
            R.relxilllp(grids[i], params[i])
        t0 = time.perf_counter()
        for i in range(n_plain):
            R.relxilllp(grids[i], params[i])
        plain = {"value": n_plain / (time.perf_counter() - t0), "unit": "spectra/s",
                 "sample": f"{n_plain} single c_lmodrelxilllp calls, output cache off"}
        R.output_cache_config(50)

    # parity spot check against the oracle (outside the timed region)
    out = d_flux.cpu().numpy()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib

    oracle_lib.lib(tdir)
    max_err = max_tot = 0.0
    for i in range(min(4, S)):
        s, ref = oracle_lib.evaluate("relxilllp", params[i], grids[i])
        got = out[offs[i] - i: offs[i + 1] - i - 1]
        m = ref > 1e-6 * ref.max()
        max_err = max(max_err, float(np.max(np.abs(got[m] / ref[m] - 1))))
        max_tot = max(max_tot, abs(float(got.sum() / ref.sum()) - 1))

    # CPU baseline on a bounded sample; the oracle also counts the integrand evaluations per set
    cpu = None
    evals_per_set = None
    if pool is not None:
        idx = np.arange(min(args.cpu_sample, S))
        cpu_rate(pool, params, grids, idx[: procs])  # warm the workers
        r, dt, evals_per_set = cpu_rate(pool, params, grids, idx)
        pool.close()
        cpu = {"value": r, "unit": "spectra/s", "cores": procs, "kind": "port",
               "sample": f"{len(idx)} sets of the workload on {procs} spawned processes ({dt:.1f} s)"}

    iongrad = None
    if not args.no_iongrad:
        iongrad = run_iongrad(R, L, torch, dev, args.steps, args.warmup)
    rrad = None
    if not args.no_rrad:
        rrad = run_rrad(R, L, torch, dev, args.steps, args.warmup)
    cp = None
    if not args.no_cp:
        cp = run_cp(R, L, torch, dev, args.steps, args.warmup, n=S)

    serve = None
    if not args.no_serve:
        serve = run_serve(R, args.serve_seconds, args.serve_rate, args.walkers, args.serve_budget_gb)

    # rooflines.  The line-profile kernel is bound by FP32 instruction issue: its algorithmic work is
    # the oracle's count of integrand evaluations (one branch each) times FLOPS_PER_EVAL, over the
    # FP32 FMA rate measured on this GPU (relx_fp32_rate); its memory term (the four transfer-function
    # corner tables of the set read and the set's interpolated table written by the table kernel, the
    # interpolated table and the radius records read, the profile written) is printed beside it.  The
    # xillver kernel reads its corner rows through L2 (sets are visited in table-row order, so
    # neighbouring sets share rows): its algorithmic row bytes over its time are an L2 rate.
    names = [L.relx_profile_name(k).decode() for k in range(N_PROF)]
    per = {names[k]: (ms_k[k] / max(n_k[k], 1), int(n_k[k])) for k in range(N_PROF)}
    total_k = sum(ms_k[k] for k in range(N_PROF))
    dom = max(range(N_PROF), key=lambda k: ms_k[k])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    L.relx_fp32_rate.argtypes = [ctypes.POINTER(ctypes.c_double)]
    fp32 = ctypes.c_double(0.0)
    fp32_gflops = fp32.value if L.relx_fp32_rate(ctypes.byref(fp32)) == 0 else None
    line_ms = per["relline"][0]
    roof = {"kernel": "relline", "launches": ["line_table_kernel", "relline_kernel"], "bound": "fp32",
            "achieved": None, "peak": None, "unit": "TFLOP/s", "frac": None,
            "traffic": None, "peak_source": "measured FP32 FMA rate (relx_fp32_rate, CUDA events)"}
    if evals_per_set is not None and fp32_gflops:
        flops = evals_per_set * FLOPS_PER_EVAL * S
        roof.update({"achieved": flops / (line_ms * 1e-3) / 1e12, "peak": fp32_gflops / 1e3,
                     "algorithmic_flops": flops, "evals_per_set": evals_per_set,
                     "flops_per_eval": FLOPS_PER_EVAL})
        roof["frac"] = roof["achieved"] / roof["peak"]
    # DRAM bytes (read + write) of the line-profile launches of one step over the 4096-set workload, from
    # the one-pass ncu capture in the profiles folder (dram_traffic_relxilllp_4096sets.md); other batch
    # sizes are scaled by their set count
    roof["traffic"] = LINE_DRAM_BYTES_4096 * S / 4096
    roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of line_table_kernel and relline_kernel, "
                              "4096-set launch, scaled by sets")
    ng, nr_tab = 40, 100
    line_bytes = (S * (4 * nr_tab * ng * 16 + nr_tab * ng * 16 + nr_tab * ng * 8 + 1000 * 64) +
                  int(st6[2]) * int(st6[1] // max(S, 1) or 1) * 4)
    roof["hbm_term"] = {"algorithmic_bytes": line_bytes, "achieved_gbs": line_bytes / (line_ms * 1e-3) / 1e9,
                        "peak_gbs": hbm_peak, "frac": line_bytes / (line_ms * 1e-3) / 1e9 / hbm_peak}
    x_pad = int(st6[3])  # floats per table row on the convolution grid
    ucount = int(st6[0])
    nz_sum = int(st6[1])
    # algorithmic bytes of the xillver kernel per launch: unique corner rows x incl x conv-grid bins (read) + zone
    # spectra (write)
    xill_bytes = ucount * 10 * x_pad * 4 + nz_sum * x_pad * 4
    xill_ms = per["xillver"][0]
    xill_roof = {"kernel": "xillver", "bound": "l2", "achieved": xill_bytes / (xill_ms * 1e-3) / 1e9,
                 "unit": "GB/s", "algorithmic_bytes": xill_bytes,
                 "note": "rows shared by neighbouring sets come from L2; DRAM sees a small fraction of the "
                         "algorithmic bytes (ncu summary in the profiles folder)"}
    kernels = {n: {"ms_per_launch": round(per[n][0], 4), "launches": per[n][1],
                   "share": round(ms_k[k] / total_k, 4) if total_k else None} for k, n in enumerate(names)}
    # the long, descriptive entries first and the headline last, so that a reader of the line's tail
    # (a log that keeps the end) still sees the numbers
    line = {
        "tuning": R.tuning_report(), "graphs": "step replayed as a CUDA graph after its second launch",
        "kernels": kernels, "rooflines_other": [xill_roof],
        "serve": serve, "ion_gradient": iongrad, "returning_radiation": rrad, "cp_flavour": cp,
        "table_load": {"seconds": table_load_s, "bytes": int(tb.value)},
        "config": {"workload": WORKLOAD, "sets_per_gpu": S, "parallelism": f"replicas x{world}",
                   "tables": f"synthetic full-size, {tb.value / 1e9:.2f} GB on the device",
                   "l2": "inputs larger than L2 (1 GB xillver table, ~2 GB workspace per step)"},
        "clocks": clk, "roofline": roof, "dominant_kernel": names[dom], "cpu_baseline": cpu,
        "max_rel_err_vs_oracle": max_err, "max_total_err_vs_oracle": max_tot, "gpu_launches": int(launches),
        "plain_gpu": plain, "batched_over_plain": (value / world / plain["value"]) if plain else None,
        "serve_p50_ms": serve["p50_ms"] if serve else None, "serve_p99_ms": serve["p99_ms"] if serve else None,
        "metric": METRIC, "unit": "spectra/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 radii, grids and normalisation sums)", "data": "synthetic",
        "e2e": e2e, "value": value,
    }
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def spawn_replicas(args) -> int:
    """--gpus N without a launcher: one process per GPU through torch.distributed.run on this node
    (RANK, LOCAL_RANK and WORLD_SIZE set for each), the same command line otherwise."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def run_dry(args) -> int:
    """The replica bookkeeping without a GPU (for tests of the launch path): gloo ranks, a fixed
    sleep per step in place of the batch, max over ranks, whole-job throughput."""
    from relxill_gb300 import replicas

    rank, world, local = replicas.rank_info()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        time.sleep(0.01)
    dt = replicas.max_over_ranks(time.perf_counter() - t0, dist)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": replicas.job_throughput(args.sets, args.steps, world, dt),
                          "unit": "spectra/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "dry_run": True, "ranks": world, "local_rank": local}))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sets", type=int, default=N_SETS)
    ap.add_argument("--cpu-sample", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-iongrad", action="store_true")
    ap.add_argument("--no-rrad", action="store_true")
    ap.add_argument("--no-cp", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--serve-rate", type=float, default=50000.0)
    ap.add_argument("--walkers", type=int, default=256)
    ap.add_argument("--serve-budget-gb", type=float, default=8.0)
    ap.add_argument("--dry-run", action="store_true", help="replica bookkeeping only, no GPU (tests)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_replicas(args)
    if args.dry_run:
        return run_dry(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
