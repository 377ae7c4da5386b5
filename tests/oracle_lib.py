"""ctypes access to the CPU oracle (oracle/librelx_oracle.so) for the tests.

The oracle is the C restatement of the reference's algorithm (test
infrastructure); it is built here with make and never used by the product.
"""
from __future__ import annotations

import ctypes
import multiprocessing as mp
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "librelx_oracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "librelxill_ref.so")
MODELS = {"relline": 0, "relconv": 1, "relxill": 2, "relxilllp": 3, "relline_lp": 4, "relconv_lp": 5, "xillver": 6,
          "xillverCp": 7, "relxillCp": 8, "relxilllpCp": 9}
_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return ORACLE_SO


def lib(table_path: str | None = None) -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(ORACLE_SO)
        L.relxo_eval.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_int, _dp]
        L.relxo_eval_ext.argtypes = [ctypes.c_int, _dp, ctypes.c_int, ctypes.c_double, _dp, ctypes.c_int, _dp]
        L.relxo_set_table_path.argtypes = [ctypes.c_char_p]
        L.relxo_rebin_spectrum.argtypes = [_dp, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int]
        L.relxo_rebin_spectrum.restype = None
        for name in ("relxo_kerr_rms",):
            getattr(L, name).argtypes = [ctypes.c_double]
            getattr(L, name).restype = ctypes.c_double
        L.relxo_gi_potential_lp.argtypes = [ctypes.c_double] * 5
        L.relxo_gi_potential_lp.restype = ctypes.c_double
        L.relxo_norm_wrt_xillver.argtypes = [_dp, _dp, ctypes.c_int]
        L.relxo_norm_wrt_xillver.restype = ctypes.c_double
        L.relxo_primary_norm_factor.argtypes = [ctypes.c_double, ctypes.c_double]
        L.relxo_primary_norm_factor.restype = ctypes.c_double
        L.relxo_norm_change.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.relxo_norm_change.restype = ctypes.c_double
        L.relxo_conv_spectrum_normalized.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int]
        L.relxo_conv_spectrum_normalized.restype = None
        L.relxo_conv_grid.argtypes = [_dp]
        L.relxo_conv_grid.restype = None
        _lib = L
    if table_path is not None:
        _lib.relxo_set_table_path(table_path.encode())
    return _lib


def p(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)


def evaluate(model: str, params, energy, flux_in=None, ion_grad_type: int = 0, iongrad_index: float = 0.0):
    """One oracle evaluation; returns (status, flux)."""
    L = lib()
    e = np.ascontiguousarray(energy, dtype=np.float64)
    par = np.ascontiguousarray(params, dtype=np.float64)
    flux = np.zeros(len(e) - 1) if flux_in is None else np.array(flux_in, dtype=np.float64)
    st = L.relxo_eval_ext(MODELS[model], par.ctypes.data_as(_dp), ion_grad_type, iongrad_index,
                          e.ctypes.data_as(_dp), len(e) - 1, flux.ctypes.data_as(_dp))
    return st, flux


def conv_grid() -> np.ndarray:
    g = np.zeros(4097)
    lib().relxo_conv_grid(g.ctypes.data_as(_dp))
    return g


def _pool_init(table_path: str, env: dict) -> None:
    os.environ.update(env)
    lib(table_path)


def _pool_eval(args):
    model, params, energy, flux_in, igt, igi = args
    return evaluate(model, params, energy, flux_in, igt, igi)


def pool(table_path: str, procs: int | None = None, env: dict | None = None):
    """A pool of spawned processes, each with the oracle on table_path (the oracle keeps the first
    tables it loads, so other tables need other processes).  env: variables the children set first
    (RELXILL_NUM_RZONES)."""
    build()
    n = procs or max(1, min(16, os.cpu_count() or 1))
    return mp.get_context("spawn").Pool(n, initializer=_pool_init, initargs=(table_path, dict(env or {})))


def evaluate_many(pl, jobs):
    """jobs: (model, params, energy, flux_in, ion_grad_type, iongrad_index) tuples; [(status, flux)]."""
    return pl.map(_pool_eval, jobs, chunksize=1)
