"""relxill_gb300: relxill's relativistic convolution path on GB300 (sm_103a).

The package is a thin host layer over the C ABI of ``librelxill_gb300.so``
(include/relxill_gb300.h).  It mirrors the reference's local-model interface:
one function per model taking the energy grid (bin edges in keV) and the
parameter array in the order of ``lmodel_relxill_public.dat`` and returning
the photon flux per bin, plus a batched call for many parameter sets with
different energy grids.

There is no CPU fallback: if the CUDA library is missing, or no GPU is
present, calls raise.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librelxill_gb300.so")

MODELS: Dict[str, int] = {"relline": 0, "relconv": 1, "relxill": 2, "relxilllp": 3, "relline_lp": 4,
                          "relconv_lp": 5, "xillver": 6, "xillverCp": 7, "relxillCp": 8, "relxilllpCp": 9}
CONV_MODELS = ("relconv", "relconv_lp")  # models that take the caller's spectrum in `flux`

# parameter names and defaults of lmodel_relxill_public.dat:1-84 (in order)
PARAMS: Dict[str, List[Tuple[str, float]]] = {
    "relline": [("lineE", 6.4), ("Index1", 3.0), ("Index2", 3.0), ("Rbr", 15.0), ("a", 0.998), ("Incl", 30.0),
                ("Rin", -1.0), ("Rout", 400.0), ("z", 0.0), ("limb", 0.0)],
    "relconv": [("Index1", 3.0), ("Index2", 3.0), ("Rbr", 15.0), ("a", 0.998), ("Incl", 30.0), ("Rin", -1.0),
                ("Rout", 400.0), ("limb", 0.0)],
    "relxill": [("Index1", 3.0), ("Index2", 3.0), ("Rbr", 15.0), ("a", 0.998), ("Incl", 30.0), ("Rin", -1.0),
                ("Rout", 400.0), ("z", 0.0), ("gamma", 2.0), ("logxi", 3.1), ("Afe", 1.0), ("Ecut", 300.0),
                ("refl_frac", 3.0)],
    "relxilllp": [("h", 6.0), ("beta", 0.0), ("a", 0.998), ("Incl", 30.0), ("Rin", -1.0), ("Rout", 400.0),
                  ("z", 0.0), ("gamma", 2.0), ("logxi", 3.1), ("Afe", 1.0), ("Ecut", 300.0), ("refl_frac", 1.0),
                  ("switch_returnrad", 1.0), ("switch_reflfrac_boost", 0.0)],
    "relline_lp": [("lineE", 6.4), ("h", 6.0), ("a", 0.998), ("Incl", 30.0), ("Rin", -1.0), ("Rout", 400.0),
                   ("z", 0.0), ("limb", 0.0), ("gamma", 2.0), ("switch_returnrad", 1.0)],
    "relconv_lp": [("h", 6.0), ("beta", 0.0), ("a", 0.998), ("Incl", 30.0), ("Rin", -1.0), ("Rout", 400.0),
                   ("limb", 0.0), ("gamma", 2.0), ("switch_returnrad", 1.0)],
    "xillver": [("gamma", 2.0), ("Afe", 1.0), ("Ecut", 300.0), ("logxi", 3.1), ("z", 0.0), ("Incl", 30.0),
                ("refl_frac", -1.0)],
    "xillverCp": [("gamma", 2.0), ("Afe", 1.0), ("kTe", 60.0), ("logxi", 3.1), ("logN", 15.0), ("z", 0.0),
                  ("Incl", 30.0), ("refl_frac", -1.0)],
    "relxillCp": [("Incl", 30.0), ("a", 0.998), ("Rin", -1.0), ("Rout", 400.0), ("Rbr", 15.0), ("Index1", 3.0),
                  ("Index2", 3.0), ("z", 0.0), ("gamma", 2.0), ("logxi", 3.1), ("logN", 15.0), ("Afe", 1.0),
                  ("kTe", 60.0), ("refl_frac", 3.0)],
    "relxilllpCp": [("Incl", 30.0), ("a", 0.998), ("Rin", -1.0), ("Rout", 400.0), ("h", 6.0), ("beta", 0.0),
                    ("gamma", 2.0), ("logxi", 3.1), ("logN", 15.0), ("Afe", 1.0), ("kTe", 60.0), ("refl_frac", 1.0),
                    ("z", 0.0), ("iongrad_index", 0.0), ("iongrad_type", 0.0), ("switch_returnrad", 1.0),
                    ("switch_reflfrac_boost", 0.0)],
}
LMOD_SYMBOL = {"relline": "c_lmodrelline", "relconv": "c_lmodrelconv", "relxill": "c_lmodrelxill",
               "relxilllp": "c_lmodrelxilllp", "relline_lp": "c_lmodrellinelp", "relconv_lp": "c_lmodrelconvlp",
               "xillver": "c_lmodxillver", "xillverCp": "c_lmodxillverdensnthcomp",
               "relxillCp": "c_lmodrelxilldensnthcomp", "relxilllpCp": "c_lmodrelxilllpdensnthcomp"}

STATUS = {0: "ok", 1: "parameter out of range", 2: "table inconsistent", 3: "unsupported option",
          4: "radial grid outside the table", 5: "relconv input sum <= 0", 6: "CUDA error",
          7: "device memory", 8: "device wait timed out", 9: "bad arguments", 10: "tables not loaded"}


class RelxillError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"relxill_gb300 status {status} ({STATUS.get(status, '?')}){': ' + message if message else ''}")


_lib: Optional[ctypes.CDLL] = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_int64)


def lib() -> ctypes.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m relxill_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    L.relx_init.argtypes = [ctypes.c_char_p]
    L.relx_init.restype = ctypes.c_int
    L.relx_last_error.restype = ctypes.c_char_p
    L.relx_last_status.restype = ctypes.c_int
    L.relx_eval_batch.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _lp, _dp, _dp, _ip, _ip, _dp]
    L.relx_eval_batch.restype = ctypes.c_int
    L.relx_eval_batch_device.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         _lp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _ip,
                                         ctypes.c_void_p, ctypes.c_void_p]
    L.relx_eval_batch_device.restype = ctypes.c_int
    L.relx_table_bytes.argtypes = [_lp]
    L.relx_table_bytes.restype = ctypes.c_int
    L.relx_tuning_config.argtypes = [ctypes.c_int, ctypes.c_int]
    L.relx_tuning_config.restype = ctypes.c_int
    L.relx_tuning_report.argtypes = [_dp, ctypes.c_int]
    L.relx_tuning_report.restype = ctypes.c_int
    L.relx_cache_config.argtypes = [ctypes.c_int]
    L.relx_cache_config.restype = ctypes.c_int
    L.relx_cache_stats.argtypes = [_lp]
    L.relx_cache_stats.restype = ctypes.c_int
    L.relx_output_cache_config.argtypes = [ctypes.c_int]
    L.relx_output_cache_config.restype = ctypes.c_int
    L.relx_output_cache_stats.argtypes = [_lp]
    L.relx_output_cache_stats.restype = ctypes.c_int
    L.relx_serve_create.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int]
    L.relx_serve_create.restype = ctypes.c_void_p
    L.relx_serve_submit.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                    ctypes.c_double]
    L.relx_serve_submit.restype = ctypes.c_int64
    L.relx_serve_poll.argtypes = [ctypes.c_void_p, _lp, _ip, _dp, ctypes.c_int]
    L.relx_serve_poll.restype = ctypes.c_int
    L.relx_serve_wait.argtypes = [ctypes.c_void_p, ctypes.c_int64, _ip]
    L.relx_serve_wait.restype = ctypes.c_int
    L.relx_serve_stats.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int]
    L.relx_serve_stats.restype = ctypes.c_int
    L.relx_serve_destroy.argtypes = [ctypes.c_void_p]
    L.relx_serve_destroy.restype = None
    for name in LMOD_SYMBOL.values():
        fn = getattr(L, name)
        fn.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, ctypes.c_char_p]
        fn.restype = None
    _lib = L
    return L


def _ptr(a: np.ndarray, t=_dp):
    return a.ctypes.data_as(t)


def init(table_path: Optional[str] = None) -> None:
    """Load the tables onto the current GPU (RELXILL_TABLE_PATH if not given)."""
    L = lib()
    st = L.relx_init(table_path.encode() if table_path else None)
    if st:
        raise RelxillError(st, L.relx_last_error().decode())


def last_error() -> str:
    return lib().relx_last_error().decode()


def _as_params(model: str, params) -> np.ndarray:
    p = np.ascontiguousarray(params, dtype=np.float64)
    npar = len(PARAMS[model])
    if p.ndim == 1:
        p = p[None, :]
    if p.shape[1] != npar:
        raise ValueError(f"{model} takes {npar} parameters, got {p.shape[1]}")
    return p


def pack_grids(energies: Sequence[np.ndarray]) -> Tuple[np.ndarray, np.ndarray]:
    """Concatenate per-set bin-edge arrays; returns (edges, offsets[n_sets+1])."""
    offs = np.zeros(len(energies) + 1, dtype=np.int64)
    for i, e in enumerate(energies):
        offs[i + 1] = offs[i] + len(e)
    return np.concatenate([np.asarray(e, dtype=np.float64) for e in energies]), offs


def eval_batch(model: str, params, energies: Sequence[np.ndarray], flux_in: Optional[Sequence[np.ndarray]] = None,
               ion_grad_type: Optional[Sequence[int]] = None, iongrad_index: Optional[Sequence[float]] = None,
               check: bool = True) -> Tuple[List[np.ndarray], np.ndarray]:
    """Evaluate many parameter sets, each on its own energy grid, in one batch.

    Returns (list of flux arrays, per-set status array)."""
    L = lib()
    p = _as_params(model, params)
    n = p.shape[0]
    if len(energies) != n:
        raise ValueError("one energy grid per parameter set")
    edges, offs = pack_grids(energies)
    nflux = int(offs[-1]) - n
    flux = np.zeros(nflux, dtype=np.float64)
    status = np.zeros(n, dtype=np.int32)
    fin = None
    if model in CONV_MODELS:
        if flux_in is None:
            raise ValueError(f"{model} needs the input spectra")
        fin = np.concatenate([np.asarray(f, dtype=np.float64) for f in flux_in])
    igt = None if ion_grad_type is None else np.ascontiguousarray(ion_grad_type, dtype=np.int32)
    igi = None if iongrad_index is None else np.ascontiguousarray(iongrad_index, dtype=np.float64)
    st = L.relx_eval_batch(MODELS[model], n, _ptr(p), _ptr(edges), _ptr(offs, _lp),
                           _ptr(fin) if fin is not None else None, _ptr(flux), _ptr(status, _ip),
                           _ptr(igt, _ip) if igt is not None else None, _ptr(igi) if igi is not None else None)
    if check and st and not np.any(status):
        raise RelxillError(st, L.relx_last_error().decode())
    out = [flux[offs[i] - i: offs[i + 1] - i - 1] for i in range(n)]
    return out, status


def _lmod(model: str, energy, params, flux_in=None) -> np.ndarray:
    L = lib()
    e = np.ascontiguousarray(energy, dtype=np.float64)
    p = _as_params(model, params)[0].copy()
    nflux = len(e) - 1
    flux = np.zeros(nflux) if flux_in is None else np.array(flux_in, dtype=np.float64)
    getattr(L, LMOD_SYMBOL[model])(_ptr(e), nflux, _ptr(p), 0, _ptr(flux), None, None)
    st = L.relx_last_status()
    if st:
        raise RelxillError(st, L.relx_last_error().decode())
    return flux


def relline(energy, params) -> np.ndarray:
    """relline photon flux per bin (c_lmodrelline)."""
    return _lmod("relline", energy, params)


def relconv(energy, params, flux) -> np.ndarray:
    """relconv applied to `flux` on the grid `energy` (c_lmodrelconv)."""
    return _lmod("relconv", energy, params, flux)


def relxill(energy, params) -> np.ndarray:
    """relxill photon flux per bin (c_lmodrelxill)."""
    return _lmod("relxill", energy, params)


def relxilllp(energy, params) -> np.ndarray:
    """relxilllp photon flux per bin (c_lmodrelxilllp)."""
    return _lmod("relxilllp", energy, params)


def relline_lp(energy, params) -> np.ndarray:
    """relline_lp photon flux per bin (c_lmodrellinelp)."""
    return _lmod("relline_lp", energy, params)


def relconv_lp(energy, params, flux) -> np.ndarray:
    """relconv_lp applied to `flux` on the grid `energy` (c_lmodrelconvlp)."""
    return _lmod("relconv_lp", energy, params, flux)


def xillver(energy, params) -> np.ndarray:
    """xillver photon flux per bin (c_lmodxillver)."""
    return _lmod("xillver", energy, params)


def xillverCp(energy, params) -> np.ndarray:
    """xillverCp photon flux per bin (c_lmodxillverdensnthcomp)."""
    return _lmod("xillverCp", energy, params)


def relxillCp(energy, params) -> np.ndarray:
    """relxillCp photon flux per bin (c_lmodrelxilldensnthcomp)."""
    return _lmod("relxillCp", energy, params)


def relxilllpCp(energy, params) -> np.ndarray:
    """relxilllpCp photon flux per bin (c_lmodrelxilllpdensnthcomp)."""
    return _lmod("relxilllpCp", energy, params)


def default_params(model: str) -> np.ndarray:
    return np.array([v for _, v in PARAMS[model]], dtype=np.float64)


def log_grid(emin: float, emax: float, nbins: int) -> np.ndarray:
    """nbins log-spaced bins (nbins+1 edges), like get_log_grid (relutility.c:399-405)."""
    return np.exp(np.linspace(np.log(emin), np.log(emax), nbins + 1))


def tuning_config(autotune: bool = True, graphs: bool = True) -> None:
    """Autotuned line-kernel tiles / pipelined chunks, and CUDA-graph replay of recurring batch shapes."""
    lib().relx_tuning_config(1 if autotune else 0, 1 if graphs else 0)


def tuning_report() -> List[Dict[str, float]]:
    out = np.zeros(64 * 6)
    n = lib().relx_tuning_report(_ptr(out), 64)
    keys = ("model", "size_class", "zones", "line_tile", "chunk", "best_ms")
    return [dict(zip(keys, out[i * 6:(i + 1) * 6].tolist())) for i in range(n)]


def cache_config(slots: int) -> None:
    """Device line-profile cache with `slots` entries (0 turns it off)."""
    st = lib().relx_cache_config(int(slots))
    if st:
        raise RelxillError(st, last_error())


def cache_stats() -> Dict[str, int]:
    out = np.zeros(3, dtype=np.int64)
    st = lib().relx_cache_stats(_ptr(out, _lp))
    if st:
        raise RelxillError(st, last_error())
    return {"lookups": int(out[0]), "hits": int(out[1]), "slots": int(out[2])}


def output_cache_config(max_entries: int) -> None:
    """Output cache of the local-model calls (relxill family): the last `max_entries` calls are kept
    (50 by default, as the reference's RelxillCache); 0 turns it off."""
    st = lib().relx_output_cache_config(int(max_entries))
    if st:
        raise RelxillError(st, last_error())


def output_cache_stats() -> Dict[str, int]:
    out = np.zeros(3, dtype=np.int64)
    st = lib().relx_output_cache_stats(_ptr(out, _lp))
    if st:
        raise RelxillError(st, last_error())
    return {"lookups": int(out[0]), "hits": int(out[1]), "entries": int(out[2])}


class Server:
    """Serving engine (relx_serve_*): continuous batching of single-spectrum requests.

    The HBM budget is allocated here (half per batch slot) and every batch is
    carved from it; a request that alone needs more than half of it completes
    with status 7.  The energy grid, the input spectrum (relconv) and the
    output array of a request must stay alive until the request completes;
    `submit` keeps references to them."""

    STATS = ("completed", "batches", "mean_batch", "p50_ms", "p99_ms", "max_ms", "waiting", "last_error")

    def __init__(self, hbm_budget_bytes: int = 8 << 30, max_batch: int = 4096, cache_slots: int = 0):
        L = lib()
        self._h = L.relx_serve_create(int(hbm_budget_bytes), int(max_batch), int(cache_slots))
        if not self._h:
            raise RelxillError(last_status_or(6), last_error())
        self._keep: Dict[int, tuple] = {}

    def submit(self, model: str, params, energy: np.ndarray, out: np.ndarray, flux_in: Optional[np.ndarray] = None,
               ion_grad_type: int = 0, iongrad_index: float = 0.0) -> int:
        p = np.ascontiguousarray(params, dtype=np.float64)
        if energy.dtype != np.float64 or not energy.flags.c_contiguous:
            raise ValueError("energy must be a contiguous float64 array")
        if out.dtype != np.float64 or not out.flags.c_contiguous or len(out) != len(energy) - 1:
            raise ValueError("out must be a contiguous float64 array of len(energy) - 1")
        rid = lib().relx_serve_submit(self._h, MODELS[model], _ptr(p), _ptr(energy), len(energy) - 1,
                                      _ptr(flux_in) if flux_in is not None else None, _ptr(out),
                                      int(ion_grad_type), float(iongrad_index))
        if rid < 0:
            raise RelxillError(int(-rid), last_error())
        self._keep[rid] = (p, energy, out, flux_in)
        return int(rid)

    def poll(self, max_n: int = 4096) -> List[Tuple[int, int, float]]:
        ids = np.zeros(max_n, dtype=np.int64)
        sts = np.zeros(max_n, dtype=np.int32)
        lat = np.zeros(max_n, dtype=np.float64)
        n = lib().relx_serve_poll(self._h, _ptr(ids, _lp), _ptr(sts, _ip), _ptr(lat), max_n)
        res = [(int(ids[i]), int(sts[i]), float(lat[i])) for i in range(n)]
        for rid, _, _ in res:
            self._keep.pop(rid, None)
        return res

    def stats(self, reset: bool = False) -> Dict[str, float]:
        out = np.zeros(8)
        lib().relx_serve_stats(self._h, _ptr(out), 8, 1 if reset else 0)
        return dict(zip(self.STATS, out.tolist()))

    def close(self) -> None:
        if self._h:
            lib().relx_serve_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def last_status_or(default: int) -> int:
    st = lib().relx_last_status()
    return st if st else default

