"""The C-ABI library builds, loads without a GPU and exports every function
declared in include/relxill_gb300.h."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "relxill_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(\w+)\s*\([^;]*\)\s*;", src)) - {"if", "while"})


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for n in ("c_lmodrelline", "c_lmodrelconv", "c_lmodrelxill", "c_lmodrelxilllp", "c_lmodrellinelp",
              "c_lmodrelconvlp", "c_lmodxillver", "c_lmodxillverdensnthcomp", "c_lmodrelxilldensnthcomp",
              "c_lmodrelxilllpdensnthcomp", "c_lmodxillverns", "c_lmodrelxillns", "relx_eval_batch",
              "relx_eval_batch_device", "relx_last_status", "relx_init"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from relxill_gb300 import build

    path = build.build()
    lib = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_layer_refuses_without_library(monkeypatch):
    import relxill_gb300 as R

    monkeypatch.setattr(R, "LIB_PATH", "/nonexistent/librelxill_gb300.so")
    monkeypatch.setattr(R, "_lib", None)
    try:
        R.lib()
    except RuntimeError as e:
        assert "missing" in str(e)
    else:
        raise AssertionError("no error without the CUDA library")


def test_unsupported_public_models_zero_flux_and_report():
    """xillverNS and relxillNS of the public model list link, return zeros and status 3 (no GPU needed)."""
    from relxill_gb300 import build

    lib = ctypes.CDLL(build.build())
    dp = ctypes.POINTER(ctypes.c_double)
    e = (ctypes.c_double * 11)(*[1.0 + i for i in range(11)])
    par = (ctypes.c_double * 13)()
    for name in ("c_lmodxillverns", "c_lmodrelxillns"):
        f = getattr(lib, name)
        f.argtypes = [dp, ctypes.c_int, dp, ctypes.c_int, dp, dp, ctypes.c_char_p]
        f.restype = None
        flux = (ctypes.c_double * 10)(*([7.0] * 10))
        f(e, 10, par, 0, flux, None, None)
        assert list(flux) == [0.0] * 10
        lib.relx_last_status.restype = ctypes.c_int
        assert lib.relx_last_status() == 3


def test_output_cache_bookkeeping_without_a_gpu():
    """The local-model output cache's configuration and counters need no GPU."""
    from relxill_gb300 import build

    lib = ctypes.CDLL(build.build())
    out = (ctypes.c_int64 * 3)()
    assert lib.relx_output_cache_config(ctypes.c_int(-1)) != 0
    assert lib.relx_output_cache_config(ctypes.c_int(3)) == 0
    assert lib.relx_output_cache_stats(out) == 0
    assert out[2] == 0
    assert lib.relx_output_cache_config(ctypes.c_int(50)) == 0
