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
              "c_lmodrelconvlp", "c_lmodxillver", "relx_eval_batch",
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
