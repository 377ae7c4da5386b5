"""Build the CUDA library of the package (librelxill_gb300.so) in-tree.

nvcc compiles every translation unit for sm_103a only, in parallel, and links
a shared library with the C ABI of include/relxill_gb300.h.  No torch build
machinery is involved: the library is plain C ABI and loads with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "librelxill_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-Xptxas", "-v"]
SOURCES = ["setup.cu", "relline.cu", "xillver.cu", "xillver_model.cu", "conv.cu", "runtime.cu", "relcache.cu", "serve.cu",
           "noalloc.cu", "table_ingest.cu", "nthcomp.cu", "measure.cu", "fits_reader.cpp"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _compile(src: str, obj: str, verbose: bool) -> str:
    cmd = [nvcc(), *ARCH, *CU_FLAGS, "-c", os.path.join(SRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr if verbose else ""


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "relxill_gb300.h"))
    objs, jobs = [], []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for s in SOURCES:
            obj = os.path.join(OUT_DIR, s.rsplit(".", 1)[0] + ".o")
            objs.append(obj)
            if force or _stale(obj, [os.path.join(SRC, s), *headers]):
                jobs.append(ex.submit(_compile, s, obj, verbose))
        logs = [j.result() for j in jobs]
    if verbose:
        for l in logs:
            sys.stderr.write(l)
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
