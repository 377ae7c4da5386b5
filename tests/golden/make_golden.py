"""Generate tests/golden/golden_small.npz with the compiled reference
(oracle/_ref/librelxill_ref.so, built by oracle/build_ref.sh from the
reference sources) on the small synthetic tables.

Run from the repository root:  python tests/golden/make_golden.py
The ionisation-gradient cases run with RELXILL_NUM_RZONES=10 and an empty
xillver cache before each evaluation (ref_reset_xillver_cache).
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from relxill_gb300 import synth_tables  # noqa: E402
from cases import CASES, CONV_MODELS, grid, conv_input  # noqa: E402

MODEL_ID = {"relline": 0, "relconv": 1, "relxill": 2, "relxilllp": 3, "relline_lp": 4, "relconv_lp": 5, "xillver": 6,
            "xillverCp": 7, "relxillCp": 8, "relxilllpCp": 9}


def main():
    tdir = os.path.join(ROOT, "_tables", "small")
    synth_tables.ensure_tables(tdir, xill="small")
    os.environ["RELXILL_TABLE_PATH"] = tdir
    os.environ["RELXILL_NUM_RZONES"] = "10"
    ref = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "librelxill_ref.so"))
    dp = ctypes.POINTER(ctypes.c_double)
    out = {}
    for name, model, params, gspec, igt, igi in CASES:
        e = grid(gspec)
        p = np.asarray(params, dtype=np.float64)
        f = conv_input(e) if model in CONV_MODELS else np.zeros(len(e) - 1)
        ref.ref_reset_xillver_cache()
        if igt:
            rc = ref.ref_eval_relxilllp_iongrad(p.ctypes.data_as(dp), igt, ctypes.c_double(igi), e.ctypes.data_as(dp),
                                                len(e) - 1, f.ctypes.data_as(dp))
        else:
            rc = ref.ref_eval(MODEL_ID[model], p.ctypes.data_as(dp), e.ctypes.data_as(dp), len(e) - 1,
                              f.ctypes.data_as(dp))
        assert rc == 0, name
        out[name] = f
        print(name, f.sum())
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_small.npz"), **out)


if __name__ == "__main__":
    main()
