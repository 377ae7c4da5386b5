"""The xillver table decoded on the GPU: a table with a value that is not
finite is refused with status 2, and reloading the good tables gives the
same spectra as before."""
import os
import shutil

import numpy as np
import pytest

from cases import log_grid

pytestmark = pytest.mark.gpu


def test_table_with_nan_is_refused_and_reload_restores(gpu, small_tables, tmp_path):
    from relxill_gb300 import fits, synth_tables

    e = log_grid(0.1, 1000.0, 800)
    p = np.array([[2.0, 1.0, 300.0, 3.1, 0.0, 30.0, -1.0]])
    want, _ = gpu.eval_batch("xillver", p, [e])
    bad = tmp_path / "bad"
    bad.mkdir()
    for name in os.listdir(small_tables):
        if name.endswith(".fits") and name != synth_tables.XILLTABLE_FILENAME:
            os.symlink(os.path.join(small_tables, name), bad / name)
    path = str(bad / synth_tables.XILLTABLE_FILENAME)
    shutil.copyfile(os.path.join(small_tables, synth_tables.XILLTABLE_FILENAME), path)
    hdu = fits.find_hdu(fits.read_hdus(path), "SPECTRA")
    col_off = 4 * 5  # PARAMVAL (5 floats) precedes INTPSPEC in a row
    with open(path, "r+b") as f:
        f.seek(hdu.offset + 7 * hdu.width + col_off + 4 * 100)
        f.write(b"\x7f\xc0\x00\x00")  # big-endian quiet NaN
    L = gpu.lib()
    try:
        st = L.relx_init(str(bad).encode())
        assert st == 2
        assert "not finite" in L.relx_last_error().decode()
    finally:
        assert L.relx_init(small_tables.encode()) == 0
    got, st = gpu.eval_batch("xillver", p, [e])
    assert not st.any()
    np.testing.assert_array_equal(got[0], want[0])
