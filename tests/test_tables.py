"""Synthetic tables: the FITS layout the reference loaders expect."""
import os

import numpy as np

from relxill_gb300 import fits, synth_tables


def test_fits_roundtrip(tmp_path):
    path = str(tmp_path / "t.fits")
    cols = [fits.Column("x", "E", 3, np.arange(12, dtype=np.float32).reshape(4, 3)),
            fits.Column("n", "J", 1, np.arange(4, dtype=np.int32)[:, None]),
            fits.Column("s", "A", 8, np.array(["ab", "cde", "f", "Incl"]))]
    with open(path, "wb") as f:
        f.write(fits.primary_header())
        f.write(fits.bintable("T1", cols, 4))
    h = fits.read_hdus(path)
    assert [x.name for x in h] == ["", "T1"]
    t = fits.read_table(path, h[1])
    np.testing.assert_array_equal(t["x"], np.arange(12, dtype=np.float32).reshape(4, 3))
    assert list(t["s"]) == ["ab", "cde", "f", "Incl"]
    assert os.path.getsize(path) % 2880 == 0


def test_relline_table_layout(small_tables):
    path = os.path.join(small_tables, synth_tables.RELTABLE_FILENAME)
    h = fits.read_hdus(path)
    a = fits.read_table(path, fits.find_hdu(h, "a"))["a"].ravel()
    mu0 = fits.read_table(path, fits.find_hdu(h, "mu0"))["mu0"].ravel()
    assert len(h) == len(a) * len(mu0) + 3            # reltable.c:290: HDU ii*n_mu0+jj+4
    assert h[3].name == "1_1" and h[-1].name == f"{len(a)}_{len(mu0)}"
    t = fits.read_table(path, h[3])
    r = t["r"].ravel()
    assert np.all(np.diff(r) < 0) and r[0] == 1000.0  # radii descend from 1000
    assert np.all(t["gmax"] > t["gmin"])


def test_xillver_table_layout(small_tables):
    path = os.path.join(small_tables, synth_tables.XILLTABLE_FILENAME)
    h = fits.read_hdus(path)
    p = fits.read_table(path, fits.find_hdu(h, "PARAMETERS"))
    assert list(p["NAME"]) == ["Gamma", "A_Fe", "logXi", "Ecut", "Incl"]  # Incl last (xilltable.c:229-233)
    n = p["NUMBVALS"].ravel()
    s = fits.find_hdu(h, "SPECTRA")
    assert s.nrows == int(np.prod(n))
    rows = fits.read_table(path, s, rows=(0, int(n[-1]) + 1))
    # incl is the fastest index of the rows (get_xillspec_rownum, xilltable.c:325-337)
    np.testing.assert_allclose(rows["PARAMVAL"][: n[-1], 4], p["VALUE"][4][: n[-1]])
    assert rows["PARAMVAL"][n[-1], 3] == p["VALUE"][3][1]


def test_tables_are_deterministic(tmp_path):
    a = synth_tables.relline_arrays(n_a=4, n_mu0=3, n_r=10, n_g=5, seed=3)
    b = synth_tables.relline_arrays(n_a=4, n_mu0=3, n_r=10, n_g=5, seed=3)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
