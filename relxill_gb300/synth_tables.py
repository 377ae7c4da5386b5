"""Seeded synthetic relxill tables, written in the reference FITS layouts.

The real tables (``rel_table_v0.5a.fits``, ``rel_lp_table_v0.5b.fits``,
``xillver-a-Ec5.fits``) are not distributed with the reference, so every run
works on synthetic tables with the same layout, shapes and value ranges:

* relline table: the layout read by ``read_relline_table``
  (reltable.c:235-311): extension ``a`` (column ``a``), extension ``mu0``
  (column ``mu0``), then one extension per (spin, mu0) pair at HDU number
  ``ii*n_mu0+jj+4`` with ``n_r`` rows and columns ``r``, ``gmin``, ``gmax``
  and the ``n_g``-vectors ``trff1``, ``trff2``, ``cosne1``, ``cosne2``
  (reltable.c:171-232).  Radii descend from 1000 to just inside the ISCO.
  gmin/gmax follow the Keplerian redshift of a ring, the transfer functions
  are smooth analytic shapes with a seeded 1% smooth perturbation.
* lamp-post table: extension ``I_h`` with one row per spin and columns ``a``,
  ``hgrid``, ``r`` and ``h{k}``, ``del{k}``, ``del_inc{k}`` for k = 1..n_h
  (reltable.c:313-381).  Intensities follow the Newtonian lamp-post
  emissivity (Relphysics.cpp:282-288) times a GR-like boost and a seeded
  smooth perturbation; the angles are geometric.
* xillver table: OGIP table model with PARAMETERS (col 1 NAME, col 9
  NUMBVALS, col 10 VALUE; Incl last), ENERGIES (cols 1-2) and SPECTRA (col 2)
  in the row order of ``get_xillspec_rownum`` (xilltable.c:325-337).  Each
  spectrum is a cut-off power law plus a 6.4 keV Gaussian whose equivalent
  width rises with logXi, scaled by 10^logXi, times lognormal noise (sigma
  0.05).
* xillverCp table (nthcomp continuum, common.h:166): the same OGIP layout
  with six parameters, Gamma, A_Fe, logXi, kTe, Dens, Incl (row order of the
  6-parameter get_xillspec_rownum, xilltable.c:325-337); spectra as above
  with a cut-off at 2.7 kTe and scaled by 10^(Dens - 15) as well (the loader
  divides by both, xilltable.c:478-485).  Small grid (4 x 3 x 4 x 4 x 3 x 10).
* returning-radiation table: extension ``SPIN`` (column ``a``), then one
  extension ``FRAC01``, ``FRAC02``, ... per spin with 50 rows (one per
  incident radial bin, Relreturn_Table.cpp:180-330) and double columns
  ``rlo``, ``rhi``, the 50-vectors ``frac_e``, ``tf_r``, ``gmin``, ``gmax``
  (one element per emitting bin), the 50x20-vector ``frac_g`` and ``f_ret``,
  ``f_bh``, ``f_inf``.  Radial bins are log-spaced from the table spin's ISCO
  to 1000; the transfer fractions fall off with the distance between the
  rings, the energy shifts follow the ratio of the radii and the g
  distributions are smooth bumps, each with a seeded perturbation.

Dimensions default to the ones the reference loaders hard-code
(common.h:69-81: 25 spins x 30 mu0 x 100 radii x 40 g*, lamp post
20 spins x 250 heights x 100 radii) so the same files can be read by the
reference's own loaders.  The xillver dimensions are read from the file by
every loader and default to 13 Gamma x 4 A_Fe x 16 logXi x 10 Ecut x 10 Incl
x 2999 energies over 0.07-1000 keV.
"""
from __future__ import annotations

import argparse
import math
import os
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import fits

RELTABLE_FILENAME = "rel_table_v0.5a.fits"
LPTABLE_FILENAME = "rel_lp_table_v0.5b.fits"
XILLTABLE_FILENAME = "xillver-a-Ec5.fits"
RRADTABLE_FILENAME = "table_returnRad_v20220301.fits"
XILLTABLE_CP_FILENAME = "xillverCp_v3.4.fits"
RRAD_NR = 50  # common.h:127-128
RRAD_NG = 20
RRAD_SPINS = (-0.998, -0.5, 0.0, 0.3, 0.5, 0.7, 0.8, 0.9, 0.95, 0.98, 0.99, 0.998)

GFAC_H = 5e-3


def kerr_rms(a: float) -> float:
    """ISCO radius (Relphysics.cpp:139-150)."""
    sign = -1.0 if a < 0 else 1.0
    z1 = 1.0 + (1.0 - a * a) ** (1.0 / 3.0) * ((1.0 + a) ** (1.0 / 3.0) + (1.0 - a) ** (1.0 / 3.0))
    z2 = math.sqrt(3.0 * a * a + z1 * z1)
    return 3.0 + z2 - sign * math.sqrt((3.0 - z1) * (3.0 + z1 + 2 * z2))


def kerr_rplus(a: float) -> float:
    return 1.0 + math.sqrt(1.0 - a * a)


def _smooth(rng: np.random.Generator, *axes: np.ndarray, amp: float = 0.01) -> np.ndarray:
    """1 + amp*sin(2 pi (sum_i u_i x_i + phi)): a seeded smooth perturbation."""
    u = rng.uniform(0.3, 1.7, size=len(axes))
    phi = rng.uniform(0.0, 1.0)
    arg = phi
    for ui, x in zip(u, axes):
        arg = arg + ui * x
    return 1.0 + amp * np.sin(2.0 * np.pi * arg)


# ----------------------------------------------------------------------------
# relline table
# ----------------------------------------------------------------------------

def relline_arrays(n_a=25, n_mu0=30, n_r=100, n_g=40, seed=1234):
    rng = np.random.default_rng(seed)
    a_grid = np.linspace(-0.998, 0.998, n_a).astype(np.float32)
    mu0_grid = np.linspace(0.0175, 1.0, n_mu0).astype(np.float32)
    gstar = GFAC_H + (1.0 - 2 * GFAC_H) / (n_g - 1) * np.arange(n_g)
    r = np.zeros((n_a, n_r))
    for i, a in enumerate(a_grid.astype(np.float64)):
        r[i] = np.exp(np.linspace(np.log(1000.0), np.log(0.995 * kerr_rms(a)), n_r))
    A = a_grid.astype(np.float64)[:, None, None]
    M = mu0_grid.astype(np.float64)[None, :, None]
    R = r[:, None, :]
    sin_i = np.sqrt(np.maximum(1.0 - M * M, 0.0))
    sq = np.sqrt(R)
    inner = np.maximum(R * R - 3 * R + 2 * A * sq, 1e-3)
    ut = (R * sq + A) / (sq * np.sqrt(inner))
    g0 = 1.0 / ut
    beta = np.minimum(0.9, 1.0 / np.sqrt(np.maximum(R - 0.5, 0.6)))
    width = 0.9 * beta * sin_i + 0.02
    gmin = g0 * (1.0 - width) * _smooth(rng, A, M, np.log(R), amp=0.002)
    gmax = g0 * (1.0 + 1.1 * width) * _smooth(rng, A, M, np.log(R), amp=0.002)
    G = gstar[None, None, None, :]
    A4, M4, R4 = A[..., None], M[..., None], R[..., None]
    base = (M4 / np.pi) * (1.0 + 0.5 / R4)
    trff1 = base * (1.0 + 0.25 * (2 * G - 1.0)) * _smooth(rng, A4, M4, np.log(R4), G)
    trff2 = base * (1.0 - 0.25 * (2 * G - 1.0)) * _smooth(rng, A4, M4, np.log(R4), G)
    sin4 = np.sqrt(np.maximum(1.0 - M4 * M4, 0.0))
    cosne1 = np.clip(M4 + 0.3 * (G - 0.5) * sin4 + 0.2 / R4, 0.02, 0.998) * _smooth(rng, A4, M4, G, amp=0.002)
    cosne2 = np.clip(M4 - 0.3 * (G - 0.5) * sin4 + 0.2 / R4, 0.02, 0.998) * _smooth(rng, A4, M4, G, amp=0.002)
    return dict(
        a=a_grid, mu0=mu0_grid,
        r=np.broadcast_to(r[:, None, :], (n_a, n_mu0, n_r)).astype(np.float32),
        gmin=gmin.astype(np.float32), gmax=gmax.astype(np.float32),
        trff1=trff1.astype(np.float32), trff2=trff2.astype(np.float32),
        cosne1=cosne1.astype(np.float32), cosne2=cosne2.astype(np.float32),
    )


def write_relline_table(path: str, **kw) -> None:
    t = relline_arrays(**kw)
    n_a, n_mu0, n_r = t["r"].shape
    n_g = t["trff1"].shape[-1]
    with open(path, "wb") as f:
        f.write(fits.primary_header())
        f.write(fits.bintable("a", [fits.Column("a", "E", 1, t["a"][:, None])], n_a))
        f.write(fits.bintable("mu0", [fits.Column("mu0", "E", 1, t["mu0"][:, None])], n_mu0))
        for ii in range(n_a):
            for jj in range(n_mu0):
                cols = [
                    fits.Column("r", "E", 1, t["r"][ii, jj][:, None]),
                    fits.Column("gmin", "E", 1, t["gmin"][ii, jj][:, None]),
                    fits.Column("gmax", "E", 1, t["gmax"][ii, jj][:, None]),
                    fits.Column("trff1", "E", n_g, t["trff1"][ii, jj]),
                    fits.Column("trff2", "E", n_g, t["trff2"][ii, jj]),
                    fits.Column("cosne1", "E", n_g, t["cosne1"][ii, jj]),
                    fits.Column("cosne2", "E", n_g, t["cosne2"][ii, jj]),
                ]
                f.write(fits.bintable(f"{ii + 1}_{jj + 1}", cols, n_r))


# ----------------------------------------------------------------------------
# lamp-post table
# ----------------------------------------------------------------------------

def lp_arrays(n_a=20, n_h=250, n_r=100, seed=1234):
    rng = np.random.default_rng(seed + 1)
    a_grid = np.linspace(-0.998, 0.998, n_a).astype(np.float32)
    hgrid = np.zeros((n_a, n_h))
    for i, a in enumerate(a_grid.astype(np.float64)):
        hgrid[i] = np.exp(np.linspace(np.log(1.0 + 0.02 * (1.0 - abs(a))), np.log(600.0), n_h))
    rad = np.exp(np.linspace(np.log(1.0), np.log(1000.0), n_r))
    A = a_grid.astype(np.float64)[:, None, None]
    H = hgrid[:, :, None]
    R = rad[None, None, :]
    newton = (1.0 / ((R / H) ** 2 + 1.0)) ** 1.5 / (2 * np.pi * H * H)
    boost = (1.0 + 2.0 / R) * (1.0 + 1.0 / H) * (1.0 + 0.1 * A / R)
    intens = newton * boost * _smooth(rng, A, np.log(H), np.log(R))
    dele = np.arctan(R / H) * (1.0 + 0.1 / (1.0 + H)) * _smooth(rng, A, np.log(H), np.log(R), amp=0.002)
    dele = np.minimum(dele, 0.5 * np.pi - 1e-3)
    del_inc = np.minimum(np.arctan(R / H) * 0.98 + 0.01, 0.5 * np.pi - 1e-2)
    return dict(
        a=a_grid, hgrid=hgrid.astype(np.float32),
        r=np.broadcast_to(rad, (n_a, n_r)).astype(np.float32),
        intens=intens.astype(np.float32), dele=dele.astype(np.float32),
        del_inc=del_inc.astype(np.float32),
    )


def write_lp_table(path: str, **kw) -> None:
    t = lp_arrays(**kw)
    n_a, n_h, n_r = t["intens"].shape
    cols = [
        fits.Column("a", "E", 1, t["a"][:, None]),
        fits.Column("hgrid", "E", n_h, t["hgrid"]),
        fits.Column("r", "E", n_r, t["r"]),
    ]
    for k in range(n_h):
        cols.append(fits.Column(f"h{k + 1}", "E", n_r, t["intens"][:, k, :]))
        cols.append(fits.Column(f"del{k + 1}", "E", n_r, t["dele"][:, k, :]))
        cols.append(fits.Column(f"del_inc{k + 1}", "E", n_r, t["del_inc"][:, k, :]))
    with open(path, "wb") as f:
        f.write(fits.primary_header())
        f.write(fits.bintable("I_h", cols, n_a))


# ----------------------------------------------------------------------------
# xillver table
# ----------------------------------------------------------------------------

@dataclass
class XillDims:
    gamma: Sequence[float]
    afe: Sequence[float]
    logxi: Sequence[float]
    ecut: Sequence[float]
    n_incl: int = 10
    n_ener: int = 2999
    emin: float = 0.07
    emax: float = 1000.0

    @property
    def incl(self) -> np.ndarray:
        mu = 1.0 - (np.arange(self.n_incl) + 0.5) / self.n_incl
        return np.degrees(np.arccos(mu))


def xill_dims(size: str = "full") -> XillDims:
    if size == "full":
        return XillDims(gamma=np.linspace(1.0, 3.4, 13), afe=[0.5, 1.0, 3.0, 10.0],
                        logxi=np.linspace(0.0, 4.7, 16), ecut=np.geomspace(5.0, 1000.0, 10))
    if size == "small":
        return XillDims(gamma=np.linspace(1.0, 3.4, 5), afe=[0.5, 1.0, 3.0],
                        logxi=np.linspace(0.0, 4.7, 5), ecut=np.geomspace(5.0, 1000.0, 5),
                        n_incl=10, n_ener=2999)
    raise ValueError(size)


def _coarse_norm(gam: np.ndarray, ect: np.ndarray) -> np.ndarray:
    """1/calcNormWrtXillverTableSpec of the cut-off power law (Xillspec.cpp:179-233)."""
    e = np.exp(np.linspace(np.log(0.1), np.log(1000.0), 501))
    em = 0.5 * (e[1:] + e[:-1])
    de = e[1:] - e[:-1]
    pl = np.exp(1.0 / ect[..., None]) * em ** (-gam[..., None]) * np.exp(-em / ect[..., None]) * de
    s = (pl * em * 1e20 * 1.602177e-09).sum(-1)
    return (1e15 / 4.0 / np.pi) / s


def write_xillver_table(path: str, dims: XillDims | None = None, seed=1234) -> None:
    dims = dims or xill_dims("full")
    rng = np.random.default_rng(seed + 2)
    gam = np.asarray(dims.gamma, dtype=np.float32)
    afe = np.asarray(dims.afe, dtype=np.float32)
    lxi = np.asarray(dims.logxi, dtype=np.float32)
    ect = np.asarray(dims.ecut, dtype=np.float32)
    inc = dims.incl.astype(np.float32)
    names = ["Gamma", "A_Fe", "logXi", "Ecut", "Incl"]
    vals = [gam, afe, lxi, ect, inc]
    nmax = max(len(v) for v in vals)
    value = np.zeros((5, nmax), dtype=np.float32)
    for i, v in enumerate(vals):
        value[i, : len(v)] = v
    zeros = np.zeros((5, 1), dtype=np.float32)
    params_cols = [
        fits.Column("NAME", "A", 12, np.array(names)),
        fits.Column("METHOD", "J", 1, np.zeros((5, 1), dtype=np.int32)),
        fits.Column("INITIAL", "E", 1, np.array([[v[len(v) // 2]] for v in vals], dtype=np.float32)),
        fits.Column("DELTA", "E", 1, zeros + 0.01),
        fits.Column("MINIMUM", "E", 1, np.array([[v[0]] for v in vals], dtype=np.float32)),
        fits.Column("BOTTOM", "E", 1, np.array([[v[0]] for v in vals], dtype=np.float32)),
        fits.Column("TOP", "E", 1, np.array([[v[-1]] for v in vals], dtype=np.float32)),
        fits.Column("MAXIMUM", "E", 1, np.array([[v[-1]] for v in vals], dtype=np.float32)),
        fits.Column("NUMBVALS", "J", 1, np.array([[len(v)] for v in vals], dtype=np.int32)),
        fits.Column("VALUE", "E", nmax, value),
    ]
    edges = np.exp(np.linspace(np.log(dims.emin), np.log(dims.emax), dims.n_ener + 1)).astype(np.float32)
    elo, ehi = edges[:-1], edges[1:]
    em = 0.5 * (elo.astype(np.float64) + ehi.astype(np.float64))
    de = ehi.astype(np.float64) - elo.astype(np.float64)
    n_rows = len(gam) * len(afe) * len(lxi) * len(ect) * len(inc)
    mu = np.cos(np.radians(inc.astype(np.float64)))
    with open(path, "wb") as f:
        f.write(fits.primary_header())
        f.write(fits.bintable("PARAMETERS", params_cols, 5))
        f.write(fits.bintable("ENERGIES", [fits.Column("ENERG_LO", "E", 1, elo[:, None]),
                                           fits.Column("ENERG_HI", "E", 1, ehi[:, None])], dims.n_ener))
        st = fits.StreamingTable(f, "SPECTRA", [("PARAMVAL", "E", 5), ("INTPSPEC", "E", dims.n_ener)], n_rows)
        for ig, g in enumerate(gam.astype(np.float64)):
            # shape (afe, lxi, ect, incl, ener)
            E = ect.astype(np.float64)
            norm = _coarse_norm(np.full(E.shape, g), E)
            cont = (np.exp(1.0 / E)[:, None] * em[None, :] ** (-g) * np.exp(-em[None, :] / E[:, None])
                    * de[None, :] * norm[:, None])
            L = lxi.astype(np.float64)[None, :, None, None, None]
            F = afe.astype(np.float64)[:, None, None, None, None]
            MU = mu[None, None, None, :, None]
            albedo = (0.25 + 0.08 * L) * (0.6 + 0.4 * MU) / (0.8 + 0.1 * np.log(F))
            ew = 0.02 * (1.0 + L) * np.sqrt(F)
            c64 = np.array([np.interp(6.4, em, cont[k] / de) for k in range(len(E))])
            gauss = np.exp(-0.5 * ((em - 6.4) / 0.12) ** 2) / (0.12 * np.sqrt(2 * np.pi)) * de
            spec = (cont[None, None, :, None, :] * albedo
                    + ew * c64[None, None, :, None, None] * gauss[None, None, None, None, :])
            spec = spec * (10.0 ** L)
            spec = np.broadcast_to(spec, (len(afe), len(lxi), len(ect), len(inc), dims.n_ener))
            noise = np.exp(0.05 * rng.standard_normal(spec.shape))
            spec = (spec * noise).astype(np.float32).reshape(-1, dims.n_ener)
            grid = np.stack(np.meshgrid(afe, lxi, ect, inc, indexing="ij"), -1).reshape(-1, 4)
            pv = np.concatenate([np.full((grid.shape[0], 1), gam[ig], np.float32), grid.astype(np.float32)], 1)
            st.write_rows(PARAMVAL=pv, INTPSPEC=spec)
        st.close()


def write_xillver_cp_table(path: str, seed: int = 1234, n_ener: int = 2999) -> None:
    rng = np.random.default_rng(seed + 3)
    gam = np.array([1.2, 1.9, 2.6, 3.4], dtype=np.float32)
    afe = np.array([0.5, 1.0, 3.0], dtype=np.float32)
    lxi = np.array([0.0, 1.5, 3.0, 4.7], dtype=np.float32)
    kte = np.array([5.0, 20.0, 60.0, 400.0], dtype=np.float32)
    dns = np.array([15.0, 17.5, 20.0], dtype=np.float32)
    inc = XillDims([1.0], [1.0], [1.0], [1.0]).incl.astype(np.float32)
    names = ["Gamma", "A_Fe", "logXi", "kTe", "Dens", "Incl"]
    vals = [gam, afe, lxi, kte, dns, inc]
    npar = len(vals)
    nmax = max(len(v) for v in vals)
    value = np.zeros((npar, nmax), dtype=np.float32)
    for i, v in enumerate(vals):
        value[i, : len(v)] = v
    zeros = np.zeros((npar, 1), dtype=np.float32)
    params_cols = [
        fits.Column("NAME", "A", 12, np.array(names)),
        fits.Column("METHOD", "J", 1, np.zeros((npar, 1), dtype=np.int32)),
        fits.Column("INITIAL", "E", 1, np.array([[v[len(v) // 2]] for v in vals], dtype=np.float32)),
        fits.Column("DELTA", "E", 1, zeros + 0.01),
        fits.Column("MINIMUM", "E", 1, np.array([[v[0]] for v in vals], dtype=np.float32)),
        fits.Column("BOTTOM", "E", 1, np.array([[v[0]] for v in vals], dtype=np.float32)),
        fits.Column("TOP", "E", 1, np.array([[v[-1]] for v in vals], dtype=np.float32)),
        fits.Column("MAXIMUM", "E", 1, np.array([[v[-1]] for v in vals], dtype=np.float32)),
        fits.Column("NUMBVALS", "J", 1, np.array([[len(v)] for v in vals], dtype=np.int32)),
        fits.Column("VALUE", "E", nmax, value),
    ]
    edges = np.exp(np.linspace(np.log(0.07), np.log(1000.0), n_ener + 1)).astype(np.float32)
    elo, ehi = edges[:-1], edges[1:]
    em = 0.5 * (elo.astype(np.float64) + ehi.astype(np.float64))
    de = ehi.astype(np.float64) - elo.astype(np.float64)
    mu = np.cos(np.radians(inc.astype(np.float64)))
    n_rows = int(np.prod([len(v) for v in vals]))
    with open(path, "wb") as f:
        f.write(fits.primary_header())
        f.write(fits.bintable("PARAMETERS", params_cols, npar))
        f.write(fits.bintable("ENERGIES", [fits.Column("ENERG_LO", "E", 1, elo[:, None]),
                                           fits.Column("ENERG_HI", "E", 1, ehi[:, None])], n_ener))
        st = fits.StreamingTable(f, "SPECTRA", [("PARAMVAL", "E", npar), ("INTPSPEC", "E", n_ener)], n_rows)
        for ig, g in enumerate(gam.astype(np.float64)):
            E = 2.7 * kte.astype(np.float64)
            norm = _coarse_norm(np.full(E.shape, g), E)
            cont = (np.exp(1.0 / E)[:, None] * em[None, :] ** (-g) * np.exp(-em[None, :] / E[:, None])
                    * de[None, :] * norm[:, None])                                   # (kte, ener)
            L = lxi.astype(np.float64)[None, :, None, None, None, None]
            F = afe.astype(np.float64)[:, None, None, None, None, None]
            D = dns.astype(np.float64)[None, None, None, :, None, None]
            MU = mu[None, None, None, None, :, None]
            soft = 1.0 + 0.3 * (D - 15.0) / 5.0 * np.exp(-em / 0.5)[None, None, None, None, None, :]
            albedo = (0.25 + 0.08 * L) * (0.6 + 0.4 * MU) / (0.8 + 0.1 * np.log(F)) * soft
            ew = 0.02 * (1.0 + L) * np.sqrt(F)
            c64 = np.array([np.interp(6.4, em, cont[k] / de) for k in range(len(E))])
            gauss = np.exp(-0.5 * ((em - 6.4) / 0.12) ** 2) / (0.12 * np.sqrt(2 * np.pi)) * de
            spec = (cont[None, None, :, None, None, :] * albedo
                    + ew * c64[None, None, :, None, None, None] * gauss[None, None, None, None, None, :])
            spec = spec * (10.0 ** L) * (10.0 ** (D - 15.0))
            spec = np.broadcast_to(spec, (len(afe), len(lxi), len(kte), len(dns), len(inc), n_ener))
            noise = np.exp(0.05 * rng.standard_normal(spec.shape))
            spec = (spec * noise).astype(np.float32).reshape(-1, n_ener)
            grid = np.stack(np.meshgrid(afe, lxi, kte, dns, inc, indexing="ij"), -1).reshape(-1, 5)
            pv = np.concatenate([np.full((grid.shape[0], 1), gam[ig], np.float32), grid.astype(np.float32)], 1)
            st.write_rows(PARAMVAL=pv, INTPSPEC=spec)
        st.close()


# ----------------------------------------------------------------------------
# returning-radiation table
# ----------------------------------------------------------------------------

def rrad_arrays(spin: float, nr: int = RRAD_NR, ng: int = RRAD_NG, seed: int = 1234):
    """Transfer fractions of one spin: row i is the incident bin, element j the emitting bin."""
    rng = np.random.default_rng(seed + 7 + int(round((spin + 1.0) * 1000)))
    edges = np.exp(np.linspace(np.log(kerr_rms(spin)), np.log(1000.0), nr + 1))
    rlo, rhi = edges[:-1], edges[1:]
    rm = 0.5 * (rlo + rhi)
    li, lj = np.log(rm)[:, None], np.log(rm)[None, :]
    area = (rhi * rhi - rlo * rlo)[:, None]
    f_ret = 0.35 * (rm[0] / rm) ** 0.8 * (0.6 + 0.4 * max(spin, 0.0))
    kern = area * np.exp(-np.abs(li - lj) / 0.7) / rm[:, None] ** 1.5 * _smooth(rng, li, lj, amp=0.02)
    tf_r = kern / kern.sum(axis=0, keepdims=True) * f_ret[None, :]
    frac_e = 0.9 * tf_r * _smooth(rng, li, lj, amp=0.02)
    gc = np.exp(0.15 * (lj - li)) * _smooth(rng, li, lj, amp=0.01)
    wid = 0.3 + 0.05 * np.sin(li + 2 * lj) ** 2
    gmin, gmax = gc * (1.0 - wid), gc * (1.0 + wid)
    x = (np.arange(ng) + 0.5) / ng
    bump = np.exp(-0.5 * ((x[None, None, :] - 0.45 - 0.1 * np.tanh(lj - li)[:, :, None]) / 0.22) ** 2)
    bump = bump * _smooth(rng, li[:, :, None], lj[:, :, None], x[None, None, :] * 3, amp=0.05)
    frac_g = bump / bump.sum(axis=2, keepdims=True)
    return dict(rlo=rlo, rhi=rhi, frac_e=frac_e, tf_r=tf_r, gmin=gmin, gmax=gmax, frac_g=frac_g, f_ret=f_ret,
                f_bh=0.3 * (rm[0] / rm), f_inf=1.0 - f_ret - 0.3 * (rm[0] / rm))


def write_rrad_table(path: str, spins: Sequence[float] = RRAD_SPINS, seed: int = 1234) -> None:
    with open(path, "wb") as f:
        f.write(fits.primary_header())
        f.write(fits.bintable("SPIN", [fits.Column("a", "D", 1, np.asarray(spins, dtype=np.float64)[:, None])],
                              len(spins)))
        for k, a in enumerate(spins):
            t = rrad_arrays(float(a), seed=seed)
            nr, ng = t["frac_g"].shape[1], t["frac_g"].shape[2]
            cols = [fits.Column("rlo", "D", 1, t["rlo"][:, None]), fits.Column("rhi", "D", 1, t["rhi"][:, None])]
            for name in ("frac_e", "tf_r", "gmin", "gmax"):
                cols.append(fits.Column(name, "D", nr, t[name]))
            cols.append(fits.Column("frac_g", "D", nr * ng, t["frac_g"].reshape(nr, nr * ng)))
            for name in ("f_ret", "f_bh", "f_inf"):
                cols.append(fits.Column(name, "D", 1, t[name][:, None]))
            f.write(fits.bintable(f"FRAC{k + 1:02d}", cols, nr))


def write_all(outdir: str, xill: str = "full", seed: int = 1234) -> str:
    os.makedirs(outdir, exist_ok=True)
    write_relline_table(os.path.join(outdir, RELTABLE_FILENAME), seed=seed)
    write_lp_table(os.path.join(outdir, LPTABLE_FILENAME), seed=seed)
    write_xillver_table(os.path.join(outdir, XILLTABLE_FILENAME), xill_dims(xill), seed=seed)
    write_rrad_table(os.path.join(outdir, RRADTABLE_FILENAME), seed=seed)
    write_xillver_cp_table(os.path.join(outdir, XILLTABLE_CP_FILENAME), seed=seed)
    return outdir


def ensure_tables(outdir: str, xill: str = "full", seed: int = 1234) -> str:
    """Write the five tables into ``outdir`` unless a complete set is there."""
    stamp = os.path.join(outdir, f".complete_{xill}_{seed}")
    if not os.path.exists(stamp):
        write_all(outdir, xill=xill, seed=seed)
    else:
        if not os.path.exists(os.path.join(outdir, RRADTABLE_FILENAME)):
            write_rrad_table(os.path.join(outdir, RRADTABLE_FILENAME), seed=seed)
        if not os.path.exists(os.path.join(outdir, XILLTABLE_CP_FILENAME)):
            write_xillver_cp_table(os.path.join(outdir, XILLTABLE_CP_FILENAME), seed=seed)
        with open(stamp, "w") as fh:
            fh.write("ok\n")
    return outdir


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("outdir")
    p.add_argument("--xill", default="full", choices=["full", "small"])
    p.add_argument("--seed", type=int, default=1234)
    a = p.parse_args(argv)
    ensure_tables(a.outdir, a.xill, a.seed)


if __name__ == "__main__":
    main()
