"""Parameter sets and energy grids of the golden fixtures (shared by the
fixture generator and the tests)."""
import numpy as np


def log_grid(emin, emax, n):
    return np.exp(np.linspace(np.log(emin), np.log(emax), n + 1))


GRID_LINE = ("line", 0.1, 20.0, 3000)      # relline: 3000 log bins 0.1-20 keV
GRID_WIDE = ("wide", 0.1, 1000.0, 3000)    # relxill / relxilllp output grid
GRID_CONV = ("convin", 0.3, 80.0, 500)      # relconv input grid
GRID_XLOW = ("xlow", 0.01, 2000.0, 1500)    # xillver: a grid reaching past both ends of the table
GRID_F1 = ("f1", 0.5722, 177.1, 1114)       # the grid of the returning-radiation set below
CONV_MODELS = ("relconv", "relconv_lp")

CASES = [
    # (name, model, params, grid, iongrad_type, iongrad_index)
    ("relline_cfg1", "relline", [6.4, 3, 3, 15, 0.998, 30, -1, 400, 0, 0], GRID_LINE, 0, 0.0),
    ("relline_b", "relline", [6.4, 4, 2.5, 8, 0.5, 60, -1.5, 300, 0.1, 1], GRID_LINE, 0, 0.0),
    ("relline_c", "relline", [1.0, 3, 3, 15, -0.5, 80, -1, 1000, 0, 2], GRID_LINE, 0, 0.0),
    ("relline_d", "relline", [6.97, 5, 3, 4, 0.9, 7, -1, 50, 0, 0], GRID_LINE, 0, 0.0),
    ("relconv_a", "relconv", [3, 3, 15, 0.9, 45, -1, 400, 0], GRID_CONV, 0, 0.0),
    ("relxill_cfg2", "relxill", [3, 3, 15, 0.9, 45, -1, 400, 0, 2.0, 3.1, 1, 300, 3], GRID_WIDE, 0, 0.0),
    ("relxill_b", "relxill", [4, 2, 10, 0.3, 20, -2, 200, 0.05, 1.7, 1.0, 3, 100, -1], GRID_WIDE, 0, 0.0),
    ("relxilllp_a", "relxilllp", [10, 0, 0.9, 45, -1, 400, 0, 2.0, 3.1, 1, 300, 1, 0, 0], GRID_WIDE, 0, 0.0),
    ("relxilllp_b", "relxilllp", [3, 0.3, 0.998, 70, -1, 400, 0.2, 2.6, 4.0, 5, 50, 2, 0, 1], GRID_WIDE, 0, 0.0),
    ("relxilllp_c", "relxilllp", [50, 0, -0.5, 10, -3, 100, 0, 1.5, 0.5, 0.7, 800, -1, 0, 0], GRID_WIDE, 0, 0.0),
    ("relxilllp_pl", "relxilllp", [10, 0, 0.9, 45, -1, 400, 0, 2.0, 3.1, 1, 300, 1, 0, 0], GRID_WIDE, 1, 0.5),
    ("relxilllp_alpha", "relxilllp", [5, 0, 0.5, 30, -1, 400, 0, 2.2, 2.0, 1, 100, 1, 0, 0], GRID_WIDE, 2, 0.0),
    ("rellinelp_a", "relline_lp", [6.4, 6, 0.998, 30, -1, 400, 0, 0, 2, 0], GRID_LINE, 0, 0.0),
    ("rellinelp_b", "relline_lp", [1.0, 3, 0.5, 60, -1, 100, 0.1, 1, 2.5, 0], GRID_LINE, 0, 0.0),
    ("rellinelp_c", "relline_lp", [6.97, 50, -0.5, 80, -3, 1000, 0, 2, 1.4, 0], GRID_LINE, 0, 0.0),
    ("relconvlp_a", "relconv_lp", [6, 0, 0.998, 30, -1, 400, 0, 2, 0], GRID_CONV, 0, 0.0),
    ("relconvlp_b", "relconv_lp", [20, 0.5, 0.3, 70, -2, 300, 2, 1.6, 0], GRID_CONV, 0, 0.0),
    ("xillver_a", "xillver", [2, 1, 300, 3.1, 0, 30, -1], GRID_WIDE, 0, 0.0),
    ("xillver_b", "xillver", [1.7, 3, 80, 1.5, 0.05, 60, 2.5], GRID_WIDE, 0, 0.0),
    # Ecut and logxi on their upper bounds, incl below the table, primary only
    ("xillver_c", "xillver", [2.5, 0.7, 1000, 4.7, 0, 5, 0], GRID_XLOW, 0, 0.0),
    # parameters on grid values or clamped (zero-weight corners), z = 1
    ("xillver_d", "xillver", [1.0, 10, 5, 0, 1.0, 87, 1], GRID_XLOW, 0, 0.0),
    # returning radiation ($switch_returnrad = 1, the reference's default for the lamp-post models)
    ("relxilllp_rr_a", "relxilllp", [10, 0, 0.9, 45, -1, 400, 0, 2.0, 3.1, 1, 300, 1, 1, 0], GRID_WIDE, 0, 0.0),
    ("relxilllp_rr_b", "relxilllp", [3, 0.3, 0.998, 70, -1, 400, 0.2, 2.6, 4.0, 5, 50, 2, 1, 1], GRID_WIDE, 0, 0.0),
    # negative spin: no xillver correction factors (Relxill.cpp:338-341)
    ("relxilllp_rr_neg", "relxilllp", [50, 0, -0.5, 10, -3, 100, 0, 1.5, 0.5, 0.7, 800, -1, 1, 0], GRID_WIDE, 0, 0.0),
    # only the returning part of the emissivity ($switch_returnrad = -1)
    ("relxilllp_rr_only", "relxilllp", [6, 0, 0.95, 30, -1, 400, 0, 2.0, 1.0, 1, 300, 1, -1, 0], GRID_WIDE, 0, 0.0),
    ("relxilllp_rr_alpha", "relxilllp", [5, 0, 0.5, 30, -1, 400, 0, 2.2, 2.0, 1, 100, 1, 1, 0], GRID_WIDE, 2, 0.0),
    ("relxilllp_rr_pl", "relxilllp", [10, 0, 0.9, 45, -1, 400, 0, 2.0, 3.1, 1, 300, 1, 1, 0], GRID_WIDE, 1, 0.5),
    ("rellinelp_rr", "relline_lp", [6.4, 6, 0.998, 30, -1, 400, 0, 0, 2.0, 1], GRID_LINE, 0, 0.0),
    ("relconvlp_rr", "relconv_lp", [6, 0.0, 0.7, 30, -1, 400, 0, 2.0, 1], GRID_CONV, 0, 0.0),
    # returning radiation that stays high out to Rout = 242.088: single outer radii dominate bins, and
    # one Romberg test of the reference sits at obtprec 0.0200002 (switch 1, then -1)
    ("relxilllp_rr_rout", "relxilllp", [7.819159105467463, 0.06318223691180253, 0.7520664936838367,
                                        20.839453254507205, -1, 242.08828763042303, 0.0, 1.2155558003015097,
                                        1.2222305853986382, 9.569424921641735, 210.91094357446238,
                                        5.727814656047778, 1, 0], GRID_F1, 0, 0.0),
    ("relxilllp_rr_rout_only", "relxilllp", [7.819159105467463, 0.06318223691180253, 0.7520664936838367,
                                             20.839453254507205, -1, 242.08828763042303, 0.0, 1.2155558003015097,
                                             1.2222305853986382, 9.569424921641735, 210.91094357446238,
                                             5.727814656047778, -1, 0], GRID_F1, 0, 0.0),
    # Cp flavour: nthcomp continuum, 6-parameter xillverCp table (lmodel_relxill_public.dat:86-129)
    ("xillvercp_a", "xillverCp", [2.0, 1.0, 60, 3.1, 15, 0, 30, -1], GRID_WIDE, 0, 0.0),
    ("xillvercp_b", "xillverCp", [1.7, 3.0, 25, 1.5, 17.0, 0.05, 60, 2.0], GRID_WIDE, 0, 0.0),
    ("relxillcp_a", "relxillCp", [30, 0.998, -1, 400, 15, 3, 3, 0, 2.0, 3.1, 15, 1, 60, 3], GRID_WIDE, 0, 0.0),
    ("relxillcp_b", "relxillCp", [60, 0.5, -2, 300, 10, 4, 2.5, 0.1, 1.8, 2.0, 18, 2.0, 100, -1], GRID_WIDE, 0, 0.0),
    ("relxilllpcp_a", "relxilllpCp", [30, 0.998, -1, 400, 6, 0, 2.0, 3.1, 15, 1, 60, 1, 0, 0, 0, 0, 0], GRID_WIDE,
     0, 0.0),
    # returning radiation with its corrections and the reflection-fraction boost
    ("relxilllpcp_rr", "relxilllpCp", [45, 0.9, -1, 400, 10, 0.2, 2.4, 2.0, 16, 3, 30, 2, 0, 0, 0, 1, 1], GRID_WIDE,
     0, 0.0),
    # the ionisation gradient is a parameter of relxilllpCp: ALPHA and power law
    ("relxilllpcp_alpha", "relxilllpCp", [70, 0.5, -1, 400, 5, 0, 2.2, 2.0, 15, 1, 100, 1, 0, 0.0, 2, 1, 0],
     GRID_WIDE, 0, 0.0),
    ("relxilllpcp_pl", "relxilllpCp", [30, 0.9, -1, 400, 10, 0, 2.0, 3.1, 15, 1, 60, 1, 0, 0.5, 1, 0, 0], GRID_WIDE,
     0, 0.0),
]


def grid(spec):
    _, lo, hi, n = spec
    return log_grid(lo, hi, n)


def conv_input(e):
    """relconv input spectrum: a power law with a Gaussian line (per bin)."""
    em = 0.5 * (e[1:] + e[:-1])
    return em ** -1.5 * np.diff(e) * (1 + 5 * np.exp(-0.5 * ((em - 6.4) / 0.2) ** 2))
