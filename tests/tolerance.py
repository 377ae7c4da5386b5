"""The parity bar of the path: FP32 bulk arithmetic within 1e-4 relative per
bin for bins above 1e-6 of the peak, and 1e-6 relative in the total flux."""
import numpy as np

REL_BIN = 1e-4
PEAK_FLOOR = 1e-6
REL_TOTAL = 1e-6


def compare(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape
    peak = np.abs(ref).max()
    m = np.abs(ref) > PEAK_FLOOR * peak
    rel = np.abs(got[m] - ref[m]) / np.abs(ref[m]) if m.any() else np.zeros(1)
    tot = abs(got.sum() / ref.sum() - 1) if ref.sum() != 0 else abs(got.sum())
    return float(rel.max()), float(tot)


def assert_close(got, ref, what=""):
    r, t = compare(got, ref)
    assert r <= REL_BIN, f"{what}: max per-bin relative error {r:.3e} > {REL_BIN}"
    assert t <= REL_TOTAL, f"{what}: total flux relative error {t:.3e} > {REL_TOTAL}"
