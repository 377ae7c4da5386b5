"""The Cp flavour on the GPU (nthcomp continuum, 6-parameter xillverCp table):
random batches of xillverCp, relxillCp and relxilllpCp against the CPU
oracle, the local-model entry points against the batched call, and a kTe
without an nthcomp grid reported as a parameter error."""
import numpy as np
import pytest

import oracle_lib
from cases import log_grid
from tolerance import assert_close

pytestmark = pytest.mark.gpu


def _check(R, model, params, grids):
    out, st = R.eval_batch(model, params, grids)
    assert not st.any(), (st, R.last_error())
    for i in range(len(grids)):
        s, orc = oracle_lib.evaluate(model, params[i], grids[i])
        assert s == 0
        assert_close(out[i], orc, f"{model} set {i}")
    return out


def test_xillvercp_random_sets(gpu, oracle):
    rng = np.random.default_rng(51)
    n = 12
    p = np.column_stack([rng.uniform(1.2, 3.4, n), rng.uniform(0.5, 3, n), rng.uniform(5, 400, n),
                         rng.uniform(0, 4.7, n), rng.uniform(15, 20, n), rng.choice([0.0, 0.1], n),
                         rng.uniform(5, 85, n), rng.choice([-1.0, 0.0, 2.0], n)])
    _check(gpu, "xillverCp", p, [log_grid(0.1, 500.0, int(rng.integers(100, 2000))) for _ in range(n)])


def test_relxillcp_random_sets(gpu, oracle):
    rng = np.random.default_rng(52)
    n = 6
    p = np.column_stack([rng.uniform(10, 80, n), rng.uniform(-0.5, 0.998, n), -np.ones(n), rng.uniform(100, 500, n),
                         rng.uniform(5, 30, n), rng.uniform(2, 4, n), rng.uniform(2, 4, n), np.zeros(n),
                         rng.uniform(1.4, 3.0, n), rng.uniform(0, 4.5, n), rng.uniform(15, 19, n),
                         rng.uniform(0.5, 3, n), rng.uniform(10, 300, n), rng.uniform(0.5, 3, n)])
    _check(gpu, "relxillCp", p, [log_grid(0.3, 80.0, int(rng.integers(300, 1500))) for _ in range(n)])


def test_relxilllpcp_random_sets(gpu, oracle, monkeypatch):
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")
    rng = np.random.default_rng(53)
    n = 6
    p = np.column_stack([rng.uniform(10, 80, n), rng.uniform(0.1, 0.998, n), -np.ones(n), np.full(n, 400.0),
                         rng.uniform(3, 50, n), np.zeros(n), rng.uniform(1.4, 3.0, n), rng.uniform(0, 4.5, n),
                         rng.uniform(15, 19, n), rng.uniform(0.5, 3, n), rng.uniform(10, 300, n), np.ones(n),
                         np.zeros(n), np.zeros(n), np.array([0, 0, 1, 2, 0, 0]), np.array([0, 1, 0, 1, 1, 0]),
                         np.zeros(n)])
    _check(gpu, "relxilllpCp", p, [log_grid(0.3, 80.0, int(rng.integers(300, 1500))) for _ in range(n)])


def test_cp_entry_points_match_batch(gpu):
    w = log_grid(0.1, 1000.0, 700)
    for model, p in (("xillverCp", gpu.default_params("xillverCp")),
                     ("relxillCp", gpu.default_params("relxillCp")),
                     ("relxilllpCp", gpu.default_params("relxilllpCp"))):
        out, _ = gpu.eval_batch(model, p[None], [w])
        np.testing.assert_array_equal(getattr(gpu, model)(w, p), out[0])


def test_kte_without_grid_is_a_parameter_error(gpu):
    w = log_grid(0.1, 1000.0, 300)
    p = gpu.default_params("xillverCp")
    p[2] = 0.0  # kTe = 0: no photon-energy grid for the Kompaneets equation
    out, st = gpu.eval_batch("xillverCp", p[None], [w], check=False)
    assert st[0] == 1 and not out[0].any()
    q = gpu.default_params("relxillCp")
    q[12] = -5.0
    out, st = gpu.eval_batch("relxillCp", q[None], [w], check=False)
    assert st[0] == 1 and not out[0].any()


@pytest.mark.parametrize("zones", [16, 20, 30])
def test_relxilllpcp_zone_counts(gpu, oracle, monkeypatch, zones):
    """The 6-parameter corners of a set come from the de-duplicated list (at most 16 zones), the
    per-zone lists (more zones) or, beyond 25 zones, per-zone lists built without de-duplication;
    ionisation gradients give every zone its own logxi and density brackets."""
    monkeypatch.setenv("RELXILL_NUM_RZONES", str(zones))
    rng = np.random.default_rng(54 + zones)
    n = 4
    p = np.column_stack([rng.uniform(10, 80, n), rng.uniform(0.1, 0.998, n), -np.ones(n), np.full(n, 400.0),
                         rng.uniform(3, 50, n), np.zeros(n), rng.uniform(1.4, 3.0, n), rng.uniform(0, 4.5, n),
                         rng.uniform(15, 19, n), rng.uniform(0.5, 3, n), rng.uniform(10, 300, n), np.ones(n),
                         np.zeros(n), np.zeros(n), np.array([1, 2, 2, 1]), np.zeros(n), np.zeros(n)])
    _check(gpu, "relxilllpCp", p, [log_grid(0.3, 80.0, int(rng.integers(300, 1500))) for _ in range(n)])


def test_relxillcp_mixed_zone_counts(gpu, oracle, monkeypatch):
    """relxillCp sets without (1 zone) and with an ionisation gradient (25 zones) in one batch."""
    monkeypatch.delenv("RELXILL_NUM_RZONES", raising=False)
    rng = np.random.default_rng(58)
    n = 4
    p = np.column_stack([rng.uniform(10, 80, n), rng.uniform(-0.5, 0.998, n), -np.ones(n), rng.uniform(100, 500, n),
                         rng.uniform(5, 30, n), rng.uniform(2, 4, n), rng.uniform(2, 4, n), np.zeros(n),
                         rng.uniform(1.4, 3.0, n), rng.uniform(0, 4.5, n), rng.uniform(15, 19, n),
                         rng.uniform(0.5, 3, n), rng.uniform(10, 300, n), rng.uniform(0.5, 3, n)])
    igt = np.array([0, 1, 0, 2], dtype=np.int32)
    igi = np.where(igt == 1, 1.2, 0.0)
    grids = [log_grid(0.3, 80.0, int(rng.integers(300, 1000))) for _ in range(n)]
    out, st = gpu.eval_batch("relxillCp", p, grids, ion_grad_type=igt, iongrad_index=igi)
    assert not st.any(), (st, gpu.last_error())
    for i in range(n):
        s, orc = oracle_lib.evaluate("relxillCp", p[i], grids[i], None, int(igt[i]), float(igi[i]))
        assert s == 0
        assert_close(out[i], orc, f"relxillCp set {i} (ion_grad_type {igt[i]})")


def test_cp_same_numbers_alone_and_in_batch(gpu, monkeypatch):
    """Few continua (one set) go through the one-CTA-per-continuum nthcomp kernel, many (64 sets of
    11 continua) through the one-thread-per-continuum one; both give the same numbers."""
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")
    rng = np.random.default_rng(57)
    n = 64
    p = np.column_stack([rng.uniform(10, 80, n), rng.uniform(0.1, 0.998, n), -np.ones(n), np.full(n, 400.0),
                         rng.uniform(3, 50, n), np.zeros(n), rng.uniform(1.4, 3.0, n), rng.uniform(0, 4.5, n),
                         rng.uniform(15, 19, n), rng.uniform(0.5, 3, n), rng.uniform(10, 300, n), np.ones(n),
                         np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)])
    grids = [log_grid(0.3, 80.0, int(rng.integers(300, 1000))) for _ in range(n)]
    big, st = gpu.eval_batch("relxilllpCp", p, grids)
    assert not st.any()
    for i in (0, 31, 63):
        one, _ = gpu.eval_batch("relxilllpCp", p[i:i + 1], grids[i:i + 1])
        np.testing.assert_array_equal(one[0], big[i])
    q = np.column_stack([rng.uniform(1.2, 3.4, 400), rng.uniform(0.5, 3, 400), rng.uniform(5, 400, 400),
                         rng.uniform(0, 4.7, 400), rng.uniform(15, 20, 400), np.zeros(400), rng.uniform(5, 85, 400),
                         -np.ones(400)])
    w = [log_grid(0.1, 500.0, 300)] * 400
    big, st = gpu.eval_batch("xillverCp", q, w)
    assert not st.any()
    for i in (0, 399):
        one, _ = gpu.eval_batch("xillverCp", q[i:i + 1], w[i:i + 1])
        np.testing.assert_array_equal(one[0], big[i])
