"""relx_eval_one_noalloc: one parameter set through the entry point whose
intermediate arrays live in a static device array, against the batched entry
point on the same inputs.  The caller's buffers come from torch; the entry
point itself allocates nothing."""
import ctypes
import os

import numpy as np
import pytest

from cases import CASES, CONV_MODELS, conv_input, grid
from tolerance import assert_close

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_small.npz")


@pytest.fixture(autouse=True)
def _zones_env(monkeypatch):
    # the golden outputs were made with ten zones for the ionisation gradients
    monkeypatch.setenv("RELXILL_NUM_RZONES", "10")


MODELS = {"relline": 0, "relconv": 1, "relxill": 2, "relxilllp": 3, "relline_lp": 4, "relconv_lp": 5, "xillver": 6,
          "xillverCp": 7, "relxillCp": 8, "relxilllpCp": 9}
RELX_ERR_ARG = 9


def _fn(R):
    L = R.lib()
    f = L.relx_eval_one_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


class _Call:
    """Device buffers of one call, made once by the caller."""

    def __init__(self, torch, model, params, e, igt=0, igi=0.0):
        dev = torch.device("cuda:0")
        self.model, self.igt, self.igi = model, igt, igi
        self.n = len(e) - 1
        self.params = torch.tensor(np.asarray(params, dtype=np.float64), device=dev)
        self.energy = torch.tensor(np.asarray(e, dtype=np.float64), device=dev)
        self.fin = torch.tensor(conv_input(e), device=dev) if model in CONV_MODELS else None
        self.flux = torch.full((self.n,), -1.0, dtype=torch.float64, device=dev)
        self.status = torch.full((1,), -1, dtype=torch.int32, device=dev)

    def run(self, f):
        return f(MODELS[self.model], self.params.data_ptr(), self.energy.data_ptr(), self.n,
                 self.fin.data_ptr() if self.fin is not None else None, self.flux.data_ptr(), self.status.data_ptr(),
                 self.igt, self.igi, None)


def _batch(R, model, params, e, igt=0, igi=0.0):
    fin = [conv_input(e)] if model in CONV_MODELS else None
    out, st = R.eval_batch(model, np.asarray(params)[None], [e], flux_in=fin,
                           ion_grad_type=[igt] if igt else None, iongrad_index=[igi] if igt else None)
    assert st[0] == 0, R.last_error()
    return out[0]


def _case(name):
    return next(c for c in CASES if c[0] == name)


def test_noalloc_matches_batch_on_two_calls_in_a_row(gpu):
    """Each case twice in a row through the no-allocation entry point, against the batched entry
    point and against the reference's own output (golden file).  relxilllpcp_alpha and
    relxilllpcp_pl carry their ionisation gradient in the parameter array (params[14] = 2 and 1)
    while the call's ion_grad_type argument stays 0."""
    torch = pytest.importorskip("torch")
    f = _fn(gpu)
    golden = np.load(GOLDEN)
    names = ["relxilllp_a", "relxill_cfg2", "relline_cfg1", "relconv_a", "relxilllp_alpha", "relxilllp_b",
             "rellinelp_b", "relconvlp_b", "xillver_b", "xillver_d", "xillvercp_a", "xillvercp_b", "relxillcp_b",
             "relxilllpcp_a", "relxilllpcp_rr", "relxilllpcp_alpha", "relxilllpcp_pl", "relxilllp_rr_a",
             "rellinelp_rr"]
    for name in names:
        _, model, params, gspec, igt, igi = _case(name)
        e = grid(gspec)
        want = _batch(gpu, model, params, e, igt, igi)
        call = _Call(torch, model, params, e, igt, igi)
        for k in range(2):
            call.flux.fill_(-1.0)
            assert call.run(f) == 0, gpu.last_error()
            torch.cuda.synchronize()
            assert int(call.status.item()) == 0
            got = call.flux.cpu().numpy()
            assert_close(got, want, f"{name} no-alloc call {k + 1} vs batch")
            assert_close(got, golden[name], f"{name} no-alloc call {k + 1} vs reference")


def test_noalloc_alternating_sets_keep_their_results(gpu):
    """Two different sets back to back share the scratch; each result matches its own batch result."""
    torch = pytest.importorskip("torch")
    f = _fn(gpu)
    a, b = _case("relxilllp_a"), _case("relxilllp_c")
    ea, eb = grid(a[3]), grid(b[3])
    ca = _Call(torch, "relxilllp", a[2], ea)
    cb = _Call(torch, "relxilllp", b[2], eb)
    assert ca.run(f) == 0 and cb.run(f) == 0, gpu.last_error()
    torch.cuda.synchronize()
    assert_close(ca.flux.cpu().numpy(), _batch(gpu, "relxilllp", a[2], ea), "set A")
    assert_close(cb.flux.cpu().numpy(), _batch(gpu, "relxilllp", b[2], eb), "set B")


def test_noalloc_allocates_no_device_memory(gpu):
    torch = pytest.importorskip("torch")
    f = _fn(gpu)
    _, model, params, gspec, _, _ = _case("relxilllp_a")
    call = _Call(torch, model, params, grid(gspec))
    assert call.run(f) == 0  # set-up on the first call of the device
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert call.run(f) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_relline_grid_beyond_limit(gpu):
    torch = pytest.importorskip("torch")
    f = _fn(gpu)
    _, _, params, _, _, _ = _case("relline_cfg1")
    e = np.exp(np.linspace(np.log(0.1), np.log(10.0), 16386))
    call = _Call(torch, "relline", params, e)
    assert call.run(f) == RELX_ERR_ARG
    assert "16384" in gpu.last_error()
