"""The device-buffer entry point (relx_eval_batch_device) against the host-buffer
one, and the host-buffer path of large batches (groups of consecutive sets on
two streams with their own staging) against the same sets in one device-buffer
launch: every set gives the same numbers whichever path and batch it runs in."""
import ctypes

import numpy as np
import pytest

import oracle_lib
from tolerance import assert_close

pytestmark = pytest.mark.gpu


def _lp_sets(n, seed, nb_lo=300, nb_hi=1200):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 14))
    p[:, 0] = rng.uniform(3, 100, n)
    p[:, 2] = rng.uniform(0, 0.998, n)
    p[:, 3] = rng.uniform(5, 85, n)
    p[:, 4], p[:, 5] = -1.0, 400.0
    p[:, 7] = rng.uniform(1.4, 2.8, n)
    p[:, 8] = rng.uniform(0, 4.5, n)
    p[:, 9], p[:, 10], p[:, 11] = 1.0, 300.0, 1.0
    grids = [np.exp(np.linspace(np.log(0.3), np.log(80.0), int(k) + 1)) for k in rng.integers(nb_lo, nb_hi, n)]
    return p, grids


def _device(R, model, params, grids):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    L = R.lib()
    n = len(grids)
    edges, offs = R.pack_grids(grids)
    d_params = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float64)).to(dev)
    d_e = torch.from_numpy(edges).to(dev)
    d_off = torch.from_numpy(offs).to(dev)
    d_flux = torch.full((int(offs[-1]) - n,), -1.0, dtype=torch.float64, device=dev)
    d_status = torch.full((n,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    st = L.relx_eval_batch_device(R.MODELS[model], n, d_params.data_ptr(), d_e.data_ptr(), d_off.data_ptr(),
                                  offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None, d_flux.data_ptr(),
                                  d_status.data_ptr(), None, None, None, stream.cuda_stream)
    assert st == 0, R.last_error()
    stream.synchronize()
    flux = d_flux.cpu().numpy()
    assert not d_status.cpu().numpy().any()
    return [flux[offs[i] - i: offs[i + 1] - i - 1] for i in range(n)]


def test_device_buffers_match_host_buffers(gpu):
    params, grids = _lp_sets(64, 31)
    host, st = gpu.eval_batch("relxilllp", params, grids)
    assert not st.any()
    dev = _device(gpu, "relxilllp", params, grids)
    for i in range(len(grids)):
        np.testing.assert_array_equal(dev[i], host[i])


def test_large_host_batch_in_groups(gpu, oracle):
    """2100 sets through the host buffers run as groups of consecutive sets (512, 1076, 512)
    alternating over two streams; each set equals the same set in one device-buffer launch of all
    2100, and the oracle."""
    params, grids = _lp_sets(2100, 32, 40, 160)
    host, st = gpu.eval_batch("relxilllp", params, grids)
    assert not st.any()
    dev = _device(gpu, "relxilllp", params, grids)
    for i in range(len(grids)):
        np.testing.assert_array_equal(host[i], dev[i])
    for i in (0, 511, 512, 1587, 1588, 2099):  # the ends of the groups
        s, orc = oracle_lib.evaluate("relxilllp", params[i], grids[i])
        assert s == 0
        assert_close(host[i], orc, f"set {i}")
