"""Host memory handed straight to the fused cylindrical pipeline: particle
arrays read in place from page-locked host memory, and results written into
host memory (evaluated in particle order), agree with the all-device call to
the order-dependence of the FP64 atomic sums; the pointer classifier reports
where buffers live."""
import ctypes
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _close(a, b, tol):
    return np.max(np.abs(a - b)) <= tol * max(np.max(np.abs(b)), 1e-300)


def _case():
    g = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    return g, os.path.join(GOLDEN, "eof_c1.cache")


def test_pointer_access_classes():
    import torch
    from exptool_gb300 import _lib
    lib = _lib.load()
    d = torch.empty(16, dtype=torch.float64, device="cuda")
    p = torch.empty(16, dtype=torch.float64, pin_memory=True)
    a = np.empty(16)
    assert lib.xt_pointer_access(ctypes.c_void_p(d.data_ptr())) == _lib.XT_PTR_DEVICE
    assert lib.xt_pointer_access(ctypes.c_void_p(p.data_ptr())) == _lib.XT_PTR_PINNED
    assert lib.xt_pointer_access(ctypes.c_void_p(a.ctypes.data)) in (_lib.XT_PTR_PAGEABLE, _lib.XT_PTR_INACCESSIBLE)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_host_inputs_and_results_match_device_call(precision):
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import eof
    g, path = _case()
    table = eof.table_from_file(path)
    n = g["m"].size
    pinned = [torch.from_numpy(np.ascontiguousarray(g[k], dtype=np.float64)).pin_memory() for k in "xyzm"]
    host_in = [dev.kernel_input(t.numpy()) for t in pinned]
    assert all(isinstance(a, np.ndarray) for a in host_in)          # passed in place, not copied
    dev_in = [t.to("cuda") for t in pinned]
    # atomic accumulation order varies between calls: FP64 sums differ in the
    # last bits, and the FP32 field can round either way
    tol = 1e-12 if precision == "f64" else 1e-6
    c0, s0, o0 = table.accumulate_eval(*dev_in, precision=precision)
    ref = dev.to_host_many([c0, s0] + list(o0))
    # particles read from host memory, results on the device (sorted evaluation)
    c1, s1, o1 = table.accumulate_eval(*host_in, precision=precision)
    got = dev.to_host_many([c1, s1] + list(o1))
    for a, b in zip(got, ref):
        assert _close(a, b, tol)
    # particles and results in host memory (evaluation in particle order)
    res = dev.pinned_empty(n, 6)
    c2, s2, _ = table.accumulate_eval(*host_in, precision=precision, outs=res)
    got = dev.to_host_many([c2, s2]) + [t.numpy() for t in res]
    for a, b in zip(got, ref):
        assert _close(a, b, tol)


def test_public_call_with_pinned_particles_matches_golden():
    import torch
    from exptool_gb300.basis import eof
    g, path = _case()

    class P:
        pass

    p = P()
    pinned = [torch.from_numpy(np.ascontiguousarray(g[k], dtype=np.float64)).pin_memory().numpy() for k in "xyzm"]
    p.xpos, p.ypos, p.zpos, p.mass = pinned
    E, res = eof.compute_coefficients_and_forces(p, path, verbose=0)
    for m in range(E.cos.shape[0]):
        assert np.max(np.abs(E.cos[m] - g["cos"][m])) <= 1e-10 * np.max(np.abs(g["cos"][m]))
    for k in range(6):
        assert np.max(np.abs(res[k] - g["aep"][k])) <= 1e-10 * np.max(np.abs(g["aep"][k]))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_coefficients_in_page_locked_memory(precision):
    """The sorted drop-in calls with their coefficients in page-locked host
    memory: the accumulation's last kernel writes them there, and the
    evaluation's field stage reads host coefficients in place.  The
    accumulation agrees with the device-output call to the order of its sums;
    the evaluation (no atomics) bit for bit with the same call on
    device coefficients."""
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import eof
    g, path = _case()
    table = eof.table_from_file(path)
    xa, ya, za, ma = (np.ascontiguousarray(g[k], dtype=np.float64) for k in "xyzm")
    d = [torch.from_numpy(a).to("cuda") for a in (xa, ya, za, ma)]
    ref = dev.to_host(table.accumulate_sorted(*d, precision=precision))
    got = table.accumulate_sorted(*d, precision=precision, host=True)
    assert isinstance(got, np.ndarray) and got.shape == ref.shape
    # FP32 path: the records' order within a cell (set by the binning's
    # atomics) changes the FP32 run sums between calls
    assert _close(got, ref, 1e-12 if precision == "f64" else 1e-6)
    shape = (table.mmax + 1, table.norder)
    hc, hs = dev.coef_pair(ref[0], ref[1], *shape)
    res_host = dev.to_host(table.eval_sorted(*d[:3], hc, hs, precision=precision))
    dc, ds = dev.coef_pair(torch.from_numpy(ref[0]).to("cuda"), torch.from_numpy(ref[1]).to("cuda"), *shape)
    res_dev = dev.to_host(table.eval_sorted(*d[:3], dc, ds, precision=precision))
    assert np.isfinite(res_dev).all()
    assert np.array_equal(res_host, res_dev)
