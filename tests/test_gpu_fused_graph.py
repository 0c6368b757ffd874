"""The fused cylindrical call replayed as a CUDA graph: the first call of a
shape runs directly, the second captures it, later calls replay it with the
binning node pointed at new particle arrays.  Every call must give the
results of a direct (ungraphed) call on the same particles."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_graph_replay_patches_particle_arrays(precision):
    import torch
    from exptool_gb300 import _lib
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import eof
    g = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    table = eof.table_from_file(os.path.join(GOLDEN, "eof_c1.cache"))
    lib = _lib.load()
    ca, sa = np.cos(0.7), np.sin(0.7)
    xa, ya, za, ma = (np.ascontiguousarray(g[k], dtype=np.float64) for k in "xyzm")
    # a second particle set of the same size: rotated about z and lifted
    sets = {"A": (xa, ya, za, ma), "B": (ca * xa - sa * ya, sa * xa + ca * ya, za + 0.01, ma * 1.5)}
    dsets = {k: [torch.from_numpy(np.ascontiguousarray(a)).to("cuda") for a in v] for k, v in sets.items()}

    def run(name, direct=False):
        r = torch.empty(xa.size, dtype=torch.float64, device="cuda")
        if direct:
            lib.xt_timing_enable(1)      # stage timing enqueues the call without a graph
        try:
            coef, res = table.accumulate_eval_blocks(*dsets[name], precision=precision, r_out=r)
            out = dev.to_host_many([coef, res, r])
        finally:
            lib.xt_timing_enable(0)
        return out

    ref = {k: run(k, direct=True) for k in sets}
    tol = 1e-12 if precision == "f64" else 1e-6
    # direct (first sighting), capture, patch to B, patch back to A, replay B again
    for name in ["A", "A", "B", "A", "B", "B"]:
        got = run(name)
        for a, b in zip(got, ref[name]):
            assert _rel(a, b) <= tol, name
    if precision == "f64":
        assert max(_rel(ref["A"][0][0][m], g["cos"][m]) for m in range(g["cos"].shape[0])) <= 1e-10
        for k in range(5):
            assert _rel(ref["A"][1][k], g["aep"][k]) <= 1e-10
        assert _rel(ref["A"][2], g["aep"][5]) <= 1e-10


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_host_results_staged_by_part(precision):
    """Results into page-locked host memory: the records are sorted by part of
    the particle range, then cell, and each part's results are copied out
    while the next is evaluated; the copies are issued outside the captured
    graph, so every call may name a new destination.  Direct, captured and
    replayed calls with a fresh destination each time (and particle counts of
    1, 7 and the golden set) agree with device-result calls to rounding (the
    deposit order differs)."""
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import eof
    g = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    table = eof.table_from_file(os.path.join(GOLDEN, "eof_c1.cache"))
    xa, ya, za, ma = (np.ascontiguousarray(g[k], dtype=np.float64) for k in "xyzm")
    tol = 1e-12 if precision == "f64" else 2e-6
    for n in (1, 7, xa.size):
        d = [torch.from_numpy(np.ascontiguousarray(a[:n])).to("cuda") for a in (xa, ya, za, ma)]
        r = torch.empty(n, dtype=torch.float64, device="cuda")
        coef, res = table.accumulate_eval_blocks(*d, precision=precision, r_out=r)
        ref_coef, ref_res = dev.to_host_many([coef, res])
        for _ in range(4):          # direct, capture, replays
            blk = torch.empty(5 * n, dtype=torch.float64, pin_memory=True)
            blk.fill_(np.nan)
            coef, none = table.accumulate_eval_blocks(*d, precision=precision, r_out=r, res_out=blk.data_ptr())
            assert none is None
            got_coef = dev.to_host(coef)       # synchronises the stream: the copies are done
            got = blk.numpy().reshape(5, n)
            assert not np.isnan(got).any(), n
            assert _rel(got_coef, ref_coef) <= tol, n
            for k in range(5):
                assert _rel(got[k], ref_res[k]) <= tol, (n, k)
