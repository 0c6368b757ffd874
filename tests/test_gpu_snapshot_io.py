"""Snapshot readers on the GPU: columns de-interleaved by the kernel from
page-locked records equal the reference readers' columns bit for bit
(tests/golden/snapshots.npz), on the host (file types) and on the device
(float columns as float64); a device-read snapshot feeds the fused EOF call
directly and gives the host-array result."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

SNAP = os.path.join(GOLDEN, "snap")
COMPS = {"OUT.f4idx": ("psp", ["star", "dark"]), "OUT.f8": ("psp", ["star"]),
         "SPL.f4": ("spl", ["star", "gas"]), "SPL.f8idx": ("spl", ["star"])}


def _reader(kind):
    from exptool_gb300.io import psp_io, spl_io
    return psp_io if kind == "psp" else spl_io


@pytest.mark.parametrize("fname", list(COMPS))
def test_columns_match_reference(fname):
    import torch
    g = np.load(os.path.join(GOLDEN, "snapshots.npz"))
    kind, comps = COMPS[fname]
    for cname in comps:
        host = _reader(kind).Input(os.path.join(SNAP, fname), comp=cname)
        devr = _reader(kind).Input(os.path.join(SNAP, fname), comp=cname, device=True)
        keys = [k.split("/")[2] for k in g.files if k.startswith(f"{fname}/{cname}/") and not k.endswith("/time")]
        assert sorted(host.data) == sorted(keys)
        assert host.time == float(g[f"{fname}/{cname}/time"])
        for k in keys:
            want = g[f"{fname}/{cname}/{k}"]
            got = host.data[k]
            assert got.dtype == want.dtype and np.array_equal(got, want), (fname, cname, k)
            d = devr.data[k]
            assert d.is_cuda
            if want.dtype.kind == "f":
                assert d.dtype == torch.float64
                assert np.array_equal(d.cpu().numpy(), want.astype(np.float64)), (fname, cname, k)
            else:
                assert np.array_equal(d.cpu().numpy(), want), (fname, cname, k)


def test_large_snapshot_round_trip(tmp_path):
    """1e6 particles, double precision with ids and attributes (84-byte
    records): every column survives the write / read / de-interleave."""
    from exptool_gb300.io import psp_io, snapshot
    rng = np.random.default_rng(9)
    n = 1_000_003
    comp = {k: rng.normal(size=n) for k in ["m", "x", "y", "z", "vx", "vy", "vz", "potE", "f_attr0"]}
    comp["i_attr0"] = rng.integers(-2**31, 2**31, n)
    comp["id"] = rng.integers(0, 2**62, n)
    path = str(tmp_path / "OUT.big")
    snapshot.write_psp(path, 3.0, {"disc": comp}, float_len=8, indexing=True)
    I = psp_io.Input(path, comp="disc")
    for k, v in comp.items():
        assert np.array_equal(I.data[k], v.astype(I.data[k].dtype)), k


def test_device_snapshot_feeds_fused_call(tmp_path):
    from exptool_gb300.basis import eof
    from exptool_gb300.io import psp_io, snapshot
    eg = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    comp = {"m": eg["m"], "x": eg["x"], "y": eg["y"], "z": eg["z"]}
    for k in ("vx", "vy", "vz", "potE"):
        comp[k] = np.zeros_like(eg["m"])
    path = str(tmp_path / "OUT.eof")
    snapshot.write_psp(path, 0.0, {"disc": comp}, float_len=8)
    cache = os.path.join(GOLDEN, "eof_c1.cache")
    Ed, rd = eof.compute_coefficients_and_forces(psp_io.Input(path, comp="disc", device=True), cache, verbose=0)
    Eh, rh = eof.compute_coefficients_and_forces(psp_io.Input(path, comp="disc"), cache, verbose=0)
    for m in range(Ed.cos.shape[0]):
        assert np.max(np.abs(Ed.cos[m] - eg["cos"][m])) <= 1e-10 * np.max(np.abs(eg["cos"][m]))
        assert np.allclose(Ed.cos[m], Eh.cos[m], rtol=0, atol=1e-12 * np.max(np.abs(Eh.cos[m])))
    for k in range(6):
        assert np.max(np.abs(rd[k] - eg["aep"][k])) <= 1e-10 * np.max(np.abs(eg["aep"][k]))
