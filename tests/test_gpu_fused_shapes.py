"""The fused accumulate + evaluate call on table shapes the golden caches do
not reach: mmax 8 (the largest deposit instantiation), mmax 5 (below its
instantiation's cap), orders that are not a multiple of the contraction's
order groups and field row batches (10, 7), and node counts that leave a
partial node block of the tiled tables.  Random tables and disc-like
particles; the oracle gives the coefficients and the forces at them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(8, 10, 40, 30), (5, 7, 33, 21)]


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _case(mmax, norder, numx, numy, seed=11, n=20000):
    from exptool_gb300.basis import eof
    rng = np.random.default_rng(seed)
    shp = (mmax + 1, norder, numx + 1, numy + 1)
    tabs = [rng.standard_normal(shp) for _ in range(6)]
    ascale, hscale, cmap = 1.0, 0.1, 1
    XMIN, XMAX, dX, YMIN, YMAX, dY = eof.set_table_params(RMAX=20.0, RMIN=0.001, ASCALE=ascale, HSCALE=hscale,
                                                          NUMX=numx, NUMY=numy, CMAP=cmap)
    R = 0.01 + rng.exponential(2.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    x, y = R * np.cos(phi), R * np.sin(phi)
    z = 0.1 * rng.standard_normal(n)
    m = np.full(n, 1.0 / n)
    par = dict(XMIN=XMIN, dX=dX, YMIN=YMIN, dY=dY, ascale=ascale, hscale=hscale, cmap=cmap)
    return tabs, (x, y, z, m), par


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "m%d_n%d_%dx%d" % s)
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_fused_shapes_against_oracle(shape, precision):
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import eof
    from oracle import eof as oeof
    mmax, norder, numx, numy = shape
    (potC, rforceC, zforceC, potS, rforceS, zforceS), (x, y, z, m), p = _case(*shape)
    table = eof.table_from_arrays(mmax, norder, numx, numy, p["cmap"], p["XMIN"], p["dX"], p["YMIN"], p["dY"],
                                  p["ascale"], p["hscale"], potC, rforceC, zforceC, potS, rforceS, zforceS)
    cos, sin, outs = table.accumulate_eval(*(dev.to_dev(a) for a in (x, y, z, m)), precision=precision)
    cos, sin = dev.to_host(cos), dev.to_host(sin)
    outs = [dev.to_host(o) for o in outs]
    c, s = oeof.accumulate(x, y, z, m, potC, potS, mmax, norder, p["XMIN"], p["dX"], p["YMIN"], p["dY"], numx, numy,
                           p["ascale"], p["hscale"], p["cmap"])
    ref = oeof.accumulated_eval_particles(x, y, z, c, s, potC, rforceC, zforceC, potS, rforceS, zforceS, p["XMIN"],
                                          p["dX"], p["YMIN"], p["dY"], numx, numy, mmax, norder, p["ascale"],
                                          p["hscale"], p["cmap"])
    # FP64 path: the parity bar; mixed path: FP32 per-particle arithmetic
    tol = 1e-10 if precision == "f64" else 2e-5
    for mm in range(mmax + 1):
        assert _rel(cos[mm], c[mm]) <= tol, ("cos", mm, _rel(cos[mm], c[mm]))
        if mm:
            assert _rel(sin[mm], s[mm]) <= tol, ("sin", mm, _rel(sin[mm], s[mm]))
    assert not np.any(sin[0])
    # forces at the GPU's own coefficients against the oracle's at its own:
    # the coefficient difference is inside the tolerance above
    for k in range(6):
        assert _rel(outs[k], ref[k]) <= tol, (k, _rel(outs[k], ref[k]))


ENGINE_SHAPES = [(8, 24, 40, 30), (0, 4, 20, 12), (6, 18, 48, 24), (5, 7, 33, 21)]


@pytest.mark.parametrize("shape", ENGINE_SHAPES, ids=lambda s: "m%d_n%d_%dx%d" % s)
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_field_engines_agree(shape, precision):
    """The field stage's bulk-copy pipeline (engine 1) and row-load kernel
    (engine 2) on the same particles: forces agree to double-float rounding
    of the field (FP64 path) or to FP32 rounding of it (mixed path), and the
    pipeline's against the oracle at the bar of the test above.  The shapes
    take the pipeline through two m-ranges per field (M = 8, Q = 24), sine
    units with no rows (M = 0), and last node blocks of 55, 17 and 9 nodes
    whose FP32 tile is written by plain stores; its wait flag stays clear."""
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import eof
    from oracle import eof as oeof
    mmax, norder, numx, numy = shape
    (potC, rforceC, zforceC, potS, rforceS, zforceS), (x, y, z, m), p = _case(*shape, seed=23, n=30000)
    table = eof.table_from_arrays(mmax, norder, numx, numy, p["cmap"], p["XMIN"], p["dX"], p["YMIN"], p["dY"],
                                  p["ascale"], p["hscale"], potC, rforceC, zforceC, potS, rforceS, zforceS)
    got = {}
    try:
        for engine in (1, 2):
            dev.cyl_field_engine(engine)
            cos, sin, outs = table.accumulate_eval(*(dev.to_dev(a) for a in (x, y, z, m)), precision=precision)
            got[engine] = [dev.to_host(o) for o in outs]
            dev.cyl_status()
    finally:
        dev.cyl_field_engine(0)
    agree = 1e-12 if precision == "f64" else 1e-6
    for k in range(6):
        assert _rel(got[1][k], got[2][k]) <= agree, (k, _rel(got[1][k], got[2][k]))
    c, s = oeof.accumulate(x, y, z, m, potC, potS, mmax, norder, p["XMIN"], p["dX"], p["YMIN"], p["dY"], numx, numy,
                           p["ascale"], p["hscale"], p["cmap"])
    ref = oeof.accumulated_eval_particles(x, y, z, c, s, potC, rforceC, zforceC, potS, rforceS, zforceS, p["XMIN"],
                                          p["dX"], p["YMIN"], p["dY"], numx, numy, mmax, norder, p["ascale"],
                                          p["hscale"], p["cmap"])
    tol = 1e-10 if precision == "f64" else 2e-5
    for k in range(6):
        assert _rel(got[1][k], ref[k]) <= tol, (k, _rel(got[1][k], ref[k]))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_empty_snapshot_between_full_ones(precision):
    """The fused call on no particles returns zero coefficients (the deposit
    grids are cleared and no node block is listed), and the workspace it
    leaves does not leak into a full call or back: empty, full, empty on one
    workspace, the full call against the oracle."""
    import torch
    from exptool_gb300 import _lib
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import eof
    from oracle import eof as oeof
    shape = (5, 7, 33, 21)
    mmax, norder, numx, numy = shape
    (potC, rforceC, zforceC, potS, rforceS, zforceS), (x, y, z, m), p = _case(*shape, seed=31, n=5000)
    table = eof.table_from_arrays(mmax, norder, numx, numy, p["cmap"], p["XMIN"], p["dX"], p["YMIN"], p["dY"],
                                  p["ascale"], p["hscale"], potC, rforceC, zforceC, potS, rforceS, zforceS)
    pc = _lib.XT_F64 if precision == "f64" else _lib.XT_F32
    ws = torch.empty(_lib.load().xt_cyl_accumulate_eval_workspace(table.handle, x.size, pc), dtype=torch.uint8,
                     device="cuda")
    none = [torch.empty(0, dtype=torch.float64, device="cuda") for _ in range(4)]
    full = [dev.to_dev(a) for a in (x, y, z, m)]
    c, s = oeof.accumulate(x, y, z, m, potC, potS, mmax, norder, p["XMIN"], p["dX"], p["YMIN"], p["dY"], numx, numy,
                           p["ascale"], p["hscale"], p["cmap"])
    tol = 1e-10 if precision == "f64" else 2e-5
    for run in ("empty", "full", "empty"):
        args = none if run == "empty" else full
        cos, sin, outs = table.accumulate_eval(*args, precision=precision, workspace=ws)
        cos, sin = dev.to_host(cos), dev.to_host(sin)
        if run == "empty":
            assert not np.any(cos) and not np.any(sin)
            assert all(o.numel() == 0 for o in outs)
        else:
            for mm in range(mmax + 1):
                assert _rel(cos[mm], c[mm]) <= tol, ("cos", mm)
                if mm:
                    assert _rel(sin[mm], s[mm]) <= tol, ("sin", mm)
