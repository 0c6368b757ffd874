"""GPU drop-in functions against the exptool reference's own outputs
(tests/golden, produced by tests/golden/make_golden.py).

Parity bar of the plain FP64 path: normwise relative error <= 1e-10
(coefficients per l / m block, evaluated fields per output array)."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    s = np.max(np.abs(b)) if b.size else 0.0
    d = np.max(np.abs(a - b)) if b.size else 0.0
    return d / s if s > 0 else d


def block_rel(a, b, lmax):
    out, row = [], 0
    for l in range(lmax + 1):
        out.append(rel(a[row:row + 2 * l + 1], b[row:row + 2 * l + 1]))
        row += 2 * l + 1
    return max(out)


class Holder:
    def __init__(self, x, y, z, m):
        self.xpos, self.ypos, self.zpos, self.mass = x, y, z, m
        self.data = {"x": x, "y": y, "z": z, "m": m}


@pytest.mark.parametrize("cmap", [0, 1, 2])
def test_sl_golden(cmap):
    from exptool_gb300.basis import spheresl
    g = np.load(os.path.join(GOLDEN, f"sl_c{cmap}.npz"))
    cache = os.path.join(GOLDEN, f"sl_c{cmap}.cache")
    model = os.path.join(GOLDEN, f"sl_c{cmap}.model")
    P = Holder(g["x"], g["y"], g["z"], g["m"])
    ec = spheresl.compute_coefficients_solitary(P, cache, model)
    assert block_rel(ec, g["expcoef"], 4) <= TOL
    assert block_rel(spheresl.compute_coefficients_solitary(P, cache, model, no_odd=True), g["expcoef_noodd"], 4) <= TOL
    so = spheresl.compute_coefficients(P, cache, model)
    assert block_rel(so.expcoef, g["expcoef"], 4) <= TOL and so.lmax == 4 and so.nmax == 6
    ec = g["expcoef"]
    for tag, kw in {"aep": {}, "aep_l02": dict(L1=0, L2=2), "aep_l13_noodd": dict(L1=1, L2=3, NO_ODD=True)}.items():
        res = spheresl.all_eval_particles(P, ec, cache, model, 0, **kw)
        for k in range(8):
            assert rel(res[k], g[tag][k]) <= TOL, (tag, k, rel(res[k], g[tag][k]))
    r, c, p = g["pt_r"], g["pt_costh"], g["pt_phi"]
    tab = (g["xi"], g["p0"], g["d0"], cmap, 1.0)
    from oracle.sl import read_cached_table
    _, _, _, _, _, _, _, _, evt, eft = read_cached_table(cache)
    for tag, no in {"all_eval": False, "all_eval_noodd": True}.items():
        res = spheresl.all_eval(r, c, p, ec, *tab, 4, 6, evt, eft, no_odd=no)
        for k in range(7):
            assert rel(res[k], g[tag][:, k]) <= TOL, (tag, k)
    for tag, (lu, nu, no) in {"force_eval": (4, 6, False), "force_eval_l2n4": (2, 4, False),
                              "force_eval_noodd": (4, 6, True)}.items():
        res = spheresl.force_eval(r, c, p, ec, *tab, lu, nu, evt, eft, no_odd=no)
        for k in range(5):
            assert rel(res[k], g[tag][:, k]) <= TOL, (tag, k, rel(res[k], g[tag][:, k]))
    # scalar call returns floats like the reference
    s = spheresl.force_eval(float(r[0]), float(c[0]), float(p[0]), ec, *tab, 4, 6, evt, eft)
    assert isinstance(s[0], float) and abs(s[0] - g["force_eval"][0, 0]) <= TOL * max(1.0, abs(s[0]))


@pytest.mark.parametrize("tag", ["c1", "c0"])
def test_eof_golden(tag):
    from exptool_gb300.basis import eof
    g = np.load(os.path.join(GOLDEN, f"eof_{tag}.npz"))
    path = os.path.join(GOLDEN, f"eof_{tag}.cache")
    potC, rforceC, zforceC, densC, potS, rforceS, zforceS, densS = eof.parse_eof(path)
    rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens = eof.eof_params(path)
    XMIN, XMAX, dX, YMIN, YMAX, dY = eof.set_table_params(RMAX=rmax, RMIN=rmin, ASCALE=ascale, HSCALE=hscale,
                                                          NUMX=numx, NUMY=numy, CMAP=cmap)
    assert np.array_equal([XMIN, XMAX, dX, YMIN, YMAX, dY], g["table_params"])
    P = Holder(g["x"], g["y"], g["z"], g["m"])
    c, s = eof.accumulate(P, potC, potS, mmax, norder, XMIN, dX, YMIN, dY, numx, numy, ascale, hscale, cmap)
    for m in range(mmax + 1):
        assert rel(c[m], g["cos"][m]) <= TOL, m
        if m:
            assert rel(s[m], g["sin"][m]) <= TOL, m
    assert not np.any(s[0])
    E = eof.compute_coefficients(P, path, verbose=0)
    assert max(rel(E.cos[m], g["cos"][m]) for m in range(mmax + 1)) <= TOL
    # the fused pipeline (double-float set-up and inner products) on the same particles
    E2, res2 = eof.compute_coefficients_and_forces(P, path, verbose=0)
    assert max(rel(E2.cos[m], g["cos"][m]) for m in range(mmax + 1)) <= TOL
    assert max(rel(E2.sin[m], g["sin"][m]) for m in range(1, mmax + 1)) <= TOL
    for k in range(6):
        assert rel(res2[k], g["aep"][k]) <= TOL, k
    E.cos, E.sin = g["cos"], g["sin"]
    res = eof.compute_forces(P, E, verbose=0)
    for k in range(6):
        assert rel(res[k], g["aep"][k]) <= TOL, k
    tabs = dict(potC=potC, rforceC=rforceC, zforceC=zforceC, potS=potS, rforceS=rforceS, zforceS=zforceS)
    kw = dict(rmin=XMIN, dR=dX, zmin=YMIN, dZ=dY, numx=numx, numy=numy, MMAX=mmax, NMAX=norder, ASCALE=ascale,
              HSCALE=hscale, CMAP=cmap, verbose=0)
    res = eof.accumulated_eval_particles(P, g["cos"], g["sin"], m1=1, m2=2, **tabs, **kw)
    for k in range(6):
        assert rel(res[k], g["aep_m12"][k]) <= TOL, k
    if "aep_dens" in g.files:
        res = eof.accumulated_eval_particles(P, g["cos"], g["sin"], density=True, verbose=0, eof_file=path)
        for k in range(8):
            assert rel(res[k], g["aep_dens"][k]) <= TOL, k
    fk = dict(rmin=XMIN, dR=dX, zmin=YMIN, dZ=dY, numx=numx, numy=numy, ASCALE=ascale, HSCALE=hscale, CMAP=cmap)
    R, Z, PH = g["pt_R"], g["pt_z"], g["pt_phi"]
    for gt, (MM, NN, NO, PT) in {"force_eval": (mmax, norder, False, False), "force_eval_noodd": (mmax, norder, True, False),
                                 "force_eval_m2n2": (min(2, mmax), 2, False, False),
                                 "force_eval_perturb": (mmax, norder, False, True)}.items():
        res = eof.force_eval(R, Z, PH, g["cos"], g["sin"], potC, rforceC, zforceC, potS, rforceS, zforceS, MMAX=MM,
                             NMAX=NN, no_odd=NO, perturb=PT, **fk)
        for k in range(len(res)):
            assert rel(res[k], g[gt][:, k]) <= TOL, (gt, k, rel(res[k], g[gt][:, k]))
    if dens:
        for gt, NO in {"acc_eval": False, "acc_eval_noodd": True}.items():
            res = eof.accumulated_eval(R, Z, PH, g["cos"], g["sin"], potC, rforceC, zforceC, densC, potS, rforceS,
                                       zforceS, densS, MMAX=mmax, NMAX=norder, no_odd=NO, **fk)
            for k in range(7):
                assert rel(res[k], g[gt][:, k]) <= TOL, (gt, k)


def make_fields():
    from exptool_gb300.basis import potential, spheresl, eof
    g = np.load(os.path.join(GOLDEN, "fields.npz"))
    sg = np.load(os.path.join(GOLDEN, "sl_c2.npz"))
    eg = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    cache, model = os.path.join(GOLDEN, "sl_c2.cache"), os.path.join(GOLDEN, "sl_c2.model")
    epath = os.path.join(GOLDEN, "eof_c1.cache")
    F = potential.Fields("none", epath, cache, model, verbose=0)
    F.EOF = eof.EOF_Object()
    F.EOF.eof_file, F.EOF.cos, F.EOF.sin = epath, eg["cos"], eg["sin"]
    F.SL = spheresl.SL_Object()
    F.SL.sph_file, F.SL.model_file, F.SL.expcoef = cache, model, sg["expcoef"]
    F.halofac = float(g["halofac"])
    F.prep_tables()
    return F, g


def test_fields_golden():
    F, g = make_fields()
    res = F.return_forces_cart(g["px"], g["py"], g["pz"], rotpos=g["rot"])
    for k in range(8):
        assert rel(res[k], g["forces_cart"][:, k]) <= TOL, (k, rel(res[k], g["forces_cart"][:, k]))
    F.set_field_parameters(no_odd=True, halo_l=2, halo_n=4, disk_m=2, disk_n=2)
    res = F.return_forces_cart(g["px"], g["py"], g["pz"], rotpos=g["rot"])
    for k in range(8):
        assert rel(res[k], g["forces_cart_trunc"][:, k]) <= TOL, k
    F.reset_field_parameters()
    s = F.return_forces_cart(float(g["px"][0]), float(g["py"][0]), float(g["pz"][0]), rotpos=float(g["rot"][0]))
    assert abs(s[0] - g["forces_cart"][0, 0]) <= TOL * np.max(np.abs(g["forces_cart"][:, 0]))


def test_leapfrog_golden():
    from exptool_gb300.utils import integrate
    F, g = make_fields()
    orbits = [([1.0, 0.0, 0.05], [0.0, 0.55, 0.02], 0.0, False, 1000, False),
              ([0.3, -1.2, 0.0], [0.4, 0.1, 0.0], 0.2, True, 1000, False),
              ([2.5, 0.5, -0.1], [-0.1, -0.4, 0.05], -0.15, False, 1, True)]
    for k, (ip, iv, rf, force, apmax, apse) in enumerate(orbits):
        F.reset_field_parameters()
        O = integrate.leapfrog_integrate(F, 60, 0.02, ip, iv, rotfreq=rf, force=force, ap_max=apmax, apse=apse)
        keys = sorted(k2[len(f"orbit{k}_"):] for k2 in g.files if k2.startswith(f"orbit{k}_"))
        assert sorted(O.keys()) == keys
        for key in keys:
            assert rel(O[key], g[f"orbit{k}_{key}"]) <= 1e-9, (k, key, rel(O[key], g[f"orbit{k}_{key}"]))
    F.reset_field_parameters()
    O = integrate.leapfrog_integrate(F, 40, 0.02, [0.8, 0.2, 0.0], [0.1, 0.6, 0.0], no_odd=True, halo_l=2, disk_m=2,
                                     disk_n=2)
    for key in O:
        assert rel(O[key], g[f"orbit3_{key}"]) <= 1e-9, key
    F.reset_field_parameters()
    ts = [integrate.compute_timestep(F, [1.0, 0.2, 0.1], [0.1, 0.5, 0.0]),
          integrate.compute_timestep(F, [4.0, -1.0, 0.3], [0.2, 0.3, 0.05], dyn_res=50.)]
    assert rel(np.array(ts), g["timestep"]) <= TOL
