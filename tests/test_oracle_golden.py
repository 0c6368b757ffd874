"""Pin the CPU oracle against golden vectors produced by the exptool reference
(``tests/golden/make_golden.py``)."""
import os

import numpy as np
import pytest

from oracle import sl as osl
from oracle import eof as oeof
from oracle import fields as ofields
from tests.conftest import GOLDEN

RTOL = 1e-12


def close(a, b, rtol=RTOL):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b)) / scale if a.size else 0.0
    assert a.shape == b.shape, (a.shape, b.shape)
    assert err <= rtol, err


def sl_table(cmap):
    return osl.load_table(os.path.join(GOLDEN, f"sl_c{cmap}.cache"), os.path.join(GOLDEN, f"sl_c{cmap}.model"))


@pytest.mark.parametrize("cmap", [0, 1, 2])
def test_sl_tables_and_bases(cmap):
    g = np.load(os.path.join(GOLDEN, f"sl_c{cmap}.npz"))
    t = sl_table(cmap)
    close(t["xi"], g["xi"], 0)
    close(t["p0"], g["p0"], 0)
    close(t["d0"], g["d0"], 0)
    close(osl.factorial_return(6), g["factorial6"], 1e-15)
    for i, x in enumerate(g["leg_x"]):
        close(osl.legendre_R(6, x)[:, :, 0], g["legendre"][i], 1e-15)
        p, dp = osl.dlegendre_R(6, x)
        close(p[:, :, 0], g["dlegendre"][i][0], 1e-15)
        close(dp[:, :, 0], g["dlegendre"][i][1], 1e-14)
    lm, nm = t["lmax"], t["nmax"]
    d, f, pt = osl.halo_dens_force_pot(g["pt_r"], lm, nm, t["ev"], t["ef"], t["xi"], t["d0"], t["p0"],
                                       t["cmap"], t["scale"], t["rmin"], t["rmax"])
    close(d, g["dens_force_pot"][:, 0], 1e-14)
    close(f, g["dens_force_pot"][:, 1], 1e-14)
    close(pt, g["dens_force_pot"][:, 2], 1e-14)
    close(osl.halo_pot_matrix(g["pt_r"], lm, nm, t["ev"], t["ef"], t["xi"], t["p0"], t["cmap"], t["scale"],
                              t["rmin"], t["rmax"]), g["pot_matrix"], 1e-14)


def _block_close(a, b, lmax, rtol):
    """Normwise relative error per l block of an expcoef matrix."""
    row = 0
    for l in range(lmax + 1):
        blk = slice(row, row + 2 * l + 1)
        s = np.max(np.abs(b[blk]))
        if s > 0:
            assert np.max(np.abs(a[blk] - b[blk])) / s <= rtol, l
        else:
            assert np.max(np.abs(a[blk])) == 0
        row += 2 * l + 1


@pytest.mark.parametrize("cmap", [0, 1, 2])
def test_sl_accumulate_and_eval(cmap):
    g = np.load(os.path.join(GOLDEN, f"sl_c{cmap}.npz"))
    t = sl_table(cmap)
    x, y, z, m = g["x"], g["y"], g["z"], g["m"]
    _block_close(osl.compute_coefficients_solitary(x, y, z, m, t), g["expcoef"], t["lmax"], 1e-13)
    _block_close(osl.compute_coefficients_solitary(x, y, z, m, t, no_odd=True), g["expcoef_noodd"], t["lmax"], 1e-13)
    ec = g["expcoef"]
    for tag, kw in {"aep": {}, "aep_l02": dict(L1=0, L2=2), "aep_l13_noodd": dict(L1=1, L2=3, NO_ODD=True)}.items():
        res = osl.all_eval_particles(x, y, z, ec, t, **kw)
        for k in range(8):
            close(res[k], g[tag][k], 1e-12)
    r, c, p = g["pt_r"], g["pt_costh"], g["pt_phi"]
    for tag, kw in {"all_eval": {}, "all_eval_noodd": dict(no_odd=True)}.items():
        res = osl.all_eval(r, c, p, ec, t, **kw)
        for k in range(7):
            close(res[k], g[tag][:, k], 1e-12)
    for tag, kw in {"force_eval": {}, "force_eval_l2n4": dict(lmax=2, nmax=4),
                    "force_eval_noodd": dict(no_odd=True)}.items():
        res = osl.force_eval(r, c, p, ec, t, **kw)
        for k in range(5):
            close(res[k], g[tag][:, k], 1e-12)


@pytest.mark.parametrize("tag", ["c1", "c0"])
def test_eof_golden(tag):
    g = np.load(os.path.join(GOLDEN, f"eof_{tag}.npz"))
    t = oeof.load_table(os.path.join(GOLDEN, f"eof_{tag}.cache"))
    close(np.array([t["XMIN"], t["XMAX"], t["dX"], t["YMIN"], t["YMAX"], t["dY"]]), g["table_params"], 0)
    x, y, z, m = g["x"], g["y"], g["z"], g["m"]
    kw = dict(MMAX=t["mmax"], NMAX=t["norder"], XMIN=t["XMIN"], dX=t["dX"], YMIN=t["YMIN"], dY=t["dY"],
              NUMX=t["numx"], NUMY=t["numy"], ASCALE=t["ascale"], HSCALE=t["hscale"], CMAP=t["cmap"])
    c, s = oeof.accumulate(x, y, z, m, t["potC"], t["potS"], **kw)
    for ref in (("cos", "sin"), ("cos_data", "sin_data"), ("cos_multi", "sin_multi")):
        for mm in range(t["mmax"] + 1):
            close(c[mm], g[ref[0]][mm], 1e-12)
            close(s[mm], g[ref[1]][mm], 1e-12) if mm else None
    ev = dict(rmin=t["XMIN"], dR=t["dX"], zmin=t["YMIN"], dZ=t["dY"], numx=t["numx"], numy=t["numy"],
              MMAX=t["mmax"], NMAX=t["norder"], ASCALE=t["ascale"], HSCALE=t["hscale"], CMAP=t["cmap"])
    tabs = [t[k] for k in ("potC", "rforceC", "zforceC", "potS", "rforceS", "zforceS")]
    a_c, a_s = g["cos"], g["sin"]
    for gt, kw2 in {"aep": {}, "aep_m12": dict(m1=1, m2=2)}.items():
        res = oeof.accumulated_eval_particles(x, y, z, a_c, a_s, *tabs, **ev, **kw2)
        for k in range(6):
            close(res[k], g[gt][k], 1e-12)
    if "aep_dens" in g.files:
        res = oeof.accumulated_eval_particles(x, y, z, a_c, a_s, *tabs, **ev, densC=t["densC"], densS=t["densS"])
        for k in range(8):
            close(res[k], g["aep_dens"][k], 1e-12)
    fk = {k: ev[k] for k in ("rmin", "dR", "zmin", "dZ", "numx", "numy", "ASCALE", "HSCALE", "CMAP")}
    R, Z, P = g["pt_R"], g["pt_z"], g["pt_phi"]
    for gt, (MM, NN, NO, PT) in {"force_eval": (t["mmax"], t["norder"], False, False),
                                 "force_eval_noodd": (t["mmax"], t["norder"], True, False),
                                 "force_eval_m2n2": (min(2, t["mmax"]), 2, False, False),
                                 "force_eval_perturb": (t["mmax"], t["norder"], False, True)}.items():
        res = oeof.force_eval(R, Z, P, a_c, a_s, *tabs, MMAX=MM, NMAX=NN, no_odd=NO, perturb=PT, **fk)
        for k in range(len(res)):
            close(res[k], g[gt][:, k], 1e-12)
    for gt, NO in {"acc_eval": False, "acc_eval_noodd": True}.items():
        res = oeof.accumulated_eval(R, Z, P, a_c, a_s, t["potC"], t["rforceC"], t["zforceC"], t["densC"], t["potS"],
                                    t["rforceS"], t["zforceS"], t["densS"], MMAX=t["mmax"], NMAX=t["norder"],
                                    no_odd=NO, **fk)
        for k in range(7):
            close(res[k], g[gt][:, k], 1e-12)
    b = oeof.return_bins(R, Z, **fk)
    for k in range(4):
        close(b[k], g["bins"][k], 0)


def fields_oracle():
    g = np.load(os.path.join(GOLDEN, "fields.npz"))
    slt = sl_table(2)
    sg = np.load(os.path.join(GOLDEN, "sl_c2.npz"))
    et = oeof.load_table(os.path.join(GOLDEN, "eof_c1.cache"))
    eg = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    F = ofields.FieldsOracle(slt, sg["expcoef"], et, eg["cos"], eg["sin"], halofac=float(g["halofac"]))
    return F, g


def test_fields_forces_and_orbits():
    F, g = fields_oracle()
    res = F.return_forces_cart(g["px"], g["py"], g["pz"], rotpos=g["rot"])
    for k in range(8):
        close(res[k], g["forces_cart"][:, k], 1e-12)
    F.set_field_parameters(no_odd=True, halo_l=2, halo_n=4, disk_m=2, disk_n=2)
    res = F.return_forces_cart(g["px"], g["py"], g["pz"], rotpos=g["rot"])
    for k in range(8):
        close(res[k], g["forces_cart_trunc"][:, k], 1e-12)
    F.reset_field_parameters()
    orbits = [([1.0, 0.0, 0.05], [0.0, 0.55, 0.02], 0.0, False, 1000, False),
              ([0.3, -1.2, 0.0], [0.4, 0.1, 0.0], 0.2, True, 1000, False),
              ([2.5, 0.5, -0.1], [-0.1, -0.4, 0.05], -0.15, False, 1, True)]
    for k, (ip, iv, rf, force, apmax, apse) in enumerate(orbits):
        F.reset_field_parameters()
        O = ofields.leapfrog_integrate(F, 60, 0.02, [ip], [iv], rotfreq=rf, force=force, ap_max=apmax, apse=apse)[0]
        keys = sorted(k2[len(f"orbit{k}_"):] for k2 in g.files if k2.startswith(f"orbit{k}_"))
        assert sorted(O.keys()) == keys
        for key in keys:
            close(O[key], g[f"orbit{k}_{key}"], 1e-11)
    F.reset_field_parameters()
    O = ofields.leapfrog_integrate(F, 40, 0.02, [[0.8, 0.2, 0.0]], [[0.1, 0.6, 0.0]], no_odd=True, halo_l=2,
                                   disk_m=2, disk_n=2)[0]
    for key in O:
        close(O[key], g[f"orbit3_{key}"], 1e-11)
    F.reset_field_parameters()
    ts = [ofields.compute_timestep(F, [1.0, 0.2, 0.1], [0.1, 0.5, 0.0]),
          ofields.compute_timestep(F, [4.0, -1.0, 0.3], [0.2, 0.3, 0.05], dyn_res=50.)]
    close(np.array(ts), g["timestep"], 1e-12)
