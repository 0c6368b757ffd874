"""Generate the golden fixtures in this directory by running the exptool
reference (imported from its source tree through ``refshim``) on small,
seeded inputs.

Run from the repository root, naming the exptool source tree root (the
directory holding the ``exptool`` package):

  python tests/golden/make_golden.py --reference <root> [snapshots | run_time]

or set EXPTOOL_REFERENCE instead of --reference.  ``snapshots`` makes only the
snapshot-reader, coefficient-file and orbit-frequency fixtures, ``run_time``
only run_time.npz.

Outputs (all small):
  sl_c{0,1,2}.cache / .model  SL basis tables (reference file formats)
  eof_c1.cache, eof_c0.cache  EOF tables (old-style header; with / without density)
  sl_c{0,1,2}.npz             particles, SL accumulate / evaluate outputs
  eof_c1.npz, eof_c0.npz      particles, EOF accumulate / evaluate outputs
  fields.npz                  Fields.return_forces_cart, leapfrog_integrate,
                              compute_timestep outputs
  orbit_grids.npz             integrate_grid / _launchy / _3D arrays and the
                              print_orbit_array(_3D) text of the reference
  centering.npz               Fields.total_coefficients centring (centres and the
                              centred particles handed to the accumulators)
  run_time.npz                Fields.total_coefficients() reading a PSP snapshot,
                              get_fields and run_time_mod (orbit text, field file)
  coef_files.npz              bytes of SL / EOF coefficient files written by the
                              reference (two dumps each), the SHA-256 and size of
                              a Fields.save_field file, rotation_curve and
                              resonance_positions outputs
The table files are built by this project's generators; every output array is
produced by the reference code.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import refshim  # noqa: E402
from exptool_gb300.tables.models import TruncatedHernquist  # noqa: E402
from exptool_gb300.tables.sl_solver import SLBasis, write_sl_cache, write_model_file  # noqa: E402
from exptool_gb300.tables.eof_builder import EOFTables  # noqa: E402
from exptool_gb300.tables.samplers import hernquist_sample, disc_sample  # noqa: E402


def P(name):
    return os.path.join(HERE, name)


class Data:
    """Container with the ``.data`` dict of ``particle.Input`` plus the holder
    attributes (``eof.accumulated_eval_particles`` reads ``.zpos`` too)."""

    def __init__(self, x, y, z, m):
        self.data = {"x": x, "y": y, "z": z, "m": m}
        self.xpos, self.ypos, self.zpos, self.mass = x, y, z, m
        self.time = 0.0
        self.filename = "synthetic"
        self.comp = "dark"


def holder(ref, x, y, z, m):
    h = ref.particle.holder()
    h.xpos, h.ypos, h.zpos, h.mass = x, y, z, m
    return h


SL_EDGE = np.array([
    [0.0, 0.0, 0.0, 1e-3],        # origin
    [0.0, 0.0, 0.7, 1e-3],        # +z axis
    [0.0, 0.0, -2.5, 1e-3],       # -z axis
    [150.0, 20.0, -30.0, 1e-3],   # beyond rmax
    [5e-5, -3e-5, 2e-5, 1e-3],    # inside rmin
    [-2.0, -0.0, 0.5, 1e-3],      # phi = -pi branch
    [-0.3, 0.4, 0.0, 2e-3],       # midplane
])


def sl_case(ref, cmap):
    lmax, nmax, numr = 4, 6, 200
    rmin, rmax, scale = 1e-3, 100.0, 1.0
    model = TruncatedHernquist(a=1.0, rtrunc=100.0)
    basis = SLBasis(model, lmax, nmax, rmin, rmax, nfine=8001)
    cache, modelf = P(f"sl_c{cmap}.cache"), P(f"sl_c{cmap}.model")
    write_sl_cache(cache, basis, numr, cmap, scale)
    write_model_file(modelf, model, rmin * 0.5, rmax, npts=300, title="truncated Hernquist a=1 rt=100")
    refshim.set_log_bounds(ref, rmin, rmax)
    x, y, z, m = hernquist_sample(200, 100 + cmap)
    x = np.concatenate([x, SL_EDGE[:, 0]])
    y = np.concatenate([y, SL_EDGE[:, 1]])
    z = np.concatenate([z, SL_EDGE[:, 2]])
    m = np.concatenate([m, SL_EDGE[:, 3]])
    sl = ref.spheresl
    out = dict(x=x, y=y, z=z, m=m)
    out["expcoef"] = sl.compute_coefficients_solitary(holder(ref, x, y, z, m), cache, modelf, 0, False)
    out["expcoef_noodd"] = sl.compute_coefficients_solitary(holder(ref, x, y, z, m), cache, modelf, 0, True)
    ec = out["expcoef"]
    for tag, (L1, L2, NO) in {"aep": (-1000, 1000, False), "aep_l02": (0, 2, False),
                               "aep_l13_noodd": (1, 3, True)}.items():
        res = sl.all_eval_particles(Data(x, y, z, m), ec, cache, modelf, 0, L1=L1, L2=L2, NO_ODD=NO)
        out[tag] = np.array(res)
    # point-wise evaluators with the tables loaded the way Fields.prep_tables does
    (lm, nm, nr, cm, r0, r1, sc, lt, evt, eft) = ref.halo_methods.read_cached_table(cache)
    xi, rarr, p0, d0 = ref.halo_methods.init_table(modelf, nr, r0, r1, cmap=cm, scale=sc)
    out.update(xi=xi, p0=p0, d0=d0)
    rng = np.random.default_rng(300 + cmap)
    npt = 24
    pr = np.concatenate([10 ** rng.uniform(-3.5, 2.3, npt - 3), [1e-10, 1e-3, 100.0]])
    pc = np.concatenate([rng.uniform(-1, 1, npt - 3), [1.0, -1.0, 0.0]])
    pp = rng.uniform(-np.pi, np.pi, npt)
    out.update(pt_r=pr, pt_costh=pc, pt_phi=pp)
    ae = []
    for i in range(npt):
        ae.append(sl.all_eval(pr[i], pc[i], pp[i], ec, xi, p0, d0, cm, sc, lm, nm, evt, eft, no_odd=False))
    out["all_eval"] = np.array(ae)
    ae = []
    for i in range(npt):
        ae.append(sl.all_eval(pr[i], pc[i], pp[i], ec, xi, p0, d0, cm, sc, lm, nm, evt, eft, no_odd=True))
    out["all_eval_noodd"] = np.array(ae)
    for tag, (lu, nu, no) in {"force_eval": (lm, nm, False), "force_eval_l2n4": (2, 4, False),
                               "force_eval_noodd": (lm, nm, True)}.items():
        fe = []
        for i in range(npt):
            fe.append(sl.force_eval(pr[i], pc[i], pp[i], ec, xi, p0, d0, cm, sc, lu, nu, evt, eft, no_odd=no))
        out[tag] = np.array(fe)
    # radial function matrices and Legendre tables
    dpf = [np.array(sl.get_halo_dens_pot_force(r, lm, nm, evt, eft, xi, d0, p0, cm, sc)) for r in pr]
    out["dens_force_pot"] = np.array(dpf)
    out["pot_matrix"] = np.array([sl.get_halo_pot_matrix(r, lm, nm, evt, eft, xi, p0, cm, sc) for r in pr])
    lx = np.array([-1.0, -0.999999999, -0.5, 0.0, 0.3, 0.99999999, 1.0])
    out["leg_x"] = lx
    out["legendre"] = np.array([sl.legendre_R(6, v) for v in lx])
    out["dlegendre"] = np.array([np.array(sl.dlegendre_R(6, v)) for v in lx])
    out["factorial6"] = sl.factorial_return(6)
    np.savez_compressed(P(f"sl_c{cmap}.npz"), **out)
    print("sl", cmap, "done")
    return cache, modelf, ec


EOF_EDGE = np.array([
    [0.0, 0.0, 0.0, 1e-3],        # origin (R = 1e-5 from the 1e-10 softening)
    [40.0, 0.0, 0.1, 1e-3],       # beyond the radial table: extrapolation
    [3.0, 4.0, 30.0, 1e-3],       # beyond the vertical table: extrapolation
    [1.0, 1.0, -30.0, 1e-3],      # below the vertical table: clamp
    [-2.0, -0.0, 0.5, 1e-3],      # phi = -pi branch
    [1e-4, 1e-4, 0.0, 1e-3],      # inside rmin: clamp
    [0.5, -0.5, 0.0, 2e-3],       # midplane
])


def eof_case(ref, tag, cmap, dens, mmax, norder, numx, seed):
    tables = EOFTables(mmax=mmax, norder=norder, numx=numx, numy=numx, rmin=0.001, rmax=30.0,
                       ascale=1.0, hscale=0.1, cmap=cmap, lmax_sph=12, nmax_sph=8,
                       nsample=20000, seed=seed)
    path = P(f"eof_{tag}.cache")
    tables.write(path, dens=dens)
    e = ref.eof
    potC, rforceC, zforceC, densC, potS, rforceS, zforceS, densS = e.parse_eof(path)
    rmin, rmax, nx, ny, mm, no, asc, hsc, cm, dn = e.eof_params(path)
    XMIN, XMAX, dX, YMIN, YMAX, dY = e.set_table_params(RMAX=rmax, RMIN=rmin, ASCALE=asc, HSCALE=hsc,
                                                        NUMX=nx, NUMY=ny, CMAP=cm)
    x, y, z, m = disc_sample(200, seed + 1)
    x = np.concatenate([x, EOF_EDGE[:, 0]])
    y = np.concatenate([y, EOF_EDGE[:, 1]])
    z = np.concatenate([z, EOF_EDGE[:, 2]])
    m = np.concatenate([m, EOF_EDGE[:, 3]])
    out = dict(x=x, y=y, z=z, m=m, table_params=np.array([XMIN, XMAX, dX, YMIN, YMAX, dY]))
    a_cos, a_sin = e.accumulate(holder(ref, x, y, z, m), potC, potS, mm, no, XMIN, dX, YMIN, dY,
                                nx, ny, asc, hsc, cm)
    out.update(cos=a_cos, sin=a_sin)
    c2, s2 = e.accumulate(Data(x, y, z, m), potC, potS, mm, no, XMIN, dX, YMIN, dY, nx, ny, asc, hsc, cm)
    out.update(cos_data=c2, sin_data=s2)
    mc = e.make_coefficients_multi(Data(x, y, z, m), 3, potC, potS, mm, no, XMIN, dX, YMIN, dY,
                                   nx, ny, asc, hsc, cm)
    out.update(cos_multi=mc[0], sin_multi=mc[1])
    kw = dict(rmin=XMIN, dR=dX, zmin=YMIN, dZ=dY, numx=nx, numy=ny, MMAX=mm, NMAX=no,
              ASCALE=asc, HSCALE=hsc, CMAP=cm, verbose=0)
    out["aep"] = np.array(e.accumulated_eval_particles(Data(x, y, z, m), a_cos, a_sin, potC, rforceC, zforceC,
                                                       potS, rforceS, zforceS, m1=0, m2=1000, **kw))
    out["aep_m12"] = np.array(e.accumulated_eval_particles(Data(x, y, z, m), a_cos, a_sin, potC, rforceC,
                                                           zforceC, potS, rforceS, zforceS, m1=1, m2=2, **kw))
    if dens:
        # the density branch is reachable only through eof_file (eof.py:1027-1035)
        out["aep_dens"] = np.array(e.accumulated_eval_particles(Data(x, y, z, m), a_cos, a_sin, density=True,
                                                                verbose=0, eof_file=path))
    rng = np.random.default_rng(seed + 7)
    npt = 20
    pR = np.concatenate([rng.uniform(0.01, 12, npt - 4), [1e-5, 40.0, 2.0, 0.5]])
    pz = np.concatenate([rng.normal(0, 0.3, npt - 4), [0.0, 0.1, 30.0, -30.0]])
    pp = rng.uniform(-np.pi, np.pi, npt)
    out.update(pt_R=pR, pt_z=pz, pt_phi=pp)
    fk = dict(rmin=XMIN, dR=dX, zmin=YMIN, dZ=dY, numx=nx, numy=ny, ASCALE=asc, HSCALE=hsc, CMAP=cm)
    for tg, (MM, NN, NO, PT) in {"force_eval": (mm, no, False, False), "force_eval_noodd": (mm, no, True, False),
                                  "force_eval_m2n2": (min(2, mm), 2, False, False),
                                  "force_eval_perturb": (mm, no, False, True)}.items():
        res = []
        for i in range(npt):
            res.append(e.force_eval(pR[i], pz[i], pp[i], a_cos, a_sin, potC, rforceC, zforceC,
                                    potS, rforceS, zforceS, MMAX=MM, NMAX=NN, no_odd=NO, perturb=PT, **fk))
        out[tg] = np.array(res)
    for tg, NO in {"acc_eval": False, "acc_eval_noodd": True}.items():
        res = []
        for i in range(npt):
            res.append(e.accumulated_eval(pR[i], pz[i], pp[i], a_cos, a_sin, potC, rforceC, zforceC, densC,
                                          potS, rforceS, zforceS, densS, MMAX=mm, NMAX=no, no_odd=NO, **fk))
        out[tg] = np.array(res)
    out["bins"] = np.array(e.return_bins(pR, pz, **fk))
    np.savez_compressed(P(f"eof_{tag}.npz"), **out)
    print("eof", tag, "done")
    return path, a_cos, a_sin


def fields_case(ref, sph_cache, sph_model, expcoef, eof_path, a_cos, a_sin):
    refshim.set_log_bounds(ref, 1e-3, 100.0)
    F = ref.potential.Fields("none", eof_path, sph_cache, sph_model, verbose=0)
    F.EOF = ref.eof.EOF_Object()
    F.EOF.eof_file, F.EOF.cos, F.EOF.sin = eof_path, a_cos, a_sin
    F.SL = ref.spheresl.SL_Object()
    F.SL.sph_file, F.SL.model_file, F.SL.expcoef = sph_cache, sph_model, expcoef
    F.halofac = 0.8
    F.prep_tables()
    rng = np.random.default_rng(900)
    npt = 16
    px = rng.normal(0, 3, npt)
    py = rng.normal(0, 3, npt)
    pz = rng.normal(0, 0.5, npt)
    rot = rng.uniform(0, 2 * np.pi, npt)
    out = dict(px=px, py=py, pz=pz, rot=rot, halofac=0.8)
    res = [F.return_forces_cart(px[i], py[i], pz[i], rotpos=rot[i]) for i in range(npt)]
    out["forces_cart"] = np.array(res)
    F.set_field_parameters(no_odd=True, halo_l=2, halo_n=4, disk_m=2, disk_n=2)
    out["forces_cart_trunc"] = np.array([F.return_forces_cart(px[i], py[i], pz[i], rotpos=rot[i])
                                         for i in range(npt)])
    F.reset_field_parameters()
    orbits = [([1.0, 0.0, 0.05], [0.0, 0.55, 0.02], 0.0, False, 1000, False),
              ([0.3, -1.2, 0.0], [0.4, 0.1, 0.0], 0.2, True, 1000, False),
              ([2.5, 0.5, -0.1], [-0.1, -0.4, 0.05], -0.15, False, 1, True)]
    for k, (ip, iv, rf, force, apmax, apse) in enumerate(orbits):
        O = ref.integrate.leapfrog_integrate(F, 60, 0.02, ip, iv, rotfreq=rf, force=force,
                                             ap_max=apmax, apse=apse)
        for key, val in O.items():
            out[f"orbit{k}_{key}"] = np.asarray(val)
    O = ref.integrate.leapfrog_integrate(F, 40, 0.02, [0.8, 0.2, 0.0], [0.1, 0.6, 0.0], no_odd=True,
                                         halo_l=2, disk_m=2, disk_n=2)
    for key, val in O.items():
        out[f"orbit3_{key}"] = np.asarray(val)
    F.reset_field_parameters()
    out["timestep"] = np.array([ref.integrate.compute_timestep(F, [1.0, 0.2, 0.1], [0.1, 0.5, 0.0]),
                                ref.integrate.compute_timestep(F, [4.0, -1.0, 0.3], [0.2, 0.3, 0.05], dyn_res=50.)])
    np.savez_compressed(P("fields.npz"), **out)
    print("fields done")


def coef_files_case(ref, sl_ec, sl_ec2, eof_cos, eof_sin):
    """Coefficient and field files written by the reference's own writers,
    from fixed metadata (relative file names, so the bytes do not depend on
    where the repository lives)."""
    import hashlib
    import tempfile
    out = {}
    tmp = tempfile.mkdtemp()
    o = ref.spheresl.SL_Object()
    o.filename, o.comp, o.nbodies, o.sph_file, o.model_file = "OUT.run0.00010", "dark", 207, "sl_c2.cache", "sl_c2.model"
    o.lmax, o.nmax = 4, 6
    sl_path = os.path.join(tmp, "sl.coef")
    # spheresl.save_sl_coefficients fails under numpy 2 (it seeks with a
    # 1-element memmap, spheresl.py:1435); frame the file as it does and let
    # the reference's own sl_coefficients_to_file write each dump
    with open(sl_path, "wb") as f:
        np.array([2], dtype="i4").tofile(f)
        for t, ec in ((0.5, sl_ec), (1.25, sl_ec2)):
            o.time, o.expcoef = t, ec
            ref.spheresl.sl_coefficients_to_file(f, o)
    last, dumps = ref.spheresl.restore_sl_coefficients(sl_path)
    out["sl_restored_times"] = np.array(sorted(dumps.keys()))
    out["sl_bytes"] = np.frombuffer(open(sl_path, "rb").read(), dtype=np.uint8)
    e = ref.eof.EOF_Object()
    e.filename, e.comp, e.nbodies, e.eof_file, e.mmax, e.nmax = "OUT.run0.00010", "star", 3000, "eof_c1.cache", 3, 3
    eof_path = os.path.join(tmp, "eof.coef")
    for t, (c, s_) in ((0.5, (eof_cos, eof_sin)), (1.25, (2.0 * eof_cos, -eof_sin))):
        e.time, e.cos, e.sin = t, c, s_
        ref.eof.save_eof_coefficients(eof_path, e)
    out["eof_bytes"] = np.frombuffer(open(eof_path, "rb").read(), dtype=np.uint8)
    last, dumps = ref.eof.restore_eof_coefficients(eof_path)
    out["eof_restored_times"] = np.array(list(dumps.keys()))
    # a whole field, with cache file names relative to this directory
    cwd = os.getcwd()
    os.chdir(HERE)
    try:
        refshim.set_log_bounds(ref, 1e-3, 100.0)
        F = ref.potential.Fields("OUT.run0.00010", "eof_c1.cache", "sl_c2.cache", "sl_c2.model", verbose=0)
        F.EOF = ref.eof.EOF_Object()
        F.EOF.eof_file, F.EOF.cos, F.EOF.sin = "eof_c1.cache", eof_cos, eof_sin
        F.SL = ref.spheresl.SL_Object()
        F.SL.sph_file, F.SL.model_file, F.SL.expcoef = "sl_c2.cache", "sl_c2.model", sl_ec
        F.halofac = 0.75
        F.time = 2.5
        F.prep_tables()
        F.xcen_disk = F.ycen_disk = F.zcen_disk = 0.0
        F.xcen_halo = F.ycen_halo = F.zcen_halo = 0.0
        fpath = os.path.join(tmp, "field.bin")
        F.save_field(fpath)
        raw = open(fpath, "rb").read()
        out["field_sha256"] = np.frombuffer(hashlib.sha256(raw).digest(), dtype=np.uint8)
        out["field_size"] = np.array(len(raw))
        G = ref.potential.restore_field(fpath)
        px = np.array([0.7, -1.3, 2.2])
        py = np.array([0.4, 0.9, -0.6])
        pz = np.array([0.05, -0.2, 0.3])
        out["restored_forces_cart"] = np.array([G.return_forces_cart(px[i], py[i], pz[i]) for i in range(3)])
        rv = np.linspace(0.05, 3.0, 12)
        F.rotation_curve(rvals=rv)
        for k in ("disk_rotation", "halo_rotation", "total_rotation", "disk_dpdr", "halo_dpdr", "total_dpdr"):
            out["rc_" + k] = np.asarray(getattr(F, k))
        F.rotation_curve(rvals=rv, mono=True, angle=0.3)
        out["rc_mono_angle_total_rotation"] = np.asarray(F.total_rotation)
        F.resonance_positions(rvals=rv)
        out["rp_omega"], out["rp_kappa"] = np.asarray(F.omega), np.asarray(F.kappa)
    finally:
        os.chdir(cwd)
    np.savez_compressed(P("coef_files.npz"), **out)
    print("coefficient files done")


def orbit_grid_case(ref, sph_cache, sph_model, expcoef, eof_path, a_cos, a_sin):
    """Orbit grids of the reference integrator in the fields_case potential."""
    import io
    refshim.set_log_bounds(ref, 1e-3, 100.0)
    F = ref.potential.Fields("none", eof_path, sph_cache, sph_model, verbose=0)
    F.EOF = ref.eof.EOF_Object()
    F.EOF.eof_file, F.EOF.cos, F.EOF.sin = eof_path, a_cos, a_sin
    F.SL = ref.spheresl.SL_Object()
    F.SL.sph_file, F.SL.model_file, F.SL.expcoef = sph_cache, sph_model, expcoef
    F.halofac = 0.8
    F.prep_tables()
    out = {}
    rads, vels = np.array([0.6, 1.4]), np.array([0.45, 0.7])
    # dt = 1e-4 is below every compute_timestep step, so each orbit keeps its own
    g = ref.integrate.integrate_grid(rads, vels, F, 30, 1e-4, 0.15, False, -1, -1, 100., 1000, 0)
    out["grid"] = g
    F.reset_field_parameters()
    out["grid_launchy"] = ref.integrate.integrate_grid_launchy(rads, vels, F, 25, 0.01, -0.2, True, 2, 2, 50., 1000, 0)
    F.reset_field_parameters()
    out["grid_3d"] = ref.integrate.integrate_grid_3D(np.array([1.0]), np.array([0.5, 0.6]), F, 20, 1e-4, 0.0,
                                                     False, -1, -1, 100., 1000, np.array([0.05, -0.1]),
                                                     np.array([0.02]), 0)
    buf = io.StringIO()
    ref.integrate.print_orbit_array(buf, g)
    out["grid_text"] = np.array(buf.getvalue())
    buf = io.StringIO()
    ref.integrate.print_orbit_array_3D(buf, out["grid_3d"])
    out["grid_3d_text"] = np.array(buf.getvalue())
    np.savez_compressed(P("orbit_grids.npz"), **out)
    print("orbit grids done")


def centering_case(ref):
    """Fields.total_coefficients with centring, the snapshot reader replaced
    by in-memory particles and the two accumulators by recorders of the
    particles they receive (the coefficient paths are pinned elsewhere)."""
    rng = np.random.default_rng(41)
    dx, dy, dz, dm = disc_sample(12000, seed=42)
    dm = dm * rng.uniform(0.5, 1.5, dm.size)
    dx, dy, dz = dx + 0.03, dy - 0.02, dz + 0.01          # an off-centre disc
    hx, hy, hz, hm = hernquist_sample(15000, seed=43)
    hx = hx - 0.05
    comps = {"star": Data(dx, dy, dz, dm), "dark": Data(hx, hy, hz, hm)}
    comps["star"].time = 1.5

    class FakeInput:
        def __init__(self, filename, comp="star", verbose=0):
            src = comps[comp]
            self.data = {k: np.array(v) for k, v in src.data.items()}
            self.time = src.time

    seen = {}

    def rec_eof(P, eof_file, verbose=0, no_odd=False, **kw):
        seen["disk"] = np.stack([P.data["x"], P.data["y"], P.data["z"], P.data["m"]])
        return ref.eof.EOF_Object()

    def rec_sl(P, sph_file, mod_file, verbose=0, no_odd=False):
        seen["halo"] = np.stack([P.data["x"], P.data["y"], P.data["z"], P.data["m"]])
        return ref.spheresl.SL_Object()

    pot = ref.potential
    keep = (pot.particle.Input, pot.eof.compute_coefficients, pot.spheresl.compute_coefficients)
    out = {}
    try:
        pot.particle.Input = FakeInput
        pot.eof.compute_coefficients = rec_eof
        pot.spheresl.compute_coefficients = rec_sl
        for mutual in (False, True):
            F = pot.Fields("fake", "eof", "sph", "mod", centering=True, mutual_center=mutual, verbose=0)
            F.total_coefficients()
            tag = "mutual" if mutual else "separate"
            out[tag + "_centers"] = np.array([F.xcen_disk, F.ycen_disk, F.zcen_disk, F.xcen_halo, F.ycen_halo,
                                              F.zcen_halo, F.halofac, F.time])
            # checksums of the centred particles handed to the accumulators
            out[tag + "_disk_sums"] = np.array([seen["disk"].sum(axis=1), (seen["disk"] ** 2).sum(axis=1)])
            out[tag + "_halo_sums"] = np.array([seen["halo"].sum(axis=1), (seen["halo"] ** 2).sum(axis=1)])
            out[tag + "_disk_first"] = seen["disk"][:, :16]
            out[tag + "_halo_first"] = seen["halo"][:, :16]
    finally:
        pot.particle.Input, pot.eof.compute_coefficients, pot.spheresl.compute_coefficients = keep
    np.savez_compressed(P("centering.npz"), **out)
    print("centering done")


def snapshot_case():
    """PSP and SPL snapshots (single and double precision, with and without
    particle ids, with integer and float attributes, several components, an
    unaligned float attribute in 84-byte records) written with
    exptool_gb300.io.snapshot's writers and read by the reference's own
    psp_io / spl_io.  PyYAML is not installed, so the reference readers'
    yaml.safe_load is supplied by exptool_gb300.io.yaml_lite: these vectors pin
    the binary layout, not the YAML parsing."""
    import json
    import types
    from exptool_gb300.io import snapshot, yaml_lite
    shim = types.ModuleType("yaml")
    shim.safe_load = yaml_lite.load
    sys.modules["yaml"] = shim
    from exptool.io import psp_io, spl_io
    psp_io.yaml = spl_io.yaml = shim        # imported earlier against the stub module
    folder = P("snap")
    os.makedirs(folder, exist_ok=True)
    rng = np.random.default_rng(7)

    def comp(n, nint, nfloat, with_id):
        c = {k: rng.normal(size=n) for k in ["m", "x", "y", "z", "vx", "vy", "vz", "potE"]}
        c["m"] = np.abs(c["m"]) * 1e-3
        for i in range(nint):
            c[f"i_attr{i}"] = rng.integers(-1000, 1000, n)
        for i in range(nfloat):
            c[f"f_attr{i}"] = rng.normal(size=n)
        if with_id:
            c["id"] = rng.integers(0, 2**40, n)
        return c

    cases = {
        "OUT.f4idx": ("psp", 4, True, {"star": comp(300, 1, 2, True), "dark": comp(200, 0, 0, True)}),
        "OUT.f8": ("psp", 8, False, {"star": comp(250, 1, 1, False)}),
        "SPL.f4": ("spl", 4, False, {"star": comp(301, 0, 1, False), "gas": comp(77, 2, 0, False)}),
        "SPL.f8idx": ("spl", 8, True, {"star": comp(150, 1, 0, True)}),
    }
    out = {}
    for fname, (kind, fl, idx, comps) in cases.items():
        path = os.path.join(folder, fname)
        if kind == "psp":
            snapshot.write_psp(path, 1.25, comps, float_len=fl, indexing=idx)
        else:
            snapshot.write_spl(path, 2.5, comps, nsub=3, float_len=fl, indexing=idx)
        for cname in comps:
            I = (psp_io if kind == "psp" else spl_io).Input(path, comp=cname)
            for k, v in I.data.items():
                out[f"{fname}/{cname}/{k}"] = v
            out[f"{fname}/{cname}/time"] = np.float64(I.time)
        out[f"{fname}/header"] = np.array(json.dumps({k: {kk: (int(vv) if isinstance(vv, np.integer) else vv)
                                                           for kk, vv in h.items()}
                                                       for k, h in I.header.items()}, sort_keys=True))
    np.savez_compressed(P("snapshots.npz"), **out)


def outcoef_case(ref):
    """EXP coefficient time series in the four layouts (new YAML-headed and old
    SphereSL / Cylinder; the old files end in a partial record), written with
    exptool_gb300.io.outcoef's writers and read by the reference's
    io/outcoef.OutCoef and eof.read_binary_eof_coefficients(_dict) (yaml.load
    supplied by exptool_gb300.io.yaml_lite: PyYAML is not installed), and by
    spheresl.read_binary_sl_coefficients.  Under numpy 2 these readers stop at
    dtype codes numpy removed ('aN' strings, np.float); they run here with
    those two codes mapped to their replacements, their logic unchanged."""
    import types
    from exptool_gb300.io import outcoef, yaml_lite
    shim = types.ModuleType("yaml")
    shim.load = lambda s, Loader=None: yaml_lite.load(s)
    shim.safe_load = yaml_lite.load
    shim.FullLoader = None
    from exptool.io import outcoef as ref_oc
    ref_oc.yaml = shim

    class _Numpy2:
        """numpy for the reference's readers with the codes numpy 2 removed
        mapped to their replacements ('aN' -> 'SN' byte strings, np.float ->
        float); everything else is numpy itself."""
        float = float

        def __getattr__(self, k):
            return getattr(np, k)

        @staticmethod
        def fromfile(f, dtype=float, count=-1, **kw):
            if isinstance(dtype, str) and dtype.startswith("a"):
                dtype = "S" + dtype[1:]
            return np.fromfile(f, dtype=dtype, count=count, **kw)

    saved = (ref_oc.np, ref.spheresl.np)
    ref_oc.np = ref.spheresl.np = _Numpy2()
    folder = P("outcoef")
    os.makedirs(folder, exist_ok=True)
    rng = np.random.default_rng(21)
    T = np.array([0.0, 0.002, 1.0e-5, 0.75, 12.5])
    sl = rng.normal(size=(5, 7 * 7, 9))
    cy = rng.normal(size=(5, 2, 7, 11))
    cy[:, 1, 0] = 0.0
    files = {"sl_new": (outcoef.write_new_spheresl, sl), "sl_old": (outcoef.write_old_spheresl, sl),
             "cyl_new": (outcoef.write_new_cylinder, cy), "cyl_old": (outcoef.write_old_cylinder, cy)}
    out = {}
    for name, (w, c) in files.items():
        path = os.path.join(folder, name)
        w(path, T, c)
        if name.endswith("old"):
            with open(path, "ab") as f:
                f.write(b"\x01" * 37)          # a partial trailing record
        O = ref_oc.OutCoef(path)
        out[f"{name}/T"], out[f"{name}/coefs"] = O.T, O.coefs
        out[f"{name}/basis"] = np.array(O.basis)
        if name == "sl_new":
            O._repackage_spherical_coefficients()
            out["sl_new/C_2_1_sin_3"] = O.C[2][1]["sin"][3]
            out["sl_new/C_3_0_cos_4"] = O.C[3][0]["cos"][4]
        if name == "cyl_new":
            O._repackage_cylindrical_coefficients()
            out["cyl_new/C_4_sin_2"] = O.C[4]["sin"][2]
            d = O._repackage_cylindrical_coefficients_compatibility()
            out["cyl_new/dict_times"] = np.array(sorted(d))
            out["cyl_new/dict_cos_at_0.75"] = d[0.75].cos
    tr, cr = ref.eof.read_binary_eof_coefficients(os.path.join(folder, "cyl_old"))
    out["eof_read_binary/T"], out["eof_read_binary/coefs"] = tr, cr
    dct = ref.eof.read_binary_eof_coefficients_dict(os.path.join(folder, "cyl_old"))
    out["eof_read_binary_dict/times"] = np.array(sorted(dct))
    out["eof_read_binary_dict/sin_at_12.5"] = dct[12.5].sin
    ts, cs = ref.spheresl.read_binary_sl_coefficients(os.path.join(folder, "sl_old"))
    out["spheresl_read_binary/T"], out["spheresl_read_binary/coefs"] = ts, cs
    ref_oc.np, ref.spheresl.np = saved
    np.savez_compressed(P("outcoef.npz"), **out)


def frequencies_case(ref):
    """Orbit maps of 48 orbits x 2048 steps (freq_signals: three sinusoids of
    distinct amplitudes per coordinate, plus noise) through the reference's
    orbits/frequencies functions (each call given a fresh window list: the
    reference's default list is modified by its calls).  The maps are stored
    as their generating parameters."""
    import freq_signals
    from exptool.orbits import frequencies as fq
    prm = freq_signals.params()
    sig = freq_signals.build(prm)
    T = sig["T"]
    O = ref.orbit.Orbits()
    for k, v in sig.items():
        O[k] = v
    out = {f"param_{k}": np.asarray(v) for k, v in prm.items()}
    fq.find_fundamental_frequency_map(O, window=[0, 10000], order=4)
    for i in (1, 2, 3):
        out[f"map_OX{i}"] = O[f"OX{i}"]
    one = {"T": T, "X": O["X"][:, 5], "VX": O["VX"][:, 5]}
    one, freq, spec = fq.find_fundamental_frequency(one, window=[0, 10000], retall=True, order=3)
    for i in (1, 2, 3):
        out[f"one_OX{i}"] = np.float64(one[f"OX{i}"])
    out["one_freq"], out["one_spec"] = freq, spec
    out["org_omega"], out["org_power"] = fq.organize_frequencies(freq, spec, order=4)
    R = np.sqrt(O["X"][:, 7] ** 2 + O["Y"][:, 7] ** 2)
    phi = np.arctan2(O["Y"][:, 7], O["X"][:, 7])
    out["orbit_freqs"] = np.array(fq.find_orbit_frequencies(T, R, phi, O["Z"][:, 7], window=[0, 10000]))
    r, t, z = fq.find_orbit_map_frequencies(O, window=[0, 10000])
    out["map_OmegaR"], out["map_OmegaT"], out["map_OmegaZ"] = r, t, z
    np.savez_compressed(P("frequencies.npz"), **out)


def run_time_case(ref):
    """potential.Fields.total_coefficients() reading its snapshot file itself
    (components 'star' and 'dark' through the reference's particle.Input and
    psp_io; yaml.safe_load supplied by exptool_gb300.io.yaml_lite), with and
    without centring; potential.get_fields; and integrate.run_time_mod, whose
    orbit text file and saved field are recorded.  eof.compute_coefficients
    goes through refshim shim 5 (numpy 2)."""
    import hashlib
    import tempfile
    import types
    import run_time_input
    from exptool_gb300.io import coefficients, yaml_lite
    shim = types.ModuleType("yaml")
    shim.safe_load = yaml_lite.load
    sys.modules["yaml"] = shim
    from exptool.io import psp_io, spl_io
    psp_io.yaml = spl_io.yaml = shim
    keep = refshim.patch_eof_compute_coefficients(ref)
    refshim.set_log_bounds(ref, 1e-3, 100.0)
    eof_path, cache, model = P("eof_c1.cache"), P("sl_c2.cache"), P("sl_c2.model")
    out = {}
    try:
        with tempfile.TemporaryDirectory() as d:
            d = d + "/"
            infile = d + "OUT.run0.00003"
            run_time_input.write_snapshot(infile)
            out["snapshot_sha256"] = np.array(hashlib.sha256(open(infile, "rb").read()).hexdigest())
            for tag, centering, mutual in (("plain", False, False), ("separate", True, False)):
                F = ref.potential.Fields(infile, eof_path, cache, model, centering=centering,
                                         mutual_center=mutual, verbose=0)
                F.total_coefficients()
                out[tag + "_cos"], out[tag + "_sin"] = (np.array(F.EOF.cos, dtype=np.float64), np.array(F.EOF.sin, dtype=np.float64))
                out[tag + "_expcoef"] = np.array(F.SL.expcoef, dtype=np.float64)
                out[tag + "_meta"] = np.array([F.time, F.halofac, F.xcen_disk, F.ycen_disk, F.zcen_disk,
                                               F.xcen_halo, F.ycen_halo, F.zcen_halo], dtype=np.float64)
            F, patt, rotfreq = ref.potential.get_fields(d, "run0", 3, eof_path, cache, model, transform=False)
            out["get_fields_cos"], out["get_fields_sin"] = (np.array(F.EOF.cos, dtype=np.float64), np.array(F.EOF.sin, dtype=np.float64))
            out["get_fields_expcoef"] = np.array(F.SL.expcoef, dtype=np.float64)
            out["get_fields_meta"] = np.array([patt, rotfreq, F.time, F.halofac, F.xcen_disk, F.ycen_disk,
                                               F.zcen_disk, F.xcen_halo, F.ycen_halo, F.zcen_halo])
            g = run_time_input.GRID
            ref.integrate.run_time_mod(d, "run0", eof_path, cache, model, 3, g["rads"], g["vels"], g["nint"],
                                       g["dt"], False, -1, -1, 100., 1000, 0, nprocs=2, omegap=g["omegap"],
                                       orbitfile=d + "omap.txt", save_field=True, field_file_name=d + "field.dat")
            out["omap_text"] = np.array(open(d + "omap.txt").read())
            rec = coefficients.read_field_record(d + "field.dat")
            out["field_size"] = np.int64(os.path.getsize(d + "field.dat"))
            for k in ("cos", "sin", "expcoef", "eof_f", "sl_f", "eof_i", "sl_i", "flags", "time"):
                out["field_" + k] = np.asarray(rec[k])
            # file names only: the recorded paths are those of the machine that ran this
            out["field_files"] = np.array([os.path.basename(bytes(v).decode().rstrip("\x00")) for v in rec["files"]])
    finally:
        ref.eof.compute_coefficients = keep
    np.savez_compressed(P("run_time.npz"), **out)
    print("run_time done")


def main(only_snapshots=False, only_run_time=False, reference=None):
    """All fixtures, or (argument ``snapshots``) only the snapshot-reader,
    coefficient-file and orbit-frequency ones, or (``run_time``) only
    run_time.npz."""
    ref = refshim.load(reference)
    if only_run_time:
        run_time_case(ref)
        return
    snapshot_case()
    outcoef_case(ref)
    frequencies_case(ref)
    if only_snapshots:
        return
    sl_out = {}
    for cmap in (0, 1, 2):
        sl_out[cmap] = sl_case(ref, cmap)
    eof_path, a_cos, a_sin = eof_case(ref, "c1", 1, True, 3, 3, 12, 500)
    eof_case(ref, "c0", 0, False, 2, 3, 8, 600)
    cache, modelf, ec = sl_out[2]
    fields_case(ref, cache, modelf, ec, eof_path, a_cos, a_sin)
    ec2 = np.load(P("sl_c2.npz"))["expcoef_noodd"]
    coef_files_case(ref, ec, ec2, a_cos, a_sin)
    orbit_grid_case(ref, cache, modelf, ec, eof_path, a_cos, a_sin)
    centering_case(ref)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="exptool source tree root (default: $EXPTOOL_REFERENCE)")
    ap.add_argument("which", nargs="?", choices=["all", "snapshots", "run_time"], default="all")
    a = ap.parse_args()
    main(only_snapshots=a.which == "snapshots", only_run_time=a.which == "run_time", reference=a.reference)
