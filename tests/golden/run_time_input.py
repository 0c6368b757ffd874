"""The PSP snapshot of the run_time fixtures, rebuilt from seeds by both the
fixture script and the tests (so no snapshot file is committed).  Only
correctly rounded IEEE operations (+ - * / sqrt) turn the PCG64 uniforms into
particles, so the file is bit-identical on every platform."""
import numpy as np

GRID = dict(rads=np.array([0.5, 1.0, 1.7]), vels=np.array([0.3, 0.55]), nint=40, dt=0.01, omegap=0.3)


def _circle(rng, n):
    """cos, sin of an angle through the rational parametrisation of the circle
    (t = tan of half the angle, uniform in [-1, 1], reflected to a full turn)."""
    t = rng.uniform(-1.0, 1.0, n)
    c = (1.0 - t * t) / (1.0 + t * t)
    s = 2.0 * t / (1.0 + t * t)
    flip = rng.uniform(0.0, 1.0, n) < 0.5
    return np.where(flip, -c, c), np.where(flip, -s, s)


def write_snapshot(path):
    """'star' = 3000 disc-like particles (R = u/(1-u) with u ~ U[0, 0.95),
    z = 0.1 (2v - 1)/(1 + |2v - 1|)) off centre by (0.02, -0.01, 0.005), masses
    1/3000 scattered by U[0.5, 1.5); 'dark' = 4000 halo particles
    (r = sqrt(u)/(1 - sqrt(u)), u ~ U[0, 0.9), isotropic by a uniform cos
    theta); velocities and potentials U[-1, 1); double precision, no ids,
    time 0.75; all from default_rng(61)."""
    from exptool_gb300.io import snapshot
    rng = np.random.default_rng(61)
    nd, nh = 3000, 4000
    u = rng.uniform(0.0, 0.95, nd)
    R = u / (1.0 - u)
    v = 2.0 * rng.uniform(0.0, 1.0, nd) - 1.0
    zd = 0.1 * v / (1.0 + np.abs(v))
    c, s = _circle(rng, nd)
    dm = (1.0 / nd) * rng.uniform(0.5, 1.5, nd)
    su = np.sqrt(rng.uniform(0.0, 0.9, nh))
    r = su / (1.0 - su)
    ct = rng.uniform(-1.0, 1.0, nh)
    st = np.sqrt((1.0 - ct) * (1.0 + ct))
    ch, sh = _circle(rng, nh)
    hm = np.full(nh, 1.0 / nh)

    def comp(x, y, z, m):
        n = x.size
        return {"m": m, "x": x, "y": y, "z": z, "vx": rng.uniform(-1.0, 1.0, n), "vy": rng.uniform(-1.0, 1.0, n),
                "vz": rng.uniform(-1.0, 1.0, n), "potE": rng.uniform(-1.0, 1.0, n)}

    comps = {"star": comp(R * c + 0.02, R * s - 0.01, zd + 0.005, dm),
             "dark": comp(r * st * ch, r * st * sh, r * ct, hm)}
    snapshot.write_psp(path, 0.75, comps, float_len=8, indexing=False)
