"""Synthetic orbit maps for the orbit-frequency fixtures: three sinusoids of
distinct amplitudes per coordinate plus Gaussian noise, rebuilt from small
stored parameters by both the fixture script and the tests."""
import numpy as np


def params(seed=31, nt=2048, no=48, dt=0.01):
    rng = np.random.default_rng(seed)
    out = {"nt": nt, "no": no, "dt": dt, "noise_seed": seed + 1}
    for name, base in (("X", 6.0), ("Y", 6.0), ("Z", 11.0)):
        out[f"{name}_w"] = base * (1.0 + 0.5 * rng.random((3, no)))
        out[f"{name}_amp"] = np.array([1.0, 0.45, 0.2])[:, None] * (1.0 + 0.1 * rng.random((3, no)))
        out[f"{name}_ph"] = 2 * np.pi * rng.random((3, no))
    return out


def build(p):
    """{'T', 'X', 'VX', 'Y', 'VY', 'Z', 'VZ'} of shape (nt,) / (nt, no)."""
    nt, no = int(p["nt"]), int(p["no"])
    T = np.arange(nt) * float(p["dt"])
    rng = np.random.default_rng(int(p["noise_seed"]))
    out = {"T": T}
    for name in ("X", "Y", "Z"):
        w, amp, ph = p[f"{name}_w"], p[f"{name}_amp"], p[f"{name}_ph"]
        x = np.zeros((nt, no))
        v = np.zeros((nt, no))
        for k in range(3):
            x += amp[k] * np.cos(w[k] * T[:, None] + ph[k])
            v -= amp[k] * w[k] * np.sin(w[k] * T[:, None] + ph[k])
        out[name] = x + 1e-3 * rng.normal(size=x.shape)
        out["V" + name] = v
    out["Y"] = out["Y"] + 0.5
    return out
