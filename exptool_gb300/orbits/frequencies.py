"""Orbit frequencies with the interface of ``exptool/orbits/frequencies.py``,
computed for whole orbit maps at once on the GPU: the spectra of all orbits
(columns) are one batched FFT (cuFFT through torch.fft), the relative maxima
and the strongest peaks of every spectrum are found with tensor operations,
in chunks of orbits that bound device memory.  The reference loops over
orbits with numpy.fft.

Conventions followed (frequencies.py):
* frequencies are numpy.fft.fftfreq(N, d = T[1] - T[0]) of the window;
* fundamental frequencies: the spectrum of pos + i vel (Hann window
  0.5 - 0.5 cos(2 pi n / (N - 1)) when hanning), relative maxima of
  |Re spectrum| that beat `order` neighbours on each side (edges clipped, as
  numpy.take with mode='clip'), positive frequencies only, sorted by that
  power (frequencies.py:94-132);
* radial / azimuthal / vertical frequencies: |frequency| of the largest
  |spectrum| of R, phi, z with the zero-frequency term of R (and, for maps,
  of z) removed (frequencies.py:135-217).
Where a spectrum has fewer than three qualifying maxima the missing
fundamental frequencies are NaN (the reference raises IndexError).  The
reference's mutable default ``window`` list is not modified here.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import device as dev

_CHUNK_BYTES = 1 << 31          # complex spectra per chunk of orbits


def _window(n, lo, hi):
    return lo, (n if hi > n else hi)


def _chunks(norb, nt):
    per = max(1, int(_CHUNK_BYTES // (16 * max(nt, 1))))
    for a in range(0, norb, per):
        yield a, min(norb, a + per)


def _relmax(a, order):
    """Strict relative maxima along dim 0 against `order` neighbours each
    side, indices clipped at the ends."""
    n = a.shape[0]
    idx = torch.arange(n, device=a.device)
    mask = torch.ones_like(a, dtype=torch.bool)
    for k in range(1, int(order) + 1):
        mask &= a > a[(idx + k).clamp(max=n - 1)]
        mask &= a > a[(idx - k).clamp(min=0)]
    return mask


def _hann(n, device):
    if n == 1:
        return torch.ones(1, dtype=torch.float64, device=device)
    k = torch.arange(n, dtype=torch.float64, device=device)
    return 0.5 - 0.5 * torch.cos(2.0 * np.pi * k / (n - 1))


def _fundamental(pos, vel, freq, hanning, order, nkeep=3):
    """pos, vel: (N, B) float64 host arrays -> (omega (nkeep, B), power (nkeep, B))."""
    N, B = pos.shape
    fr = torch.as_tensor(freq, dtype=torch.float64, device=dev.device())
    om = np.full((nkeep, B), np.nan)
    pw = np.full((nkeep, B), np.nan)
    w = _hann(N, dev.device())[:, None] if hanning else None
    for a, b in _chunks(B, N):
        p = dev.to_dev(np.ascontiguousarray(pos[:, a:b]))
        v = dev.to_dev(np.ascontiguousarray(vel[:, a:b]))
        ft = torch.complex(p, v)
        if w is not None:
            ft = ft * w
        spec = torch.fft.fft(ft, dim=0)
        amp = spec.real.abs()
        mask = _relmax(amp, order) & (fr > 0)[:, None]
        vals = torch.where(mask, amp, torch.full_like(amp, -np.inf))
        k = min(nkeep, N)
        tv, ti = torch.topk(vals, k, dim=0)
        ok = torch.isfinite(tv)
        om[:k, a:b] = dev.to_host(torch.where(ok, fr[ti], torch.full_like(tv, np.nan)))
        pw[:k, a:b] = dev.to_host(torch.where(ok, tv, torch.full_like(tv, np.nan)))
    return om, pw


def find_fundamental_frequency_map(OrbitInstance, time="T", pos="X", vel="VX", hanning=True, window=(0, 10000),
                                   order=4):
    """frequencies.py:25-66: adds O<pos>1..3 arrays (one value per orbit)."""
    T = np.asarray(OrbitInstance[time])
    lo, hi = _window(T.shape[-1], window[0], window[1])
    freq = np.fft.fftfreq(T[lo:hi].shape[-1], d=(T[1] - T[0]))
    P = np.asarray(OrbitInstance[pos], dtype=np.float64)[lo:hi]
    V = np.asarray(OrbitInstance[vel], dtype=np.float64)[lo:hi]
    om, _pw = _fundamental(P, V, freq, hanning, order)
    for i in range(3):
        OrbitInstance["O" + pos + str(i + 1)] = om[i]
    return OrbitInstance


def find_fundamental_frequency(OrbitInstance, time="T", pos="X", vel="VX", hanning=True, window=(0, 10000),
                               retall=False, order=3):
    """frequencies.py:69-91 for one orbit: adds scalar O<pos>1..3."""
    T = np.asarray(OrbitInstance[time])
    lo, hi = _window(T.shape[-1], window[0], window[1])
    freq = np.fft.fftfreq(T[lo:hi].shape[-1], d=(T[1] - T[0]))
    P = np.asarray(OrbitInstance[pos], dtype=np.float64)[lo:hi][:, None]
    V = np.asarray(OrbitInstance[vel], dtype=np.float64)[lo:hi][:, None]
    om, _pw = _fundamental(P, V, freq, hanning, order)
    for i in range(3):
        OrbitInstance["O" + pos + str(i + 1)] = om[i, 0]
    if retall:
        ft = torch.complex(dev.to_dev(P[:, 0]), dev.to_dev(V[:, 0]))
        if hanning:
            ft = ft * _hann(ft.shape[0], dev.device())
        return OrbitInstance, freq, dev.to_host(torch.fft.fft(ft))
    return OrbitInstance


def organize_frequencies(freq, fftarr, order=4):
    """frequencies.py:94-132: (positive-frequency relative maxima of
    |Re fftarr|, their power), strongest first."""
    a = torch.as_tensor(np.abs(np.asarray(fftarr).real), dtype=torch.float64, device=dev.device())
    mask = dev.to_host(_relmax(a[:, None], order)[:, 0])
    vals = np.where(mask)[0]
    g = np.where(np.asarray(freq)[vals] > 0.0)[0]
    gomegas = np.asarray(freq)[vals[g]]
    gvals = np.abs(np.asarray(fftarr).real)[vals[g]]
    o = (-1.0 * gvals).argsort()
    return gomegas[o], gvals[o]


def _peak_freqs(cols, freq, zero_first):
    """|freq| of the largest |spectrum| of each column of each array; the
    zero-frequency term removed where zero_first[i]."""
    fr = torch.as_tensor(freq, dtype=torch.float64, device=dev.device())
    N, B = cols[0].shape
    outs = [np.empty(B) for _ in cols]
    for a, b in _chunks(B, N):
        for i, c in enumerate(cols):
            sp = torch.fft.fft(dev.to_dev(np.ascontiguousarray(c[:, a:b])).to(torch.complex128), dim=0)
            mag = sp.abs()
            if zero_first[i]:
                mag[0] = 0.0
            outs[i][a:b] = dev.to_host(fr[mag.argmax(dim=0)].abs())
    return outs


def find_orbit_frequencies(T, R, PHI, Z, window=(0, 10000)):
    """frequencies.py:135-168 for one orbit: (Omega_R, Omega_T, Omega_Z)."""
    lo, hi = window[0], (np.asarray(R).shape[0] if window[1] == 10000 else window[1])
    T = np.asarray(T)
    freq = np.fft.fftfreq(T[lo:hi].shape[-1], d=(T[1] - T[0]))
    cols = [np.asarray(a, dtype=np.float64)[lo:hi][:, None] for a in (R, PHI, Z)]
    r, t, z = _peak_freqs(cols, freq, (True, False, False))
    return r[0], t[0], z[0]


def find_orbit_map_frequencies(OrbitInstance, window=(0, 10000)):
    """frequencies.py:171-217 for all orbits of a map: (Omega_R, Omega_T,
    Omega_Z) arrays.  Polar coordinates are added when missing."""
    if "Rp" not in OrbitInstance:
        print("orbit.find_orbit_frequencies: must have polar_coordinates. calculating...")
        OrbitInstance.polar_coordinates()
    phi = np.asarray(OrbitInstance["Phi"])
    lo, hi = window[0], (phi.shape[0] - 1 if window[1] == 10000 else window[1])
    T = np.asarray(OrbitInstance["T"])
    freq = np.fft.fftfreq(T[lo:hi].shape[-1], d=(T[1] - T[0]))

    def cols2(a):
        a = np.asarray(a, dtype=np.float64)[lo:hi]
        return a if a.ndim == 2 else a[:, None]

    r, t, z = _peak_freqs([cols2(OrbitInstance["Rp"]), cols2(phi), cols2(OrbitInstance["Z"])], freq,
                          (True, False, True))
    if phi.ndim == 1:
        return r[0], t[0], z[0]
    return r, t, z
