"""Orbit frequencies with the interface of ``exptool/orbits/frequencies.py``,
computed for whole orbit maps at once on the GPU by one kernel of this library
(``xt_orbit_spectra``): one CTA per orbit takes the N-point DFT of its signal
in double-float arithmetic in shared memory (radix-4 Stockham FFT for N a
power of two, Bluestein's transform otherwise) and searches the spectrum for its peaks in
place, so only indices and powers leave the device.  The reference loops over
orbits with numpy.fft.

Conventions followed (frequencies.py):
* frequencies are numpy.fft.fftfreq(N, d = T[1] - T[0]) of the window;
* fundamental frequencies: the spectrum of pos + i vel (numpy.hanning window
  when hanning), relative maxima of |Re spectrum| that beat `order`
  neighbours on each side (edges clipped, as numpy.take with mode='clip'),
  positive frequencies only, sorted by that power (frequencies.py:94-132);
* radial / azimuthal / vertical frequencies: |frequency| of the largest
  |spectrum| of R, phi, z with the zero-frequency term of R (and, for maps,
  of z) removed (frequencies.py:135-217).
Where a spectrum has fewer than three qualifying maxima the missing
fundamental frequencies are NaN (the reference raises IndexError).  The
reference's mutable default ``window`` list is not modified here.  Signals are
limited to 4096 samples for a power-of-two length and 2048 otherwise (the
transform of one signal lives in shared memory).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _lib
from .. import device as dev

_CHUNK_BYTES = 1 << 31          # device bytes of signal columns per chunk of orbits
_MAX_M = 4096
_TABLES = {}


def _window(n, lo, hi):
    return lo, (n if hi > n else hi)


def _chunks(norb, nt, arrays=1):
    per = max(1, int(_CHUNK_BYTES // (8 * arrays * max(nt, 1))))
    for a in range(0, norb, per):
        yield a, min(norb, a + per)


def _split(z):
    """Complex FP64 values -> (k, 4) float32 (re hi, re lo, im hi, im lo)."""
    z = np.asarray(z, dtype=np.complex128)
    rh = z.real.astype(np.float32)
    ih = z.imag.astype(np.float32)
    out = np.empty((z.size, 4), dtype=np.float32)
    out[:, 0] = rh
    out[:, 1] = (z.real - rh.astype(np.float64)).astype(np.float32)
    out[:, 2] = ih
    out[:, 3] = (z.imag - ih.astype(np.float64)).astype(np.float32)
    return out


def _tables(n):
    """(m, twiddles, chirp, chirp transform) device tables for signals of n
    samples, cached per n.  Chirp angles are reduced exactly in integers
    before the FP64 exponentials."""
    if n in _TABLES:
        return _TABLES[n]
    if n < 2:
        raise ValueError(f"orbit signals need at least 2 samples, got {n}")
    pow2 = n & (n - 1) == 0
    m = n if pow2 else 1 << int(np.ceil(np.log2(2 * n - 1)))
    if m > _MAX_M:
        raise ValueError(f"orbit signals of {n} samples exceed the transform limit ({_MAX_M} for powers of two, "
                         f"{_MAX_M // 2} otherwise)")
    t = np.arange(m // 2, dtype=np.int64)
    tw = np.exp(-2j * np.pi * (t / m))
    chirp = chirp_f = None
    if not pow2:
        j = np.arange(n, dtype=np.int64)
        w = np.exp(-1j * np.pi * ((j * j) % (2 * n)) / n)          # exp(-i pi j^2 / n)
        b = np.zeros(m, dtype=np.complex128)
        b[:n] = np.conj(w)
        b[m - n + 1:] = np.conj(w[1:])[::-1]
        chirp = dev.to_dev(_split(w), dtype=torch.float32)
        chirp_f = dev.to_dev(_split(np.fft.fft(b)), dtype=torch.float32)
    out = (m, dev.to_dev(_split(tw), dtype=torch.float32), chirp, chirp_f)
    _TABLES[n] = out
    return out


def spectra_device(mode, re, im, win=None, order=4, zero_first=False, freq_sign=1, want_spec=False):
    """One xt_orbit_spectra launch over device signals: re, im (None for a
    real signal) are (N, B) float64 CUDA tensors, column b one orbit's
    samples; win a device window of N values or None.  mode 0 returns the
    three strongest relative maxima of |Re X| at frequencies of sign
    freq_sign beating `order` neighbours on each side, mode 1 the index of
    the largest |X| (the zero-frequency term dropped when zero_first).
    Returns device (idx (B, 3) int32, value (B, 3) float64, spectra (B, N, 2)
    float64 or None); unused slots hold index -1."""
    lib = _lib.load()
    N, B = re.shape
    m, tw, chirp, chirp_f = _tables(N)
    io = torch.empty((B, 3), dtype=torch.int32, device=re.device)
    vo = torch.empty((B, 3), dtype=torch.float64, device=re.device)
    so = torch.empty((B, N, 2), dtype=torch.float64, device=re.device) if want_spec else None
    _lib.check(lib.xt_orbit_spectra(int(mode), B, N, dev.dptr(re), dev.dptr(im), B, dev.dptr(win), int(order),
                                    int(bool(zero_first)), int(freq_sign), m, dev.dptr(tw), dev.dptr(chirp),
                                    dev.dptr(chirp_f), dev.dptr(io), dev.dptr(vo), dev.dptr(so),
                                    dev.stream_ptr()), "xt_orbit_spectra")
    return io, vo, so


def _spectra(mode, re, im, win, order, zero_first, freq_sign, want_spec=False):
    """spectra_device over (N, B) host arrays in chunks of orbits that bound
    the device memory.  Returns host (idx (B, 3), val (B, 3), spectra (B, N)
    complex or None)."""
    N, B = re.shape
    idx = np.empty((B, 3), dtype=np.int32)
    val = np.empty((B, 3))
    spec = np.empty((B, N), dtype=np.complex128) if want_spec else None
    w = dev.to_dev(np.asarray(win, dtype=np.float64)) if win is not None else None
    for a, b in _chunks(B, N, 1 if im is None else 2):
        rd = dev.to_dev(np.ascontiguousarray(re[:, a:b]))
        idd = dev.to_dev(np.ascontiguousarray(im[:, a:b])) if im is not None else None
        io, vo, so = spectra_device(mode, rd, idd, w, order, zero_first, freq_sign, want_spec)
        idx[a:b] = dev.to_host(io)
        val[a:b] = dev.to_host(vo)
        if want_spec:
            sh = dev.to_host(so)
            spec[a:b] = sh[..., 0] + 1j * sh[..., 1]
    return idx, val, spec


def _fundamental(pos, vel, freq, hanning, order, nkeep=3, want_spec=False):
    """pos, vel: (N, B) float64 host arrays -> (omega (nkeep, B), power (nkeep, B)[, spectra (B, N)])."""
    N, B = pos.shape
    win = np.hanning(N) if hanning else None
    sign = 1 if (N < 2 or freq[1] > 0) else -1
    idx, val, spec = _spectra(0, pos, vel, win, order, False, sign, want_spec)
    ok = idx[:, :nkeep] >= 0
    om = np.where(ok, np.asarray(freq)[np.clip(idx[:, :nkeep], 0, None)], np.nan).T
    pw = np.where(ok, val[:, :nkeep], np.nan).T
    return (om, pw, spec) if want_spec else (om, pw)


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
    om, _pw, spec = _fundamental(P, V, freq, hanning, order, want_spec=True)
    for i in range(3):
        OrbitInstance["O" + pos + str(i + 1)] = om[i, 0]
    if retall:
        return OrbitInstance, freq, spec[0]
    return OrbitInstance


def organize_frequencies(freq, fftarr, order=4):
    """frequencies.py:94-132: (positive-frequency relative maxima of
    |Re fftarr|, their power), strongest first.  A host utility on a given
    spectrum, as in the reference."""
    amp = np.abs(np.asarray(fftarr).real)
    n = amp.size
    k = np.arange(n)
    mask = np.ones(n, dtype=bool)
    for j in range(1, int(order) + 1):
        mask &= amp > amp[np.clip(k + j, 0, n - 1)]
        mask &= amp > amp[np.clip(k - j, 0, n - 1)]
    vals = np.where(mask)[0]
    g = np.where(np.asarray(freq)[vals] > 0.0)[0]
    gomegas = np.asarray(freq)[vals[g]]
    gvals = amp[vals[g]]
    o = (-1.0 * gvals).argsort()
    return gomegas[o], gvals[o]


def _peak_freqs(cols, freq, zero_first):
    """|freq| of the largest |spectrum| of each column of each array; the
    zero-frequency term removed where zero_first[i]."""
    outs = []
    for i, c in enumerate(cols):
        idx, _val, _ = _spectra(1, c, None, None, 0, zero_first[i], 1)
        outs.append(np.abs(np.asarray(freq)[idx[:, 0]]))
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
