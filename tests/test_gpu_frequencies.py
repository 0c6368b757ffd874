"""Orbit frequencies on the GPU (batched FFT, relative maxima, strongest
peaks) against the reference's orbits/frequencies on the same orbit maps
(tests/golden/frequencies.npz; maps rebuilt by tests/golden/freq_signals).
Frequencies are values of the FFT grid and must agree exactly; powers and
spectra to FFT rounding."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _case():
    from tests.golden import freq_signals
    g = np.load(os.path.join(GOLDEN, "frequencies.npz"))
    prm = {k[len("param_"):]: g[k] for k in g.files if k.startswith("param_")}
    return g, freq_signals.build(prm)


def test_fundamental_frequencies_match_reference():
    from exptool_gb300.orbits import frequencies as fq
    from exptool_gb300.orbits.orbit import Orbits
    g, sig = _case()
    O = Orbits()
    for k, v in sig.items():
        O[k] = v
    fq.find_fundamental_frequency_map(O, window=(0, 10000), order=4)
    for i in (1, 2, 3):
        assert np.array_equal(O[f"OX{i}"], g[f"map_OX{i}"]), i
    one = {"T": sig["T"], "X": sig["X"][:, 5], "VX": sig["VX"][:, 5]}
    one, freq, spec = fq.find_fundamental_frequency(one, window=(0, 10000), retall=True, order=3)
    for i in (1, 2, 3):
        assert one[f"OX{i}"] == float(g[f"one_OX{i}"]), i
    assert np.array_equal(freq, g["one_freq"])
    assert np.max(np.abs(spec - g["one_spec"])) <= 1e-12 * np.max(np.abs(g["one_spec"]))
    om, pw = fq.organize_frequencies(freq, g["one_spec"], order=4)
    assert np.array_equal(om, g["org_omega"])
    assert np.array_equal(pw, g["org_power"])


def test_orbit_frequencies_match_reference():
    from exptool_gb300.orbits import frequencies as fq
    from exptool_gb300.orbits.orbit import Orbits
    g, sig = _case()
    R = np.sqrt(sig["X"][:, 7] ** 2 + sig["Y"][:, 7] ** 2)
    phi = np.arctan2(sig["Y"][:, 7], sig["X"][:, 7])
    got = np.array(fq.find_orbit_frequencies(sig["T"], R, phi, sig["Z"][:, 7]))
    assert np.array_equal(got, g["orbit_freqs"])
    O = Orbits()
    for k, v in sig.items():
        O[k] = v
    r, t, z = fq.find_orbit_map_frequencies(O)
    assert np.array_equal(r, g["map_OmegaR"])
    assert np.array_equal(t, g["map_OmegaT"])
    assert np.array_equal(z, g["map_OmegaZ"])


def _np_fundamental(freq, spec, order):
    """The reference's selection (frequencies.py:94-132) on a numpy.fft
    spectrum: positive-frequency relative maxima of |Re spectrum| (edges
    clipped), strongest first."""
    amp = np.abs(spec.real)
    n = amp.size
    k = np.arange(n)
    mask = np.ones(n, dtype=bool)
    for j in range(1, order + 1):
        mask &= amp > amp[np.clip(k + j, 0, n - 1)]
        mask &= amp > amp[np.clip(k - j, 0, n - 1)]
    v = np.where(mask)[0]
    v = v[freq[v] > 0.0]
    return freq[v[np.argsort(-amp[v], kind="stable")]]


@pytest.mark.parametrize("hi", [1500, 1000, 2047, 17])
def test_non_power_of_two_windows(hi):
    """Windows whose length is not a power of two run Bluestein's transform:
    the spectrum equals numpy.fft.fft of the Hann-windowed x + i vx to 1e-12
    of its largest term, and the three fundamental frequencies (map and
    single orbit) and the R / phi / z peak frequencies equal the ones the
    reference's numpy selection gives on that spectrum."""
    from exptool_gb300.orbits import frequencies as fq
    from exptool_gb300.orbits.orbit import Orbits
    _g, sig = _case()
    T = sig["T"]
    freq = np.fft.fftfreq(hi, d=T[1] - T[0])
    one = {"T": T, "X": sig["X"][:, 3], "VX": sig["VX"][:, 3]}
    one, f1, spec = fq.find_fundamental_frequency(one, window=(0, hi), retall=True, order=3)
    ref = np.fft.fft(np.hanning(hi) * (sig["X"][:hi, 3] + 1j * sig["VX"][:hi, 3]))
    assert np.array_equal(f1, freq)
    assert np.max(np.abs(spec - ref)) <= 1e-12 * np.max(np.abs(ref))
    want = _np_fundamental(freq, ref, 3)
    got = [one[f"OX{i}"] for i in (1, 2, 3)]
    for i in range(3):
        if i < want.size:
            assert got[i] == want[i], (i, got, want[:3])
        else:
            assert np.isnan(got[i])
    O = Orbits()
    for k, v in sig.items():
        O[k] = v
    fq.find_fundamental_frequency_map(O, window=(0, hi), order=4)
    for b in range(sig["X"].shape[1]):
        w = _np_fundamental(freq, np.fft.fft(np.hanning(hi) * (sig["X"][:hi, b] + 1j * sig["VX"][:hi, b])), 4)
        for i in range(min(3, w.size)):
            assert O[f"OX{i + 1}"][b] == w[i], (b, i)
    R = np.sqrt(sig["X"][:hi] ** 2 + sig["Y"][:hi] ** 2)
    phi = np.arctan2(sig["Y"][:hi], sig["X"][:hi])
    got = np.array(fq.find_orbit_frequencies(T[:hi], R[:, 2], phi[:, 2], sig["Z"][:hi, 2]))
    fR = np.fft.fft(R[:, 2])
    fR[0] = 0.0
    want = [np.abs(freq[np.argmax(np.abs(fR))]), np.abs(freq[np.argmax(np.abs(np.fft.fft(phi[:, 2])))]),
            np.abs(freq[np.argmax(np.abs(np.fft.fft(sig["Z"][:hi, 2])))])]
    assert np.array_equal(got, want), (got, want)
