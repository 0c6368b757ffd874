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
