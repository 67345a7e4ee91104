"""The bisector-injection restatement against golden vectors made by the reference's
own BIS_inject_spectral_quiet / _active (tests/golden/make_golden_bis.py)."""
import os

import numpy as np
import pytest

import oracle

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_bis.npz"))


def test_quiet_injection_matches_reference():
    out = oracle.bisector_inject(GOLD["wave"], GOLD["flux"], 0, GOLD["q_coeffs"], scale=float(GOLD["scale"]))
    assert np.array_equal(out, GOLD["quiet"])


def test_active_injection_matches_reference():
    out = oracle.bisector_inject(GOLD["wave"], GOLD["flux"], 1, GOLD["up"], GOLD["low"], GOLD["dep_cut"],
                                 GOLD["vcut"], GOLD["vshift"], float(GOLD["scale"]))
    assert np.array_equal(out, GOLD["active"])
    # the fixture covers every branch, including the pixels on the branch points
    f = GOLD["flux"]
    assert np.any(f == 0.5) and np.any(f <= 0.5) and np.any(f > GOLD["dep_cut"].max())


def test_folded_grid_is_refused():
    wave = GOLD["wave"]
    with pytest.raises(ValueError):
        oracle.bisector_inject(wave, GOLD["flux"], 0, np.array([[3e7, 0.0, 0.0, 0.0]]), scale=1.0)
