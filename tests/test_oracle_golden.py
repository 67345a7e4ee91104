"""The oracle against golden vectors produced by the reference's own Python code
(tests/golden/make_golden.py: CCF_func.py, run_all_SOAP.py's LB_params,
mask_templates and CCF apodisation), plus the product's host-side mirrors of those
functions."""
import os

import numpy as np
import pytest

import oracle
from soap_gpu_gb300 import config

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def _dense_mask():
    M = np.zeros(tuple(GOLD["mask_shape"]))
    M[GOLD["mask_rows"], GOLD["mask_cols"]] = GOLD["mask_vals"]
    return M


def test_ccf_mask_matches_reference():
    wave = GOLD["ccf_wave"]
    M = oracle.ccf_mask(GOLD["ccf_vel"], GOLD["ccf_lines"], GOLD["ccf_weights"], wave, 0.005)
    ref = _dense_mask()
    assert M.shape == ref.shape
    assert np.array_equal(M != 0, ref != 0), "mask support differs"
    assert np.max(np.abs(M - ref)) <= 1e-12


def test_ccf_values_match_reference():
    M = _dense_mask()
    for s in range(GOLD["ccf_spectra"].shape[0]):
        got = oracle.ccf(M, GOLD["ccf_spectra"][s])
        ref = GOLD["ccf_raw"][s]
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_ccf_normalise_matches_reference():
    for s in range(GOLD["ccf_raw"].shape[0]):
        got = oracle.ccf_normalise(GOLD["ccf_raw"][s])
        assert np.max(np.abs(got - GOLD["ccf_norm"][s])) <= 1e-14


def test_lb_params_match_reference():
    for tab, t, ref in zip(GOLD["lb_tables"], GOLD["lb_temps"], GOLD["lb_params"]):
        tarr = np.array([5778, 5240, 3750])
        a = oracle.lb_params(int(t), tab[0], tab[1], tab[2], tarr)
        b = config.lb_params(int(t), tab[0], tab[1], tab[2], tarr)
        assert np.allclose(a, ref, rtol=0, atol=1e-13)
        assert np.array_equal(a, b)


def test_mask_template_names():
    for t, name in zip((6100, 5770, 5300, 4350, 3000), GOLD["mask_names"]):
        assert config.mask_template_name(t) == str(name)


def test_mask_slice_mismatch_is_an_error():
    """At a 0.01 A grid the reference's literal 20000-pixel slice does not give the
    trimmed size (CCF_func.py:8-9 vs run_all_SOAP.py:292): the oracle refuses."""
    wave = 5000.0 + np.arange(2000) * 0.01
    with pytest.raises(ValueError):
        oracle.ccf_mask(np.array([0.0]), np.array([5005.0]), np.array([1.0]), wave, 0.01, index_old=20000)
    M = oracle.ccf_mask(np.array([0.0]), np.array([5005.0]), np.array([1.0]), wave, 0.01, mask_step=0.01,
                        index_old=10000)
    assert M.shape == (1, 2000) and M.sum() > 0
