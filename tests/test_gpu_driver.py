"""The in-process driver (soap_gpu_gb300/driver.py) against the oracle: the same
files as the stage executables, and RV / BIS / FWHM series equal to the oracle's
CCF + Gaussian fit applied to the written spectra."""
import os

import numpy as np
import pytest

import oracle
from oracle import ref_run
from soap_gpu_gb300 import config, driver, rv, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driven(tmp_path_factory):
    root = str(tmp_path_factory.mktemp("driver"))
    case = synth.small_case(seed=11, grid=36, n=4200, n_phase=4, n_mu=5)
    inp = synth.generate(case)
    cfg = synth.write_reference_layout(inp, root)
    out = driver.run(cfg, form="plain64", verbose=False)
    return case, inp, config.load_config(cfg), root, out


def test_npz_outputs(driven):
    case, inp, rc, root, out = driven
    for name in ("tot", "flux", "bconv"):
        d = np.load(os.path.join(root, rc.output_prefix, rc.file_prefix + "_RV_%s_GPU.npz" % name))
        assert d["RV"].shape == (case.n_phase,)
        assert d["ccf"].shape == (case.n_phase + 1, len(case.velocities))
        assert d["bis"].shape == (case.n_phase + 1, 91)
        assert np.all(np.isfinite(d["RV"]))
    s = np.load(os.path.join(root, rc.output_prefix, rc.file_prefix + "_GPU_SOAP_RV_data.npz"))
    assert set(s.files) == {"time", "tot", "flux", "bconv"}


def test_rv_series_match_oracle_fit(driven):
    case, inp, rc, root, out = driven
    n_eff = case.n_eff
    wave = inp.wave[:n_eff]
    wt = rv.trim(wave)
    mask = np.loadtxt(os.path.join(root, rc.input_prefix + rc.mask_prefix + config.mask_template_name(rc.t_star)))
    lw, lwt = rv.select_lines(wt, mask[:, 0], mask[:, 1])
    M = oracle.ccf_mask(case.velocities, lw, lwt, wt, case.step)
    base = os.path.join(root, rc.output_prefix)
    for name, qname in (("tot", "_SED_quiet_sun_lower_spec.bin"), ("flux", "_SED_quiet_sun_lower_spec.bin"),
                        ("bconv", "_quiet_sun_lower_spec.bin")):
        v0 = []
        for p in range(case.n_phase + 1):
            if p < case.n_phase:
                spec = np.fromfile(os.path.join(base, "SOAP_resolution", rc.file_prefix +
                                                "_lower_spec_%s_%d_.bin" % (name, p)))
            else:
                spec = np.fromfile(os.path.join(base, rc.file_prefix + qname))
            c = oracle.ccf_normalise(oracle.ccf(M, rv.trim(spec)))
            v0.append(oracle.gauss_bis(case.velocities, c)["par"][3])
        v0 = np.array(v0)
        ref_rv = (v0 - v0[-1])[:-1]
        assert np.max(np.abs(out[name]["RV"] - ref_rv)) < 1e-4      # m/s: 0.01 cm/s


def test_spectra_match_the_stage_executables(driven, tmp_path):
    case, inp, rc, root, out = driven
    from soap_gpu_gb300 import build
    r2 = str(tmp_path / "tools")
    inp2, cfg2 = ref_run.prepare(synth.small_case(seed=11, grid=36, n=4200, n_phase=4, n_mu=5), r2)
    rc2 = config.load_config(cfg2)
    ref_run.run_impl(rc2, r2, build.BINDIR, env=dict(os.environ, SOAPGB_FORM="plain64"))
    for p in range(case.n_phase):
        for name in ("tot", "flux", "bconv"):
            rel = os.path.join("SOAP_resolution", rc.file_prefix + "_lower_spec_%s_%d_.bin" % (name, p))
            a = np.fromfile(os.path.join(root, rc.output_prefix, rel))
            b = np.fromfile(os.path.join(r2, rc2.output_prefix, rel))
            assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
