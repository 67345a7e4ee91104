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


def _write_real_layout(root, rc, phases, regions):
    """The files a 'real' run reuses (run_all_SOAP.py:148-157): the phase locator and
    one region table per phase, written by hand here (a phase may have none)."""
    for d in (rc.output_prefix, rc.maps_dir, rc.raw_dir, rc.final_spec_dir):
        os.makedirs(os.path.join(root, d), exist_ok=True)
    np.savetxt(os.path.join(root, rc.output_prefix + "/" + rc.file_prefix + "_phase_locator.txt"), phases)
    info = np.zeros((len(phases), 2))
    for i, reg in enumerate(regions):
        if len(reg):
            np.savetxt(os.path.join(root, rc.maps_dir + "maps%d_for_all.txt" % i), reg)
        info[i] = (i, len(reg))
    np.savetxt(os.path.join(root, rc.maps_dir + "final_info.txt"), info)


def test_keyword_real_reuses_external_maps(tmp_path):
    """keyword 'real': the driver takes the phases and the per-phase region tables from
    existing files instead of the configuration.  The same files run through the stage
    executables give the same spectra; the phase without a region has zero deficits."""
    from soap_gpu_gb300 import build
    case = synth.small_case(seed=13, grid=36, n=4200, n_phase=4, n_mu=5)
    phases = np.array([0.42, 0.47, 0.5, 0.55, 0.61])
    regions = [case.regions, case.regions[:1], np.zeros((0, 4)),
               np.array([[10.0, 200.0, 0.15, 0.0], [-25.0, 160.0, 0.22, 1.0], [15.0, 170.0, 0.1, 0.0]]),
               case.regions[::-1]]
    roots = []
    for tag in ("driver", "tools"):
        root = str(tmp_path / tag)
        inp = synth.generate(case)
        cfg = synth.write_reference_layout(inp, root, keyword="real")
        rc = config.load_config(cfg)
        assert rc.keyword == "real"
        _write_real_layout(root, rc, phases, regions)
        roots.append((root, cfg, rc))
    (r1, cfg1, rc1), (r2, cfg2, rc2) = roots
    out = driver.run(cfg1, form="plain64", verbose=False)
    assert out["tot"]["RV"].shape == (len(phases),)
    assert np.array_equal(out["tot"]["time"], phases)
    ref_run.run_impl(rc2, r2, build.BINDIR, env=dict(os.environ, SOAPGB_FORM="plain64"), write=False)
    visible = 0
    for p in range(len(phases)):
        for name in ("tot", "flux", "bconv"):
            raw = os.path.join(rc1.raw_dir, rc1.file_prefix + "_Spec_%s_%d_.bin" % (name, p))
            a = np.fromfile(os.path.join(r1, raw))
            b = np.fromfile(os.path.join(r2, raw))
            if p == 2:
                assert not np.any(a) and not np.any(b), "a phase without regions has zero deficits"
            else:
                assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
                visible += bool(np.any(b))
            low = os.path.join(rc1.final_spec_dir, rc1.file_prefix + "_lower_spec_%s_%d_.bin" % (name, p))
            a = np.fromfile(os.path.join(r1, low))
            b = np.fromfile(os.path.join(r2, low))
            assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
    assert visible >= 3 * 3, "too few phases with a visible region in the test"
