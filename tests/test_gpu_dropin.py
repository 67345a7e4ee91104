"""The drop-in executables through run_all_SOAP.py's argv / file contract, on a small
synthetic case, against the oracle (run_all_SOAP.py:160-250 builds the same
command lines; oracle/ref_run.py restates that part of the driver)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from oracle import ref_run
from soap_gpu_gb300 import build, config, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def run_dir(tmp_path_factory):
    build.build()
    root = str(tmp_path_factory.mktemp("dropin"))
    case = synth.small_case(seed=9, grid=36, n=4200, n_phase=3, n_mu=5)
    inp, cfg_path = ref_run.prepare(case, root)
    rc = config.load_config(cfg_path)
    env = dict(os.environ, SOAPGB_FORM="plain64")
    ref_run.run_impl(rc, root, build.BINDIR, env=env)
    return case, inp, rc, root


def _f(root, rc, rel):
    return np.fromfile(os.path.join(root, rc.output_prefix, rel))


def test_maps_and_quiet_spectra(run_dir):
    case, inp, rc, root = run_dir
    om = oracle.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                          inp.mu_boundary, inp.lb)
    pre = rc.file_prefix
    assert np.array_equal(np.fromfile(os.path.join(root, rc.output_prefix, pre + "region_map.bin"), dtype=np.int32),
                          om["region"])
    for k, name in (("delta", "delta_map"), ("limb", "limb_map"), ("mu", "mu_map"), ("lb", "LB_map")):
        assert np.array_equal(_f(root, rc, pre + name + ".bin"), om[k]), name
    n_eff = case.n_eff
    q = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, case.grid, case.step)
    got = _f(root, rc, pre + "_quiet_sun_spec.bin")
    assert got.size == n_eff
    assert np.max(np.abs(got - q[:n_eff])) <= 1e-13 * np.max(q)
    low, _, _ = oracle.lower_resolution(inp.wave, q, n_eff, case.sigma_v, step_mult=case.step, step_exp=0.005)
    gl = _f(root, rc, pre + "_quiet_sun_lower_spec.bin")
    assert np.max(np.abs(gl - low)) <= 1e-11 * np.max(np.abs(low))
    assert np.array_equal(_f(root, rc, pre + "_quiet_sun_wave.bin"), inp.wave[:n_eff])


def test_phase_spectra_and_resolution(run_dir):
    case, inp, rc, root = run_dir
    om = oracle.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                          inp.mu_boundary, inp.lb)
    pre, n, n_eff = rc.file_prefix, case.n, case.n_eff
    q = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, case.grid, case.step)
    qs = oracle.quiet_disk(inp.wave, inp.q_sed, n_eff, om, case.grid, case.step)
    raw_dir = rc.raw_dir.split("/", 1)[1]
    spec_dir = rc.final_spec_dir.split("/", 1)[1]
    active = 0
    for p, ph in enumerate(rc.phases):
        t, b = oracle.phase_maps(case.grid, case.nrho, case.incl, ph, case.regions, case.t_star, case.t_diff_spot,
                                 case.t_diff_fac)
        active += int(np.sum(b >= 0))
        assert np.array_equal(_f(root, rc, raw_dir + pre + "_temp_map_%d_.bin" % p), t)
        assert np.array_equal(_f(root, rc, raw_dir + pre + "_spot_binary_map_%d_.bin" % p), b)
        fl, bc, tt = oracle.phase_integrate(inp.wave, n_eff, case.grid, t, b, om, inp.q_norm, inp.q_sed,
                                            inp.spot_norm, inp.fac_norm, inp.spot_sed[0], inp.fac_sed[0], case.step)
        for name, ref, base in (("tot", tt, qs), ("flux", fl, qs), ("bconv", bc, q)):
            got = _f(root, rc, raw_dir + pre + "_Spec_%s_%d_.bin" % (name, p))
            scale = max(np.max(np.abs(ref)), 1e-300)
            assert np.max(np.abs(got - ref[:n_eff])) <= 1e-12 * scale
            a = np.zeros(n)
            a[:n_eff] = base[:n_eff] - ref[:n_eff]
            low, _, _ = oracle.lower_resolution(inp.wave, a, n_eff, case.sigma_v)
            gl = _f(root, rc, spec_dir + pre + "_lower_spec_%s_%d_.bin" % (name, p))
            assert np.max(np.abs(gl - low)) <= 1e-11 * np.max(np.abs(low))
    assert active > 0


def test_bis_fit2_files(tmp_path):
    build.build()
    x = np.arange(-20000.0, 20001.0, 500.0)
    sig = 3500.0
    y = 1.1 - 0.15 * np.exp(-(x - 420.0) ** 2 / (2 * sig * sig)) + 1e-4 * np.cos(x / 999.0)
    np.savetxt(tmp_path / "CCF_data.txt", np.array([x, y]).T)
    np.savetxt(tmp_path / "CCF_error.txt", np.ones(x.size).T)
    p = subprocess.run([os.path.join(build.BINDIR, "BIS_FIT2"), str(x.size)], cwd=tmp_path, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    assert p.returncode == 0, p.stdout
    xr = np.loadtxt(tmp_path / "CCF_data.txt")
    ref = oracle.gauss_bis(xr[:, 0], xr[:, 1])
    par = np.fromfile(tmp_path / "ccf_parameter.bin")
    assert par.size == 5 and abs(par[3] - ref["par"][3]) < 1e-4 and abs(par[4] - ref["par"][4]) < 1e-4
    assert np.fromfile(tmp_path / "ccf_model.bin").size == x.size
    assert np.max(np.abs(np.fromfile(tmp_path / "ccf_bis.bin") - ref["bis"])) < 1e-4
    assert np.max(np.abs(np.fromfile(tmp_path / "ccf_depth.bin") - ref["depth"])) < 1e-9
