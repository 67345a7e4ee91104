"""Code paths the benchmark workload does not reach:
* a fast rotator with large regions, whose tiles overflow the precomputed plans, so
  the integration kernel plans them itself (against the PLAIN64 form and the oracle);
* a grid beyond the box-list limit (760 x 760 cells), where the pipeline's collapsed
  forms build their phase lists from the G*G maps instead of the region boxes."""
import ctypes

import numpy as np
import pytest

import oracle
from soap_gpu_gb300 import synth
from soap_gpu_gb300._lib import Star

from _cases import activity, cubes, rel_err

pytestmark = pytest.mark.gpu


def _fast_rotator():
    case = synth.small_case(seed=3, grid=48, n=8300, n_phase=2, n_mu=6)
    case.vsini = 250.0   # Doppler slope 8.3e-4: shifts of up to ~830 px on this grid
    case.regions = np.array([[15.0, 180.0, 0.5, 1.0], [10.0, 170.0, 0.3, 0.0]])
    return case


def test_plan_overflow_tiles_match_plain64(ctx):
    case = _fast_rotator()
    inp = synth.generate(case)
    maps = oracle.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                            inp.mu_boundary, inp.lb)
    act = activity(case)
    regions = [case.regions for _ in case.phases]
    temp, bi = ctx.phase_maps(case.grid, case.incl, case.phases, regions, act)
    assert np.sum((bi >= -0.5) & (bi <= 1.5)) > 200
    n_eff = 8192
    ref = ctx.phase_integrate("plain64", inp.wave, n_eff, case.grid, temp, bi, maps, cubes(inp), case.step, act)
    for form, tol in (("fast64", 2e-10), ("fast32", 1e-6)):
        got = ctx.phase_integrate(form, inp.wave, n_eff, case.grid, temp, bi, maps, cubes(inp), case.step, act)
        for r, g in zip(ref, got):
            for p in range(case.n_phase):
                scale = max(np.max(np.abs(r[p])), 1e-300)
                assert rel_err(g[p], r[p], scale) <= tol, form
    # and the PLAIN64 form against the oracle, on one phase
    rf, rb, rt = oracle.phase_integrate(inp.wave, n_eff, case.grid, temp[0], bi[0], maps, inp.q_norm, inp.q_sed,
                                        inp.spot_norm, inp.fac_norm, inp.spot_sed[0], inp.fac_sed[0], case.step)
    assert rel_err(ref[0][0], rf) <= 1e-12 and rel_err(ref[2][0], rt) <= 1e-12


def test_pipeline_beyond_box_list_grid(ctx):
    case = synth.small_case(seed=5, grid=760, n=4200, n_phase=2, n_mu=6)
    inp = synth.generate(case)
    n_eff = (case.n // 512) * 512
    maps = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                         inp.mu_boundary, inp.lb)
    cb = cubes(inp)
    cb["spot_sed"] = inp.spot_sed[0]
    cb["fac_sed"] = inp.fac_sed[0]
    act = activity(case)
    regions = [case.regions for _ in case.phases]
    star = Star(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                (ctypes.c_double * 4)(*inp.lb))
    q_norm = ctx.quiet_disk("fast32", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    q_sed = ctx.quiet_disk("fast32", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    low, raw = ctx.phase_pipeline("fast32", inp.wave, n_eff, star, maps, cb, case.step, act, case.phases, regions,
                                  q_sed, q_norm, case.sigma_v, conv_step=case.step, want_raw=True)
    temp, bi = ctx.phase_maps(case.grid, case.incl, case.phases, regions, act)
    assert np.sum((bi >= -0.5) & (bi <= 1.5)) > 0
    flux, bconv, tot = ctx.phase_integrate("fast32", inp.wave, n_eff, case.grid, temp, bi, maps, cb, case.step, act)
    for k, spec in enumerate((tot, flux, bconv)):
        assert np.array_equal(raw[:, k], spec[:, :n_eff])
    assert np.all(np.isfinite(low))
