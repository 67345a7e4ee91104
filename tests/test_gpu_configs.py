"""Parity at the full sizes of the standard workloads, through the library's own calls.

* The 100x100-grid, 20,000-pixel star (one spot, 25 phases) in the plain FP64 form:
  disk maps, both quiet spectra, every phase's deficit spectra and normalised spectra
  against the oracle, and the RV / bisector-span / FWHM of every spectrum through
  soapgb_ccf + soapgb_gauss_bis against the oracle's CCF and fit.
* The 300x300-grid, 310,000-pixel star (facula + overlapping spot): the plain FP64
  pipeline against the oracle on three phases with a visible region (and the quiet
  disk on the whole grid), then the FP32 pipeline -- the call the benchmark times --
  against the plain FP64 pipeline on all 100 phases.
* The solar variant of the facula intensity (SOAP_integration_solar.cu:427,433) at
  the 310,000-pixel size.

Tolerances are the contract of the plain FP64 form and of the precision form: 1e-10
of the spectrum's scale on the interior pixels [210, N_eff - 210) for FP64 against the
oracle, 1e-6 relative flux error on the normalised spectra for FP32 against FP64, and
1 cm/s on RV, bisector span and FWHM.  The spectra are trimmed by 210 pixels before the
CCF (run_all_SOAP.py:259,266), so the edge pixels, where no source owns an output
pixel, never reach the RV.
"""
import numpy as np
import pytest

import oracle
from soap_gpu_gb300 import rv, synth

from _cases import activity, rel_err

pytestmark = pytest.mark.gpu

EDGE = 210
FP64_TOL = 1e-10
FLUX_TOL = 1e-6
CMS = 0.01          # 1 cm/s in m/s


def _interior(a):
    return a[..., EDGE:-EDGE]


def _star(case, lb):
    import ctypes
    from soap_gpu_gb300._lib import Star
    return Star(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                (ctypes.c_double * 4)(*lb))


def _cubes(inp):
    return dict(q_norm=inp.q_norm, q_sed=inp.q_sed, spot_norm=inp.spot_norm, fac_norm=inp.fac_norm,
                spot_sed=inp.spot_sed[0], fac_sed=inp.fac_sed[0])


def _oracle_fit(case, inp, spectra):
    """RV (v0), bisector span and FWHM of each spectrum by the oracle's CCF and fit."""
    n_eff = case.n_eff
    wt = rv.trim(inp.wave[:n_eff])
    lw, lwt = rv.select_lines(wt, inp.mask_wave, inp.mask_weight)
    M = oracle.ccf_mask(case.velocities, lw, lwt, wt, case.step, mask_step=case.step,
                        index_old=int(rv.WAVE_EXTEND / case.step))
    out = {"rv": [], "span": [], "fwhm": []}
    for s in spectra.reshape(-1, n_eff):
        f = oracle.gauss_bis(case.velocities, oracle.ccf_normalise(oracle.ccf(M, rv.trim(s))))
        out["rv"].append(f["par"][3])
        out["span"].append(f["par"][2])
        out["fwhm"].append(f["par"][4])
    return {k: np.array(v).reshape(spectra.shape[:-1]) for k, v in out.items()}


def _gpu_fit(ctx, case, inp, spectra, form="plain64"):
    r = rv.ccf_fit(ctx, case.step, case.velocities, inp.wave[:case.n_eff], spectra, inp.mask_wave,
                   inp.mask_weight, form=form)
    assert np.all(r["iters"] >= 0), "a Gaussian fit did not converge"
    return r


def _assert_fits_close(a, b, what):
    for k in ("rv", "span", "fwhm"):
        d = float(np.max(np.abs(np.asarray(a[k]) - np.asarray(b[k]))))
        assert d <= CMS, "%s: %s differs by %.3g m/s (bound 1 cm/s)" % (what, k, d)


# ---------------------------------------------------------------------------
# 100x100 grid, 20,000 px, one spot, 25 phases: plain FP64 against the oracle
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def small_star(ctx):
    case = synth.make_case(0)
    inp = synth.generate(case)
    n_eff = case.n_eff
    om = oracle.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                          inp.mu_boundary, inp.lb)
    maps = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                         inp.mu_boundary, inp.lb)
    q_norm = ctx.quiet_disk("plain64", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    q_sed = ctx.quiet_disk("plain64", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    oq_norm = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, case.grid, case.step)
    oq_sed = oracle.quiet_disk(inp.wave, inp.q_sed, n_eff, om, case.grid, case.step)
    act = activity(case)
    regions = [case.regions for _ in case.phases]
    low, raw = ctx.phase_pipeline("plain64", inp.wave, n_eff, _star(case, inp.lb), maps, _cubes(inp), case.step,
                                  act, case.phases, regions, q_sed, q_norm, case.sigma_v, conv_step=case.step,
                                  want_raw=True)
    o_raw = np.zeros((case.n_phase, 3, n_eff))
    o_low = np.zeros((case.n_phase, 3, n_eff))
    for p, ph in enumerate(case.phases):
        temp, bi = oracle.phase_maps(case.grid, case.nrho, case.incl, ph, case.regions, case.t_star,
                                     case.t_diff_spot, case.t_diff_fac)
        f, b, t = oracle.phase_integrate(inp.wave, n_eff, case.grid, temp, bi, om, inp.q_norm, inp.q_sed,
                                         inp.spot_norm, inp.fac_norm, inp.spot_sed[0], inp.fac_sed[0], case.step)
        for k, (spec, base) in enumerate(((t, oq_sed), (f, oq_sed), (b, oq_norm))):
            o_raw[p, k] = spec[:n_eff]
            o_low[p, k], _, _ = oracle.lower_resolution(inp.wave, base - spec, n_eff, case.sigma_v,
                                                        step_mult=case.step, step_exp=case.step)
    return dict(case=case, inp=inp, maps=maps, om=om, q=(q_sed, q_norm), oq=(oq_sed, oq_norm), low=low, raw=raw,
                o_low=o_low, o_raw=o_raw)


def test_small_star_maps_and_quiet_disk(small_star):
    s = small_star
    for k in ("delta", "limb", "mu", "lb"):
        assert np.array_equal(s["maps"][k], s["om"][k]), k
    assert np.array_equal(s["maps"]["region"], s["om"]["region"])
    for g, o in zip(s["q"], s["oq"]):
        assert rel_err(_interior(g[:s["case"].n_eff]), _interior(o[:s["case"].n_eff]), np.max(np.abs(o))) <= FP64_TOL


def test_small_star_all_phases_match_oracle(small_star):
    s = small_star
    assert np.count_nonzero(np.any(s["o_raw"] != 0, axis=(1, 2))) >= 5, "too few phases with a visible spot"
    for p in range(s["case"].n_phase):
        for k in range(3):
            scale = max(np.max(np.abs(s["o_raw"][p, k])), 1e-300)
            assert rel_err(_interior(s["raw"][p, k]), _interior(s["o_raw"][p, k]), scale) <= FP64_TOL, (p, k)
            assert rel_err(_interior(s["low"][p, k]), _interior(s["o_low"][p, k])) <= FP64_TOL, (p, k)


def test_small_star_rv_bis_fwhm_match_oracle_fit(ctx, small_star):
    s = small_star
    case, inp = s["case"], s["inp"]
    g = _gpu_fit(ctx, case, inp, s["low"])
    o = _oracle_fit(case, inp, s["o_low"])
    _assert_fits_close(g, o, "100x100 grid, 25 phases")
    # the series run_all_SOAP.py reports: RV relative to the quiet star (:351-362)
    q_low = np.stack([oracle.lower_resolution(inp.wave, s["oq"][i], case.n_eff, case.sigma_v,
                                              step_mult=case.step, step_exp=case.step)[0] for i in (0, 0, 1)])
    qo = _oracle_fit(case, inp, q_low)
    assert np.ptp((o["rv"] - qo["rv"][None, :])[:, 0]) > 0.1, "the spot leaves no RV signal"


# ---------------------------------------------------------------------------
# 300x300 grid, 310,000 px, facula + overlapping spot
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def big_star(ctx):
    case = synth.make_case(1)
    inp = synth.generate(case)
    n_eff = case.n_eff
    om = oracle.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                          inp.mu_boundary, inp.lb)
    maps = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                         inp.mu_boundary, inp.lb)
    q = {f: (ctx.quiet_disk(f, inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step),
             ctx.quiet_disk(f, inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step))
         for f in ("plain64", "fast32")}
    # three phases with a visible region, spread over the visible stretch of the rotation
    visible = []
    for ph in case.phases:
        _, bi = oracle.phase_maps(case.grid, case.nrho, case.incl, ph, case.regions, case.t_star, case.t_diff_spot,
                                  case.t_diff_fac)
        if np.any(bi >= 0):
            visible.append(ph)
    assert len(visible) >= 3
    pick = np.array([visible[len(visible) // 6], visible[len(visible) // 2], visible[(5 * len(visible)) // 6]])
    return dict(case=case, inp=inp, maps=maps, om=om, q=q, pick=pick, n_visible=len(visible))


def _oracle_phases(s, phases, solar=False):
    case, inp, om = s["case"], s["inp"], s["om"]
    n_eff = case.n_eff
    oq_sed, oq_norm = s["oq"]
    o_raw = np.zeros((len(phases), 3, n_eff))
    o_low = np.zeros((len(phases), 3, n_eff))
    for p, ph in enumerate(phases):
        temp, bi = oracle.phase_maps(case.grid, case.nrho, case.incl, ph, case.regions, case.t_star,
                                     case.t_diff_spot, case.t_diff_fac)
        f, b, t = oracle.phase_integrate(inp.wave, n_eff, case.grid, temp, bi, om, inp.q_norm, inp.q_sed,
                                         inp.spot_norm, inp.fac_norm, inp.spot_sed[0], inp.fac_sed[0], case.step,
                                         solar=solar, t_star=case.t_star, t_diff_fac=case.t_diff_fac)
        for k, (spec, base) in enumerate(((t, oq_sed), (f, oq_sed), (b, oq_norm))):
            o_raw[p, k] = spec[:n_eff]
            o_low[p, k], _, _ = oracle.lower_resolution(inp.wave, base - spec, n_eff, case.sigma_v,
                                                        step_mult=case.step, step_exp=case.step)
    return o_raw, o_low


@pytest.fixture(scope="module")
def big_oracle(big_star):
    s = big_star
    case, inp = s["case"], s["inp"]
    # the synthetic quiet cube with continuum equals the normalised one, so one oracle
    # disk sum over the whole 300x300 grid serves both quiet spectra
    assert np.array_equal(inp.q_sed, inp.q_norm)
    oq = oracle.quiet_disk(inp.wave, inp.q_norm, case.n_eff, s["om"], case.grid, case.step)
    s["oq"] = (oq, oq)
    return s


def _pipeline(ctx, s, form, phases, solar=False, want_raw=True):
    case, inp = s["case"], s["inp"]
    q_sed, q_norm = s["q"][form]
    return ctx.phase_pipeline(form, inp.wave, case.n_eff, _star(case, inp.lb), s["maps"], _cubes(inp), case.step,
                              activity(case, solar), phases, [case.regions for _ in phases], q_sed, q_norm,
                              case.sigma_v, conv_step=case.step, want_raw=want_raw)


def test_big_star_quiet_disk_matches_oracle(big_oracle):
    s = big_oracle
    n_eff = s["case"].n_eff
    for k in ("delta", "limb", "mu", "lb", "region"):
        assert np.array_equal(s["maps"][k], s["om"][k]), k
    for g in s["q"]["plain64"]:
        assert rel_err(_interior(g[:n_eff]), _interior(s["oq"][0][:n_eff])) <= FP64_TOL


@pytest.mark.parametrize("solar", [False, True])
def test_big_star_plain64_pipeline_matches_oracle(ctx, big_oracle, solar):
    s = big_oracle
    phases = s["pick"] if not solar else s["pick"][1:2]
    low, raw = _pipeline(ctx, s, "plain64", phases, solar)
    o_raw, o_low = _oracle_phases(s, phases, solar)
    for p in range(len(phases)):
        for k in range(3):
            scale = np.max(np.abs(o_raw[p, k]))
            assert scale > 0, "phase %g has no visible region" % phases[p]
            assert rel_err(_interior(raw[p, k]), _interior(o_raw[p, k]), scale) <= FP64_TOL, (p, k)
            assert rel_err(_interior(low[p, k]), _interior(o_low[p, k])) <= FP64_TOL, (p, k)
    if not solar:
        _assert_fits_close(_gpu_fit(ctx, s["case"], s["inp"], low), _oracle_fit(s["case"], s["inp"], o_low),
                           "300x300 grid, plain FP64 vs oracle")


@pytest.mark.parametrize("solar", [False, True])
def test_big_star_fp32_pipeline_within_budget(ctx, big_star, solar):
    """The benchmarked call (FP32 form, all 100 phases) against the plain FP64 form."""
    s = big_star
    case, inp = s["case"], s["inp"]
    low32 = _pipeline(ctx, s, "fast32", case.phases, solar, want_raw=False)
    low64 = _pipeline(ctx, s, "plain64", case.phases, solar, want_raw=False)
    scale = np.max(np.abs(low64), axis=2, keepdims=True)
    flux = float(np.max(np.abs(low32 - low64) / scale))
    assert flux <= FLUX_TOL, "normalised flux error %.3g" % flux
    g32 = _gpu_fit(ctx, case, inp, low32)
    g64 = _gpu_fit(ctx, case, inp, low64)
    _assert_fits_close(g32, g64, "300x300 grid, FP32 vs FP64")
    # and relative to the quiet star, as the RV series is reported
    ql = [ctx.lower_resolution(f, inp.wave, np.zeros_like(s["q"][f][0]), case.n_eff, case.sigma_v,
                               base=s["q"][f][0], step_mult=case.step, step_exp=case.step)[0] for f in ("fast32",
                                                                                                     "plain64")]
    q32 = _gpu_fit(ctx, case, inp, np.asarray(ql[0]).reshape(1, -1))
    q64 = _gpu_fit(ctx, case, inp, np.asarray(ql[1]).reshape(1, -1))
    d = np.max(np.abs((g32["rv"] - q32["rv"][0]) - (g64["rv"] - q64["rv"][0])))
    assert d <= CMS, "RV series differ by %.3g m/s" % d
    assert s["n_visible"] >= 30
