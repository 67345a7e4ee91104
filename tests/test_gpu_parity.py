"""GPU parity of every stage of the per-phase synthesis path against the oracle.

Tolerances: integer / index outputs (mu bins, visibility, region maps, CCF mask
entries) bit-exact; PLAIN64 spectra within 1e-12 relative to the spectrum's scale
(the reference's arithmetic, one rounding per operation);
FAST64 within 2e-10: the collapsed form re-associates the cell sum and takes the
interpolation weight from the analytic shifted position, while the reference forms
it as (l_j - l'_i) / (l'_{i+1} - l'_i) from ~5000 A values 0.005 A apart, which
carries ~1e-10 relative rounding per cell (the PLAIN64 form reproduces that
rounding bit for bit);
FAST32 within 2e-6 of scale (the precision form's flux budget is 1e-6 on the final
normalised spectra, checked at full size by bench.py's accuracy report).
"""
import numpy as np
import pytest

import oracle
from _cases import activity, cubes, oracle_maps, regions_per_phase, rel_err, small_inputs, star_args

pytestmark = pytest.mark.gpu


def test_disk_maps_exact(ctx):
    inp = small_inputs()
    om = oracle_maps()
    gm = ctx.disk_maps(**star_args(inp))
    assert np.array_equal(gm["region"], om["region"])
    for k in ("delta", "limb", "mu", "lb"):
        assert np.array_equal(gm[k], om[k]), k


@pytest.mark.parametrize("grid,n", [(40, 4200), (33, 4096), (17, 2100)])
def test_quiet_disk_plain64(ctx, grid, n):
    inp = small_inputs(grid=grid, n=n)
    om = oracle_maps(grid=grid, n=n)
    n_eff = (n // 512) * 512
    ref = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, grid, inp.case.step)
    got = ctx.quiet_disk("plain64", inp.wave, inp.q_norm, n_eff, om, grid, inp.case.step)
    assert np.all(got[n_eff:] == 0)
    assert rel_err(got, ref) <= 1e-13


@pytest.mark.parametrize("form,tol", [("fast64", 2e-10), ("fast32", 1e-6)])
@pytest.mark.parametrize("grid,n", [(40, 4200), (33, 4096), (17, 2100)])
def test_quiet_disk_fast(ctx, form, tol, grid, n):
    inp = small_inputs(grid=grid, n=n)
    om = oracle_maps(grid=grid, n=n)
    n_eff = (n // 512) * 512
    ref = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, grid, inp.case.step)
    got = ctx.quiet_disk(form, inp.wave, inp.q_norm, n_eff, om, grid, inp.case.step)
    assert np.all(got[n_eff:] == 0)
    assert rel_err(got, ref) <= tol


def test_quiet_disk_v0_column_copies(ctx):
    """Cells with v == 0 copy the cube row (SOAP_initialize.cu:149-152)."""
    inp = small_inputs()
    om = {k: v.copy() for k, v in oracle_maps().items()}
    vis = om["limb"] > -998
    om["delta"][vis] = 0.0
    n_eff = 4096
    got = ctx.quiet_disk("plain64", inp.wave, inp.q_norm, n_eff, om, 40, inp.case.step)
    expect = np.zeros(inp.wave.size)
    for k in np.nonzero(vis)[0]:
        expect[:n_eff] = expect[:n_eff] + inp.q_norm[om["region"][k], :n_eff] * om["limb"][k]
    assert rel_err(got, expect) <= 1e-13


@pytest.mark.parametrize("form,tol", [("plain64", 1e-12), ("fast64", 1e-11), ("fast32", 2e-6)])
def test_lower_resolution(ctx, form, tol):
    inp = small_inputs()
    om = oracle_maps()
    n_eff = 4096
    q = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, 40, inp.case.step)
    ref, conv, mm = oracle.lower_resolution(inp.wave, q, n_eff, inp.case.sigma_v, step_mult=0.005)
    got, gmm = ctx.lower_resolution(form, inp.wave, q, n_eff, inp.case.sigma_v, step_mult=0.005)
    assert rel_err(got, ref) <= tol
    assert gmm[0, 0] == mm[0]
    assert abs(gmm[0, 1] - mm[1]) <= tol * abs(mm[1])


@pytest.mark.parametrize("form,tol", [("plain64", 1e-12), ("fast64", 1e-11), ("fast32", 2e-6)])
def test_lower_resolution_with_base(ctx, form, tol):
    inp = small_inputs()
    n, n_eff = inp.wave.size, 4096
    rng = np.random.default_rng(3)
    base = np.zeros(n)
    base[:n_eff] = 1000.0 * inp.q_sed[0, :n_eff]
    spec = np.zeros((3, n))
    spec[:, :n_eff] = 50.0 * rng.uniform(0, 1, (3, n_eff)) * inp.q_norm[1, :n_eff]
    got, gmm = ctx.lower_resolution(form, inp.wave, spec, n_eff, inp.case.sigma_v, base=base)
    for s in range(3):
        ref, _, mm = oracle.lower_resolution(inp.wave, base - spec[s], n_eff, inp.case.sigma_v)
        assert rel_err(got[s], ref) <= tol
        if form == "fast32":   # the FP32 form rounds the spectra to FP32 before the exact FP64 minimum
            assert abs(gmm[s, 0] - mm[0]) <= 1e-7 * np.max(np.abs(spec[s]))
        else:
            assert gmm[s, 0] == mm[0]


def test_phase_maps_exact(ctx):
    inp = small_inputs()
    c = inp.case
    act = activity(c)
    temp, bi = ctx.phase_maps(c.grid, c.incl, c.phases, regions_per_phase(c), act)
    for p, ph in enumerate(c.phases):
        t_ref, b_ref = oracle.phase_maps(c.grid, c.nrho, c.incl, ph, c.regions, c.t_star, c.t_diff_spot,
                                         c.t_diff_fac)
        assert np.array_equal(temp[p], t_ref)
        assert np.array_equal(bi[p], b_ref)
    assert np.sum(bi >= 0) > 0, "no active cell in the test case"


def test_region_overwrite_order(ctx):
    """Later regions overwrite earlier ones (SOAP_integration.cu:724-785)."""
    inp = small_inputs()
    c = inp.case
    act = activity(c)
    r = c.regions
    t1, b1 = ctx.phase_maps(c.grid, c.incl, [0.5], [r], act)
    t2, b2 = ctx.phase_maps(c.grid, c.incl, [0.5], [r[::-1]], act)
    _, ba = ctx.phase_maps(c.grid, c.incl, [0.5], [r[:1]], act)
    _, bb = ctx.phase_maps(c.grid, c.incl, [0.5], [r[1:]], act)
    both = (ba[0] >= 0) & (bb[0] >= 0)
    assert np.any(both), "regions should overlap in the test case"
    assert np.all(b1[0][both] == r[-1, 3]) and np.all(b2[0][both] == r[0, 3])
    only_a = (ba[0] >= 0) & ~both
    assert np.all(b1[0][only_a] == r[0, 3]) and np.all(b2[0][only_a] == r[0, 3])


@pytest.mark.parametrize("solar", [False, True])
def test_phase_integrate_plain64(ctx, solar):
    inp = small_inputs()
    c = inp.case
    om = oracle_maps()
    act = activity(c, solar)
    temp, bi = ctx.phase_maps(c.grid, c.incl, c.phases, regions_per_phase(c), act)
    n_eff = 4096
    flux, bconv, tot = ctx.phase_integrate("plain64", inp.wave, n_eff, c.grid, temp, bi, om, cubes(inp), c.step,
                                           act)
    for p in range(c.n_phase):
        rf, rb, rt = oracle.phase_integrate(inp.wave, n_eff, c.grid, temp[p], bi[p], om, inp.q_norm, inp.q_sed,
                                            inp.spot_norm, inp.fac_norm, inp.spot_sed[0], inp.fac_sed[0], c.step,
                                            solar=solar, t_star=c.t_star, t_diff_fac=c.t_diff_fac)
        tol = 1e-12
        assert rel_err(flux[p], rf) <= tol
        assert rel_err(bconv[p], rb) <= tol
        assert rel_err(tot[p], rt) <= tol


@pytest.mark.parametrize("form,tol", [("fast64", 2e-10), ("fast32", 1e-6)])
@pytest.mark.parametrize("solar", [False, True])
def test_phase_integrate_fast(ctx, form, tol, solar):
    inp = small_inputs()
    c = inp.case
    om = oracle_maps()
    act = activity(c, solar)
    temp, bi = ctx.phase_maps(c.grid, c.incl, c.phases, regions_per_phase(c), act)
    n_eff = 4096
    ref = ctx.phase_integrate("plain64", inp.wave, n_eff, c.grid, temp, bi, om, cubes(inp), c.step, act)
    got = ctx.phase_integrate(form, inp.wave, n_eff, c.grid, temp, bi, om, cubes(inp), c.step, act)
    for r, g in zip(ref, got):
        for p in range(c.n_phase):
            scale = max(np.max(np.abs(r[p])), 1e-300)
            assert np.all(g[p, n_eff:] == 0)
            assert rel_err(g[p], r[p], scale) <= tol


def test_phase_without_active_cells_is_zero(ctx):
    """A phase with no visible active cell has zero deficit (RV = 0 downstream)."""
    inp = small_inputs()
    c = inp.case
    om = oracle_maps()
    act = activity(c)
    # a region on the far side at phase 0 (longitude 0 faces away with this convention)
    far = np.array([[0.0, 0.0, 0.1, 0.0]])
    temp, bi = ctx.phase_maps(c.grid, c.incl, [0.0, 0.5], [far, far], act)
    vis = [np.any(b >= 0) for b in bi]
    flux, bconv, tot = ctx.phase_integrate("plain64", inp.wave, 4096, c.grid, temp, bi, om, cubes(inp), c.step,
                                           act)
    for p in range(2):
        if not vis[p]:
            assert np.all(flux[p] == 0) and np.all(bconv[p] == 0) and np.all(tot[p] == 0)
    assert not all(vis), "expected one invisible phase"


def test_ccf_matches_oracle(ctx):
    inp = small_inputs()
    c = inp.case
    n_eff = 4096
    wave = inp.wave[:n_eff][200:-200][10:-10]
    rng = np.random.default_rng(5)
    spectra = 1.0 - 0.3 * rng.uniform(0, 1, (3, wave.size)) * inp.q_norm[0, 210:n_eff - 210][None, :]
    sel = (inp.mask_wave > wave.min()) & (inp.mask_wave < wave.max())
    lw, lwt = inp.mask_wave[sel], inp.mask_weight[sel] * rng.uniform(0.5, 1.0, sel.sum())
    vel = c.velocities
    index_old = int(100.0 / c.step)
    M = oracle.ccf_mask(vel, lw, lwt, wave, c.step, 100.0, 0.005, index_old)
    for form, tol in (("plain64", 1e-12), ("fast32", 1e-7)):
        raw = ctx.ccf(form, vel, lw, lwt, wave, c.step, spectra, normalise=False, index_old=index_old)
        nrm = ctx.ccf(form, vel, lw, lwt, wave, c.step, spectra, normalise=True, index_old=index_old)
        for s in range(3):
            ref = oracle.ccf(M, spectra[s])
            assert rel_err(raw[s], ref) <= tol
            assert rel_err(nrm[s], oracle.ccf_normalise(ref)) <= tol


def test_gauss_bis_matches_oracle(ctx):
    rng = np.random.default_rng(11)
    x = np.arange(-20000.0, 20001.0, 500.0)
    ys = []
    for _ in range(6):
        c, k, x0, fw = 1.05, -rng.uniform(0.05, 0.4), rng.uniform(-3000, 3000), rng.uniform(6000, 12000)
        sig = fw / (2 * np.sqrt(2 * np.log(2)))
        y = c + k * np.exp(-(x - x0) ** 2 / (2 * sig * sig)) + 1e-4 * np.sin(x / 777.0)
        ys.append(y)
    ys = np.array(ys)
    got = ctx.gauss_bis(x, ys)
    for s in range(len(ys)):
        ref = oracle.gauss_bis(x, ys[s])
        assert got["iters"][s] >= 0 and ref["iters"] >= 0
        assert abs(got["par"][s, 3] - ref["par"][3]) < 1e-4          # v0 [m/s]: 0.01 cm/s
        assert abs(got["par"][s, 4] - ref["par"][4]) < 1e-4          # fwhm [m/s]
        assert abs(got["par"][s, 2] - ref["par"][2]) < 1e-4          # span [m/s]
        assert np.max(np.abs(got["bis"][s] - ref["bis"])) < 1e-4
        assert rel_err(got["model"][s], ref["model"]) < 1e-9
