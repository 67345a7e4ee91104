"""Properties of the oracle that follow from the reference's math (CPU only)."""
import numpy as np
import pytest

import oracle
from _cases import oracle_maps, small_inputs


def test_zero_velocity_cells_copy_the_row():
    inp = small_inputs()
    om = {k: v.copy() for k, v in oracle_maps().items()}
    vis = om["limb"] > -998
    om["delta"][vis] = 0.0
    n_eff = 4096
    got = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, 40, inp.case.step)
    expect = np.zeros(inp.wave.size)
    for k in np.nonzero(vis)[0]:
        expect[:n_eff] = expect[:n_eff] + inp.q_norm[om["region"][k], :n_eff] * om["limb"][k]
    assert np.array_equal(got, expect)


def test_scatter_and_gather_differ_only_at_holes_collisions_and_edges():
    """The reference's scatter (SOAP_initialize.cu:142-165) and the interval-owning
    gather agree except where two sources hit one pixel, none does, or at the ends."""
    inp = small_inputs()
    om = oracle_maps()
    n_eff = 4096
    g = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, 40, inp.case.step)
    s = oracle.quiet_disk(inp.wave, inp.q_norm, n_eff, om, 40, inp.case.step, sem=oracle.SEM_SCATTER)
    interior = slice(64, n_eff - 64)
    diff = np.abs(g[interior] - s[interior]) / np.max(g)
    assert np.count_nonzero(diff) < 0.01 * diff.size
    assert np.max(diff) < 1e-4


def test_limb_darkening_is_linear():
    inp = small_inputs()
    c = inp.case

    def q(u1, u2):
        m = oracle.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, u1, u2, inp.mu_boundary, inp.lb)
        return oracle.quiet_disk(inp.wave, inp.q_norm, 4096, m, c.grid, c.step)

    q00, q10, q01 = q(0.0, 0.0), q(1.0, 0.0), q(0.0, 1.0)
    expect = q00 - 0.29 * (q00 - q10) - 0.34 * (q00 - q01)
    assert np.max(np.abs(q(0.29, 0.34) - expect)) <= 1e-12 * np.max(q00)


def test_invisible_region_gives_no_active_cell():
    c = small_inputs().case
    # a small spot on the far side at phase 0 (it faces the observer at phase 0.5)
    reg = np.array([[0.0, 180.0, 0.1, 0.0]])
    bd = oracle.region_bbox(0.1, 180.0, 0.0, c.incl, c.nrho, 0.0, c.grid)
    assert bd[4] == 0
    t, b = oracle.phase_maps(c.grid, c.nrho, c.incl, 0.0, reg, c.t_star, c.t_diff_spot, c.t_diff_fac)
    assert np.all(b == -9999.0) and np.all(t == -9999.0)
    t, b = oracle.phase_maps(c.grid, c.nrho, c.incl, 0.5, reg, c.t_star, c.t_diff_spot, c.t_diff_fac)
    assert np.sum(b == 0.0) > 0
    assert np.all(t[b == 0.0] == c.t_star - c.t_diff_spot)


def test_facula_temperature_is_truncated_polynomial():
    c = small_inputs().case
    reg = np.array([[10.0, 180.0, 0.3, 1.0]])
    m = oracle_maps()
    t, b = oracle.phase_maps(c.grid, c.nrho, c.incl, 0.5, reg, c.t_star, c.t_diff_spot, c.t_diff_fac)
    sel = b == 1.0
    assert np.any(sel)
    mu = m["mu"][sel]
    expect = (c.t_star + c.t_diff_fac + 0.9 - 407.7 * mu + 190.9 * mu * mu).astype(np.int64)
    assert np.array_equal(t[sel].astype(np.int64), expect)


def test_mirror_symmetric_spots_give_opposite_deficit_shift():
    """Two spots mirrored about the central meridian (incl 90, no differential
    rotation) produce flux deficits whose centroids shift in opposite directions."""
    inp = small_inputs()
    c = inp.case
    m = oracle.disk_maps(c.grid, c.period, 0.0, 90.0, c.radius_km, c.u1, c.u2, inp.mu_boundary, inp.lb)
    n_eff = 4096

    def deficit(lon):
        reg = np.array([[0.0, lon, 0.2, 0.0]])
        t, b = oracle.phase_maps(c.grid, c.nrho, 90.0, 0.5, reg, c.t_star, c.t_diff_spot, c.t_diff_fac)
        f, _, _ = oracle.phase_integrate(inp.wave, n_eff, c.grid, t, b, m, inp.q_norm, inp.q_norm,
                                         inp.q_norm, inp.q_norm, np.zeros(inp.wave.size), np.zeros(inp.wave.size),
                                         c.step)
        return f[:n_eff]

    fa, fb = deficit(150.0), deficit(210.0)
    # the cell grid is mirror symmetric up to its first column (y = -1 has no mirror)
    assert np.sum(fa) > 0 and abs(np.sum(fa) - np.sum(fb)) < 1e-3 * np.sum(fa)
    # to first order in v the deficits are f0 +- v f0': their departures from the
    # central-meridian deficit are anti-correlated
    f0 = deficit(180.0)
    sl = slice(300, n_eff - 300)
    da = fa[sl] / np.sum(fa[sl]) - f0[sl] / np.sum(f0[sl])
    db = fb[sl] / np.sum(fb[sl]) - f0[sl] / np.sum(f0[sl])
    assert np.corrcoef(da, db)[0, 1] < -0.5   # the discrete cell sets mirror only approximately


def test_gauss_fit_reaches_the_minpack_optimum():
    """The fit restates GSL's trust-region LM (GSL is not available here); pin its
    optimum against scipy's MINPACK Levenberg-Marquardt on the same model."""
    scipy_opt = pytest.importorskip("scipy.optimize")
    rng = np.random.default_rng(7)
    x = np.arange(-20000.0, 20001.0, 250.0)
    for _ in range(5):
        c, k, x0, fw = 1.1, -rng.uniform(0.05, 0.3), rng.uniform(-2000, 2000), rng.uniform(5000, 11000)
        sig = fw / (2 * np.sqrt(2 * np.log(2)))
        y = c + k * np.exp(-(x - x0) ** 2 / (2 * sig * sig)) + 2e-4 * rng.standard_normal(x.size)
        r = oracle.gauss_bis(x, y)
        assert r["iters"] >= 0
        xr = x - x[0]

        def res(p):
            s = p[3] / 2 / np.sqrt(2 * np.log(2))
            return p[0] + p[1] * np.exp(-(xr - p[2]) ** 2 / 2 / s / s) - y

        p0 = np.array([r["par"][0], -r["par"][1], r["par"][3] - x[0], r["par"][4]]) * (1 + 1e-4)
        sol = scipy_opt.least_squares(res, p0, method="lm", xtol=1e-15, ftol=1e-15, gtol=1e-15)
        v0_scipy = sol.x[2] + x[0]
        assert abs(v0_scipy - r["par"][3]) < 1e-4          # m/s: 0.01 cm/s
        assert abs(sol.x[3] - r["par"][4]) < 1e-4
        assert abs(abs(sol.x[1]) - r["par"][1]) < 1e-10
