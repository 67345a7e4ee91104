"""Small seeded workloads shared by the tests (sizes the oracle finishes in seconds)."""
from __future__ import annotations

import functools

import numpy as np

import oracle
from soap_gpu_gb300 import synth


@functools.lru_cache(maxsize=None)
def small_inputs(seed=7, grid=40, n=4200, n_phase=4, n_mu=6, distinct_sed=True):
    case = synth.small_case(seed=seed, grid=grid, n=n, n_phase=n_phase, n_mu=n_mu)
    inp = synth.generate(case)
    if distinct_sed:
        # make the SED / continuum cubes differ from the normalised ones so every
        # input of the integration is exercised
        rng = np.random.default_rng(seed + 100)
        slope = 1.0 + 0.2 * (inp.wave - inp.wave.mean()) / np.ptp(inp.wave)
        inp.q_sed = inp.q_norm * slope[None, :] * rng.uniform(0.9, 1.1, (case.n_mu, 1))
        inp.spot_sed = np.tile(0.3 + 0.05 * slope, (case.n_mu, 1))
        inp.fac_sed = np.tile(1.0 + 0.1 * slope, (case.n_mu, 1))
    return inp


def star_args(inp):
    c = inp.case
    return dict(grid=c.grid, period=c.period, omega_ratio=c.w_ratio, incl=c.incl, radius_km=c.radius_km,
                u1=c.u1, u2=c.u2, mu_boundary=inp.mu_boundary, lb=inp.lb)


@functools.lru_cache(maxsize=None)
def oracle_maps(seed=7, grid=40, n=4200, n_phase=4, n_mu=6):
    inp = small_inputs(seed, grid, n, n_phase, n_mu)
    c = inp.case
    return oracle.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, inp.mu_boundary,
                            inp.lb)


def regions_per_phase(case):
    return [case.regions for _ in range(case.n_phase)]


def activity(case, solar=False):
    from soap_gpu_gb300._lib import Activity
    return Activity(case.t_star, case.t_diff_spot, case.t_diff_fac, case.nrho, int(bool(solar)))


def cubes(inp):
    return dict(q_norm=inp.q_norm, q_sed=inp.q_sed, spot_norm=inp.spot_norm, fac_norm=inp.fac_norm,
                spot_sed=inp.spot_sed, fac_sed=inp.fac_sed)


def rel_err(a, b, scale=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.max(np.abs(b)) if scale is None else scale
    if s == 0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b)) / s)
