"""Seeded synthetic inputs in the reference's file formats.

The seed cubes and the wavelength grid the reference reads (``input_spec/*.bin``)
come from PHOENIX downloads and an observed solar atlas that are not available
offline, so every workload here is synthetic.  ``make_case(k)`` gives the five
standard workloads:

* 0 -- 100x100 grid, 20,000 px on 5000-5100 A at 0.005 A, 150 lines, 10 mu bins,
       one spot (lat 20, 1 % of the hemisphere), 25 phases, 60-line binary mask,
       81 CCF velocities (-20..20 km/s at 0.5 km/s).
* 1 -- 300x300 grid, 310,000 px on 3800-6900 A at 0.01 A, 6,000 lines, 20 mu bins,
       a facula (3 %) then an overlapping spot (1 %), 100 phases, 4,000-line mask,
       161 CCF velocities (-20..20 km/s at 0.25 km/s).
* 2 -- the star of 1 (computed in the FP32 compensated form by the caller).
* 3 -- many stars of uneven sizes sharing the 310k-px seeds (batched form,
       ``make_batch``).
* 4 -- 200x200 grid, 100,000 px, 3 regions, 50 phases (differentiable form).

Spectra: continuum 1 minus Gaussian lines with centres U(range), depths U(0.05, 0.9)
and sigma U(0.03, 0.08) A, clipped at 0.  Spot lines take depths x U(0.9, 1.2),
facula lines x U(0.95, 1.05).  Per mu bin a cubic bisector rv(flux) with
coefficients U(-300, 300) m/s is injected the way ``CB_injection_faculae.py:227-244``
(BIS_inject_spectral_quiet) does it: each pixel moves by the relativistic shift of
rv(flux) and the spectrum is re-interpolated onto the grid (0 outside the shifted
range).  Spots get the same cubic x 0.5, faculae x 0.7.  The continuum cubes are
constant: quiet 1.0, spot 0.35, facula 1.05.  All draws come from
``numpy.random.default_rng(seed)`` in a fixed order.
"""
from __future__ import annotations

import dataclasses
import os
from typing import List, Optional

import numpy as np

C_LIGHT = 299792458.0
R_SUN_KM = 696000


@dataclasses.dataclass
class Case:
    name: str
    grid: int
    n: int
    lambda0: float
    step: float
    n_lines: int
    n_mu: int
    regions: np.ndarray            # (n_reg, 4): lat, long, size, type -- applied in order
    n_phase: int
    rot_step: float
    n_mask_lines: int
    ccf_window: float              # m/s
    ccf_size: float                # m/s
    vsini: float = 2.0             # km/s
    incl: float = 90.0
    u1: float = 0.29
    u2: float = 0.34
    w_ratio: float = -0.18
    radius: float = 1.0            # solar radii
    t_star: int = 5778
    t_diff_spot: int = 663
    t_diff_fac: int = 250
    inst_reso: int = 115000
    nrho: int = 20
    spot_conti: float = 0.35
    fac_conti: float = 1.05
    seed: int = 0

    @property
    def n_eff(self) -> int:
        return (self.n // 512) * 512

    @property
    def radius_km(self) -> float:
        return self.radius * R_SUN_KM

    @property
    def period(self) -> float:
        """Rotation period [d] giving the requested vsini at the equator."""
        return 2 * np.pi * self.radius_km / (self.vsini * 86400.0)

    @property
    def sigma_v(self) -> float:
        """Instrument Gaussian sigma [m/s] (run_all_SOAP.py:63-65)."""
        fwhm = C_LIGHT / float(self.inst_reso)
        return fwhm / (2 * np.sqrt(2 * np.log(2)))

    @property
    def rot_num(self) -> float:
        return self.n_phase * self.rot_step

    @property
    def phases(self) -> np.ndarray:
        """run_all_SOAP.py:191"""
        return np.arange(0.0, self.rot_num, self.rot_step)

    @property
    def velocities(self) -> np.ndarray:
        """run_all_SOAP.py:262"""
        return np.arange(-1 * self.ccf_window, self.ccf_window + 1.0, self.ccf_size)


def make_case(k: int) -> Case:
    if k == 0:
        return Case("config0", grid=100, n=20000, lambda0=5000.0, step=0.005, n_lines=150, n_mu=10,
                    regions=np.array([[20.0, 180.0, 0.1, 0.0]]), n_phase=25, rot_step=0.04,
                    n_mask_lines=60, ccf_window=20000.0, ccf_size=500.0, seed=0)
    if k in (1, 2):
        return Case("config%d" % k, grid=300, n=310000, lambda0=3800.0, step=0.01, n_lines=6000, n_mu=20,
                    regions=np.array([[25.0, 185.0, 0.1732, 1.0], [20.0, 180.0, 0.1, 0.0]]),
                    n_phase=100, rot_step=0.01, n_mask_lines=4000, ccf_window=20000.0, ccf_size=250.0,
                    seed=1)
    if k == 4:
        return Case("config4", grid=200, n=100000, lambda0=5000.0, step=0.01, n_lines=2000, n_mu=10,
                    regions=np.array([[15.0, 170.0, 0.1, 0.0], [30.0, 200.0, 0.1414, 1.0],
                                      [-20.0, 150.0, 0.12, 0.0]]),
                    n_phase=50, rot_step=0.02, n_mask_lines=1000, ccf_window=20000.0, ccf_size=500.0,
                    seed=4)
    raise ValueError("unknown case %r" % k)


def small_case(seed: int = 7, grid: int = 40, n: int = 4096, n_phase: int = 4, n_mu: int = 6) -> Case:
    """A reduced case for parity tests that the oracle finishes in seconds."""
    return Case("small", grid=grid, n=n, lambda0=5000.0, step=0.005, n_lines=40, n_mu=n_mu,
                regions=np.array([[25.0, 185.0, 0.25, 1.0], [20.0, 175.0, 0.2, 0.0]]),
                n_phase=n_phase, rot_step=1.0 / max(n_phase, 1), n_mask_lines=12,
                ccf_window=20000.0, ccf_size=500.0, vsini=4.0, seed=seed)


def make_batch(n_star: int = 256, seed: int = 3, grid=(100, 400), n_regions=(1, 12), size_pct=(0.1, 3.0),
               lat=(-60.0, 60.0), n_phase=(20, 200), vsini=(1.0, 10.0)) -> List[Case]:
    """The stars of the batched form: per star a grid side U{grid}, U{n_regions} spots
    and faculae (type U{0, 1}) of size U(size_pct) % of the hemisphere (chord radius
    sqrt(f)), latitude U(lat), longitude U(0, 360), U{n_phase} phases over one rotation
    and vsini U(vsini) km/s; everything else as the 300x300-grid star.  The seed spectra
    are shared (``generate(make_case(1))`` at full size)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_star):
        g = int(rng.integers(grid[0], grid[1] + 1))
        nr = int(rng.integers(n_regions[0], n_regions[1] + 1))
        f = rng.uniform(size_pct[0], size_pct[1], nr) / 100.0
        regions = np.column_stack([rng.uniform(lat[0], lat[1], nr), rng.uniform(0.0, 360.0, nr), np.sqrt(f),
                                   rng.integers(0, 2, nr).astype(np.float64)])
        npk = int(rng.integers(n_phase[0], n_phase[1] + 1))
        out.append(Case("batch%d" % k, grid=g, n=310000, lambda0=3800.0, step=0.01, n_lines=6000, n_mu=20,
                        regions=regions, n_phase=npk, rot_step=1.0 / npk, n_mask_lines=4000,
                        ccf_window=20000.0, ccf_size=250.0, vsini=float(rng.uniform(vsini[0], vsini[1])),
                        seed=seed))
    return out


@dataclasses.dataclass
class Inputs:
    case: Case
    wave: np.ndarray               # (n,)
    mu_boundary: np.ndarray        # (n_mu - 1,)  descending
    q_norm: np.ndarray             # (n_mu, n)  new_noconti_convec_T_eff_<T*>
    q_sed: np.ndarray              # (n_mu, n)  new_conti_convec_T_eff_<T*>
    spot_norm: np.ndarray          # (n_mu, n)  new_noconti_convec_T_eff_<T*-dT_spot>
    fac_norm: np.ndarray           # (n_mu, n)  new_noconti_convec_T_eff_<T*+dT_fac>
    spot_sed: np.ndarray           # (n_mu, n)  new_conti_T_eff_<T*-dT_spot>
    fac_sed: np.ndarray            # (n_mu, n)  new_conti_T_eff_<T*+dT_fac>
    lb_table: dict                 # Limb_brightening_info.npz content
    mask_wave: np.ndarray          # mask line wavelengths
    mask_weight: np.ndarray        # mask contrasts

    @property
    def lb(self) -> np.ndarray:
        from .config import lb_params
        t = self.lb_table
        return lb_params(self.case.t_star, t["LB_G2"], t["LB_K0"], t["LB_M0"], t["Temp_array"])


def _delta_wavelength(v, wave0):
    beta = v / C_LIGHT
    return wave0 * (np.sqrt((1 + beta) / (1 - beta)) - 1)


def _line_spectrum(wave, centres, depths, sigmas, lambda0, step):
    out = np.ones_like(wave)
    n = wave.size
    for c, d, s in zip(centres, depths, sigmas):
        half = int(np.ceil(9 * s / step))
        j = int(round((c - lambda0) / step))
        lo, hi = max(0, j - half), min(n, j + half + 1)
        if lo >= hi:
            continue
        x = wave[lo:hi]
        out[lo:hi] -= d * np.exp(-((x - c) ** 2) / (2 * s * s))
    return np.clip(out, 0.0, None)


def _inject_bisector(wave, flux, coeffs):
    """CB_injection_faculae.py:227-244 with np.interp for scipy's linear interp1d."""
    rv = np.polyval(coeffs, flux)
    wave_new = wave + _delta_wavelength(rv, wave)
    if np.any(np.diff(wave_new) <= 0):
        raise ValueError("bisector injection produced a non-monotonic grid")
    out = np.zeros_like(flux)
    sel = (wave < wave_new.max()) & (wave > wave_new.min())
    out[sel] = np.interp(wave[sel], wave_new, flux)
    return out


def generate(case: Case) -> Inputs:
    rng = np.random.default_rng(case.seed)
    n, step, l0 = case.n, case.step, case.lambda0
    wave = l0 + np.arange(n, dtype=np.float64) * step
    lo, hi = wave[0] + 0.5, wave[-1] - 0.5
    centres = np.sort(rng.uniform(lo, hi, case.n_lines))
    depths = rng.uniform(0.05, 0.9, case.n_lines)
    sigmas = rng.uniform(0.03, 0.08, case.n_lines)
    spot_scale = rng.uniform(0.9, 1.2, case.n_lines)
    fac_scale = rng.uniform(0.95, 1.05, case.n_lines)
    bis = rng.uniform(-300.0, 300.0, (case.n_mu, 4))
    base_q = _line_spectrum(wave, centres, depths, sigmas, l0, step)
    base_s = _line_spectrum(wave, centres, np.minimum(depths * spot_scale, 0.99), sigmas, l0, step)
    base_f = _line_spectrum(wave, centres, np.minimum(depths * fac_scale, 0.99), sigmas, l0, step)
    q_norm = np.empty((case.n_mu, n))
    spot_norm = np.empty((case.n_mu, n))
    fac_norm = np.empty((case.n_mu, n))
    for b in range(case.n_mu):
        q_norm[b] = _inject_bisector(wave, base_q, bis[b])
        spot_norm[b] = _inject_bisector(wave, base_s, bis[b] * 0.5)
        fac_norm[b] = _inject_bisector(wave, base_f, bis[b] * 0.7)
    q_sed = q_norm * 1.0
    spot_sed = np.full((case.n_mu, n), case.spot_conti)
    fac_sed = np.full((case.n_mu, n), case.fac_conti)
    mu_boundary = np.linspace(0.95, 0.15, case.n_mu - 1) if case.n_mu > 1 else np.zeros(0)
    # limb-brightening table in the Limb_brightening_info.npz layout (mu = 0.1..1)
    mu = np.linspace(0.1, 1.0, 10)
    amp = rng.uniform(0.1, 0.25, 3) * np.array([1.0, 0.6, 0.5])
    lb_table = {"LB_G2": amp[0] * (1 - mu) ** 1.3, "LB_K0": amp[1] * (1 - mu) ** 1.4,
                "LB_M0": amp[2] * (1 - mu) ** 1.6, "Temp_array": np.array([5778, 5240, 3750])}
    # mask: the deepest lines well inside the trimmed range, binary weights
    margin = 600 * step
    inside = (centres > wave[0] + margin) & (centres < wave[-1] - margin)
    cand = np.nonzero(inside)[0]
    order = cand[np.argsort(-depths[cand])]
    pick = np.sort(order[: case.n_mask_lines])
    mask_wave = centres[pick]
    mask_weight = np.ones(pick.size)
    return Inputs(case, wave, mu_boundary, q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed,
                  lb_table, mask_wave, mask_weight)


# --------------------------------------------------------------------------
# reference-layout writer: what run_all_SOAP.py + config_hpc.cfg expect
# --------------------------------------------------------------------------

def cube_names(case: Case) -> dict:
    """run_all_SOAP.py:94-100"""
    t = case.t_star
    return {
        "q_norm": "new_noconti_convec_T_eff_%d.bin" % t,
        "spot_norm": "new_noconti_convec_T_eff_%d.bin" % (t - case.t_diff_spot),
        "fac_norm": "new_noconti_convec_T_eff_%d.bin" % (t + case.t_diff_fac),
        "q_sed": "new_conti_convec_T_eff_%d.bin" % t,
        "spot_sed": "new_conti_T_eff_%d.bin" % (t - case.t_diff_spot),
        "fac_sed": "new_conti_T_eff_%d.bin" % (t + case.t_diff_fac),
    }


def mask_name(t_star: float) -> str:
    """run_all_SOAP.py:38-46 mask_templates"""
    types = ['F9', 'G2', 'G8', 'G9', 'K2', 'K5', 'K6', 'M0', 'M2', 'M3', 'M4', 'M5']
    teff = np.array([6050, 5770, 5480, 5380, 5100, 4400, 4300, 3800, 3400, 3250, 3100, 2800])
    return types[int(np.argmin(np.abs(teff - t_star)))] + '_mask.txt'


def write_reference_layout(inp: Inputs, root: str, output_prefix: str = "", file_prefix: str = "syn",
                           keyword: str = "nreal") -> str:
    """Write input_spec/, input_mask/ and config_hpc.cfg under ``root``.

    The layout is the one ``run_all_SOAP.py`` reads (``config_hpc.cfg`` keys at
    ``run_all_SOAP.py:56-127``); returns the config path.  ``file_prefix`` must not be
    empty: the driver joins argv with spaces for ``os.system``, so an empty prefix
    would vanish from the command line and shift every later argument.
    """
    case = inp.case
    spec_dir = os.path.join(root, "input_spec")
    mask_dir = os.path.join(root, "input_mask")
    os.makedirs(spec_dir, exist_ok=True)
    os.makedirs(mask_dir, exist_ok=True)
    for key, name in cube_names(case).items():
        np.ascontiguousarray(getattr(inp, key), dtype=np.float64).tofile(os.path.join(spec_dir, name))
    inp.wave.astype(np.float64).tofile(os.path.join(spec_dir, "solar_wavelength.bin"))
    inp.mu_boundary.astype(np.float64).tofile(os.path.join(spec_dir, "mu_boundary_array.bin"))
    np.savez(os.path.join(spec_dir, "Limb_brightening_info.npz"), **inp.lb_table)
    np.savetxt(os.path.join(mask_dir, mask_name(case.t_star)),
               np.stack([inp.mask_wave, inp.mask_weight], axis=1))
    lines = ["[main]", "", "grid     : %d" % case.grid, "nrho     : %d" % case.nrho,
             "instrument_reso : %d" % case.inst_reso, "rot_num: %r" % case.rot_num,
             "rot_step: %r" % case.rot_step, "", "", "[star]", "",
             "radius_sun : %d" % R_SUN_KM, "radius     : %r" % case.radius, "prot       : %r" % float(case.period),
             "W_ratio    : %r" % case.w_ratio, "I          : %r" % case.incl,
             "Tstar      : %d" % case.t_star, "Tdiff_spot : %d" % case.t_diff_spot,
             "Tdiff_faculae : %d" % case.t_diff_fac, "limb1      : %r" % case.u1,
             "limb2      : %r" % case.u2, "N_act: %d" % len(case.regions), ""]
    for i, (lat, lon, size, typ) in enumerate(case.regions):
        lines += ["[active_regions_%d]" % (i + 1), "longitude: %r" % float(lon), "latitude: %r" % float(lat),
                  "size: %r" % float(size), "type: %d" % int(typ), ""]
    lines += ["[data_io]", "no_thread: 512", "input_prefix: .", "output_prefix: %s" % output_prefix,
              "file_prefix: %s" % file_prefix, "input_dir: /input_spec/", "maps_dir: /SOAP_density/",
              "raw_dir: /SOAP_raw_spec/", "spec_dir: /SOAP_resolution/",
              "mu_array_name: mu_boundary_array.bin", "wave_array_name: solar_wavelength.bin",
              "CCF_window: %r" % case.ccf_window, "CCF_size: %r" % case.ccf_size,
              "BIS_prefix: /input_BIS/", "mask_prefix: /input_mask/", "keyword: %s" % keyword, ""]
    cfg = os.path.join(root, "config_hpc.cfg")
    with open(cfg, "w") as f:
        f.write("\n".join(lines))
    return cfg
