"""Run configuration in the reference's ``config_hpc.cfg`` layout.

``load_config(path)`` reads the INI file the way ``run_all_SOAP.py:50-145`` does and
returns every derived quantity the driver forwards to the stage executables
(instrument sigma, grid step, vector sizes, limb-brightening coefficients, file
names).  ``lb_params`` is the limb-brightening fit of ``run_all_SOAP.py:8-34``.
"""
from __future__ import annotations

import configparser
import dataclasses
import os
from typing import List

import numpy as np

C_LIGHT = 299792458.0


def lb_boundary(t_eff):
    """run_all_SOAP.py:8-19"""
    if t_eff > 5778:
        return np.array([0, 1])
    if 5240 <= t_eff <= 5778:
        return np.array([0, 1])
    if 3750 <= t_eff < 5240:
        return np.array([1, 2])
    return np.array([1, 2])


def lb_params(t_star, lb_g2, lb_k0, lb_m0, temp_array):
    """run_all_SOAP.py:21-34 and :140 -- facula limb-brightening cubic in mu,
    returned lowest order first (LB0..LB3)."""
    mu_array = np.linspace(0.1, 1, 10)
    lb = np.zeros(mu_array.size)
    bnd = lb_boundary(t_star)
    temp_array = np.asarray(temp_array)
    for i in range(10):
        der = np.array([lb_g2[i], lb_k0[i], lb_m0[i]])
        params = np.polyfit(temp_array[bnd], der[bnd], 1)
        lb[i] = np.poly1d(params)(t_star)
    return np.polyfit(mu_array, lb, 3)[::-1]


def mask_template_name(t_eff):
    """run_all_SOAP.py:38-46"""
    types = ['F9', 'G2', 'G8', 'G9', 'K2', 'K5', 'K6', 'M0', 'M2', 'M3', 'M4', 'M5']
    teff = np.array([6050, 5770, 5480, 5380, 5100, 4400, 4300, 3800, 3400, 3250, 3100, 2800])
    return types[int(np.argmin(np.abs(teff - t_eff)))] + '_mask.txt'


@dataclasses.dataclass
class RunConfig:
    grid: int
    nrho: int
    inst_reso: int
    rot_num: float
    rot_step: float
    inst_sigma: float
    radius_km: float
    period: float
    omega_ratio: float
    incl: float
    limb1: float
    limb2: float
    t_star: int
    t_diff_spot: int
    t_diff_fac: int
    regions: np.ndarray          # (N_act, 4): lat, long, size, type
    input_prefix: str
    input_dir: str
    output_prefix: str
    maps_dir: str
    raw_dir: str
    final_spec_dir: str
    file_prefix: str
    mu_array_name: str
    wave_array_name: str
    ccf_window: float
    ccf_size: float
    keyword: str
    mask_prefix: str
    no_thread: int

    @property
    def cube_paths(self) -> dict:
        t = self.t_star
        d = self.input_dir
        return {"q_norm": d + 'new_noconti_convec_T_eff_%d.bin' % t,
                "spot_norm": d + 'new_noconti_convec_T_eff_%d.bin' % (t - self.t_diff_spot),
                "fac_norm": d + 'new_noconti_convec_T_eff_%d.bin' % (t + self.t_diff_fac),
                "q_sed": d + 'new_conti_convec_T_eff_%d.bin' % t,
                "spot_sed": d + 'new_conti_T_eff_%d.bin' % (t - self.t_diff_spot),
                "fac_sed": d + 'new_conti_T_eff_%d.bin' % (t + self.t_diff_fac)}

    @property
    def phases(self) -> np.ndarray:
        return np.arange(0.0, self.rot_num, self.rot_step)

    @property
    def velocities(self) -> np.ndarray:
        return np.arange(-1 * self.ccf_window, self.ccf_window + 1., self.ccf_size)


def load_config(path: str) -> RunConfig:
    cfg = configparser.ConfigParser()
    if not cfg.read(path):
        raise FileNotFoundError(path)
    g = cfg.get
    inst_reso = int(g('main', 'instrument_reso'))
    sigma = 0.0
    if inst_reso > 0:
        fwhm = C_LIGHT / float(inst_reso)
        sigma = fwhm / (2 * np.sqrt(2 * np.log(2)))
    t_star = int(g('star', 'Tstar'))
    n_act = int(g('star', 'N_act'))
    regions = np.zeros((n_act, 4))
    for i in range(n_act):
        k = 'active_regions_%d' % (i + 1)
        regions[i] = [float(g(k, 'latitude')), float(g(k, 'longitude')), float(g(k, 'size')),
                      float(g(k, 'type'))]
    input_prefix = g('data_io', 'input_prefix')
    output_prefix = g('data_io', 'output_prefix') + '_phoenix' + str(t_star)
    return RunConfig(
        grid=int(g('main', 'grid')), nrho=int(g('main', 'nrho')), inst_reso=inst_reso,
        rot_num=float(g('main', 'rot_num')), rot_step=float(g('main', 'rot_step')), inst_sigma=sigma,
        radius_km=float(g('star', 'radius')) * int(g('star', 'radius_sun')), period=float(g('star', 'prot')),
        omega_ratio=float(g('star', 'W_ratio')), incl=float(g('star', 'I')), limb1=float(g('star', 'limb1')),
        limb2=float(g('star', 'limb2')), t_star=t_star, t_diff_spot=int(g('star', 'Tdiff_spot')),
        t_diff_fac=int(g('star', 'Tdiff_faculae')), regions=regions, input_prefix=input_prefix,
        input_dir=input_prefix + g('data_io', 'input_dir'), output_prefix=output_prefix,
        maps_dir=output_prefix + g('data_io', 'maps_dir'), raw_dir=output_prefix + g('data_io', 'raw_dir'),
        final_spec_dir=output_prefix + g('data_io', 'spec_dir'), file_prefix=g('data_io', 'file_prefix'),
        mu_array_name=g('data_io', 'mu_array_name'), wave_array_name=g('data_io', 'wave_array_name'),
        ccf_window=float(g('data_io', 'CCF_window')), ccf_size=float(g('data_io', 'CCF_size')),
        keyword=g('data_io', 'keyword'), mask_prefix=g('data_io', 'mask_prefix'),
        no_thread=int(g('data_io', 'no_thread')))
