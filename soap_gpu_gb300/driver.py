"""In-process replacement of run_all_SOAP.py's pipeline on the GPU library.

``python -m soap_gpu_gb300.driver [config_hpc.cfg] [--form plain64|fast64|fast32]``
reads the same configuration file and input layout as ``run_all_SOAP.py`` and writes
the same outputs -- the disk maps, quiet spectra, per-phase raw and convolved
spectra (``--write-spectra``), and the ``*_RV_{tot,flux,bconv}_GPU.npz`` /
``*_GPU_SOAP_RV_data.npz`` series (run_all_SOAP.py:400-412,443-449) -- without
spawning one process per stage and per spectrum: maps, integration, convolution,
CCF and fits each run as one batched call.

Differences from the reference driver, all deliberate:
* no plot (the PNG and the copy of Plot_animation.py are left out);
* the output directory is not removed with ``rm -r`` when it exists;
* on grids other than 0.005 A the CCF mask uses the real grid step instead of the
  literal 0.005 A and 20000-pixel slice of CCF_func.py:8-9,62-63 (which would fail
  with a shape mismatch there); at 0.005 A both are identical.
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

from . import config as cfgmod
from . import rv as rvmod
from ._lib import Activity, Star
from .api import Context


def _write(path, arr, dtype=np.float64):
    np.ascontiguousarray(arr, dtype=dtype).tofile(path)


def evolving_sizes(phases, sizes, period, area_rate):
    """Region sizes per phase for a linear change of area, as run_all_SOAP_evo.py:16-20,
    213-230 forms them: t = (phase - phase_min) * P [d], area = size^2 - area_rate * t,
    size = sqrt(area).  Returns an n_phase x n_region array."""
    t = (np.asarray(phases, dtype=np.float64) - np.min(phases)) * period
    area = np.asarray(sizes, dtype=np.float64)[None, :] ** 2 - area_rate * t[:, None]
    return np.sqrt(area)


def run(config_path: str, form: str = "plain64", write_spectra: bool = True, device: int = 0, verbose=True,
        area_rate: float = None):
    """area_rate: the spot-size evolution of run_all_SOAP_evo.py (change of region area
    per day); None keeps the sizes of the configuration."""
    rc = cfgmod.load_config(config_path)
    rc.area_rate = area_rate
    base_dir = os.path.dirname(os.path.abspath(config_path))
    cwd = os.getcwd()
    os.chdir(base_dir)
    try:
        return _run(rc, form, write_spectra, device, verbose)
    finally:
        os.chdir(cwd)


def _run(rc, form, write_spectra, device, verbose):
    t0 = time.time()
    wave = np.fromfile(rc.input_dir + rc.wave_array_name)
    step = round(wave[3] - wave[2], 5)                       # run_all_SOAP.py:124
    n = int(wave.size)
    no_block = int(n / rc.no_thread)
    n_eff = no_block * rc.no_thread
    mu_b = np.fromfile(rc.input_dir + rc.mu_array_name)
    n_mu = mu_b.size + 1
    lbf = np.load(rc.input_dir + "Limb_brightening_info.npz")
    lb = cfgmod.lb_params(rc.t_star, lbf["LB_G2"], lbf["LB_K0"], lbf["LB_M0"], lbf["Temp_array"])
    cubes = {k: np.fromfile(p).reshape(n_mu, n) for k, p in rc.cube_paths.items()}
    for d in (rc.output_prefix, rc.maps_dir, rc.raw_dir, rc.final_spec_dir):
        os.makedirs(d, exist_ok=True)
    if rc.keyword == 'real':                                  # run_all_SOAP.py:148-157
        phases = np.atleast_1d(np.loadtxt(rc.output_prefix + '/' + rc.file_prefix + '_phase_locator.txt'))
        info = np.atleast_2d(np.loadtxt(rc.maps_dir + 'final_info.txt'))
        ids = info[:, 0].astype(int)
        regions = [np.atleast_2d(np.loadtxt(rc.maps_dir + 'maps%d_for_all.txt' % i)).reshape(-1, 4)
                   if info[k, 1] > 0 else np.zeros((0, 4)) for k, i in enumerate(ids)]
    else:                                                     # run_all_SOAP.py:178-220
        phases = rc.phases
        np.savetxt(rc.output_prefix + '/' + rc.file_prefix + '_phase_locator.txt', phases.T)
        regions = [rc.regions for _ in phases]
        if getattr(rc, "area_rate", None) is not None:        # run_all_SOAP_evo.py:213-230
            sizes = evolving_sizes(phases, rc.regions[:, 2], rc.period, rc.area_rate)
            regions = [np.column_stack((rc.regions[:, 0], rc.regions[:, 1], sizes[i], rc.regions[:, 3]))
                       for i in range(phases.size)]
        info = np.zeros((phases.size, 2))
        for i in range(phases.size):
            np.savetxt(rc.maps_dir + 'maps' + str(int(i)) + '_for_all.txt', regions[i])
            info[i] = (i, regions[i].shape[0])
        np.savetxt(rc.maps_dir + 'final_info.txt', info)
        ids = np.arange(phases.size)
    prefix = rc.output_prefix + "/" + rc.file_prefix
    act = Activity(rc.t_star, rc.t_diff_spot, rc.t_diff_fac, rc.nrho, 0)
    star = Star(rc.grid, rc.period, rc.omega_ratio, rc.incl, rc.radius_km, rc.limb1, rc.limb2, (
        __import__("ctypes").c_double * 4)(*lb))
    with Context(device) as ctx:
        maps = ctx.disk_maps(rc.grid, rc.period, rc.omega_ratio, rc.incl, rc.radius_km, rc.limb1, rc.limb2, mu_b, lb)
        for key, name in (("mu", "mu_map"), ("delta", "delta_map"), ("limb", "limb_map"), ("lb", "LB_map")):
            _write(prefix + name + ".bin", maps[key])
        _write(prefix + "region_map.bin", maps["region"], np.int32)
        q_norm = ctx.quiet_disk(form, wave, cubes["q_norm"], n_eff, maps, rc.grid, step)
        q_sed = ctx.quiet_disk(form, wave, cubes["q_sed"], n_eff, maps, rc.grid, step)
        low_norm, _ = ctx.lower_resolution(form, wave, q_norm, n_eff, rc.inst_sigma, step_mult=step, step_exp=0.005)
        low_sed, _ = ctx.lower_resolution(form, wave, q_sed, n_eff, rc.inst_sigma, step_mult=step, step_exp=0.005)
        for q, low, pre in ((q_norm, low_norm, prefix), (q_sed, low_sed, prefix + "_SED")):
            _write(pre + "_quiet_sun_spec.bin", q[:n_eff])
            _write(pre + "_quiet_sun_wave.bin", wave[:n_eff])
            _write(pre + "_quiet_sun_lower_spec.bin", low)
        lower, raw = ctx.phase_pipeline(form, wave, n_eff, star, maps, cubes, step, act, phases, regions, q_sed,
                                        q_norm, rc.inst_sigma, conv_step=0.005, want_raw=True)
        t_gpu = time.time() - t0
        if verbose:
            print("GPU Calculation time (s):", t_gpu)
        if write_spectra:
            for p, pid in enumerate(ids):
                for t, name in enumerate(("tot", "flux", "bconv")):
                    _write(rc.raw_dir + rc.file_prefix + "_Spec_%s_%d_.bin" % (name, pid), raw[p, t])
                    _write(rc.final_spec_dir + rc.file_prefix + "_lower_spec_%s_%d_.bin" % (name, p), lower[p, t])
        # ---- RV series (run_all_SOAP.py:256-412) ---------------------------------------
        t1 = time.time()
        mask = np.loadtxt(rc.input_prefix + rc.mask_prefix + cfgmod.mask_template_name(rc.t_star))
        vel = rc.velocities
        literal = abs(step - 0.005) < 1e-12
        all_spec = np.concatenate([lower.reshape(-1, n_eff), np.stack([low_sed, low_sed, low_norm])], axis=0)
        fit = rvmod.ccf_fit(ctx, step, vel, wave[:n_eff], all_spec, mask[:, 0], mask[:, 1], form="plain64",
                            literal_step=literal)
        n_ph = len(phases)
        out = {}
        for t, name in enumerate(("tot", "flux", "bconv")):
            rows = [p * 3 + t for p in range(n_ph)] + [3 * n_ph + t]
            vr = fit["rv"][rows].copy()
            vr -= vr[-1]
            data = {"time": phases, "RV": vr[:-1], "ccf": fit["ccf"][rows], "model": fit["model"][rows],
                    "continuum": fit["continuum"][rows], "contrast": fit["contrast"][rows],
                    "span": fit["span"][rows], "fwhm": fit["fwhm"][rows], "depth": fit["depth"][rows],
                    "bis": fit["bis"][rows]}
            np.savez(rc.output_prefix + '/' + rc.file_prefix + '_' + 'RV_' + name + '_GPU.npz', **data)
            out[name] = data
        np.savez(rc.output_prefix + '/' + rc.file_prefix + '_GPU_SOAP_RV_data.npz', time=phases,
                 tot=out["tot"]["RV"], flux=out["flux"]["RV"], bconv=out["bconv"]["RV"])
        if verbose:
            print("RV Calculation time (s):", time.time() - t1)
            print("Computing time (s):", time.time() - t0)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("config", nargs="?", default="config_hpc.cfg")
    ap.add_argument("--form", default="plain64", choices=["plain64", "fast64", "fast32"])
    ap.add_argument("--no-spectra", action="store_true", help="do not write the per-phase spectra files")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--area-rate", type=float, default=None,
                    help="spot-size evolution: change of region area per day (run_all_SOAP_evo.py)")
    a = ap.parse_args()
    run(a.config, a.form, not a.no_spectra, a.device, area_rate=a.area_rate)


if __name__ == "__main__":
    main()
