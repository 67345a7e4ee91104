"""Generate golden vectors from the reference's own Python code.

Run in a container where the reference checkout is available:

    python tests/golden/make_golden.py /path/to/SOAP_GPU/SOAP_code

It imports ``CCF_func.py`` (numpy only) and executes, from ``run_all_SOAP.py``, the
function definitions ``LB_boundary`` / ``LB_params`` / ``mask_templates`` and the
CCF normalisation / apodisation statements (lines 306-313), all extracted from
the source with ``ast`` so the driver's module-level side effects (config
parsing, plotting, process spawning) never run.  Inputs are seeded synthetic data.
The output ``golden.npz`` is committed; the tests read only that file.
"""
from __future__ import annotations

import ast
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_ccf_func(src_dir):
    spec = importlib.util.spec_from_file_location("ref_ccf_func", os.path.join(src_dir, "CCF_func.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def driver_namespace(src_dir):
    """Function defs of run_all_SOAP.py, executed in a fresh namespace."""
    with open(os.path.join(src_dir, "run_all_SOAP.py")) as f:
        tree = ast.parse(f.read())
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef)
            and n.name in ("LB_boundary", "LB_params", "mask_templates")]
    ns = {"np": np}
    exec(compile(ast.Module(body=keep, type_ignores=[]), "run_all_SOAP.py", "exec"), ns)
    return ns


def apodisation_statements(src_dir):
    """The driver's CCF normalisation / apodisation block (run_all_SOAP.py:299,306-313)."""
    with open(os.path.join(src_dir, "run_all_SOAP.py")) as f:
        tree = ast.parse(f.read())
    names = {"nb_zeros_on_sides", "period_appodisation", "len_appodisation", "a", "b", "appod",
             "CCF_quiet_Sun"}
    body = []
    for n in tree.body:
        if isinstance(n, (ast.Assign, ast.AugAssign)):
            tgt = n.targets[0] if isinstance(n, ast.Assign) else n.target
            if isinstance(tgt, ast.Name) and tgt.id in names and 306 <= n.lineno <= 314:
                body.append(n)
    return compile(ast.Module(body=body, type_ignores=[]), "run_all_SOAP.py", "exec")


def main(src_dir):
    rng = np.random.default_rng(2024)
    ccf_func = load_ccf_func(src_dir)
    drv = driver_namespace(src_dir)
    out = {}
    # ---- CCF (CCF_func.py with the driver's extended grid, run_all_SOAP.py:292-296) ----
    step = 0.005
    n_w = 12000
    wavelength = 5050.0 + np.arange(n_w) * step
    no_points = int(100.0 / step)
    before = np.linspace(np.min(wavelength) - step * no_points, np.min(wavelength), no_points)
    after = np.linspace(wavelength[-1], wavelength[-1] + step * no_points, no_points)
    wave_ext = np.concatenate((before, wavelength, after))
    vel = np.arange(-1 * 20000.0, 20000.0 + 1., 500.0)
    while True:
        n_lines = 40
        lines = np.sort(rng.uniform(wavelength[30], wavelength[-30], n_lines))
        lines[5] = lines[4] + 0.004          # an overlapping pair: the later line overwrites
        weights = rng.uniform(0.15, 1.0, n_lines)
        with np.errstate(divide="ignore", invalid="ignore"):
            mask = ccf_func.calculate_CCF_1(vel, wavelength, lines, weights, wave_ext)
        # lines near the ends move into the linspace extensions at large |v|; keep a
        # draw where no hole lands on the duplicated grid points (a 0/0 in calc_mask)
        if np.all(np.isfinite(mask)):
            break
    spectra = 1.0 - 0.5 * rng.uniform(0, 1, (2, n_w))
    ccfs = np.array([ccf_func.calculate_CCF_2(vel, s, mask) for s in spectra])
    nz = np.nonzero(mask)
    out.update(ccf_wave=wavelength, ccf_lines=lines, ccf_weights=weights, ccf_vel=vel, ccf_spectra=spectra,
               ccf_raw=ccfs, mask_rows=nz[0].astype(np.int32), mask_cols=nz[1].astype(np.int32),
               mask_vals=mask[nz], mask_shape=np.array(mask.shape))
    # ---- normalisation + apodisation (run_all_SOAP.py:299,306-313) --------------------
    code = apodisation_statements(src_dir)
    norm = []
    for c in ccfs:
        ns = {"np": np, "vrad_ccf2": vel, "CCF_quiet_Sun": c.copy()}
        ns["CCF_quiet_Sun"] /= np.max(ns["CCF_quiet_Sun"])
        exec(code, ns)
        norm.append(ns["CCF_quiet_Sun"])
    out["ccf_norm"] = np.array(norm)
    out["appod"] = ns["appod"]
    # ---- limb-brightening coefficients (run_all_SOAP.py:8-34,140) ---------------------
    mu = np.linspace(0.1, 1.0, 10)
    tables, temps, params = [], [], []
    for t_star in (6100, 5778, 5500, 5240, 4500, 3750, 3500):
        g2 = rng.uniform(0.1, 0.3) * (1 - mu) ** 1.3
        k0 = rng.uniform(0.05, 0.2) * (1 - mu) ** 1.4
        m0 = rng.uniform(0.03, 0.15) * (1 - mu) ** 1.6
        tarr = np.array([5778, 5240, 3750])
        drv["temp_derived_array"] = tarr
        p = drv["LB_params"](t_star, g2, k0, m0)[::-1]
        tables.append(np.stack([g2, k0, m0]))
        temps.append(t_star)
        params.append(p)
    out.update(lb_tables=np.array(tables), lb_temps=np.array(temps), lb_params=np.array(params))
    out["mask_names"] = np.array([drv["mask_templates"](t) for t in (6100, 5770, 5300, 4350, 3000)])
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"))


if __name__ == "__main__":
    checkout = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SOAP_GPU_REF")
    if not checkout:
        sys.exit("usage: %s <reference SOAP_code directory>  (or set SOAP_GPU_REF)" % sys.argv[0])
    main(checkout)
