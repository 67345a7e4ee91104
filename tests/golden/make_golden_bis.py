"""Generate golden vectors for the bisector injection from the reference's own code.

Run in a container where the reference checkout is available:

    python tests/golden/make_golden_bis.py /path/to/SOAP_GPU/SOAP_code

It extracts ``Delta_wavelength``, ``BIS_inject_spectral_quiet`` and
``BIS_inject_spectral_active`` from ``CB_injection_faculae.py`` with ``ast`` (the
script's module-level statements read configuration and data files and never run)
and executes them with numpy and scipy's ``interp1d`` on seeded synthetic spectra.
The output ``golden_bis.npz`` is committed; the tests read only that file.
"""
from __future__ import annotations

import ast
import os
import sys

import numpy as np
from scipy.interpolate import interp1d

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ("Delta_wavelength", "BIS_inject_spectral_quiet", "BIS_inject_spectral_active")


def injection_namespace(src_dir):
    with open(os.path.join(src_dir, "CB_injection_faculae.py")) as f:
        tree = ast.parse(f.read())
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in NAMES]
    assert len(keep) == len(NAMES)
    ns = {"np": np, "interp1d": interp1d}
    exec(compile(ast.Module(body=keep, type_ignores=[]), "CB_injection_faculae.py", "exec"), ns)
    return ns


def line_spectrum(rng, wave, n_lines):
    flux = np.ones_like(wave)
    centres = rng.uniform(wave[40], wave[-40], n_lines)
    depths = rng.uniform(0.05, 0.95, n_lines)
    sigmas = rng.uniform(0.03, 0.08, n_lines)
    for c, d, s in zip(centres, depths, sigmas):
        flux -= d * np.exp(-((wave - c) ** 2) / (2 * s * s))
    return np.clip(flux, 0.0, None)


def main(src_dir):
    ns = injection_namespace(src_dir)
    rng = np.random.default_rng(77)
    n, n_mu = 6000, 4
    wave = 5000.0 + np.arange(n) * 0.01
    flux = line_spectrum(rng, wave, 60)
    # a few pixels exactly on the active form's branch points
    flux[100], flux[101] = 0.5, 0.8
    scale = 1.37
    q_coeffs = rng.uniform(-300.0, 300.0, (n_mu, 4))
    up = rng.uniform(-200.0, 200.0, (n_mu, 3))
    low = rng.uniform(-200.0, 200.0, (n_mu, 3))
    dep_cut = np.array([0.8, 0.85, 0.9, 0.95])
    vcut = rng.uniform(-100.0, 100.0, n_mu)
    vshift = rng.uniform(-50.0, 50.0, n_mu)
    quiet = np.array([ns["BIS_inject_spectral_quiet"](wave, flux, q_coeffs[b], scale) for b in range(n_mu)])
    active = np.array([ns["BIS_inject_spectral_active"](wave, flux, up[b], low[b], dep_cut[b], vcut[b], vshift[b],
                                                        scale) for b in range(n_mu)])
    np.savez_compressed(os.path.join(HERE, "golden_bis.npz"), wave=wave, flux=flux, scale=np.array(scale),
                        q_coeffs=q_coeffs, up=up, low=low, dep_cut=dep_cut, vcut=vcut, vshift=vshift,
                        quiet=quiet, active=active)
    print("wrote", os.path.join(HERE, "golden_bis.npz"))


if __name__ == "__main__":
    checkout = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SOAP_GPU_REF")
    if not checkout:
        sys.exit("usage: %s <reference SOAP_code directory>  (or set SOAP_GPU_REF)" % sys.argv[0])
    main(checkout)
