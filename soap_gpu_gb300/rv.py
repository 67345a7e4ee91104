"""RV / bisector / FWHM series from the normalised phase spectra.

The in-process form of run_all_SOAP.py:256-412: trim the spectra ([200:-200] then
[10:-10]), select the mask lines inside the trimmed range with contrast > 0.1,
build the CCF on the 100 A-extended grid, normalise and apodise it, fit the
Gaussian and the bisector, and subtract the quiet-star velocity.  The reference
spawns one BIS_FIT2 process per spectrum and writes text files for each; here all
spectra of all types go through one batched CCF call and one batched fit call.
"""
from __future__ import annotations

import numpy as np

CUTOFF = 200      # run_all_SOAP.py:259
CUTOFF_NEW = 10   # run_all_SOAP.py:266
WAVE_EXTEND = 100.0


def trim(a):
    return a[..., CUTOFF:-CUTOFF][..., CUTOFF_NEW:-CUTOFF_NEW]


def select_lines(wave_trim, line_wave, line_weight):
    """run_all_SOAP.py:285-290"""
    sel = (line_wave > wave_trim.min()) & (line_wave < wave_trim.max()) & (line_weight > 0.1)
    return line_wave[sel], line_weight[sel]


def ccf_fit(ctx, step, velocities, wave_neff, spectra, line_wave, line_weight, form="plain64",
            literal_step=False):
    """CCF + Gaussian/bisector fit of spectra[..., n_eff] (any leading shape).

    literal_step=True keeps CCF_func.py's hard-coded 0.005 A mask step and 20000-pixel
    slice (valid only on a 0.005 A grid); otherwise the real step is used."""
    wave_trim = trim(np.asarray(wave_neff))
    lw, lwt = select_lines(wave_trim, np.asarray(line_wave), np.asarray(line_weight))
    shape = spectra.shape[:-1]
    flat = np.ascontiguousarray(trim(np.asarray(spectra)).reshape(-1, wave_trim.size))
    no_points = int(WAVE_EXTEND / step)
    mask_step = 0.005 if literal_step else step
    index_old = 20000 if literal_step else no_points
    ccf = ctx.ccf(form, velocities, lw, lwt, wave_trim, step, flat, normalise=True, wave_extend=WAVE_EXTEND,
                  mask_step=mask_step, index_old=index_old)
    fit = ctx.gauss_bis(np.asarray(velocities, dtype=np.float64), ccf)
    out = {"ccf": ccf.reshape(shape + (len(velocities),)),
           "model": fit["model"].reshape(shape + (len(velocities),)),
           "continuum": fit["par"][:, 0].reshape(shape), "contrast": fit["par"][:, 1].reshape(shape),
           "span": fit["par"][:, 2].reshape(shape), "rv": fit["par"][:, 3].reshape(shape),
           "fwhm": fit["par"][:, 4].reshape(shape), "depth": fit["depth"].reshape(shape + (91,)),
           "bis": fit["bis"].reshape(shape + (91,)), "iters": fit["iters"].reshape(shape)}
    return out


def rv_series(ctx, case, wave_neff, lower, line_wave, line_weight, quiet=None, form="plain64"):
    """lower: [n_phase, 3 (tot, flux, bconv), n_eff].  If quiet = (quiet_sed_lower,
    quiet_norm_lower) is given, the RVs are relative to the quiet star
    (run_all_SOAP.py:351-362,396-397); otherwise the raw fitted centres."""
    res = ccf_fit(ctx, case.step, case.velocities, wave_neff, lower, line_wave, line_weight, form=form)
    if quiet is not None:
        q = np.stack([quiet[0], quiet[0], quiet[1]])       # tot, flux use SED; bconv the normalised
        qr = ccf_fit(ctx, case.step, case.velocities, wave_neff, q, line_wave, line_weight, form=form)
        res["rv"] = res["rv"] - qr["rv"][None, :]
        res["quiet"] = qr
    return res
