"""ORACLE -- test infrastructure only.

ctypes binding to ``oracle/liboracle.so``, the plain-C restatement of the reference
SOAP-GPU per-phase synthesis path (``oracle/soap_oracle.c``), plus two numpy
restatements of the reference's Python steps (``ccf_mask_numpy`` follows
``CCF_func.py:5-24,39-91``; ``lb_params`` follows ``run_all_SOAP.py:8-34``).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this package, and only as the checker.  The product path
(``soap_gpu_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
SEM_GATHER = 0
SEM_SCATTER = 1
C_LIGHT = 299792458.0

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction: identical bits on x86 and Arm)."""
    src = os.path.join(_HERE, "soap_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        tmp = _LIB_PATH + ".tmp.%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                               "-o", tmp, src, "-lm"])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_delta_lambda_cpu.restype = ctypes.c_double
        L.orc_delta_lambda_cpu.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_conv_halfwidth.restype = ctypes.c_int
        L.orc_conv_halfwidth.argtypes = [_dp, ctypes.c_double, ctypes.c_double]
        L.orc_disk_maps.restype = None
        L.orc_disk_maps.argtypes = [ctypes.c_int] + [ctypes.c_double] * 6 + [ctypes.c_int, _dp] + \
            [ctypes.c_double] * 4 + [_dp, _dp, _dp, _ip, _dp]
        L.orc_quiet_disk.restype = None
        L.orc_quiet_disk.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                     _dp, _dp, _ip, ctypes.c_double, _dp]
        L.orc_lower_resolution.restype = None
        L.orc_lower_resolution.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp] + [ctypes.c_double] * 5 + \
            [_dp, _dp, _dp]
        L.orc_region_bbox.restype = None
        L.orc_region_bbox.argtypes = [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.c_double, ctypes.c_int, _ip]
        L.orc_inverse_rotation_matrix.restype = None
        L.orc_inverse_rotation_matrix.argtypes = [ctypes.c_double] * 4 + [_dp]
        L.orc_phase_maps.restype = None
        L.orc_phase_maps.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]
        L.orc_phase_integrate.restype = None
        L.orc_phase_integrate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int,
                                          _dp, _dp, _dp, _dp, _ip, _dp,
                                          _dp, _dp, _dp, _dp, _dp, _dp,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          _dp, _dp, _dp]
        L.orc_ccf_mask.restype = ctypes.c_int
        L.orc_ccf_mask.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp]
        L.orc_ccf.restype = None
        L.orc_ccf.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        L.orc_ccf_normalise.restype = None
        L.orc_ccf_normalise.argtypes = [ctypes.c_int, _dp]
        L.orc_gauss_bis.restype = ctypes.c_int
        L.orc_gauss_bis.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def conv_halfwidth(wave, sigma_v, window_width=50.0):
    w = _c64(wave)
    return lib().orc_conv_halfwidth(_d(w), sigma_v, window_width)


def disk_maps(grid, period, omega_ratio, incl, radius_km, u1, u2, mu_b, lb):
    mu_b = _c64(mu_b)
    g2 = grid * grid
    out = [np.empty(g2) for _ in range(3)]
    region = np.empty(g2, dtype=np.int32)
    lbm = np.empty(g2)
    lib().orc_disk_maps(grid, period, omega_ratio, incl, radius_km, u1, u2, len(mu_b) + 1, _d(mu_b),
                        lb[0], lb[1], lb[2], lb[3], _d(out[0]), _d(out[1]), _d(out[2]), _i(region), _d(lbm))
    return dict(delta=out[0], limb=out[1], mu=out[2], region=region, lb=lbm)


def quiet_disk(wave, cube, n_eff, maps, grid, step, sem=SEM_GATHER):
    wave = _c64(wave)
    cube = _c64(cube)
    n = wave.size
    out = np.zeros(n)
    lib().orc_quiet_disk(sem, n, n_eff, _d(wave), _d(cube), grid, _d(_c64(maps["delta"])),
                         _d(_c64(maps["limb"])), _i(np.ascontiguousarray(maps["region"], dtype=np.int32)),
                         step, _d(out))
    return out


def lower_resolution(wave, a, n_eff, sigma_v, window_width=50.0, step_mult=0.005, step_exp=0.005,
                     sentinel=-60000.0):
    """Returns (normalised[n_eff], conv[n_eff], (minA, maxC))."""
    wave = _c64(wave)
    a = _c64(a)
    n = wave.size
    out = np.empty(n_eff)
    conv = np.empty(n_eff)
    mm = np.empty(2)
    lib().orc_lower_resolution(n, n_eff, _d(wave), _d(a), sigma_v, window_width, step_mult, step_exp,
                               sentinel, _d(conv), _d(out), _d(mm))
    return out, conv, (mm[0], mm[1])


def region_bbox(s, lon, lat, incl, nrho, phase, grid):
    b = np.empty(5, dtype=np.int32)
    lib().orc_region_bbox(s, lon, lat, incl, nrho, phase, grid, _i(b))
    return b


def inverse_rotation_matrix(lon, lat, incl, phase):
    r = np.empty(9)
    lib().orc_inverse_rotation_matrix(lon, lat, incl, phase, _d(r))
    return r.reshape(3, 3)


def phase_maps(grid, nrho, incl, phase, regions, t_star, t_diff_spot, t_diff_fac):
    regions = _c64(np.asarray(regions, dtype=np.float64).reshape(-1, 4))
    temp = np.empty(grid * grid)
    bi = np.empty(grid * grid)
    lib().orc_phase_maps(grid, nrho, incl, phase, regions.shape[0], _d(regions), t_star, t_diff_spot,
                         t_diff_fac, _d(temp), _d(bi))
    return temp, bi


def phase_integrate(wave, n_eff, grid, temp, bi, maps, q_norm, q_sed, spot_norm, fac_norm, spot_sed,
                    fac_sed, step, solar=False, t_star=5778, t_diff_fac=250, sem=SEM_GATHER):
    wave = _c64(wave)
    n = wave.size
    flux, bconv, tot = np.zeros(n), np.zeros(n), np.zeros(n)
    args = [_c64(x) for x in (q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed)]
    lib().orc_phase_integrate(sem, n, n_eff, _d(wave), grid, _d(_c64(temp)), _d(_c64(bi)),
                              _d(_c64(maps["delta"])), _d(_c64(maps["limb"])),
                              _i(np.ascontiguousarray(maps["region"], dtype=np.int32)),
                              _d(_c64(maps["lb"])), *[_d(x) for x in args], step, int(bool(solar)),
                              t_star, t_diff_fac, _d(flux), _d(bconv), _d(tot))
    return flux, bconv, tot


def ccf_mask(vel, line_wave, line_weight, wave_trim, step_size, wave_extend=100.0, mask_step=0.005,
             index_old=20000):
    vel, lw, lwt, wt = (_c64(x) for x in (vel, line_wave, line_weight, wave_trim))
    M = np.zeros((vel.size, wt.size))
    rc = lib().orc_ccf_mask(vel.size, _d(vel), lw.size, _d(lw), _d(lwt), wt.size, _d(wt), step_size,
                            wave_extend, mask_step, index_old, _d(M))
    if rc != 0:
        raise ValueError("oracle ccf_mask: line window outside the extended wavelength array "
                         "or slice size mismatch")
    return M


def ccf(M, spec):
    M = _c64(M)
    spec = _c64(spec)
    out = np.empty(M.shape[0])
    lib().orc_ccf(M.shape[0], M.shape[1], _d(M), _d(spec), _d(out))
    return out


def ccf_normalise(ccf_raw):
    c = _c64(ccf_raw).copy()
    lib().orc_ccf_normalise(c.size, _d(c))
    return c


def gauss_bis(x, y, err=None):
    x, y = _c64(x), _c64(y)
    n = x.size
    err = np.ones(n) if err is None else _c64(err)
    model = np.empty(n)
    par = np.empty(5)
    depth = np.empty(91)
    bis = np.empty(91)
    it = lib().orc_gauss_bis(n, _d(x), _d(y), _d(err), _d(model), _d(par), _d(depth), _d(bis))
    return dict(model=model, par=par, depth=depth, bis=bis, iters=it)


def num_threads():
    return lib().orc_num_threads()


# --------------------------------------------------------------------------
# numpy restatements of the reference's Python steps
# --------------------------------------------------------------------------

def lb_params(t_star, lb_g2, lb_k0, lb_m0, temp_array):
    """run_all_SOAP.py:8-34 LB_boundary / LB_params, reversed as at :140."""
    if t_star > 5778:
        bnd = np.array([0, 1])
    elif 5240 <= t_star <= 5778:
        bnd = np.array([0, 1])
    elif 3750 <= t_star < 5240:
        bnd = np.array([1, 2])
    else:
        bnd = np.array([1, 2])
    mu = np.linspace(0.1, 1, 10)
    lb = np.zeros(mu.size)
    temp_array = np.asarray(temp_array)
    for i in range(10):
        der = np.array([lb_g2[i], lb_k0[i], lb_m0[i]])
        p = np.polyfit(temp_array[bnd], der[bnd], 1)
        lb[i] = np.poly1d(p)(t_star)
    return np.polyfit(mu, lb, 3)[::-1]


def bisector_inject(wave, flux, mode, coeffs, coeffs_low=None, dep_cut=None, vcut=None, vshift=None, scale=1.0):
    """Bisector injection of one spectrum into every mu bin (numpy restatement).

    Follows CB_injection_faculae.py:191-244 (BIS_inject_spectral_active for mode 1,
    BIS_inject_spectral_quiet for mode 0) with Delta_wavelength (:119-123):
    * rv of pixel k from np.poly1d (Horner, highest power first);
    * in mode 1 the branches are taken in the reference's order:
      0.5 < f < dep_cut -> (up(f) + vshift) scale; f <= 0.5 -> (low(f) + vshift) scale;
      f > dep_cut -> (vcut + vshift) scale; otherwise no shift;
    * wave_new = wave + wave (sqrt((1 + b) / (1 - b)) - 1), b = rv / c;
    * the spectrum is re-sampled at wave by scipy's linear interp1d, which for 1-D
      float64 data delegates to numpy.interp: interval j with wn[j] <= x < wn[j + 1];
      y = f[j] where x == wn[j], else ((f[j + 1] - f[j]) / (wn[j + 1] - wn[j])) (x - wn[j])
      + f[j] (separate multiply and add), on the pixels strictly inside
      (min wave_new, max wave_new), 0 elsewhere.
    Returns n_mu x n.  Raises ValueError for a non-increasing shifted grid (scipy
    would sort it)."""
    wave = np.asarray(wave, dtype=np.float64)
    f = np.asarray(flux, dtype=np.float64)
    coeffs = np.atleast_2d(np.asarray(coeffs, dtype=np.float64))
    n_mu, n = coeffs.shape[0], wave.size
    out = np.zeros((n_mu, n))
    for b in range(n_mu):
        if mode == 0:
            rv = np.polyval(coeffs[b], f) * scale
            moved = np.ones(n, dtype=bool)
        else:
            up = (f < dep_cut[b]) & (f > 0.5)
            low = ~up & (f <= 0.5)
            cut = ~up & ~low & (f > dep_cut[b])
            rv = np.zeros(n)
            rv[up] = (np.polyval(coeffs[b], f[up]) + vshift[b]) * scale
            rv[low] = (np.polyval(np.asarray(coeffs_low)[b], f[low]) + vshift[b]) * scale
            rv[cut] = (vcut[b] + vshift[b]) * scale
            moved = up | low | cut
        beta = rv / C_LIGHT
        wn = np.where(moved, wave + wave * (np.sqrt((1 + beta) / (1 - beta)) - 1), wave)
        if not np.all(np.diff(wn) > 0):
            raise ValueError("bisector injection: shifted grid not increasing")
        sel = (wave < wn.max()) & (wave > wn.min())
        x = wave[sel]
        j = np.searchsorted(wn, x, side="right") - 1
        slope = (f[j + 1] - f[j]) / (wn[j + 1] - wn[j])
        y = slope * (x - wn[j]) + f[j]
        out[b, sel] = np.where(wn[j] == x, f[j], y)
    return out
