"""Python interface over libsoapgb.

``Context`` wraps one ``soapgb_ctx`` (one device, one stream).  Every method takes
either numpy arrays (host mode: the library copies in and out inside the call) or
CUDA ``torch`` tensors (device mode: no copies, asynchronous on the current torch
stream); results come back in the same kind.  Array layouts follow
``include/soapgb.h``.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import FORMS, Activity, BatchDesc, Cubes, Maps, SoapError, Star

try:  # torch is plumbing for device buffers and streams; numpy callers do not need it
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_dev(x):
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


# cudaStreamLegacy: the handle that names the legacy default stream explicitly
_CUDA_STREAM_LEGACY = 0x1


def torch_stream_handle(device: int) -> int:
    """The cudaStream_t of torch's current stream on ``device``, for soapgb_set_stream.

    torch's default stream is the legacy default stream, whose handle is 0; the C
    interface reads a null stream as "the context's own stream", a non-blocking stream
    with no ordering against the caller's work, so 0 becomes cudaStreamLegacy."""
    h = torch.cuda.current_stream(device).cuda_stream
    return h if h else _CUDA_STREAM_LEGACY


def _form(form):
    if isinstance(form, str):
        return FORMS[form]
    return int(form)


class _Args:
    """Collects pointers of one call, all host (numpy) or all device (torch)."""

    def __init__(self, device_mode: bool, device: int):
        self.dev = device_mode
        self.device = device
        self.keep = []

    def inp(self, x, dtype):
        if x is None:
            return None
        if self.dev:
            t = x if _is_dev(x) else torch.as_tensor(np.asarray(x), device="cuda:%d" % self.device)
            t = t.to(dtype=torch.float64 if dtype == np.float64 else torch.int32).contiguous()
            self.keep.append(t)
            return ctypes.c_void_p(t.data_ptr())
        a = np.ascontiguousarray(x, dtype=dtype)
        self.keep.append(a)
        return ctypes.c_void_p(a.ctypes.data)

    def desc(self, x, dtype):
        """A small descriptor array (phases, region tables): kept in host memory when it
        is given there, so that a device-buffer call need not synchronise to read it."""
        if x is None:
            return None
        if _is_dev(x):
            return self.inp(x, dtype)
        a = np.ascontiguousarray(x, dtype=dtype)
        self.keep.append(a)
        return ctypes.c_void_p(a.ctypes.data)

    def out(self, shape, dtype):
        if self.dev:
            t = torch.empty(shape, dtype=torch.float64 if dtype == np.float64 else torch.int32,
                            device="cuda:%d" % self.device)
            self.keep.append(t)
            return t, ctypes.c_void_p(t.data_ptr())
        a = np.empty(shape, dtype=dtype)
        self.keep.append(a)
        return a, ctypes.c_void_p(a.ctypes.data)

    @property
    def mem(self):
        return _lib.DEVICE if self.dev else _lib.HOST


class Context:
    def __init__(self, device: int = 0):
        self.L = _lib.load()
        self.device = device
        h = ctypes.c_void_p()
        rc = self.L.soapgb_ctx_create(device, ctypes.byref(h))
        self.h = h
        if rc != 0:
            msg = self.L.soapgb_last_error(h).decode() if h.value else "context creation failed"
            raise SoapError(rc, msg)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.soapgb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- helpers ----------------------------------------------------------------
    def _check(self, rc):
        if rc != 0:
            raise SoapError(rc, self.L.soapgb_last_error(self.h).decode())

    def _args(self, *xs):
        dev = any(_is_dev(x) for x in xs if x is not None)
        if dev:
            self.L.soapgb_set_stream(self.h, ctypes.c_void_p(torch_stream_handle(self.device)))
        else:
            self.L.soapgb_set_stream(self.h, None)
        return _Args(dev, self.device)

    def synchronize(self):
        self._check(self.L.soapgb_synchronize(self.h))

    def set_compensated(self, on: bool = True):
        """Compensated (Kahan) instead of plain FP32 output sums in the FP32 form's
        per-phase integration (soapgb_set_compensated)."""
        self._check(self.L.soapgb_set_compensated(self.h, 1 if on else 0))

    @property
    def launches(self) -> int:
        return int(self.L.soapgb_launch_count(self.h))

    def trace(self, on: bool = True):
        """Start (or stop) recording CUDA-event times of the library's kernels."""
        self._check(self.L.soapgb_trace_enable(self.h, 1 if on else 0))

    def trace_report(self) -> dict:
        """{kernel: (launches, total ms)} recorded since tracing started or the last report."""
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self.L.soapgb_trace_report(self.h, buf, len(buf)))
        out = {}
        for ln in buf.value.decode().splitlines():
            name, cnt, ms = ln.rsplit(" ", 2)
            out[name] = (int(cnt), float(ms))
        return out

    # -- a3 ---------------------------------------------------------------------
    def disk_maps(self, grid, period, omega_ratio, incl, radius_km, u1, u2, mu_boundary, lb):
        a = self._args(mu_boundary)
        st = Star(int(grid), period, omega_ratio, incl, radius_km, u1, u2, (ctypes.c_double * 4)(*lb))
        mu_p = a.inp(mu_boundary if len(mu_boundary) else np.zeros(1), np.float64)
        gm = int(grid) * int(grid)
        outs = {}
        ptrs = {}
        for k in ("delta", "limb", "mu", "lb"):
            outs[k], ptrs[k] = a.out(gm, np.float64)
        outs["region"], ptrs["region"] = a.out(gm, np.int32)
        m = Maps(ptrs["delta"], ptrs["limb"], ptrs["mu"], ptrs["region"], ptrs["lb"])
        self._check(self.L.soapgb_disk_maps(self.h, ctypes.byref(st), len(mu_boundary) + 1, mu_p, a.mem,
                                            ctypes.byref(m)))
        return outs

    # -- a4-a7 ------------------------------------------------------------------
    def quiet_disk(self, form, wave, cube, n_eff, maps, grid, step):
        a = self._args(wave, cube, maps["delta"])
        cube_shape = cube.shape
        n = int(wave.shape[0])
        n_mu = int(cube_shape[0]) if len(cube_shape) == 2 else 1
        out, op = a.out(n, np.float64)
        self._check(self.L.soapgb_quiet_disk(self.h, _form(form), n, int(n_eff), a.inp(wave, np.float64),
                                             a.inp(cube, np.float64), n_mu, int(grid),
                                             a.inp(maps["delta"], np.float64), a.inp(maps["limb"], np.float64),
                                             a.inp(maps["region"], np.int32), float(step), a.mem, op))
        return out

    # -- a8 / a14 ---------------------------------------------------------------
    def lower_resolution(self, form, wave, spec, n_eff, sigma_v, base=None, window=50.0, step_mult=0.005,
                         step_exp=0.005, sentinel=-60000.0):
        """Returns (out[n_spec, n_eff] or out[n_eff], minmax[n_spec, 2])."""
        a = self._args(wave, spec, base)
        single = len(spec.shape) == 1
        n = int(wave.shape[0])
        n_spec = 1 if single else int(spec.shape[0])
        out, op = a.out((n_spec, int(n_eff)), np.float64)
        mm, mp = a.out((n_spec, 2), np.float64)
        self._check(self.L.soapgb_lower_resolution(self.h, _form(form), n, int(n_eff), n_spec,
                                                   a.inp(wave, np.float64), a.inp(base, np.float64),
                                                   a.inp(spec, np.float64), sigma_v, window, step_mult, step_exp,
                                                   sentinel, a.mem, op, mp))
        return (out[0] if single else out), mm

    def lower_resolution_adjoint(self, wave, spec, n_eff, sigma_v, g_out, base=None, window=50.0, step_mult=0.005,
                                 step_exp=0.005, sentinel=-60000.0, want_base=True):
        """Gradients of a scalar through lower_resolution (PLAIN64 arithmetic), given its
        gradient g_out (n_spec x n_eff) w.r.t. the output: (grad_spec (n_spec x n),
        grad_base (n) or None), grad_base summed over the spectra."""
        a = self._args(wave, spec, base, g_out)
        n = int(wave.shape[0])
        n_spec = int(spec.shape[0])
        gs, gsp = a.out((n_spec, n), np.float64)
        gb, gbp = a.out((n,), np.float64) if (base is not None and want_base) else (None, None)
        self._check(self.L.soapgb_lower_resolution_adjoint(
            self.h, n, int(n_eff), n_spec, a.inp(wave, np.float64), a.inp(base, np.float64), a.inp(spec, np.float64),
            sigma_v, window, step_mult, step_exp, sentinel, a.inp(g_out, np.float64), a.mem, gsp, gbp))
        return gs, gb

    # -- seed preparation: bisector injection (CB_injection_faculae.py:191-244) ----------
    def bisector_inject(self, wave, flux, coeffs, coeffs_low=None, dep_cut=None, vcut=None, vshift=None,
                        scale=1.0):
        """Inject a per-mu-bin bisector into one spectrum: out[n_mu, n].

        coeffs (n_mu x n_coef, highest power first) alone gives the quiet form
        (BIS_inject_spectral_quiet); with coeffs_low, dep_cut, vcut and vshift (one row
        or value per mu bin) the active form (BIS_inject_spectral_active)."""
        a = self._args(wave, flux, coeffs)
        active = coeffs_low is not None
        c = coeffs if a.dev else np.atleast_2d(np.asarray(coeffs, dtype=np.float64))
        n_mu, n_coef = int(c.shape[0]), int(c.shape[1])
        n = int(wave.shape[0])
        out, op = a.out((n_mu, n), np.float64)
        self._check(self.L.soapgb_bisector_inject(
            self.h, 1 if active else 0, n, n_mu, n_coef, a.inp(wave, np.float64), a.inp(flux, np.float64),
            a.inp(c, np.float64), a.inp(coeffs_low, np.float64) if active else None,
            a.inp(dep_cut, np.float64) if active else None, a.inp(vcut, np.float64) if active else None,
            a.inp(vshift, np.float64) if active else None, float(scale), a.mem, op))
        return out

    # -- a9-a10 -----------------------------------------------------------------
    @staticmethod
    def _regions(regions_per_phase: Sequence[np.ndarray]):
        off = np.zeros(len(regions_per_phase) + 1, dtype=np.int32)
        rows = []
        for p, r in enumerate(regions_per_phase):
            r = np.asarray(r, dtype=np.float64).reshape(-1, 4)
            rows.append(r)
            off[p + 1] = off[p] + r.shape[0]
        reg = np.concatenate(rows, axis=0) if rows and off[-1] > 0 else np.zeros((1, 4))
        return off, reg

    def phase_maps(self, grid, incl, phases, regions_per_phase, act: Activity):
        a = self._args(phases)
        off, reg = self._regions(regions_per_phase)
        n_phase = len(phases)
        gm = int(grid) ** 2
        temp, tp = a.out((n_phase, gm), np.float64)
        bi, bp = a.out((n_phase, gm), np.float64)
        self._check(self.L.soapgb_phase_maps(self.h, int(grid), float(incl), n_phase, a.inp(phases, np.float64),
                                             a.inp(off, np.int32), a.inp(reg, np.float64), ctypes.byref(act), a.mem,
                                             tp, bp))
        return temp, bi

    # -- a11-a12 ----------------------------------------------------------------
    def phase_integrate(self, form, wave, n_eff, grid, temp, bi, maps, cubes: dict, step, act: Activity):
        a = self._args(wave, temp, cubes["q_norm"])
        n = int(wave.shape[0])
        n_phase = int(temp.shape[0])
        n_mu = int(cubes["q_norm"].shape[0])
        m = Maps(a.inp(maps["delta"], np.float64), a.inp(maps["limb"], np.float64), None,
                 a.inp(maps["region"], np.int32), a.inp(maps["lb"], np.float64))
        c = Cubes(*[a.inp(cubes[k], np.float64) for k in ("q_norm", "q_sed", "spot_norm", "fac_norm")],
                  a.inp(cubes["spot_sed"][0] if len(cubes["spot_sed"].shape) == 2 else cubes["spot_sed"],
                        np.float64),
                  a.inp(cubes["fac_sed"][0] if len(cubes["fac_sed"].shape) == 2 else cubes["fac_sed"], np.float64),
                  n_mu)
        flux, fp = a.out((n_phase, n), np.float64)
        bconv, bp = a.out((n_phase, n), np.float64)
        tot, tp = a.out((n_phase, n), np.float64)
        self._check(self.L.soapgb_phase_integrate(self.h, _form(form), n, int(n_eff), a.inp(wave, np.float64),
                                                  int(grid), n_phase, a.inp(temp, np.float64),
                                                  a.inp(bi, np.float64), ctypes.byref(m), ctypes.byref(c),
                                                  float(step), ctypes.byref(act), a.mem, fp, bp, tp))
        return flux, bconv, tot

    def phase_integrate_adjoint(self, wave, n_eff, grid, temp, bi, maps, cubes: dict, step, act: Activity,
                                g_flux, g_bconv, g_tot):
        """Gradients of a scalar through phase_integrate (PLAIN64 arithmetic), given its
        gradients g_flux, g_bconv, g_tot (n_phase x n) w.r.t. the outputs: a dict with the
        four cubes (n_mu x n), the two continuum rows ("spot_sed", "fac_sed", n), the limb
        map ("limb", G*G) and the velocity map ("delta", G*G), each summed over the phases."""
        a = self._args(wave, temp, cubes["q_norm"])
        n = int(wave.shape[0])
        n_phase = int(temp.shape[0])
        n_mu = int(cubes["q_norm"].shape[0])
        m = Maps(a.inp(maps["delta"], np.float64), a.inp(maps["limb"], np.float64), None,
                 a.inp(maps["region"], np.int32), a.inp(maps["lb"], np.float64))
        c = Cubes(*[a.inp(cubes[k], np.float64) for k in ("q_norm", "q_sed", "spot_norm", "fac_norm")],
                  a.inp(cubes["spot_sed"][0] if len(cubes["spot_sed"].shape) == 2 else cubes["spot_sed"],
                        np.float64),
                  a.inp(cubes["fac_sed"][0] if len(cubes["fac_sed"].shape) == 2 else cubes["fac_sed"], np.float64),
                  n_mu)
        out = {}
        ptrs = []
        for k, shape in (("q_norm", (n_mu, n)), ("q_sed", (n_mu, n)), ("spot_norm", (n_mu, n)),
                         ("fac_norm", (n_mu, n)), ("spot_sed", (n,)), ("fac_sed", (n,)), ("limb", (int(grid) ** 2,)),
                         ("delta", (int(grid) ** 2,))):
            out[k], pk = a.out(shape, np.float64)
            ptrs.append(pk)
        self._check(self.L.soapgb_phase_integrate_adjoint(
            self.h, n, int(n_eff), a.inp(wave, np.float64), int(grid), n_phase, a.inp(temp, np.float64),
            a.inp(bi, np.float64), ctypes.byref(m), ctypes.byref(c), float(step), ctypes.byref(act),
            a.inp(g_flux, np.float64), a.inp(g_bconv, np.float64), a.inp(g_tot, np.float64), a.mem, *ptrs))
        return out

    # -- a15-a16 ----------------------------------------------------------------
    def ccf(self, form, vel, line_wave, line_weight, wave_trim, step_size, spectra, normalise=True,
            wave_extend=100.0, mask_step=0.005, index_old=20000):
        a = self._args(spectra, wave_trim)
        single = len(spectra.shape) == 1
        n_spec = 1 if single else int(spectra.shape[0])
        n_v = len(vel)
        out, op = a.out((n_spec, n_v), np.float64)
        self._check(self.L.soapgb_ccf(self.h, _form(form), n_v, a.inp(vel, np.float64), len(line_wave),
                                      a.inp(line_wave, np.float64), a.inp(line_weight, np.float64),
                                      int(wave_trim.shape[0]), a.inp(wave_trim, np.float64), float(step_size),
                                      float(wave_extend), float(mask_step), int(index_old), n_spec,
                                      a.inp(spectra, np.float64), int(bool(normalise)), a.mem, op))
        return out[0] if single else out

    def ccf_adjoint(self, vel, line_wave, line_weight, wave_trim, step_size, g_ccf, ccf_raw=None, normalise=True,
                    wave_extend=100.0, mask_step=0.005, index_old=20000):
        """Gradient (n_spec x n_w) of a scalar w.r.t. the spectra of ccf, given its
        gradient g_ccf (n_spec x n_v) w.r.t. the CCF; ccf_raw: the raw sums (needed when
        normalise is set)."""
        a = self._args(g_ccf, wave_trim)
        n_spec, n_v = int(g_ccf.shape[0]), len(vel)
        out, op = a.out((n_spec, int(wave_trim.shape[0])), np.float64)
        self._check(self.L.soapgb_ccf_adjoint(self.h, n_v, a.inp(vel, np.float64), len(line_wave),
                                              a.inp(line_wave, np.float64), a.inp(line_weight, np.float64),
                                              int(wave_trim.shape[0]), a.inp(wave_trim, np.float64), float(step_size),
                                              float(wave_extend), float(mask_step), int(index_old), n_spec,
                                              a.inp(ccf_raw, np.float64), int(bool(normalise)),
                                              a.inp(g_ccf, np.float64), a.mem, op))
        return out

    def gauss_fit_adjoint(self, x, y, model, par, g_par, err=None):
        """Gradient (n_spec x n) of a scalar w.r.t. the fitted CCFs y, given its gradient
        g_par (n_spec x 5) w.r.t. the fit's par = (c, |k|, span, v0, fwhm), the bisector
        span's with its per-depth crossing intervals held fixed."""
        a = self._args(y, x)
        n_spec, n = int(y.shape[0]), int(x.shape[0])
        out, op = a.out((n_spec, n), np.float64)
        self._check(self.L.soapgb_gauss_fit_adjoint(self.h, n_spec, n, a.inp(x, np.float64), a.inp(y, np.float64),
                                                    a.inp(err, np.float64), a.inp(model, np.float64),
                                                    a.inp(par, np.float64), a.inp(g_par, np.float64), a.mem, op))
        return out

    # -- a17-a18 ----------------------------------------------------------------
    def gauss_bis(self, x, y, err=None):
        a = self._args(y, x)
        single = len(y.shape) == 1
        n_spec = 1 if single else int(y.shape[0])
        n = int(x.shape[0])
        model, mp = a.out((n_spec, n), np.float64)
        par, pp = a.out((n_spec, 5), np.float64)
        depth, dp = a.out((n_spec, 91), np.float64)
        bis, bp = a.out((n_spec, 91), np.float64)
        it, ip = a.out(n_spec, np.int32)
        self._check(self.L.soapgb_gauss_bis(self.h, n_spec, n, a.inp(x, np.float64), a.inp(y, np.float64),
                                            a.inp(err, np.float64), a.mem, mp, pp, dp, bp, ip))
        res = dict(model=model, par=par, depth=depth, bis=bis, iters=it)
        if single:
            res = {k: v[0] for k, v in res.items()}
        return res

    # -- composite --------------------------------------------------------------
    def phase_pipeline(self, form, wave, n_eff, star: Star, maps, cubes: dict, step, act: Activity, phases,
                       regions_per_phase, quiet_sed, quiet_norm, sigma_v, conv_step=0.005, sentinel=-60000.0,
                       want_raw=False, out=None, raw_out=None):
        """lower[n_phase, 3, n_eff] (tot, flux, bconv) and optionally raw[n_phase, 3, n_eff]."""
        a = self._args(wave, cubes["q_norm"], quiet_sed)
        n = int(wave.shape[0])
        n_phase = len(phases)
        n_mu = int(cubes["q_norm"].shape[0])
        off, reg = self._regions(regions_per_phase)
        m = Maps(a.inp(maps["delta"], np.float64), a.inp(maps["limb"], np.float64), None,
                 a.inp(maps["region"], np.int32), a.inp(maps["lb"], np.float64))
        c = Cubes(*[a.inp(cubes[k], np.float64) for k in ("q_norm", "q_sed", "spot_norm", "fac_norm")],
                  a.inp(cubes["spot_sed"][0] if len(cubes["spot_sed"].shape) == 2 else cubes["spot_sed"],
                        np.float64),
                  a.inp(cubes["fac_sed"][0] if len(cubes["fac_sed"].shape) == 2 else cubes["fac_sed"], np.float64),
                  n_mu)
        if out is not None:
            lower, lp = out, ctypes.c_void_p(out.data_ptr() if a.dev else out.ctypes.data)
        else:
            lower, lp = a.out((n_phase, 3, int(n_eff)), np.float64)
        raw, rp = None, None
        if want_raw:
            if raw_out is not None:
                raw, rp = raw_out, ctypes.c_void_p(raw_out.data_ptr() if a.dev else raw_out.ctypes.data)
            else:
                raw, rp = a.out((n_phase, 3, int(n_eff)), np.float64)
        self._check(self.L.soapgb_phase_pipeline(self.h, _form(form), n, int(n_eff), a.inp(wave, np.float64),
                                                 ctypes.byref(star), ctypes.byref(m), ctypes.byref(c), float(step),
                                                 ctypes.byref(act), n_phase, a.desc(phases, np.float64),
                                                 a.desc(off, np.int32), a.desc(reg, np.float64),
                                                 a.inp(quiet_sed, np.float64), a.inp(quiet_norm, np.float64),
                                                 float(sigma_v), float(conv_step), float(sentinel), a.mem, lp, rp))
        return (lower, raw) if want_raw else lower


class Batch:
    """Many stars through the per-phase path in one job (soapgb_batch_create / _run).

    The stars share the wavelength grid ``wave`` and the seed cubes (CUDA tensors, kept
    alive by this object); ``stars`` is a list of Star structures, ``phases`` a list of
    per-star phase arrays and ``regions`` a list (per star) of lists (per phase) of
    (n, 4) region tables.  ``run()`` enqueues the whole job on torch's current stream
    without reading host memory or synchronising, so it may be captured in a CUDA graph;
    it returns the (total phases, 3, n_eff) normalised spectra, star s at rows
    ``offsets[s]:offsets[s + 1]``."""

    def __init__(self, ctx: "Context", wave, n_eff, cubes: dict, mu_boundary, step, act: Activity, sigma_v,
                 stars: Sequence[Star], phases: Sequence, regions: Sequence, conv_step=None, sentinel=-60000.0,
                 chunk=0, blocks_per_sm=0, form="fast32"):
        self.ctx = ctx
        L = ctx.L
        dev = "cuda:%d" % ctx.device
        T = lambda a: (a if _is_dev(a) else torch.as_tensor(np.ascontiguousarray(a), device=dev)).to(
            torch.float64).contiguous()
        self.wave = T(wave)
        self.n = int(self.wave.shape[0])
        self.n_eff = int(n_eff)
        self.cube_t = {k: T(cubes[k]) for k in ("q_norm", "q_sed", "spot_norm", "fac_norm")}
        for k in ("spot_sed", "fac_sed"):
            v = cubes[k]
            self.cube_t[k] = T(v[0] if len(v.shape) == 2 else v)
        n_mu = int(self.cube_t["q_norm"].shape[0])
        self.cubes = Cubes(*[ctypes.c_void_p(self.cube_t[k].data_ptr()) for k in
                             ("q_norm", "q_sed", "spot_norm", "fac_norm", "spot_sed", "fac_sed")], n_mu)
        self.n_star = len(stars)
        self.offsets = np.zeros(self.n_star + 1, dtype=np.int32)
        for s, ph in enumerate(phases):
            self.offsets[s + 1] = self.offsets[s] + len(ph)
        ph_all = np.ascontiguousarray(np.concatenate([np.asarray(p, dtype=np.float64) for p in phases]))
        reg_rows = [np.asarray(r, dtype=np.float64).reshape(-1, 4) for per_star in regions for r in per_star]
        if len(reg_rows) != ph_all.size:
            raise ValueError("one region table per phase")
        roff = np.zeros(ph_all.size + 1, dtype=np.int32)
        roff[1:] = np.cumsum([r.shape[0] for r in reg_rows])
        reg = np.ascontiguousarray(np.concatenate(reg_rows) if roff[-1] > 0 else np.zeros((1, 4)))
        mu_b = np.ascontiguousarray(np.asarray(mu_boundary, dtype=np.float64))
        self.stars = (Star * self.n_star)(*stars)
        self._host = (ph_all, roff, reg, mu_b)
        desc = BatchDesc(_form(form), self.n, self.n_eff, ctypes.c_void_p(self.wave.data_ptr()),
                         ctypes.pointer(self.cubes), ctypes.c_void_p(mu_b.ctypes.data), float(step), act,
                         float(sigma_v), float(step if conv_step is None else conv_step), float(sentinel),
                         self.n_star, self.stars, ctypes.c_void_p(self.offsets.ctypes.data),
                         ctypes.c_void_p(ph_all.ctypes.data), ctypes.c_void_p(roff.ctypes.data),
                         ctypes.c_void_p(reg.ctypes.data), int(chunk), int(blocks_per_sm))
        h = ctypes.c_void_p()
        ctx.L.soapgb_set_stream(ctx.h, ctypes.c_void_p(torch_stream_handle(ctx.device)))
        ctx._check(L.soapgb_batch_create(ctx.h, ctypes.byref(desc), ctypes.byref(h)))
        self.h = h
        self.total_phases = int(self.offsets[-1])

    @property
    def device_bytes(self) -> int:
        return int(self.ctx.L.soapgb_batch_device_bytes(self.h))

    @property
    def items(self) -> int:
        return int(self.ctx.L.soapgb_batch_items(self.h))

    def tune(self, chunk: int, blocks_per_sm: int):
        self.ctx._check(self.ctx.L.soapgb_batch_tune(self.h, int(chunk), int(blocks_per_sm)))

    def run(self, out=None, quiet=None):
        """Enqueues the batch on torch's current stream (torch.ops.soapgb.batch_run)."""
        from .torch_ops import ops
        return ops(self.ctx).batch_run(self, out, quiet)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.ctx.L.soapgb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def version() -> str:
    return _lib.load().soapgb_version().decode()
