"""torch operators over libsoapgb: ``torch.ops.soapgb.*`` (csrc/torch/soapgb_torch.cpp).

The differentiable form's autograd Functions (``differentiable.py``) and the batched
form's runs (``api.Batch.run``) call the library through these operators: CUDA tensors in, CUDA tensors out (allocated by torch on the
inputs' device), on torch's current stream, an error status raised with the library's
message.  ``Ops(ctx)`` binds them to an ``api.Context`` with the argument conventions
of the context's own methods.  The operators are built by ``build.build()`` into
``lib/soapgb_torch.so``; without it the import fails (there is no other path).
"""
from __future__ import annotations

import os

import torch

from . import _lib
from ._lib import FORMS, Activity

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "soapgb_torch.so")
OPS = ("disk_maps", "quiet_disk", "phase_integrate", "phase_integrate_adjoint", "lower_resolution",
       "lower_resolution_adjoint", "ccf", "ccf_adjoint", "gauss_bis", "gauss_fit_adjoint", "batch_run", "synchronize")
_loaded = False


def load():
    """torch.ops.soapgb (loads lib/soapgb_torch.so once; libsoapgb first, so that the
    operators and the ctypes contexts share one library)."""
    global _loaded
    if not _loaded:
        if not os.path.exists(PATH):
            raise ImportError("soapgb_torch.so not built (%s); run __graft_entry__.build()" % PATH)
        _lib.load()
        if not _registered():   # (a build in this process has loaded its own copy)
            torch.ops.load_library(PATH)
        _loaded = True
    return torch.ops.soapgb


def _registered() -> bool:
    try:
        torch.ops.soapgb.synchronize
        return True
    except (AttributeError, RuntimeError):
        return False


def _form(form) -> int:
    return FORMS[form] if isinstance(form, str) else int(form)


def _act(act: Activity):
    return [int(act.t_star), int(act.t_diff_spot), int(act.t_diff_fac), int(act.nrho), int(act.solar)]


def _t(x):
    """float64, contiguous (None stays None)."""
    return None if x is None else x.to(torch.float64).contiguous()


def _row(t):
    """A continuum row: row 0 of an n_mu x n cube, or the row itself."""
    return _t(t[0] if t.dim() == 2 else t)


class Ops:
    """The operators bound to one context, with ``api.Context``'s signatures (device
    tensors only)."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.h = int(ctx.h.value)
        self.o = load()

    def disk_maps(self, grid, period, omega_ratio, incl, radius_km, u1, u2, mu_boundary, lb):
        d, l, mu, lbm, reg = self.o.disk_maps(self.h, int(grid), float(period), float(omega_ratio), float(incl),
                                              float(radius_km), float(u1), float(u2), _t(mu_boundary),
                                              [float(x) for x in lb])
        return {"delta": d, "limb": l, "mu": mu, "lb": lbm, "region": reg}

    def quiet_disk(self, form, wave, cube, n_eff, maps, grid, step):
        return self.o.quiet_disk(self.h, _form(form), _t(wave), _t(cube), int(n_eff), int(grid), maps["delta"],
                                 maps["limb"], maps["region"], float(step))

    def _mc(self, maps, cubes):
        return (_t(maps["delta"]), _t(maps["limb"]), maps["region"].to(torch.int32).contiguous(), _t(maps["lb"]),
                _t(cubes["q_norm"]), _t(cubes["q_sed"]), _t(cubes["spot_norm"]), _t(cubes["fac_norm"]),
                _row(cubes["spot_sed"]), _row(cubes["fac_sed"]))

    def phase_integrate(self, form, wave, n_eff, grid, temp, bi, maps, cubes, step, act: Activity):
        return self.o.phase_integrate(self.h, _form(form), _t(wave), int(n_eff), int(grid), _t(temp), _t(bi),
                                      *self._mc(maps, cubes), float(step), _act(act))

    def phase_integrate_adjoint(self, wave, n_eff, grid, temp, bi, maps, cubes, step, act: Activity, g_flux, g_bconv,
                                g_tot):
        g = self.o.phase_integrate_adjoint(self.h, _t(wave), int(n_eff), int(grid), _t(temp), _t(bi),
                                           *self._mc(maps, cubes), float(step), _act(act), _t(g_flux), _t(g_bconv),
                                           _t(g_tot))
        return dict(zip(("q_norm", "q_sed", "spot_norm", "fac_norm", "spot_sed", "fac_sed", "limb", "delta"), g))

    def lower_resolution(self, form, wave, spec, n_eff, sigma_v, base=None, window=50.0, step_mult=0.005,
                         step_exp=0.005, sentinel=-60000.0):
        single = spec.dim() == 1
        out, mm = self.o.lower_resolution(self.h, _form(form), _t(wave), _t(spec.reshape(1, -1) if single else spec),
                                          int(n_eff), float(sigma_v), _t(base), float(window), float(step_mult),
                                          float(step_exp), float(sentinel))
        return (out[0] if single else out), mm

    def lower_resolution_adjoint(self, wave, spec, n_eff, sigma_v, g_out, base=None, window=50.0, step_mult=0.005,
                                 step_exp=0.005, sentinel=-60000.0, want_base=True):
        return self.o.lower_resolution_adjoint(self.h, _t(wave), _t(spec), int(n_eff), float(sigma_v), _t(g_out),
                                               _t(base), float(window), float(step_mult), float(step_exp),
                                               float(sentinel), bool(want_base))

    def ccf(self, form, vel, line_wave, line_weight, wave_trim, step_size, spectra, normalise=True,
            wave_extend=100.0, mask_step=0.005, index_old=20000):
        single = spectra.dim() == 1
        out = self.o.ccf(self.h, _form(form), _t(vel), _t(line_wave), _t(line_weight), _t(wave_trim),
                         float(step_size), _t(spectra.reshape(1, -1) if single else spectra), bool(normalise),
                         float(wave_extend), float(mask_step), int(index_old))
        return out[0] if single else out

    def ccf_adjoint(self, vel, line_wave, line_weight, wave_trim, step_size, g_ccf, ccf_raw=None, normalise=True,
                    wave_extend=100.0, mask_step=0.005, index_old=20000):
        return self.o.ccf_adjoint(self.h, _t(vel), _t(line_wave), _t(line_weight), _t(wave_trim), float(step_size),
                                  _t(g_ccf), _t(ccf_raw), bool(normalise), float(wave_extend), float(mask_step),
                                  int(index_old))

    def gauss_bis(self, x, y, err=None):
        single = y.dim() == 1
        res = dict(zip(("model", "par", "depth", "bis", "iters"),
                       self.o.gauss_bis(self.h, _t(x), _t(y.reshape(1, -1) if single else y), _t(err))))
        return {k: v[0] for k, v in res.items()} if single else res

    def gauss_fit_adjoint(self, x, y, model, par, g_par, err=None):
        return self.o.gauss_fit_adjoint(self.h, _t(x), _t(y), _t(model), _t(par), _t(g_par), _t(err))

    def batch_run(self, batch, out=None, quiet=None):
        """One run of an ``api.Batch`` into ``out`` (allocated when None)."""
        return self.o.batch_run(self.h, int(batch.h.value), int(batch.total_phases), int(batch.n_eff),
                                int(self.ctx.device), out, quiet)

    def synchronize(self):
        self.o.synchronize(self.h)


def ops(ctx) -> Ops:
    """The operators bound to ``ctx`` (one binding per context)."""
    b = getattr(ctx, "_torch_ops", None)
    if b is None or b.h != int(ctx.h.value):
        b = Ops(ctx)
        ctx._torch_ops = b
    return b
