"""Differentiable per-phase integration (the first slice of the differentiable form).

``DeficitSpectra`` is a ``torch.autograd.Function`` over ``soapgb_phase_integrate`` in
the PLAIN64 arithmetic (SOAP_integration.cu:392-447, spot_integrate): the three deficit
spectra (flux, bconv, tot) of every phase as a function of

* the limb-darkening coefficients u1, u2 (through the limb map of the disk,
  L = 1 - u1 (1 - mu) - u2 (1 - mu)^2, SOAP_initialize.cu:365-366),
* vsini (the cells' velocities scale with it: the rotation period is
  2 pi R / (vsini 86400)), and
* the seed spectra: the quiet normalised and SED cubes, the spot and facula
  normalised cubes, and the spot and facula continuum rows.

Its backward runs the hand-written adjoint kernels of ``soapgb_phase_integrate_adjoint``
(deterministic gathers, no atomics) and applies the chain rules dL/du1 = -(1 - mu),
dL/du2 = -(1 - mu)^2 to the limb-map gradient and d delta / d vsini = delta / vsini to
the velocity-map gradient.  The outputs are linear in the limb values and the seed
spectra (gradients exact up to rounding) and continuous, piecewise smooth in the
velocities; the tests check them against FP64 central differences and a dot-product
identity.

``LowerResolution`` continues the chain through the resolution step
(SOAP_resolution.cu:216-310, PLAIN64): the Gaussian convolution and the min/max
normalisation of base - spec, by the hand-written adjoint of
``soapgb_lower_resolution_adjoint``.  ``NormalisedCcf`` (CCF_func.py:5-91) and
``GaussFit`` (BIS_FIT2.cpp:97-192) carry it to the RV: the mask CCF's transpose
(``soapgb_ccf_adjoint``) and the fit's implicit derivative at its optimum
(``soapgb_gauss_fit_adjoint``), so a loss on an RV curve reaches u1, u2 and vsini.

``QuietSpectrum`` differentiates the quiet-star disk sum (SOAP_initialize.cu:339-395)
in the same parameters: it is the integration of every visible cell with the quiet
cube's row, so its adjoint is ``soapgb_phase_integrate_adjoint`` on one phase in which
every visible cell is active (bconv = the quiet sum when the spot rows are zero).

The star vector is (u1, u2, vsini[, inclination in degrees]).  The inclination enters
the cells' velocities, v = y omega sin(i) (SOAP_initialize.cu:351), so d delta / d i =
delta cot(i); the region maps' coverage, which also moves with the inclination (the rim
rotation, SOAP_integration.cu:125-161), stays discrete like the regions' positions and
sizes.  The region contrast is the level of the spot and facula continuum rows
(SOAP_integration.cu:309-323: the Planck ratio of a spot is exactly 1, so its intensity
is its continuum row): a caller scales those rows by contrast parameters and autograd
carries the continuum-row gradients to them.

``GaussFitBis`` adds the bisector span (BIS_FIT2.cpp:214-268) to the fitted parameters;
``rv_series_checkpointed`` runs the chain phase chunk by phase chunk under
``torch.utils.checkpoint``, keeping only each chunk's fitted parameters for the backward
pass and recomputing the chunk's spectra there.

Region positions and sizes stay discrete (cell coverage), as in the reference.

Every call into the library here goes through the torch operators of
``torch_ops`` (``torch.ops.soapgb.*``, the C++ extension over the C ABI): CUDA tensors
in and out, on torch's current stream.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import torch

from ._lib import Activity
from .api import Context
from .torch_ops import ops

CUBE_KEYS = ("q_norm", "q_sed", "spot_norm", "fac_norm", "spot_sed", "fac_sed")


@dataclasses.dataclass
class IntegrationSetup:
    """What the integration depends on besides the differentiated inputs (device
    buffers): the star's disk geometry, the phases' region maps, the grid step."""
    ctx: Context
    wave: torch.Tensor           # (n,) float64
    n_eff: int
    grid: int
    period: float
    omega_ratio: float
    incl: float
    radius_km: float
    mu_boundary: torch.Tensor    # (n_mu - 1,) float64
    lb: tuple                    # facula limb-brightening cubic
    temp: torch.Tensor           # (n_phase, G*G) from Context.phase_maps
    bi: torch.Tensor
    step: float
    act: Activity

    @classmethod
    def build(cls, ctx, wave, n_eff, grid, period, omega_ratio, incl, radius_km, mu_boundary, lb, phases,
              regions_per_phase, act, step, device="cuda:0"):
        dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=device)
        temp, bi = ctx.phase_maps(grid, incl, np.asarray(phases, dtype=np.float64), regions_per_phase, act)
        return cls(ctx, dev(wave), int(n_eff), int(grid), float(period), float(omega_ratio), float(incl),
                   float(radius_km), dev(mu_boundary), tuple(float(x) for x in lb), dev(temp), dev(bi), float(step),
                   act)

    @property
    def vsini(self) -> float:
        """Equatorial velocity [km/s] of the setup's rotation period."""
        return 2 * np.pi * self.radius_km / (self.period * 86400.0)

    def maps(self, u1: float, u2: float, vsini: float, incl: float = None) -> dict:
        """The disk maps for limb-darkening coefficients (u1, u2), vsini and the
        inclination (default: the setup's, which fixed the region maps), on the device."""
        period = 2 * np.pi * self.radius_km / (vsini * 86400.0)
        return ops(self.ctx).disk_maps(self.grid, period, self.omega_ratio, self.incl if incl is None else incl,
                                  self.radius_km, u1, u2, self.mu_boundary, self.lb)

    def phases(self, p0: int, p1: int) -> "IntegrationSetup":
        """The same setup restricted to phases [p0, p1)."""
        return dataclasses.replace(self, temp=self.temp[p0:p1], bi=self.bi[p0:p1])

    @property
    def n_phase(self) -> int:
        return int(self.temp.shape[0])


def _star_maps(setup: IntegrationSetup, star):
    incl = float(star[3]) if star.numel() > 3 else None
    return setup.maps(float(star[0]), float(star[1]), float(star[2]), incl), incl


def _star_grad(star, maps, gl, gd, vsini, incl):
    """Chain rules from the limb and velocity map gradients to (u1, u2, vsini[, incl])
    over the visible cells: L = 1 - u1 (1 - mu) - u2 (1 - mu)^2, delta proportional to
    vsini and to sin(i)."""
    vis = maps["limb"] > -998.0
    zero = torch.zeros_like(maps["mu"])
    om = torch.where(vis, 1.0 - maps["mu"], zero)
    dl = torch.where(vis, maps["delta"], zero)
    g = [-(gl * om).sum(), -(gl * om * om).sum(), (gd * dl).sum() / vsini]
    if star.numel() > 3:
        rad = np.pi / 180.0
        g.append((gd * dl).sum() * rad * np.cos(incl * rad) / np.sin(incl * rad))
    return torch.stack(g).to(star.dtype)


class DeficitSpectra(torch.autograd.Function):
    """out[p, (flux, bconv, tot), :] = phase_integrate(star, cubes), star = (u1, u2, vsini);
    see the module text."""

    @staticmethod
    def forward(fctx, star, q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed, setup: IntegrationSetup):
        vsini = float(star[2])
        maps, incl = _star_maps(setup, star)
        fctx.vsini, fctx.incl, fctx.star = vsini, incl, star.detach()
        cubes = dict(zip(CUBE_KEYS, (q_norm.detach(), q_sed.detach(), spot_norm.detach(), fac_norm.detach(),
                                     spot_sed.detach(), fac_sed.detach())))
        flux, bconv, tot = ops(setup.ctx).phase_integrate("plain64", setup.wave, setup.n_eff, setup.grid,
                                                          setup.temp, setup.bi, maps, cubes, setup.step, setup.act)
        fctx.setup = setup
        fctx.maps = maps
        fctx.cubes = cubes
        return torch.stack((flux, bconv, tot), dim=1)

    @staticmethod
    def backward(fctx, g):
        setup, maps = fctx.setup, fctx.maps
        g = g.to(torch.float64)
        gr = ops(setup.ctx).phase_integrate_adjoint(setup.wave, setup.n_eff, setup.grid, setup.temp, setup.bi,
                                                    maps, fctx.cubes, setup.step, setup.act, g[:, 0].contiguous(),
                                                    g[:, 1].contiguous(), g[:, 2].contiguous())
        grad_star = _star_grad(fctx.star, maps, gr["limb"], gr["delta"], fctx.vsini, fctx.incl)
        return (grad_star, gr["q_norm"], gr["q_sed"], gr["spot_norm"], gr["fac_norm"], gr["spot_sed"],
                gr["fac_sed"], None)


def deficit_spectra(star, q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed, setup: IntegrationSetup):
    """Differentiable (n_phase, 3, n) deficit spectra, star = (u1, u2, vsini); see
    ``DeficitSpectra``."""
    return DeficitSpectra.apply(star, q_norm, q_sed, spot_norm, fac_norm, spot_sed, fac_sed, setup)


class QuietSpectrum(torch.autograd.Function):
    """The quiet-star disk sum of one cube (``soapgb_quiet_disk``, PLAIN64,
    SOAP_initialize.cu:339-395) as a function of star = (u1, u2, vsini[, incl]) and the
    cube.  Backward: the integration adjoint on one phase in which every visible cell is
    active with the quiet cube as its normalised row and zero active rows, so that its
    bconv output is exactly the quiet sum."""

    @staticmethod
    def forward(fctx, star, cube, setup: IntegrationSetup):
        maps, incl = _star_maps(setup, star)
        c = cube.detach().contiguous()
        out = ops(setup.ctx).quiet_disk("plain64", setup.wave, c, setup.n_eff, maps, setup.grid, setup.step)
        fctx.setup, fctx.maps, fctx.cube, fctx.star = setup, maps, c, star.detach()
        fctx.vsini, fctx.incl = float(star[2]), incl
        return out.reshape(-1)

    @staticmethod
    def backward(fctx, g):
        setup, maps = fctx.setup, fctx.maps
        act = setup.act
        vis = (maps["limb"] > -998.0).reshape(1, -1)
        # every visible cell a spot (the spot intensity ratio is 1, so its temperature is moot)
        bi = torch.where(vis, 0.0, -9999.0).to(torch.float64)
        temp = torch.where(vis, float(act.t_star - act.t_diff_spot), -9999.0).to(torch.float64)
        zc = torch.zeros_like(fctx.cube)
        zr = torch.zeros_like(setup.wave)
        cubes = dict(q_norm=fctx.cube, q_sed=zc, spot_norm=zc, fac_norm=zc, spot_sed=zr, fac_sed=zr)
        # only bconv carries a gradient: the adjoint skips the continuum rows' pass
        gr = ops(setup.ctx).phase_integrate_adjoint(setup.wave, setup.n_eff, setup.grid, temp, bi, maps, cubes,
                                                    setup.step, act, None,
                                                    g.to(torch.float64).reshape(1, -1).contiguous(), None)
        return _star_grad(fctx.star, maps, gr["limb"], gr["delta"], fctx.vsini, fctx.incl), gr["q_norm"], None


def quiet_spectrum(star, cube, setup: IntegrationSetup):
    """Differentiable (n,) quiet-star spectrum of ``cube``; see ``QuietSpectrum``."""
    return QuietSpectrum.apply(star, cube, setup)


@dataclasses.dataclass
class ResolutionSetup:
    """The fixed arguments of the resolution step (SOAP_resolution.cu:216-310): the
    wavelength grid (device, float64), n_eff and the instrument's sigma_v, the window
    and the reference's step constants."""
    ctx: Context
    wave: torch.Tensor
    n_eff: int
    sigma_v: float
    window: float = 50.0
    step_mult: float = 0.005
    step_exp: float = 0.005
    sentinel: float = -60000.0

    def kwargs(self) -> dict:
        return dict(window=self.window, step_mult=self.step_mult, step_exp=self.step_exp, sentinel=self.sentinel)


class LowerResolution(torch.autograd.Function):
    """out[s] = 1 - C_s (1 - min A_s) / max C_s with A_s = base - spec[s] and C_s the
    instrumental Gaussian convolution of 1 - A_s (``soapgb_lower_resolution``, PLAIN64).
    The backward runs ``soapgb_lower_resolution_adjoint``: the transposed tap gather and
    the normalisation's derivative, the extrema differentiated at their first pixel."""

    @staticmethod
    def forward(fctx, spec, base, setup: ResolutionSetup):
        spec_d, base_d = spec.detach().contiguous(), base.detach().contiguous()
        out, _ = ops(setup.ctx).lower_resolution("plain64", setup.wave, spec_d, setup.n_eff, setup.sigma_v,
                                                 base=base_d, **setup.kwargs())
        fctx.setup, fctx.spec, fctx.base = setup, spec_d, base_d
        fctx.want_base = base.requires_grad
        return out

    @staticmethod
    def backward(fctx, g):
        setup = fctx.setup
        gs, gb = ops(setup.ctx).lower_resolution_adjoint(setup.wave, fctx.spec, setup.n_eff, setup.sigma_v,
                                                         g.to(torch.float64).contiguous(), base=fctx.base,
                                                         want_base=fctx.want_base, **setup.kwargs())
        return gs, gb, None


def lower_resolution(spec, base, setup: ResolutionSetup):
    """Differentiable (n_spec, n_eff) normalised low-resolution spectra of
    base - spec[s]; see ``LowerResolution``."""
    return LowerResolution.apply(spec, base, setup)


@dataclasses.dataclass
class CcfSetup:
    """The fixed arguments of the mask CCF (CCF_func.py:5-91, run_all_SOAP.py:292-314)
    and the Gaussian fit (BIS_FIT2.cpp:97-192): velocities, mask lines, the trimmed
    wavelengths (device, float64) and the grid step."""
    ctx: Context
    vel: torch.Tensor
    line_wave: torch.Tensor
    line_weight: torch.Tensor
    wave_trim: torch.Tensor
    step: float
    wave_extend: float = 100.0
    mask_step: float = 0.005
    index_old: int = 20000

    def kwargs(self) -> dict:
        return dict(wave_extend=self.wave_extend, mask_step=self.mask_step, index_old=self.index_old)


class NormalisedCcf(torch.autograd.Function):
    """ccf[s] = the normalised, apodised mask CCF of spectra[s] (``soapgb_ccf``, FP64);
    backward: ``soapgb_ccf_adjoint`` (the mask's transpose, the max at its first index)."""

    @staticmethod
    def forward(fctx, spectra, setup: CcfSetup):
        sp = spectra.detach().contiguous()
        c = ops(setup.ctx)
        args = (setup.vel, setup.line_wave, setup.line_weight, setup.wave_trim, setup.step, sp)
        raw = c.ccf("plain64", *args, normalise=False, **setup.kwargs())
        out = c.ccf("plain64", *args, normalise=True, **setup.kwargs())
        fctx.setup, fctx.raw = setup, raw
        return out

    @staticmethod
    def backward(fctx, g):
        s = fctx.setup
        grad = ops(s.ctx).ccf_adjoint(s.vel, s.line_wave, s.line_weight, s.wave_trim, s.step,
                                 g.to(torch.float64).contiguous(), ccf_raw=fctx.raw, normalise=True, **s.kwargs())
        return grad, None


class GaussFit(torch.autograd.Function):
    """(c, |k|, v0, fwhm) of the Gaussian fit of each CCF (``soapgb_gauss_bis``);
    backward: ``soapgb_gauss_fit_adjoint`` (implicit function theorem at the optimum
    with the full Hessian).  The bisector span is not differentiated."""

    @staticmethod
    def forward(fctx, ccf, setup: CcfSetup):
        y = ccf.detach().contiguous()
        res = ops(setup.ctx).gauss_bis(setup.vel, y)
        if bool((res["iters"] < 0).any()):
            raise RuntimeError("Gaussian fit did not converge; its gradient is undefined")
        fctx.setup, fctx.y, fctx.model, fctx.par = setup, y, res["model"], res["par"]
        return res["par"][:, [0, 1, 3, 4]].clone()

    @staticmethod
    def backward(fctx, g):
        gp = torch.zeros_like(fctx.par)
        gp[:, [0, 1, 3, 4]] = g.to(torch.float64)
        s = fctx.setup
        gy = ops(s.ctx).gauss_fit_adjoint(s.vel, fctx.y, fctx.model, fctx.par, gp)
        # a singular system gives a zero gradient and a device status: raise here, as the
        # forward does for a fit that did not converge, rather than return that zero
        ops(s.ctx).synchronize()
        return gy, None


class GaussFitBis(torch.autograd.Function):
    """(c, |k|, span, v0, fwhm) of the Gaussian fit and bisector of each CCF
    (``soapgb_gauss_bis``); backward: ``soapgb_gauss_fit_adjoint`` with the span's
    gradient (its per-depth crossing intervals held fixed)."""

    @staticmethod
    def forward(fctx, ccf, setup: CcfSetup):
        y = ccf.detach().contiguous()
        res = ops(setup.ctx).gauss_bis(setup.vel, y)
        if bool((res["iters"] < 0).any()):
            raise RuntimeError("Gaussian fit did not converge; its gradient is undefined")
        fctx.setup, fctx.y, fctx.model, fctx.par = setup, y, res["model"], res["par"]
        return res["par"].clone()

    @staticmethod
    def backward(fctx, g):
        s = fctx.setup
        gy = ops(s.ctx).gauss_fit_adjoint(s.vel, fctx.y, fctx.model, fctx.par, g.to(torch.float64).contiguous())
        ops(s.ctx).synchronize()
        return gy, None


def gauss_fit_bis(ccf, setup: CcfSetup):
    """Differentiable (n_spec, 5) fit parameters (c, |k|, span, v0, fwhm); see ``GaussFitBis``."""
    return GaussFitBis.apply(ccf, setup)


def rv_series_checkpointed(star, cubes: dict, setup: IntegrationSetup, rsetup: ResolutionSetup, csetup: CcfSetup,
                           chunk: int = 10, kind=0, quiet_cube: str = None, recompute: bool = True):
    """RV, span and FWHM series over the setup's phases, relative to the quiet star, with
    the quiet spectra differentiated too.  kind selects the deficit (0 flux, 1 bconv,
    2 tot) or is a tuple of them; each pairs with its quiet base as run_all_SOAP.py pairs
    them (q_sed for flux and tot, q_norm for bconv; quiet_cube overrides it for a single
    kind).  Returns {"rv", "span", "fwhm", "par", "quiet"} for a single kind, else a dict
    of those per kind.

    The phases run in chunks of `chunk` under torch.utils.checkpoint: the forward keeps
    each chunk's fitted parameters only, and the backward recomputes the chunk's deficit,
    low-resolution spectra and CCFs before running their adjoints, so the memory held for
    the backward grows with the fitted parameters, not with the spectra.  recompute=False
    keeps every chunk's intermediates instead (no second forward; memory grows with the
    phases)."""
    from torch.utils.checkpoint import checkpoint
    kinds = (kind,) if isinstance(kind, int) else tuple(kind)
    base_key = {0: "q_sed", 1: "q_norm", 2: "q_sed"}
    if quiet_cube is not None and len(kinds) == 1:
        base_key = {kinds[0]: quiet_cube}
    cube_list = [cubes[k] for k in CUBE_KEYS]
    bases = {key: quiet_spectrum(star, cubes[key], setup) for key in sorted({base_key[k] for k in kinds})}
    zero = torch.zeros((1, setup.wave.shape[0]), dtype=torch.float64, device=setup.wave.device)
    q_par = {key: gauss_fit_bis(normalised_ccf(_trim(lower_resolution(zero, b, rsetup)), csetup), csetup)[0]
             for key, b in bases.items()}
    keys = sorted(bases)

    def chunk_par(p0, p1, star_, *rest):
        bl = dict(zip(keys, rest[:len(keys)]))
        cl = rest[len(keys):]
        d = deficit_spectra(star_, *cl, setup.phases(p0, p1))
        out = []
        for k in kinds:
            low = lower_resolution(d[:, k].contiguous(), bl[base_key[k]], rsetup)
            out.append(gauss_fit_bis(normalised_ccf(_trim(low), csetup), csetup))
        return torch.stack(out)

    pars = []
    for p0 in range(0, setup.n_phase, chunk):
        p1 = min(setup.n_phase, p0 + chunk)
        args = (p0, p1, star, *[bases[k] for k in keys], *cube_list)
        # the re-entrant form runs the chunk without a graph and reruns it under grad in the
        # backward pass: the autograd Functions here keep their inputs on their contexts,
        # which the non-re-entrant form's saved-tensor hooks would not release
        pars.append(checkpoint(chunk_par, *args, use_reentrant=True) if recompute else chunk_par(*args))
    par = torch.cat(pars, dim=1)    # (kinds, phases, 5)
    res = {}
    for i, k in enumerate(kinds):
        qp = q_par[base_key[k]]
        res[k] = {"rv": par[i, :, 3] - qp[3], "span": par[i, :, 2], "fwhm": par[i, :, 4], "par": par[i],
                  "quiet": qp}
    return res[kinds[0]] if isinstance(kind, int) else res


def _trim(a):
    """The [200:-200][10:-10] trim of run_all_SOAP.py:259,266 (a view)."""
    return a[..., 210:-210]


def normalised_ccf(spectra, setup: CcfSetup):
    """Differentiable (n_spec, n_v) normalised CCFs; see ``NormalisedCcf``."""
    return NormalisedCcf.apply(spectra, setup)


def gauss_fit(ccf, setup: CcfSetup):
    """Differentiable (n_spec, 4) fit parameters (c, |k|, v0, fwhm); see ``GaussFit``."""
    return GaussFit.apply(ccf, setup)
