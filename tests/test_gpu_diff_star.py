"""The rest of the differentiable form: the quiet-disk adjoint, the inclination, the
region contrast, the bisector span, phase checkpointing, and a fit of contrast and limb
darkening to an RV curve through the whole chain.

* The quiet spectrum (soap_gpu_gb300.differentiable.QuietSpectrum) against FP64 central
  differences in u1, u2 (linear: 1e-6 of the derivative), vsini and the inclination
  (piecewise smooth: 1e-4), and its cube gradient by the dot-product identity (1e-10).
* The deficit spectra's inclination gradient at i = 60 deg (at 90 deg it is zero by
  symmetry), the region maps' coverage held at the setup's inclination.
* The contrast: the spot continuum row scaled by c_spot, d/dc_spot by autograd over the
  continuum-row gradient, against central differences (linear: 1e-8).
* The span (BIS_FIT2.cpp:214-268) of the Gaussian fit + bisector against central
  differences of refits (1e-3 of the gradient's largest entry: the refits converge to
  xtol 1e-8 and the span's crossing intervals stay put for steps of 1e-5).
* The checkpointed chain gives the same gradient, to rounding (1e-12), whatever the
  chunking of its phases.
* 200 Adam steps fit (spot contrast, u1, u2) to a seeded RV curve of the same star.
"""
import numpy as np
import pytest

from _cases import activity, small_inputs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda:0")


def _setup(ctx, seed=7, incl=None, n_phase=4):
    import dataclasses
    from soap_gpu_gb300.differentiable import IntegrationSetup
    inp = small_inputs(seed=seed, grid=40, n=4200, n_phase=n_phase)
    c = inp.case if incl is None else dataclasses.replace(inp.case, incl=incl)
    n_eff = (c.n // 512) * 512
    setup = IntegrationSetup.build(ctx, inp.wave, n_eff, c.grid, c.period, c.w_ratio, c.incl, c.radius_km,
                                   inp.mu_boundary, inp.lb, c.phases, [c.regions for _ in c.phases], activity(c),
                                   c.step)
    cubes = [_dev(inp.q_norm), _dev(inp.q_sed), _dev(inp.spot_norm), _dev(inp.fac_norm), _dev(inp.spot_sed[0]),
             _dev(inp.fac_sed[0])]
    star = _dev([c.u1, c.u2, c.vsini, c.incl])
    return inp, setup, star, cubes


def _central(f, x, k, h):
    xp, xm = x.clone(), x.clone()
    xp[k] += h
    xm[k] -= h
    with torch.no_grad():
        return (float(f(xp)) - float(f(xm))) / (2 * h)


def test_quiet_spectrum_gradients(ctx):
    from soap_gpu_gb300.differentiable import quiet_spectrum
    inp, setup, star, cubes = _setup(ctx, incl=60.0)
    rng = np.random.default_rng(3)
    W = _dev(rng.standard_normal(inp.wave.size))
    cube = cubes[0]
    loss = lambda s, c=cube: (quiet_spectrum(s, c, setup) * W).sum()
    sg = star.clone().requires_grad_(True)
    cg = cube.clone().requires_grad_(True)
    loss(sg, cg).backward()
    for k, tol in ((0, 1e-6), (1, 1e-6), (2, 1e-4), (3, 1e-4)):
        h = 1e-6 * abs(float(star[k]))
        fd = _central(lambda s: loss(s), star, k, h)
        got = float(sg.grad[k])
        assert abs(fd) > 0, k
        assert abs(got - fd) <= tol * abs(fd), (k, got, fd)
    # linear in the cube: <W, dQ/dcube V> = <grad, V>
    V = _dev(rng.standard_normal(tuple(cube.shape)))
    with torch.no_grad():
        lv = float(loss(star, V))
    assert abs(float((cg.grad * V).sum()) - lv) <= 1e-10 * max(abs(lv), 1.0)


def test_inclination_and_contrast_gradients(ctx):
    from soap_gpu_gb300.differentiable import deficit_spectra
    inp, setup, star, cubes = _setup(ctx, incl=60.0)
    rng = np.random.default_rng(4)
    W = _dev(rng.standard_normal((len(inp.case.phases), 3, inp.wave.size)))
    spot_row = cubes[4]

    def loss(s, c_spot):
        cb = list(cubes)
        cb[4] = c_spot * spot_row
        return (deficit_spectra(s, *cb, setup) * W).sum()

    sg = star.clone().requires_grad_(True)
    cg = _dev([1.0]).requires_grad_(True)
    loss(sg, cg[0]).backward()
    h = 1e-6 * 60.0
    fd = _central(lambda s: loss(s, 1.0), star, 3, h)
    assert abs(fd) > 0
    assert abs(float(sg.grad[3]) - fd) <= 1e-4 * abs(fd), (float(sg.grad[3]), fd)
    one = _dev([1.0])
    fdc = _central(lambda c: loss(star, c[0]), one, 0, 1e-6)
    assert abs(fdc) > 0
    assert abs(float(cg.grad[0]) - fdc) <= 1e-8 * abs(fdc), (float(cg.grad[0]), fdc)


def test_span_gradient_matches_refits(ctx):
    from soap_gpu_gb300.differentiable import CcfSetup, gauss_fit_bis
    inp = small_inputs()
    vel = inp.case.velocities
    rng = np.random.default_rng(13)
    n_spec = 3
    sig = 3000.0
    # asymmetric line profiles: a second, shifted component gives a span of tens of m/s
    y = np.stack([1.0 - (0.35 + 0.05 * s) * np.exp(-(vel - 250.0 * (s - 1)) ** 2 / (2 * sig ** 2))
                  - 0.04 * np.exp(-(vel - 2500.0) ** 2 / (2 * (1.5 * sig) ** 2))
                  + 0.001 * rng.standard_normal(vel.size) for s in range(n_spec)])
    cs = CcfSetup(ctx, _dev(vel), None, None, None, 0.005)
    yd = _dev(y).requires_grad_(True)
    Wp = _dev([[0.0, 0.0, 1.0, 0.2, 0.1]] * n_spec)   # loss = span + 0.2 v0 + 0.1 fwhm
    par = gauss_fit_bis(yd, cs)
    assert float(torch.max(torch.abs(par.detach()[:, 2]))) > 1.0, "the test profiles have no span"
    (par * Wp).sum().backward()
    g = yd.grad
    scale = float(torch.max(torch.abs(g)))
    assert scale > 0
    loss = lambda t: float((gauss_fit_bis(t, cs) * Wp).sum())
    picks = list(torch.topk(g.abs().reshape(-1), 4).indices.cpu().numpy()) + list(rng.integers(0, g.numel(), 6))
    for f in picks:
        s, i = divmod(int(f), vel.size)
        h = 1e-5
        yp, ym = _dev(y), _dev(y)
        yp[s, i] += h
        ym[s, i] -= h
        with torch.no_grad():
            fd = (loss(yp) - loss(ym)) / (2 * h)
        assert abs(float(g[s, i]) - fd) <= 1e-3 * scale, (s, i, float(g[s, i]), fd)


def _chain(ctx, inp, setup):
    from soap_gpu_gb300.differentiable import CcfSetup, ResolutionSetup
    n_eff = setup.n_eff
    c = inp.case
    wave = inp.wave[:n_eff][210:n_eff - 210]
    sel = (inp.mask_wave > wave.min()) & (inp.mask_wave < wave.max())
    cs = CcfSetup(ctx, _dev(c.velocities), _dev(inp.mask_wave[sel]), _dev(inp.mask_weight[sel]), _dev(wave),
                  float(c.step), index_old=int(100.0 / c.step))
    rs = ResolutionSetup(ctx, setup.wave, n_eff, float(c.sigma_v))
    return rs, cs


def test_checkpointed_chain_matches_plain_chain(ctx):
    from soap_gpu_gb300.differentiable import rv_series_checkpointed
    inp, setup, star, cubes = _setup(ctx, n_phase=6)
    rs, cs = _chain(ctx, inp, setup)
    keys = ("q_norm", "q_sed", "spot_norm", "fac_norm", "spot_sed", "fac_sed")
    grads = []
    for chunk in (2, 6):
        sg = star.clone().requires_grad_(True)
        cb = {k: v.clone().requires_grad_(True) for k, v in zip(keys, cubes)}
        out = rv_series_checkpointed(sg, cb, setup, rs, cs, chunk=chunk)
        w = _dev(np.linspace(1.0, 2.0, out["rv"].numel()))
        ((out["rv"] * w).sum() + 0.1 * (out["span"] * w).sum()).backward()
        grads.append((sg.grad.clone(), cb["q_sed"].grad.clone(), cb["spot_sed"].grad.clone()))
    # the same adjoints, summed over the chunks in a different order: equal to rounding
    for a, b in zip(*grads):
        assert float(torch.max(torch.abs(a - b))) <= 1e-12 * float(torch.max(torch.abs(b)))
    assert float(torch.max(torch.abs(grads[0][0]))) > 0


def test_adam_fit_of_contrast_and_limb_darkening_to_an_rv_curve(ctx):
    """200 Adam steps on (spot contrast, u1, u2) from a start 15 % off, against the RV
    series of the true star (quiet spectrum included, so u1 and u2 also move the
    reference line); vsini and the inclination held.  Loss: squared RV differences,
    scaled to 1 at the start."""
    from soap_gpu_gb300.differentiable import rv_series_checkpointed
    inp, setup, star, cubes = _setup(ctx, n_phase=6)
    rs, cs = _chain(ctx, inp, setup)
    keys = ("q_norm", "q_sed", "spot_norm", "fac_norm", "spot_sed", "fac_sed")
    base = dict(zip(keys, cubes))

    def rv(p):
        cb = dict(base)
        cb["spot_sed"] = p[0] * base["spot_sed"]
        s = torch.cat((p[1:3], star[2:]))
        return rv_series_checkpointed(s, cb, setup, rs, cs, chunk=3)["rv"]

    truth = _dev([1.0, float(star[0]), float(star[1])])
    with torch.no_grad():
        target = rv(truth)
    assert float(torch.max(torch.abs(target))) > 0.1
    p = (truth * _dev([1.15, 0.85, 1.15])).requires_grad_(True)
    with torch.no_grad():
        l0 = float(((rv(p) - target) ** 2).sum())
    opt = torch.optim.Adam([p], lr=0.01)
    sched = torch.optim.lr_scheduler.ExponentialLR(opt, gamma=0.985)
    for _ in range(200):
        opt.zero_grad()
        loss = ((rv(p) - target) ** 2).sum() / l0
        loss.backward()
        opt.step()
        sched.step()
    assert float(loss.detach()) < 1e-2, float(loss.detach())
    assert abs(float(p.detach()[0]) - 1.0) < 2e-2, p.detach()
