"""The adjoints of the mask CCF (soapgb_ccf_adjoint) and of the Gaussian fit
(soapgb_gauss_fit_adjoint), and the chain from (u1, u2, vsini) to the RV series:

* the raw CCF is linear in the spectra: <W, C V> = <C^T W, V> to 1e-12;
* the normalised CCF against central differences (1e-7 of the largest entry);
* the fit's v0 and fwhm against central differences of refits (the fit converges to
  far below the steps used; 1e-4 of the largest entry);
* (u1, u2, vsini) -> deficit spectra -> low-resolution spectra -> normalised CCF ->
  fitted v0 against Richardson-extrapolated central differences of the whole
  forward (3e-3 relative; steps of 1e-2 relative, large enough that the refits'
  convergence does not show)."""
import numpy as np
import pytest

from _cases import small_inputs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda:0")


def _ccf_setup(ctx, inp, n_eff, seed=5):
    from soap_gpu_gb300.differentiable import CcfSetup
    c = inp.case
    wave = inp.wave[:n_eff][210:n_eff - 210]
    sel = (inp.mask_wave > wave.min()) & (inp.mask_wave < wave.max())
    rng = np.random.default_rng(seed)
    lw, lwt = inp.mask_wave[sel], inp.mask_weight[sel] * rng.uniform(0.5, 1.0, sel.sum())
    return CcfSetup(ctx, _dev(c.velocities), _dev(lw), _dev(lwt), _dev(wave), float(c.step),
                    index_old=int(100.0 / c.step))


def test_ccf_adjoint_is_the_transpose(ctx):
    from soap_gpu_gb300.differentiable import normalised_ccf
    inp = small_inputs()
    n_eff = 4096
    cs = _ccf_setup(ctx, inp, n_eff)
    rng = np.random.default_rng(6)
    nw = cs.wave_trim.numel()
    spectra = _dev(1.0 - 0.3 * rng.uniform(0, 1, (3, nw)) * inp.q_norm[0, 210:n_eff - 210][None, :])
    n_v = cs.vel.numel()
    W = _dev(rng.standard_normal((3, n_v)))
    V = _dev(rng.standard_normal((3, nw)))
    args = (cs.vel, cs.line_wave, cs.line_weight, cs.wave_trim, cs.step)
    cv = ctx.ccf("plain64", *args, V, normalise=False, **cs.kwargs())
    gt = ctx.ccf_adjoint(*args, W, normalise=False, **cs.kwargs())
    lhs, rhs = float((W * cv).sum()), float((gt * V).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0), (lhs, rhs)

    # normalised: central differences on a few pixels, the largest gradients among them
    sp = spectra.clone().requires_grad_(True)
    (normalised_ccf(sp, cs) * W).sum().backward()
    g = sp.grad
    scale = float(torch.max(torch.abs(g)))
    assert scale > 0
    loss = lambda x: float((normalised_ccf(x, cs) * W).sum())
    picks = list(torch.topk(g.abs().reshape(-1), 3).indices.cpu().numpy()) + list(rng.integers(0, g.numel(), 5))
    for f in picks:
        s, p = divmod(int(f), nw)
        h = 1e-6
        xp, xm = spectra.clone(), spectra.clone()
        xp[s, p] += h
        xm[s, p] -= h
        with torch.no_grad():
            fd = (loss(xp) - loss(xm)) / (2 * h)
        assert abs(float(g[s, p]) - fd) <= 1e-7 * scale, (s, p, float(g[s, p]), fd)


def test_gauss_fit_adjoint_matches_refits(ctx):
    from soap_gpu_gb300.differentiable import CcfSetup, gauss_fit
    inp = small_inputs()
    vel = inp.case.velocities
    rng = np.random.default_rng(12)
    n_spec = 3
    sig = 3000.0
    y = np.stack([1.0 - (0.35 + 0.05 * s) * np.exp(-(vel - 250.0 * (s - 1)) ** 2 / (2 * sig ** 2))
                  + 0.002 * rng.standard_normal(vel.size) for s in range(n_spec)])
    cs = CcfSetup(ctx, _dev(vel), None, None, None, 0.005)
    yd = _dev(y).requires_grad_(True)
    Wp = _dev([[0.0, 0.0, 1.0, 0.3]] * n_spec)   # loss = v0 + 0.3 fwhm, summed
    (gauss_fit(yd, cs) * Wp).sum().backward()
    g = yd.grad
    scale = float(torch.max(torch.abs(g)))
    assert scale > 0
    loss = lambda t: float((gauss_fit(t, cs) * Wp).sum())
    picks = list(torch.topk(g.abs().reshape(-1), 3).indices.cpu().numpy()) + list(rng.integers(0, g.numel(), 5))
    for f in picks:
        s, i = divmod(int(f), vel.size)
        h = 1e-4
        yp, ym = _dev(y), _dev(y)
        yp[s, i] += h
        ym[s, i] -= h
        with torch.no_grad():
            fd = (loss(yp) - loss(ym)) / (2 * h)
        assert abs(float(g[s, i]) - fd) <= 1e-4 * scale, (s, i, float(g[s, i]), fd)


def test_chain_star_to_rv(ctx):
    """(u1, u2, vsini) -> flux deficit -> low-resolution spectrum of quiet - deficit
    -> normalised CCF -> fitted v0 of every phase; loss = a fixed combination of the
    RVs, as a fit to an RV curve would use."""
    from test_gpu_adjoint import _setup
    from soap_gpu_gb300.differentiable import (ResolutionSetup, deficit_spectra, gauss_fit, lower_resolution,
                                               normalised_ccf)
    inp, setup, u, cubes = _setup(ctx, seed=7)
    n_eff = setup.n_eff
    n_phase = len(inp.case.phases)
    base = torch.zeros_like(setup.wave)
    base[:n_eff] = 1000.0 * cubes[1][0, :n_eff]
    rs = ResolutionSetup(ctx, setup.wave, n_eff, float(inp.case.sigma_v))
    cs = _ccf_setup(ctx, inp, n_eff)
    wr = _dev(np.linspace(1.0, 2.0, n_phase))

    def rv(star):
        flux = deficit_spectra(star, *cubes, setup)[:, 0].contiguous()
        low = lower_resolution(flux, base, rs)[:, 210:n_eff - 210].contiguous()
        return gauss_fit(normalised_ccf(low, cs), cs)[:, 2]

    u_g = u.clone().requires_grad_(True)
    (rv(u_g) * wr).sum().backward()

    def central(k, h):
        up, um = u.clone(), u.clone()
        up[k] += h
        um[k] -= h
        with torch.no_grad():
            return (float((rv(up) * wr).sum()) - float((rv(um) * wr).sum())) / (2 * h)

    for k in range(3):
        # the fit stops at xtol = 1e-8 relative on x0 - x[0] (~10^4 m/s), so a refit's v0
        # carries up to ~1e-4 m/s: steps of 1e-2 relative keep that below 1e-4 of the
        # difference, and Richardson's (4 D(h/2) - D(h)) / 3 removes the O(h^2) term
        h = 1e-2 * abs(float(u[k]))
        fd = (4 * central(k, h / 2) - central(k, h)) / 3
        got = float(u_g.grad[k])
        assert abs(fd) > 1e-6, ("RV gradient unexpectedly zero", k)
        assert abs(got - fd) <= 3e-3 * abs(fd), (k, got, fd)


def test_adam_fit_of_vsini_to_an_rv_curve(ctx):
    """120 Adam steps on vsini (u1, u2 held at their true values; the RV curve hardly
    constrains them) from a start 10 % off, against the RV series of the true star:
    each step runs the whole forward (integration, resolution, CCF, fit) and the four
    hand-written adjoints.  Loss: squared RV differences, scaled to 1 at the start."""
    from test_gpu_adjoint import _setup
    from soap_gpu_gb300.differentiable import (ResolutionSetup, deficit_spectra, gauss_fit, lower_resolution,
                                               normalised_ccf)
    inp, setup, u, cubes = _setup(ctx, seed=7)
    n_eff = setup.n_eff
    base = torch.zeros_like(setup.wave)
    base[:n_eff] = 1000.0 * cubes[1][0, :n_eff]
    rs = ResolutionSetup(ctx, setup.wave, n_eff, float(inp.case.sigma_v))
    cs = _ccf_setup(ctx, inp, n_eff)

    def rv(star):
        flux = deficit_spectra(star, *cubes, setup)[:, 0].contiguous()
        low = lower_resolution(flux, base, rs)[:, 210:n_eff - 210].contiguous()
        return gauss_fit(normalised_ccf(low, cs), cs)[:, 2]

    with torch.no_grad():
        target = rv(u)
    vs = float(u[2])
    z = torch.tensor([1.10], dtype=torch.float64, device="cuda:0", requires_grad=True)
    star = lambda zz: torch.cat((u[:2], zz * vs))
    with torch.no_grad():
        l0 = float(((rv(star(z)) - target) ** 2).sum())
    assert l0 > 0
    opt = torch.optim.Adam([z], lr=0.01)
    sched = torch.optim.lr_scheduler.ExponentialLR(opt, gamma=0.97)
    for _ in range(120):
        opt.zero_grad()
        loss = ((rv(star(z)) - target) ** 2).sum() / l0
        loss.backward()
        opt.step()
        sched.step()
    assert float(loss.detach()) < 1e-2
    assert abs(float(z.detach()) - 1.0) < 5e-3, float(z.detach())
