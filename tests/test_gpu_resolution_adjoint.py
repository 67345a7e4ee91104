"""The adjoint of the resolution step (soapgb_lower_resolution_adjoint) behind
soap_gpu_gb300.differentiable.LowerResolution, checked in FP64 against central
differences of the PLAIN64 forward:

* spectrum and base entries, among them the pixel holding min A and the pixels whose
  taps reach the pixel holding max C (the normalisation's extrema carry gradient
  there); the steps are far smaller than the gap to the second extremum, so the
  differences see one smooth piece;
* the chain (u1, u2, vsini) -> deficit spectra -> low-resolution spectra through both
  hand-written adjoints (tolerances as for the integration alone).

Loss: sum of W * out for a fixed random W.  Central differences at 1e-6 relative carry
an error of ~1e-9 of the derivative's scale (second-order term plus FP64 rounding of a
loss of ~10^4 terms); the tolerance is 1e-6 of the largest gradient entry."""
import numpy as np
import pytest

from _cases import small_inputs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _res_case(ctx, seed=3, n_spec=3):
    from soap_gpu_gb300.differentiable import ResolutionSetup
    inp = small_inputs()
    n, n_eff = inp.wave.size, 4096
    rng = np.random.default_rng(seed)
    base = np.zeros(n)
    base[:n_eff] = 1000.0 * inp.q_sed[0, :n_eff]
    spec = np.zeros((n_spec, n))
    spec[:, :n_eff] = 50.0 * rng.uniform(0, 1, (n_spec, n_eff)) * inp.q_norm[1, :n_eff]
    dev = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda:0")
    setup = ResolutionSetup(ctx, dev(inp.wave), n_eff, float(inp.case.sigma_v))
    W = dev(rng.standard_normal((n_spec, n_eff)))
    return setup, dev(spec), dev(base), W, rng


def test_resolution_adjoint_matches_finite_differences(ctx):
    from soap_gpu_gb300.differentiable import lower_resolution
    setup, spec, base, W, rng = _res_case(ctx)
    loss = lambda sp, b: float((lower_resolution(sp, b, setup) * W).sum())
    sp_g, b_g = spec.clone().requires_grad_(True), base.clone().requires_grad_(True)
    (lower_resolution(sp_g, b_g, setup) * W).sum().backward()
    gs, gb = sp_g.grad, b_g.grad
    scale = float(torch.max(torch.abs(gs)))
    assert scale > 0
    n_eff = setup.n_eff

    # the forward's extrema: first pixel of min A and of max C, per spectrum
    out, mm = ctx.lower_resolution("plain64", setup.wave, spec, n_eff, setup.sigma_v, base=base)
    A = (base[None, :] - spec).cpu().numpy()
    picks = []
    for s in range(spec.shape[0]):
        a = A[s]
        im = int(np.argmin(a))
        gap = np.partition(np.unique(a), 1)[1] - a[im]
        # C from out: out = 1 - C f, f = (1 - mn) / mx
        f = (1.0 - mm[s, 0]) / mm[s, 1]
        C = (1.0 - out[s].cpu().numpy()) / float(f)
        ix = int(np.argmax(np.where(np.abs(C) > 0, C, -np.inf)))
        picks.append((s, im, gap, ix))
    for s, im, gap, ix in picks:
        cand = [im, ix, ix - 3, ix + 3] + list(rng.integers(0, n_eff, 6))
        for m in cand:
            m = int(m)
            h = 1e-6 * max(abs(float(spec[s, m])), 1.0)
            if m == im:
                assert gap > 10 * h, "min A not isolated enough for a finite difference"
            sp_p, sp_m = spec.clone(), spec.clone()
            sp_p[s, m] += h
            sp_m[s, m] -= h
            with torch.no_grad():
                fd = (loss(sp_p, base) - loss(sp_m, base)) / (2 * h)
            got = float(gs[s, m])
            assert abs(got - fd) <= 1e-6 * scale, (s, m, got, fd)
    # base entries: summed over the spectra
    bscale = float(torch.max(torch.abs(gb)))
    for m in [picks[0][1], picks[0][3]] + list(rng.integers(0, n_eff, 4)):
        m = int(m)
        h = 1e-6 * max(abs(float(base[m])), 1.0)
        bp, bm = base.clone(), base.clone()
        bp[m] += h
        bm[m] -= h
        with torch.no_grad():
            fd = (loss(spec, bp) - loss(spec, bm)) / (2 * h)
        assert abs(float(gb[m]) - fd) <= 1e-6 * bscale, (m, float(gb[m]), fd)
    assert torch.isfinite(gs).all() and torch.isfinite(gb).all()


def test_resolution_adjoint_host_and_device_agree(ctx):
    setup, spec, base, W, _ = _res_case(ctx, seed=4, n_spec=2)
    gd, bd = ctx.lower_resolution_adjoint(setup.wave, spec, setup.n_eff, setup.sigma_v, W, base=base)
    gh, bh = ctx.lower_resolution_adjoint(setup.wave.cpu().numpy(), spec.cpu().numpy(), setup.n_eff,
                                          setup.sigma_v, W.cpu().numpy(), base=base.cpu().numpy())
    assert np.array_equal(gd.cpu().numpy(), gh)
    assert np.array_equal(bd.cpu().numpy(), bh)
    # deterministic: a second run gives the same bits
    gd2, bd2 = ctx.lower_resolution_adjoint(setup.wave, spec, setup.n_eff, setup.sigma_v, W, base=base)
    assert torch.equal(gd, gd2) and torch.equal(bd, bd2)
    # without a base, A = spec and the gradient changes sign against the base form's
    gn, bn = ctx.lower_resolution_adjoint(setup.wave, base[None, :] - spec, setup.n_eff, setup.sigma_v, W)
    assert bn is None
    assert torch.allclose(gn, -gd, rtol=0, atol=1e-12 * float(torch.max(torch.abs(gd))))


def test_chain_star_to_low_resolution_spectra(ctx):
    """(u1, u2, vsini) -> flux deficit of every phase (integration adjoint) -> normalised
    low-resolution spectra of quiet - deficit (resolution adjoint)."""
    from test_gpu_adjoint import _setup
    from soap_gpu_gb300.differentiable import ResolutionSetup, deficit_spectra, lower_resolution
    inp, setup, u, cubes = _setup(ctx, seed=7)
    n_eff = setup.n_eff
    n_phase = len(inp.case.phases)
    base = torch.zeros_like(setup.wave)
    base[:n_eff] = 1000.0 * cubes[1][0, :n_eff]
    rs = ResolutionSetup(ctx, setup.wave, n_eff, float(inp.case.sigma_v))
    rng = np.random.default_rng(11)
    W = torch.as_tensor(rng.standard_normal((n_phase, n_eff)), device="cuda:0")

    def loss(star):
        flux = deficit_spectra(star, *cubes, setup)[:, 0].contiguous()
        return (lower_resolution(flux, base, rs) * W).sum()

    u_g = u.clone().requires_grad_(True)
    loss(u_g).backward()
    for k, tol in ((0, 1e-6), (1, 1e-6), (2, 1e-4)):
        h = 1e-6 * abs(float(u[k]))
        up, um = u.clone(), u.clone()
        up[k] += h
        um[k] -= h
        with torch.no_grad():
            fd = (float(loss(up)) - float(loss(um))) / (2 * h)
        got = float(u_g.grad[k])
        assert abs(fd) > 1e-9, "star gradient unexpectedly zero"
        assert abs(got - fd) <= tol * abs(fd) + 1e-9, (k, got, fd)
