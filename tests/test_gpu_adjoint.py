"""The adjoint of the per-phase integration (soapgb_phase_integrate_adjoint) behind the
torch.autograd.Function of soap_gpu_gb300.differentiable, checked in FP64:

* u1, u2 and vsini against central differences of the forward (step 1e-6 relative;
  the outputs are piecewise smooth in the velocities, linear in the rest);
* cube and continuum-row entries against central differences (the outputs are linear
  in them, so any step gives the exact derivative up to rounding);
* the whole cube gradient by the dot-product identity <W, J V> = <J^T W, V> for a
  random direction V (the outputs are jointly linear in the four cubes).

Loss: sum of W * out for a fixed random W.  Tolerances are relative to the
derivative's magnitude and reflect FP64 rounding of sums over ~10^5 terms."""
import numpy as np
import pytest

from _cases import activity, small_inputs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _setup(ctx, seed=7):
    from soap_gpu_gb300.differentiable import IntegrationSetup
    inp = small_inputs(seed=seed, grid=40, n=4200, n_phase=4)
    c = inp.case
    n_eff = (c.n // 512) * 512
    setup = IntegrationSetup.build(ctx, inp.wave, n_eff, c.grid, c.period, c.w_ratio, c.incl, c.radius_km,
                                   inp.mu_boundary, inp.lb, c.phases, [c.regions for _ in c.phases], activity(c),
                                   c.step)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda:0")
    cubes = [dev(inp.q_norm), dev(inp.q_sed), dev(inp.spot_norm), dev(inp.fac_norm), dev(inp.spot_sed[0]),
             dev(inp.fac_sed[0])]
    u = dev([c.u1, c.u2, c.vsini])
    return inp, setup, u, cubes


def _loss_fn(setup, W):
    from soap_gpu_gb300.differentiable import deficit_spectra

    def loss(u, cubes):
        return (deficit_spectra(u, *cubes, setup) * W).sum()
    return loss


def test_adjoint_matches_finite_differences(ctx):
    inp, setup, u, cubes = _setup(ctx)
    n_phase = len(inp.case.phases)
    rng = np.random.default_rng(5)
    W = torch.as_tensor(rng.standard_normal((n_phase, 3, inp.wave.size)), device="cuda:0")
    loss = _loss_fn(setup, W)
    u_g = u.clone().requires_grad_(True)
    cubes_g = [c.clone().requires_grad_(True) for c in cubes]
    L0 = loss(u_g, cubes_g)
    L0.backward()
    assert torch.isfinite(L0)

    # limb darkening and vsini: central differences at 1e-6 relative (vsini: the
    # outputs are piecewise smooth, so the difference carries the kinks it straddles)
    for k, tol in ((0, 1e-6), (1, 1e-6), (2, 1e-4)):
        h = 1e-6 * abs(float(u[k]))
        up, um = u.clone(), u.clone()
        up[k] += h
        um[k] -= h
        with torch.no_grad():
            fd = (float(loss(up, cubes)) - float(loss(um, cubes))) / (2 * h)
        got = float(u_g.grad[k])
        assert abs(got - fd) <= tol * abs(fd) + 1e-9, (k, got, fd)
        assert abs(fd) > 1e-3, "star gradient unexpectedly zero"

    # seed spectra: entries where the gradient is largest and a few random ones
    for ci, c in enumerate(cubes):
        g = cubes_g[ci].grad
        flat = g.reshape(-1)
        idx = list(torch.topk(flat.abs(), 3).indices.cpu().numpy())
        idx += list(rng.integers(0, flat.numel(), 3))
        for f in idx:
            h = 1e-2 * max(abs(float(c.reshape(-1)[f])), 1.0)
            cp, cm = [x.clone() for x in cubes], [x.clone() for x in cubes]
            cp[ci].reshape(-1)[f] += h
            cm[ci].reshape(-1)[f] -= h
            with torch.no_grad():
                fd = (float(loss(u, cp)) - float(loss(u, cm))) / (2 * h)
            got = float(flat[f])
            assert abs(got - fd) <= 1e-8 * max(abs(fd), 1.0), (ci, int(f), got, fd)


def test_adjoint_dot_product_identity(ctx):
    inp, setup, u, cubes = _setup(ctx, seed=8)
    from soap_gpu_gb300.differentiable import deficit_spectra
    n_phase = len(inp.case.phases)
    rng = np.random.default_rng(9)
    W = torch.as_tensor(rng.standard_normal((n_phase, 3, inp.wave.size)), device="cuda:0")
    cubes_g = [c.clone().requires_grad_(i < 4) for i, c in enumerate(cubes)]
    (deficit_spectra(u, *cubes_g, setup) * W).sum().backward()
    V = [torch.as_tensor(rng.standard_normal(tuple(c.shape)), device="cuda:0") for c in cubes[:4]]
    with torch.no_grad():
        jv = deficit_spectra(u, *V, cubes[4], cubes[5], setup)
    lhs = float((W * jv).sum())
    rhs = sum(float((cubes_g[i].grad * V[i]).sum()) for i in range(4))
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), 1.0), (lhs, rhs)
    # the gradient is zero on the pixels beyond n_eff and on the rows no active cell reads
    n_eff = setup.n_eff
    for i in range(4):
        assert torch.all(cubes_g[i].grad[:, n_eff:] == 0)


def test_adam_fit_recovers_limb_darkening_and_vsini(ctx):
    """200 Adam steps on (u1, u2, vsini), from a start 10-15 % off, against a target
    deficit-spectrum series of the same star made with the true values: each step runs
    the forward and the hand-written adjoint on the device.  The loss is the squared
    difference of the spectra, scaled to 1 at the start."""
    from soap_gpu_gb300.differentiable import deficit_spectra
    inp, setup, u_true, cubes = _setup(ctx, seed=7)
    with torch.no_grad():
        target = deficit_spectra(u_true, *cubes, setup)
    start = u_true * torch.as_tensor([1.15, 0.88, 1.10], dtype=torch.float64, device="cuda:0")
    # optimise in units of the true values so one learning rate suits all three
    scale = u_true.clone()
    z = (start / scale).clone().requires_grad_(True)
    opt = torch.optim.Adam([z], lr=0.01)
    sched = torch.optim.lr_scheduler.ExponentialLR(opt, gamma=0.98)   # Adam's steps do not shrink by themselves
    with torch.no_grad():
        l0 = float(((deficit_spectra(start, *cubes, setup) - target) ** 2).sum())
    assert l0 > 0
    for _ in range(200):
        opt.zero_grad()
        loss = ((deficit_spectra(z * scale, *cubes, setup) - target) ** 2).sum() / l0
        loss.backward()
        opt.step()
        sched.step()
    got = (z.detach() * scale).cpu().numpy()
    want = u_true.cpu().numpy()
    assert float(loss.detach()) < 1e-4
    assert np.all(np.abs(got / want - 1.0) < 2e-3), (got, want)
