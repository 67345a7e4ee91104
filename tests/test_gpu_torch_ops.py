"""The torch operators over the C ABI (torch.ops.soapgb.*, soap_gpu_gb300.torch_ops)
give the context's device-buffer calls bit for bit, run on torch's current stream, and
raise the library's error message."""
import numpy as np
import pytest

from _cases import activity, small_inputs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda:0")


def test_operators_equal_context_calls(ctx):
    from soap_gpu_gb300.torch_ops import ops
    inp = small_inputs(seed=5, grid=32, n=4200, n_phase=3)
    c = inp.case
    n_eff = (c.n // 512) * 512
    o = ops(ctx)
    mu_b = _dev(inp.mu_boundary)
    m_ctx = ctx.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, mu_b, inp.lb)
    m_op = o.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, mu_b, inp.lb)
    for k in ("delta", "limb", "mu", "lb", "region"):
        assert torch.equal(m_ctx[k], m_op[k]), k
    wave = _dev(inp.wave)
    cube = _dev(inp.q_norm)
    for form in ("plain64", "fast64", "fast32"):
        a = ctx.quiet_disk(form, wave, cube, n_eff, m_ctx, c.grid, c.step)
        b = o.quiet_disk(form, wave, cube, n_eff, m_op, c.grid, c.step)
        assert torch.equal(a, b), form
    act = activity(c)
    temp, bi = ctx.phase_maps(c.grid, c.incl, np.asarray(c.phases), [c.regions for _ in c.phases], act)
    temp, bi = _dev(temp), _dev(bi)
    cubes = dict(q_norm=cube, q_sed=_dev(inp.q_sed), spot_norm=_dev(inp.spot_norm), fac_norm=_dev(inp.fac_norm),
                 spot_sed=_dev(inp.spot_sed[0]), fac_sed=_dev(inp.fac_sed[0]))
    fa = ctx.phase_integrate("plain64", wave, n_eff, c.grid, temp, bi, m_ctx, cubes, c.step, act)
    fb = o.phase_integrate("plain64", wave, n_eff, c.grid, temp, bi, m_op, cubes, c.step, act)
    for x, y in zip(fa, fb):
        assert torch.equal(x, y)
    assert float(torch.max(torch.abs(fa[0]))) > 0, "no active cell"
    g = [torch.ones_like(fa[0]) * w for w in (1.0, 0.5, -0.25)]
    ga = ctx.phase_integrate_adjoint(wave, n_eff, c.grid, temp, bi, m_ctx, cubes, c.step, act, *g)
    gb = o.phase_integrate_adjoint(wave, n_eff, c.grid, temp, bi, m_op, cubes, c.step, act, *g)
    for k in ga:
        assert torch.equal(ga[k], gb[k]), k
    base = ctx.quiet_disk("plain64", wave, _dev(inp.q_sed), n_eff, m_ctx, c.grid, c.step)
    la, ma = ctx.lower_resolution("plain64", wave, fa[0], n_eff, c.sigma_v, base=base, step_mult=c.step,
                                  step_exp=c.step)
    lb_, mb = o.lower_resolution("plain64", wave, fb[0], n_eff, c.sigma_v, base=base, step_mult=c.step,
                                 step_exp=c.step)
    assert torch.equal(la, lb_) and torch.equal(ma, mb)
    gl = torch.ones_like(la)
    sa, ba = ctx.lower_resolution_adjoint(wave, fa[0], n_eff, c.sigma_v, gl, base=base, step_mult=c.step,
                                          step_exp=c.step)
    sb, bb = o.lower_resolution_adjoint(wave, fb[0], n_eff, c.sigma_v, gl, base=base, step_mult=c.step,
                                        step_exp=c.step)
    assert torch.equal(sa, sb) and torch.equal(ba, bb)


def test_operators_follow_the_current_stream_and_raise(ctx):
    from soap_gpu_gb300.torch_ops import ops
    inp = small_inputs(seed=6, grid=24, n=2600, n_phase=2)
    c = inp.case
    o = ops(ctx)
    mu_b = _dev(inp.mu_boundary)
    side = torch.cuda.Stream()
    ref = o.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, mu_b, inp.lb)
    with torch.cuda.stream(side):
        got = o.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, mu_b, inp.lb)
        # read on the side stream, in order after the operator's kernels there
        limb = got["limb"].clone()
    side.synchronize()
    assert torch.equal(limb, ref["limb"])
    with pytest.raises(RuntimeError, match="soapgb"):
        o.disk_maps(0, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, mu_b, inp.lb)
