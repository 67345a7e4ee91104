"""A batch of stars of mixed shapes through one context, the shape of the survey's
measurement config 3 at parity-test sizes: grid sides 24-100, 1-5 regions of 0.1-3 %
of the hemisphere at latitudes within 60 degrees, 2-8 phases, vsini 1-10 km/s, and
shared seed spectra (4200 px, 6 mu bins).

With device buffers the FP32 pipeline calls of all stars are queued back to back on
the stream without a synchronisation (each star grows or reuses the context's work
space while earlier calls are in flight); each star's spectra must then match the
PLAIN64 pipeline of the same star, whose arithmetic is pinned to the oracle by the
parity tests, within the FP32 form's 2e-6 of scale."""
import ctypes
import dataclasses

import numpy as np
import pytest

from soap_gpu_gb300._lib import Star

from _cases import activity, cubes, rel_err, small_inputs

pytestmark = pytest.mark.gpu


def _mixed_stars(count, seed=303):
    rng = np.random.default_rng(seed)
    base = small_inputs(seed=7, grid=40, n=4200)
    stars = []
    for _ in range(count):
        n_reg = int(rng.integers(1, 6))
        frac = rng.uniform(0.001, 0.03, n_reg)   # 0.1 - 3 % of the hemisphere: s = sqrt(f)
        regions = np.column_stack((rng.uniform(-60.0, 60.0, n_reg), rng.uniform(0.0, 360.0, n_reg),
                                   np.sqrt(frac), rng.integers(0, 2, n_reg).astype(np.float64)))
        n_phase = int(rng.integers(2, 9))
        case = dataclasses.replace(base.case, grid=int(rng.integers(24, 101)), regions=regions, n_phase=n_phase,
                                   rot_step=1.0 / n_phase, vsini=float(rng.uniform(1.0, 10.0)))
        stars.append(case)
    return base, stars


def _star(case, lb):
    return Star(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                (ctypes.c_double * 4)(*lb))


def test_mixed_stars_queued_on_one_stream(ctx):
    torch = pytest.importorskip("torch")
    inp, stars = _mixed_stars(6)
    n_eff = (inp.wave.size // 512) * 512
    cb = cubes(inp)
    cb["spot_sed"] = inp.spot_sed[0]
    cb["fac_sed"] = inp.fac_sed[0]
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")
    wave_d = dev(inp.wave)
    cb_d = {k: dev(v) for k, v in cb.items()}
    queued, checks = [], []
    for case in stars:
        act = activity(case)
        maps = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                             inp.mu_boundary, inp.lb)
        regions = [case.regions for _ in range(case.n_phase)]
        star = _star(case, inp.lb)
        qn32 = ctx.quiet_disk("fast32", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
        qs32 = ctx.quiet_disk("fast32", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
        maps_d = {k: dev(v) for k, v in maps.items()}
        out = ctx.phase_pipeline("fast32", wave_d, n_eff, star, maps_d, cb_d, case.step, act, case.phases,
                                 regions, dev(qs32), dev(qn32), case.sigma_v, conv_step=case.step)
        queued.append((out, maps_d))   # keep the device inputs alive until the stream is done
        qn64 = ctx.quiet_disk("plain64", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
        qs64 = ctx.quiet_disk("plain64", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
        checks.append((maps, regions, star, act, qs64, qn64))
    ctx.synchronize()
    torch.cuda.synchronize()
    n_active = 0
    for case, (out, _), (maps, regions, star, act, qs64, qn64) in zip(stars, queued, checks):
        got = out.cpu().numpy()
        ref = ctx.phase_pipeline("plain64", inp.wave, n_eff, star, maps, cb, case.step, act, case.phases, regions,
                                 qs64, qn64, case.sigma_v, conv_step=case.step)
        assert got.shape == ref.shape == (case.n_phase, 3, n_eff)
        assert np.all(np.isfinite(got))
        assert rel_err(got, ref) <= 2e-6, (case.grid, case.n_phase, case.vsini)
        # phases whose spectra differ from the star's first phase (a region moved into
        # or across the disk)
        n_active += int(np.sum([not np.array_equal(ref[p], ref[0]) for p in range(1, case.n_phase)]))
    assert n_active > 0, "the batch needs phases with a visible region"
