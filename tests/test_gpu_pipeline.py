"""The composite per-phase pipeline (soapgb_phase_pipeline): maps -> integration ->
convolution / normalisation in one call, against the separate stage calls, and its
host-buffer path (phases in chunks, copies overlapping the next chunk) against its
device-buffer path."""
import ctypes

import numpy as np
import pytest

from soap_gpu_gb300 import synth
from soap_gpu_gb300._lib import Star

from _cases import activity, cubes, rel_err

pytestmark = pytest.mark.gpu


def _star(case, lb):
    return Star(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                (ctypes.c_double * 4)(*lb))


@pytest.fixture(scope="module")
def setup(ctx):
    case = synth.small_case(seed=11, grid=48, n=8300, n_phase=10, n_mu=6)
    inp = synth.generate(case)
    n_eff = (case.n // 512) * 512
    maps = ctx.disk_maps(case.grid, case.period, case.w_ratio, case.incl, case.radius_km, case.u1, case.u2,
                         inp.mu_boundary, inp.lb)
    cb = cubes(inp)
    cb["spot_sed"] = inp.spot_sed[0]
    cb["fac_sed"] = inp.fac_sed[0]
    act = activity(case)
    regions = [case.regions for _ in case.phases]
    return case, inp, n_eff, maps, cb, act, regions


@pytest.mark.parametrize("form,tol,solar", [("fast32", 2e-6, False), ("fast32", 2e-6, True), ("fast64", 1e-12, False),
                                            ("plain64", 1e-12, False)])
def test_pipeline_matches_stages(ctx, setup, form, tol, solar):
    """The collapsed forms' pipeline builds its phase lists from the region boxes, the
    separate integration from the maps: the lists, and so the deficit spectra, agree
    bit for bit (the solar variant puts the faculae in the directly evaluated class)."""
    case, inp, n_eff, maps, cb, act, regions = setup
    act = activity(case, solar)
    q_norm = ctx.quiet_disk(form, inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    q_sed = ctx.quiet_disk(form, inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    low, raw = ctx.phase_pipeline(form, inp.wave, n_eff, _star(case, inp.lb), maps, cb, case.step, act,
                                  case.phases, regions, q_sed, q_norm, case.sigma_v, conv_step=case.step,
                                  want_raw=True)
    temp, bi = ctx.phase_maps(case.grid, case.incl, case.phases, regions, act)
    flux, bconv, tot = ctx.phase_integrate(form, inp.wave, n_eff, case.grid, temp, bi, maps, cb, case.step, act)
    assert np.sum(bi >= 0) > 0, "no active cell in the test case"
    assert np.sum(bi == 0) > 0 and np.sum(bi == 1) > 0, "the case needs spot and facula cells"
    for k, spec in enumerate((tot, flux, bconv)):
        assert np.array_equal(raw[:, k], spec[:, :n_eff])
    base = (q_sed, q_sed, q_norm)
    for k, spec in enumerate((tot, flux, bconv)):
        ref, _ = ctx.lower_resolution(form, inp.wave, spec, n_eff, case.sigma_v, base=base[k],
                                      step_mult=case.step, step_exp=case.step)
        assert rel_err(low[:, k], ref) <= tol


def test_pipeline_host_chunks_equal_device(ctx, setup):
    """The host path runs the phases in chunks with the copies on a second stream; every
    kernel computes the same values as in the device path's single pass."""
    torch = pytest.importorskip("torch")
    case, inp, n_eff, maps, cb, act, regions = setup
    q_norm = ctx.quiet_disk("fast32", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    q_sed = ctx.quiet_disk("fast32", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    star = _star(case, inp.lb)
    low_h, raw_h = ctx.phase_pipeline("fast32", inp.wave, n_eff, star, maps, cb, case.step, act, case.phases,
                                      regions, q_sed, q_norm, case.sigma_v, conv_step=case.step, want_raw=True)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")
    maps_d = {k: dev(v) for k, v in maps.items()}
    cb_d = {k: dev(v) for k, v in cb.items()}
    low_d, raw_d = ctx.phase_pipeline("fast32", dev(inp.wave), n_eff, star, maps_d, cb_d, case.step, act,
                                      dev(case.phases), regions, dev(q_sed), dev(q_norm), case.sigma_v,
                                      conv_step=case.step, want_raw=True)
    torch.cuda.synchronize()
    assert np.array_equal(low_h, low_d.cpu().numpy())
    assert np.array_equal(raw_h, raw_d.cpu().numpy())
    assert np.all(np.isfinite(low_h)) and np.any(low_h != 1.0)


def test_pipeline_descriptors_and_wave_edges(ctx, setup):
    """Device buffers: phase descriptors from host memory (no synchronisation) and from
    device memory give the same spectra; a device wavelength array changed in place
    after its edge values were cached is reported by the next synchronisation, and the
    call after that reads the array again."""
    torch = pytest.importorskip("torch")
    case, inp, n_eff, maps, cb, act, regions = setup
    q_norm = ctx.quiet_disk("fast32", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    q_sed = ctx.quiet_disk("fast32", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    star = _star(case, inp.lb)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")
    maps_d = {k: dev(v) for k, v in maps.items()}
    cb_d = {k: dev(v) for k, v in cb.items()}
    wave_d = dev(inp.wave)

    def run(phases):
        out = ctx.phase_pipeline("fast32", wave_d, n_eff, star, maps_d, cb_d, case.step, act, phases, regions,
                                 dev(q_sed), dev(q_norm), case.sigma_v, conv_step=case.step)
        ctx.synchronize()
        return out.cpu().numpy()

    a = run(np.asarray(case.phases))        # host descriptors
    b = run(dev(case.phases))               # device descriptors
    c = run(np.asarray(case.phases))        # cached edges, confirmed on the device
    assert np.array_equal(a, b) and np.array_equal(a, c)
    w1 = wave_d[1].clone()
    wave_d[1] = w1 + 1e-9                   # same array, new second value
    ctx.phase_pipeline("fast32", wave_d, n_eff, star, maps_d, cb_d, case.step, act, np.asarray(case.phases),
                       regions, dev(q_sed), dev(q_norm), case.sigma_v, conv_step=case.step)
    with pytest.raises(RuntimeError, match="status 51"):
        ctx.synchronize()
    wave_d[1] = w1
    d = run(np.asarray(case.phases))        # read again after the report
    assert np.array_equal(a, d)


def test_pipeline_per_phase_regions(ctx, setup):
    """Region tables that change from phase to phase -- sizes that evolve as in
    run_all_SOAP_evo.py, a phase without regions, a phase with three -- through the
    pipeline's box lists agree bit for bit with the map-based stage calls."""
    from soap_gpu_gb300.driver import evolving_sizes
    case, inp, n_eff, maps, cb, act, _ = setup
    sizes = evolving_sizes(case.phases, case.regions[:, 2], 1.0, 0.002)
    regions = [np.column_stack((case.regions[:, 0], case.regions[:, 1], sizes[p], case.regions[:, 3]))
               for p in range(case.n_phase)]
    regions[1] = np.zeros((0, 4))
    regions[2] = np.vstack([regions[2], [[-30.0, 90.0, 0.15, 0.0]]])
    q_norm = ctx.quiet_disk("fast32", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    q_sed = ctx.quiet_disk("fast32", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    low, raw = ctx.phase_pipeline("fast32", inp.wave, n_eff, _star(case, inp.lb), maps, cb, case.step, act,
                                  case.phases, regions, q_sed, q_norm, case.sigma_v, conv_step=case.step,
                                  want_raw=True)
    temp, bi = ctx.phase_maps(case.grid, case.incl, case.phases, regions, act)
    flux, bconv, tot = ctx.phase_integrate("fast32", inp.wave, n_eff, case.grid, temp, bi, maps, cb, case.step, act)
    assert not np.any((bi[1] >= -0.5) & (bi[1] <= 1.5)), "phase 1 has no region"
    for k, spec in enumerate((tot, flux, bconv)):
        assert np.array_equal(raw[:, k], spec[:, :n_eff])
    assert np.all(raw[1] == 0.0)


@pytest.mark.parametrize("device_mode", [False, True])
def test_zero_phases_need_no_raw_rows(ctx, setup, device_mode):
    """Phases without a visible region: the FP32 resolution stage takes their deficits
    as zero without reading their rows, which are then left unwritten.  A first call
    leaves non-zero rows behind in the context's buffers; a call in which those phases
    have no region gives, without raw outputs, the same spectra bit for bit as with
    them (when their rows are zero-filled)."""
    torch = pytest.importorskip("torch")
    case, inp, n_eff, maps, cb, act, regions = setup
    q_norm = ctx.quiet_disk("fast32", inp.wave, inp.q_norm, n_eff, maps, case.grid, case.step)
    q_sed = ctx.quiet_disk("fast32", inp.wave, inp.q_sed, n_eff, maps, case.grid, case.step)
    star = _star(case, inp.lb)
    if device_mode:
        dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")
        back = lambda t: t.cpu().numpy()
    else:
        dev = back = lambda a: a
    maps_x = {k: dev(v) for k, v in maps.items()}
    cb_x = {k: dev(v) for k, v in cb.items()}
    args = (dev(inp.wave), n_eff, star, maps_x, cb_x, case.step, act)

    def run(regs, want_raw):
        r = ctx.phase_pipeline("fast32", *args, np.asarray(case.phases), regs, dev(q_sed), dev(q_norm),
                               case.sigma_v, conv_step=case.step, want_raw=want_raw)
        ctx.synchronize()
        return tuple(back(x) for x in r) if want_raw else back(r)

    _, raw_a = run(regions, True)
    lit = [p for p in range(case.n_phase) if np.any(raw_a[p] != 0.0)]
    assert len(lit) >= 4, "the case needs phases with a visible region"
    empty = lit[1::3]                      # interior phases: their batches mix zero and non-zero rows
    regs_b = [np.zeros((0, 4)) if p in empty else regions[p] for p in range(case.n_phase)]
    low_b = run(regs_b, False)             # rows of `empty` still hold the first call's deficits
    low_c, raw_c = run(regs_b, True)       # zero-filled rows
    assert all(np.all(raw_c[p] == 0.0) for p in empty)
    assert np.array_equal(low_b, low_c)
    for p in empty[1:]:                    # a zero phase's spectra are the base's alone
        assert np.array_equal(low_b[p], low_b[empty[0]])
