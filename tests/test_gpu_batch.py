"""The batched form (soapgb_batch_create / soapgb_batch_run): stars of mixed grids,
region counts, phase counts and rotation speeds, sharing the seed spectra, integrated in
one persistent launch.

Every star's rows of the batch output must equal, bit for bit, the FP32 composite
pipeline (soapgb_phase_pipeline) run on that star alone: the same per-tile arithmetic
runs whichever block takes a (star, phase, tile) item.  Against each star's plain FP64
pipeline (the reference's arithmetic) the FP32 tolerance of the other pipeline tests
holds.  The launch shapes of the tuner, and a replay of the run captured in a CUDA graph,
give the same bits.
"""
import ctypes

import numpy as np
import pytest

from soap_gpu_gb300 import synth
from soap_gpu_gb300._lib import Star

from _cases import activity, rel_err

pytestmark = pytest.mark.gpu

FP32_TOL = 2e-6   # normalised spectra, FP32 form against plain FP64 (test_gpu_pipeline.py)


def _star(c, lb):
    return Star(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, (ctypes.c_double * 4)(*lb))


@pytest.fixture(scope="module")
def batch_case(ctx):
    torch = pytest.importorskip("torch")
    seed_case = synth.small_case(seed=21, grid=40, n=8300, n_phase=4, n_mu=6)
    inp = synth.generate(seed_case)
    stars = synth.make_batch(n_star=20, seed=5, grid=(24, 100), n_regions=(1, 5), size_pct=(1.0, 6.0),
                             n_phase=(2, 8), vsini=(1.0, 10.0))
    dev = "cuda:0"
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)
    cubes = dict(q_norm=T(inp.q_norm), q_sed=T(inp.q_sed), spot_norm=T(inp.spot_norm), fac_norm=T(inp.fac_norm),
                 spot_sed=T(inp.spot_sed[0]), fac_sed=T(inp.fac_sed[0]))
    return seed_case, inp, stars, T(inp.wave), cubes


def _make(ctx, batch_case, **kw):
    from soap_gpu_gb300.api import Batch
    seed_case, inp, stars, wave, cubes = batch_case
    n_eff = (seed_case.n // 512) * 512
    return Batch(ctx, wave, n_eff, cubes, inp.mu_boundary, seed_case.step, activity(seed_case),
                 seed_case.sigma_v, [_star(c, inp.lb) for c in stars], [c.phases for c in stars],
                 [[c.regions for _ in c.phases] for c in stars], conv_step=seed_case.step, **kw)


def test_batch_rows_equal_each_stars_own_pipeline(ctx, batch_case):
    torch = pytest.importorskip("torch")
    seed_case, inp, stars, wave, cubes = batch_case
    n_eff = (seed_case.n // 512) * 512
    b = _make(ctx, batch_case)
    quiet = torch.empty((len(stars), 2, seed_case.n), dtype=torch.float64, device="cuda:0")
    low = b.run(quiet=quiet).cpu().numpy()
    quiet = quiet.cpu().numpy()
    assert b.items > 0
    act = activity(seed_case)
    n_vis_stars = 0
    for s, c in enumerate(stars):
        maps = ctx.disk_maps(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, inp.mu_boundary, inp.lb)
        regions = [c.regions for _ in c.phases]
        rows = low[b.offsets[s]:b.offsets[s + 1]]
        ref = {}
        for form in ("fast32", "plain64"):
            qn = ctx.quiet_disk(form, inp.wave, inp.q_norm, n_eff, maps, c.grid, seed_case.step)
            qs = ctx.quiet_disk(form, inp.wave, inp.q_sed, n_eff, maps, c.grid, seed_case.step)
            if form == "fast32":
                assert np.array_equal(quiet[s, 0], qs) and np.array_equal(quiet[s, 1], qn), s
            ref[form] = ctx.phase_pipeline(form, inp.wave, n_eff, _star(c, inp.lb), maps,
                                           {k: v.cpu().numpy() for k, v in cubes.items()}, seed_case.step, act,
                                           c.phases, regions, qs, qn, seed_case.sigma_v, conv_step=seed_case.step)
        assert np.array_equal(rows, ref["fast32"]), "star %d (grid %d, %d phases)" % (s, c.grid, c.n_phase)
        assert rel_err(rows, ref["plain64"]) <= FP32_TOL, s
        _, bi = ctx.phase_maps(c.grid, c.incl, c.phases, regions, act)
        n_vis_stars += int(np.any(bi >= 0))
    assert n_vis_stars >= len(stars) // 2, "too few stars with a visible region"
    b.close()


@pytest.mark.parametrize("chunk,bps", [(1, 0), (7, 1), (64, 2), (0, 1)])
def test_batch_launch_shapes_give_the_same_bits(ctx, batch_case, chunk, bps):
    b = _make(ctx, batch_case)
    ref = b.run().cpu().numpy()
    b.tune(chunk, bps)
    assert np.array_equal(b.run().cpu().numpy(), ref)
    b.close()


def test_batch_run_replays_from_a_cuda_graph(ctx, batch_case):
    torch = pytest.importorskip("torch")
    b = _make(ctx, batch_case)
    ref = b.run().cpu().numpy()
    out = torch.zeros((b.total_phases, 3, b.n_eff), dtype=torch.float64, device="cuda:0")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        b.run(out)           # outside the capture first: the kernels' attributes are set once
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    out.zero_()
    with torch.cuda.graph(g, capture_error_mode="relaxed"):
        b.run(out)
    for _ in range(2):
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref)
    ctx.synchronize()
    b.close()
