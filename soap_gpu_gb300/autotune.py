"""Launch shapes of the batched form, chosen by measurement and cached per batch class.

The batched integration (soapgb_batch_run) walks every (star, phase, tile) item of a
batch in one persistent launch.  Two shapes of that walk are free:

* ``chunk`` -- the items are dealt to the blocks round robin in chunks of this many
  consecutive positions (0: one contiguous share per block);
* ``blocks_per_sm`` -- resident blocks per SM (1 or 2; 0: as many as fit).

``tune(batch)`` times ``batch.run()`` with CUDA events for each candidate and returns
the fastest; ``shape_for(batch)`` returns the cached choice for the batch's class, where
a class is (pixels, mean grid side, mean visible phases per star) rounded to buckets, so
one measurement serves similar batches.  ``python -m soap_gpu_gb300.autotune`` tunes the
batched workload of 256 stars (grids 100-400, 20-200 phases, 1-12 regions, vsini 1-10
km/s, 310,000 px) and writes the cache, ``tuned_shapes.json`` beside this file.
"""
from __future__ import annotations

import json
import math
import os
from typing import Dict, Iterable, Optional, Tuple

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned_shapes.json")
CANDIDATES: Tuple[Tuple[int, int], ...] = ((0, 0), (0, 1), (1, 0), (4, 0), (16, 0), (64, 0), (256, 0), (16, 1))


def batch_class(n: int, grids: Iterable[int], visible_phases: int, n_star: int) -> str:
    """Bucketed key of a batch: pixels (powers of 2), mean grid side (steps of 50) and
    mean visible phases per star (powers of 2)."""
    grids = list(grids)
    g = sum(grids) / max(len(grids), 1)
    v = visible_phases / max(n_star, 1)
    return "n%d_g%d_v%d" % (2 ** round(math.log2(max(n, 1))), 50 * round(g / 50.0), 2 ** round(math.log2(max(v, 1))))


def key_of(batch, grids) -> str:
    return batch_class(batch.n, grids, batch.items, batch.n_star)


def load_cache(path: str = CACHE) -> Dict[str, dict]:
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def shape_for(batch, grids, path: str = CACHE) -> Optional[Tuple[int, int]]:
    """The cached (chunk, blocks_per_sm) of the batch's class, or None."""
    e = load_cache(path).get(key_of(batch, grids))
    return (int(e["chunk"]), int(e["blocks_per_sm"])) if e else None


def time_run(batch, reps: int = 3) -> float:
    """ms per batch.run() (CUDA events on torch's current stream, one warm-up run)."""
    import torch
    out = torch.empty((batch.total_phases, 3, batch.n_eff), dtype=torch.float64,
                      device="cuda:%d" % batch.ctx.device)
    batch.run(out)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        batch.run(out)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(batch, candidates=CANDIDATES, reps: int = 3):
    """Times every candidate shape; leaves the batch on the fastest and returns
    ((chunk, blocks_per_sm), {shape: ms})."""
    table = {}
    for c, b in candidates:
        batch.tune(c, b)
        table[(c, b)] = time_run(batch, reps)
    best = min(table, key=table.get)
    batch.tune(*best)
    return best, table


def record(batch, grids, best, table, path: str = CACHE):
    cache = load_cache(path)
    cache[key_of(batch, grids)] = {"chunk": best[0], "blocks_per_sm": best[1],
                                   "ms": {"%d,%d" % k: round(v, 3) for k, v in table.items()}}
    with open(path, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)


def main():
    import argparse
    import ctypes

    import numpy as np
    import torch

    from . import synth
    from ._lib import Activity, Star
    from .api import Batch, Context

    ap = argparse.ArgumentParser()
    ap.add_argument("--stars", type=int, default=64, help="stars of the 256-star batch to tune on")
    ap.add_argument("--out", default=CACHE)
    a = ap.parse_args()
    case = synth.make_case(1)
    inp = synth.generate(case)
    stars = synth.make_batch(256, seed=3)[:a.stars]
    dev = "cuda:0"
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x), device=dev)
    cubes = dict(q_norm=T(inp.q_norm), q_sed=T(inp.q_sed), spot_norm=T(inp.spot_norm), fac_norm=T(inp.fac_norm),
                 spot_sed=T(inp.spot_sed[0]), fac_sed=T(inp.fac_sed[0]))
    with Context(0) as ctx:
        sts = [Star(c.grid, c.period, c.w_ratio, c.incl, c.radius_km, c.u1, c.u2, (ctypes.c_double * 4)(*inp.lb))
               for c in stars]
        b = Batch(ctx, T(inp.wave), case.n_eff, cubes, inp.mu_boundary, case.step,
                  Activity(case.t_star, case.t_diff_spot, case.t_diff_fac, case.nrho, 0), case.sigma_v, sts,
                  [c.phases for c in stars], [[c.regions for _ in c.phases] for c in stars], conv_step=case.step)
        best, table = tune(b)
        record(b, [c.grid for c in stars], best, table, a.out)
        print(json.dumps({"class": key_of(b, [c.grid for c in stars]), "best": best,
                          "ms": {"%d,%d" % k: round(v, 3) for k, v in table.items()}}))
        b.close()


if __name__ == "__main__":
    main()
