"""Phase sharding over replicas with the gloo backend on CPU (world size 2): the
gathered per-phase results equal the single-process ones.  The per-phase work here
is the oracle's region-map scan, so the test needs no GPU."""
import os
import socket

import numpy as np
import pytest

from soap_gpu_gb300.replicas import phase_shard, run_sharded


def test_phase_shard_covers_all_phases():
    for n in (0, 1, 7, 100):
        for w in (1, 2, 3, 8):
            blocks = [phase_shard(n, w, r) for r in range(w)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            for (a, b), (c, d) in zip(blocks, blocks[1:]):
                assert b == c
            sizes = [b - a for a, b in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        phase_shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_q):
    import torch.distributed as dist
    import oracle
    from soap_gpu_gb300 import synth
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    case = synth.small_case(seed=1, grid=24, n=2600, n_phase=5, n_mu=4)

    def work(start, stop):
        res = []
        for ph in case.phases[start:stop]:
            t, b = oracle.phase_maps(case.grid, case.nrho, case.incl, ph, case.regions, case.t_star,
                                     case.t_diff_spot, case.t_diff_fac)
            res.append(int(np.sum(b >= 0)) * 1000003 + int(np.sum(t[b >= 0])))
        return res

    got = run_sharded(len(case.phases), work)
    out_q.put((rank, got))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_gather_in_phase_order():
    import multiprocessing as mp
    import oracle
    from soap_gpu_gb300 import synth
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    case = synth.small_case(seed=1, grid=24, n=2600, n_phase=5, n_mu=4)
    ref = []
    for ph in case.phases:
        t, b = oracle.phase_maps(case.grid, case.nrho, case.incl, ph, case.regions, case.t_star, case.t_diff_spot,
                                 case.t_diff_fac)
        ref.append(int(np.sum(b >= 0)) * 1000003 + int(np.sum(t[b >= 0])))
    assert results[0] == ref and results[1] == ref
