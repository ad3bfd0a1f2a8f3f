"""The bench's N>1 path on CPU with gloo, world size 2: each rank is an
independent replica (its own grid sample, no data exchange); the job time is
the maximum over ranks and throughput counts every rank's models."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import sys
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = bench.max_over_ranks(100.0 * (rank + 1), torch.device("cpu"), world)
    q.put((rank, ms, bench.job_models_per_s(8, world, 1, ms)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [200.0, 200.0]
    assert all(abs(o[2] - 16 / 0.2) < 1e-9 for o in out)


def test_grid_samples_differ_per_rank():
    from uclchem_gb300.params import grid_params
    a = grid_params(4, seed=20261203 + 0)
    b = grid_params(4, seed=20261203 + 1)
    assert a != b and len(a) == len(b) == 4


def test_serving_mix_matches_the_workload_description():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    reqs = bench.serve_requests(2000)
    ff = [d for d in reqs if d.get("freefall")]
    assert 0.25 < len(ff) / len(reqs) < 0.35
    assert all(d["initialDens"] == 1e2 and d["finalDens"] == 1e6 for d in ff)
    ft = [d["finalTime"] for d in reqs]
    assert 1e4 <= min(ft) and max(ft) <= 1e7
