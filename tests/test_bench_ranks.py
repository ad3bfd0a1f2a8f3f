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
    q.put((rank, ms, bench.job_models_per_s(8, world, ms)))
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


def test_roofline_flops_do_not_depend_on_the_step_count():
    """The LU + solve rate is the device-counted work of the one timed launch
    over that launch's time: splitting the grid into more steps changes
    ms_per_step, not the achieved rate."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    n, nlu, nni, ms = 336, 1.0e6, 4.0e6, 250e3
    want = (2.0 / 3.0 * n ** 3 * nlu + 2.0 * n * n * nni) / (ms / 1e3) / 1e12
    assert abs(bench.lu_solve_tflops(n, nlu, nni, ms) - want) < 1e-12 * want


def test_stratified_sample_covers_every_density_stratum():
    from uclchem_gb300.params import grid_params, stratified_sample
    import numpy as np
    dicts = grid_params(4096)
    idx = stratified_sample(dicts, 64)
    assert idx == stratified_sample(dicts, 64) and len(set(idx)) == 64
    ranks = np.argsort(np.argsort([d["initialDens"] for d in dicts]))
    assert sorted(int(ranks[i]) // 64 for i in idx) == list(range(64))


def test_element_drift_counts_successful_rows_only():
    import sys
    import numpy as np
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    tot = np.ones((2, 4, 3))
    tot[0, 2, 1] = 1.0 + 3e-9
    tot[1, 3, 0] = 2.0  # failed model and a row past nrows: ignored
    assert abs(bench.element_drift(tot, np.array([3, 4]), np.array([0, -5])) - 3e-9) < 1e-15
