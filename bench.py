"""Benchmark: models/s of the batched mixed-precision CLOUD-grid solve on one
GB300, against the plain-FP64 GPU path, with p50/p99 per-model latency.

Workload: the 4096-point static CLOUD grid (seeded log-uniform density
1e2-1e7 cm^-3, temperature 10-50 K, zeta and radfield 1-1e3, 1e6 yr, default
335-species network, reltol 1e-8).  One step = integrating every model of
the grid to 1e6 yr (46 output intervals each).

  value      models/s, mixed path, inputs and outputs resident in HBM
  e2e        models/s through ucl_solve_models with host buffers (copies in
             the timed region)
  fp64       plain-FP64 path and mixed path on an identical subset (ratio
             and max |dex| between the two)
  cpu_baseline  the CPU oracle (C restatement of the reference solver) on
             the host cores, on a bounded sample of the same grid

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Models/s batched-mixed vs plain-FP64 GPU at <=0.01 dex; p50/p99 latency"
UNIT = "models/s"
def workload(models: int, final_time: float) -> str:
    return (f"{models}-point static CLOUD grid (seeded), default network (335 species, 3203 reactions), "
            f"{final_time:g} yr, reltol 1e-8")
MAX_ROWS = 64
# DRAM bytes (read + write) of the mixed solver per model-step, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the 152-model,
# 1e4-yr grid launch: 113.6 GB over 152 x 4094 model-steps.  Traffic scales
# with model-steps once the slots' working set exceeds L2.
DRAM_BYTES_PER_MODEL_STEP = 1.83e5
SEED = 20261203


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--models", type=int, default=4096)
    ap.add_argument("--subset", type=int, default=16, help="models in the FP64 comparison subset")
    ap.add_argument("--subset-final-time", type=float, default=1e5,
                    help="finalTime (yr) of the FP64-vs-mixed comparison subset")
    ap.add_argument("--warmup-models", type=int, default=152, help="models per warm-up step")
    ap.add_argument("--warmup-final-time", type=float, default=1e3, help="finalTime (yr) of warm-up models")
    ap.add_argument("--cpu-seconds", type=float, default=30.0)
    ap.add_argument("--final-time", type=float, default=1e6, help="finalTime (yr) of the grid models")
    ap.add_argument("--dump", default="", help="write per-model parameters, flags and device stats of the "
                                                "timed step to this .npz")
    ap.add_argument("--serve", type=int, default=0, help="serving run: number of Poisson-arriving requests")
    ap.add_argument("--rate", type=float, default=20.0, help="serving arrival rate (requests/s)")
    ap.add_argument("--kernel", default="solve", choices=["solve", "lu"],
                    help="lu: time the batched Newton-matrix LU alone (--models matrices)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# --------------------------------------------------------------------------
def max_over_ranks(ms: float, device, world: int) -> float:
    """The job's time is the slowest rank's (one replica per GPU, no data
    exchange between them)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def full_grid_conservation(ab_d, nrows, flags, dev):
    """Largest relative drift of the H, He, C, N, O and S totals over every
    output row of every successful model (computed on the device), or None
    if it cannot be formed."""
    try:
        import torch
        from uclchem_gb300 import network
        from uclchem_gb300.analysis import element_counts
        species = network.load_default().species
        E = np.stack([element_counts(species, e) for e in ("H", "HE", "C", "N", "O", "S")], axis=1)
        tot = torch.matmul(ab_d, torch.from_numpy(E.astype(np.float64)).to(dev)).cpu().numpy()
        worst = 0.0
        for m in np.nonzero(flags == 0)[0]:
            r = int(nrows[m])
            if r < 2:
                continue
            t0 = tot[m, 0]
            ok = t0 > 0
            worst = max(worst, float(np.abs(tot[m, 1:r][:, ok] / t0[ok] - 1.0).max()))
        return worst
    except Exception:
        return None


def job_models_per_s(models_per_rank: int, world: int, steps: int, ms: float) -> float:
    """Whole-job throughput: every rank integrates its own grid sample."""
    return models_per_rank * world * steps / (ms / 1e3)


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
def _cpu_one(d):
    """One model on the oracle in a worker process; returns its wall time."""
    global _ORACLE
    if _ORACLE is None:
        from oracle.oracle import Oracle
        _ORACLE = Oracle()
    t = time.time()
    _ORACLE.cloud(d, max_rows=MAX_ROWS)
    return time.time() - t


_ORACLE = None


def cpu_baseline(dicts, seconds: float, procs: int):
    """The oracle (C restatement of the reference solver) on the host cores:
    one model per worker process (spawned, as the reference's grid script runs
    one model per process), grid points taken in order, counting the models
    completed within a wall-clock window of `seconds`; unfinished models are
    abandoned at the deadline (which favours the CPU: slow models drop out)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(procs)
    t0 = time.time()
    done = 0
    it = pool.imap_unordered(_cpu_one, dicts)
    try:
        while True:
            left = seconds - (time.time() - t0)
            if left <= 0:
                break
            it.next(timeout=left)
            done += 1
    except (StopIteration, mp.TimeoutError):
        pass
    dt = time.time() - t0
    pool.terminate()
    pool.join()
    return {"value": done / dt, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{done} models completed in a {dt:.1f} s window by {procs} worker processes "
                      f"(grid points in order, one model per process)"}


def reference_arm(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from uclchem_gb300.params import grid_params
    dicts = grid_params(args.models, seed=SEED, final_time=args.final_time)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(max(args.warmup, 0)):
        pass  # the oracle has no warm-up state
    for _ in range(max(args.steps, 1)):
        cb = cpu_baseline(dicts, args.cpu_seconds, threads)
        vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * args.cpu_seconds, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload(args.models, args.final_time), "models": args.models, "seed": SEED},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
def our_arm(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from uclchem_gb300 import _lib, network
    from uclchem_gb300.params import PARAMS_DTYPE, grid_params, make_param_array

    ctx = _lib.Context(network.DEFAULT_BLOB, device=local)
    nspec, neq = ctx.nspec, ctx.neq
    M = args.models
    dicts = grid_params(M, seed=SEED + rank, final_time=args.final_time)
    params = make_param_array(dicts)
    dev = torch.device("cuda", local)
    p_d = torch.from_numpy(params.view(np.uint8).reshape(M, -1).copy()).to(dev)
    phys_d = torch.empty((M, MAX_ROWS, 8), dtype=torch.float64, device=dev)
    ab_d = torch.empty((M, MAX_ROWS, nspec), dtype=torch.float64, device=dev)
    nr_d = torch.empty(M, dtype=torch.int32, device=dev)
    fl_d = torch.empty(M, dtype=torch.int32, device=dev)
    st_d = torch.empty((M, _lib.STATS_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    # a dedicated stream: the C ABI maps a NULL stream handle (torch's default
    # stream) to the context's own stream, which the events would not bracket
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)

    def solve(n, prec):
        ctx.solve_models_device(n, p_d.data_ptr(), None, MAX_ROWS, phys_d.data_ptr(), ab_d.data_ptr(),
                                nr_d.data_ptr(), fl_d.data_ptr(), st_d.data_ptr(), prec, 0, stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def upload(arr):
        p_d[: arr.size].copy_(torch.from_numpy(arr.view(np.uint8).reshape(arr.size, -1).copy()))

    # warm-up steps: the same kernels on the first grid points, integrated to a short time
    wm = min(args.warmup_models, M)
    upload(make_param_array(grid_params(M, seed=SEED + rank, final_time=args.warmup_final_time)[:wm]))
    for _ in range(args.warmup):
        solve(wm, _lib.PREC_MIXED)
    upload(params)
    barrier()
    clk = ClockSampler(local)
    clk.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    ev0.record(stream)
    for _ in range(args.steps):
        solve(M, _lib.PREC_MIXED)
    ev1.record(stream)
    barrier()
    wall = time.time() - t0
    clocks = clk.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dev, world)
    ms_per_step = ms / args.steps
    value = job_models_per_s(M, world, args.steps, ms)
    stats = st_d.cpu().numpy().view(_lib.STATS_DTYPE).reshape(M)
    flags = fl_d.cpu().numpy()
    nrows = nr_d.cpu().numpy()
    if args.dump and rank == 0:
        np.savez(args.dump, params=params, flags=flags, nrows=nrows, stats=stats)
    lat = stats["solve_ms"]
    conservation = full_grid_conservation(ab_d, nrows, flags, dev)

    # work counted by the device (for the roofline of the megakernel)
    n = neq
    lu_flop = 2.0 / 3.0 * n ** 3 * stats["nlu"].sum()
    solve_flop = 2.0 * n * n * stats["nni"].sum()
    mat_tflops = (lu_flop + solve_flop) / (ms_per_step / 1e3) / 1e12 / args.steps

    # plain FP64 vs mixed on an identical subset (same wave structure)
    S = min(args.subset, M)
    upload(make_param_array(grid_params(M, seed=SEED + rank, final_time=args.subset_final_time)[:S]))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solve(S, _lib.PREC_FP64)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    fp64_ms = e0.elapsed_time(e1)
    f_ab = ab_d[:S].cpu().numpy()
    f_nr = nr_d[:S].cpu().numpy()
    f_fl = fl_d[:S].cpu().numpy()
    e0.record(stream)
    solve(S, _lib.PREC_MIXED)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    mix_sub_ms = e0.elapsed_time(e1)
    mix_ab = ab_d[:S].cpu().numpy()
    mix_nr = nr_d[:S].cpu().numpy()
    mix_fl = fl_d[:S].cpu().numpy()
    ok = (f_fl == 0) & (mix_fl == 0) & (f_nr == mix_nr)
    dex = 0.0
    for k in np.nonzero(ok)[0]:
        r = int(f_nr[k])
        a, b = mix_ab[k, :r], f_ab[k, :r]
        sel = (a > 1e-14) | (b > 1e-14)
        if sel.any():
            dex = max(dex, float(np.where(sel, np.abs(np.log10(np.maximum(a, 1e-300)) -
                                                       np.log10(np.maximum(b, 1e-300))), 0).max()))

    # end to end through the host-buffer C ABI (copies inside the timed region)
    t0 = time.time()
    phys_h, ab_h, nr_h, fl_h, st_h = ctx.solve_models(params, MAX_ROWS, precision=_lib.PREC_MIXED)
    e2e_s = time.time() - t0
    h2d = params.nbytes
    d2h = phys_h.nbytes + ab_h.nbytes + nr_h.nbytes + fl_h.nbytes + st_h.nbytes

    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    cpu = cpu_baseline(dicts, args.cpu_seconds, os.cpu_count() or 1) if world == 1 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded parameter grid; default UCLCHEM network)",
        "config": {"workload": workload(M, args.final_time), "models": M, "seed": SEED, "precision": "mixed (FP32 LU)",
                   "l2": "inputs larger than L2: 152 resident model slots x ~1.1 MB (J, P, factors, scratch) = ~167 MB "
                      "> 129 MB L2, rewritten throughout the step; one step is one launch"},
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "failed_models": int((flags != 0).sum()),
        # size-independent parity property over the whole timed grid: element
        # totals (H, He, C, N, O, S) relative to each model's first row
        "max_element_drift": conservation,
        "fp64": {"models": S, "final_time_yr": args.subset_final_time, "fp64_models_per_s": S / (fp64_ms / 1e3),
                 "mixed_models_per_s": S / (mix_sub_ms / 1e3), "speedup": fp64_ms / mix_sub_ms,
                 "max_dex_mixed_vs_fp64": dex, "compared": int(ok.sum())},
        "e2e": {"value": M / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        # per step: the persistent solver, plus the admission-order sort when
        # the batch exceeds the resident slots
        "gpu_launches": args.steps * (2 if M > ctx.slots(_lib.PREC_MIXED) else 1),
        "clocks": clocks,
        "counters": {k: float(stats[k].mean()) for k in ("nst", "nfe", "nje", "nlu", "nni")},
        # device phase timers of the timed step (globaltimer, per call and share of model time)
        "phase_us_per_call": {
            "rhs": 1e3 * float(stats["t_rhs_ms"].sum() / max(stats["nfe"].sum(), 1)),
            "jacobian": 1e3 * float(stats["t_jac_ms"].sum() / max(stats["nje"].sum(), 1)),
            "lu": 1e3 * float(stats["t_lu_ms"].sum() / max(stats["nlu"].sum(), 1)),
            "solve": 1e3 * float(stats["t_solve_ms"].sum() / max(stats["nni"].sum(), 1))},
        "phase_share": {k: float(stats[f"t_{k}_ms"].sum() / max(stats["solve_ms"].sum(), 1e-30))
                        for k in ("rates", "rhs", "jac", "lu", "solve")},
        "roofline": {"bound": "tensor", "achieved": mat_tflops, "peak": peak, "unit": "TFLOP/s",
                     "frac": mat_tflops / peak,
                     "traffic": DRAM_BYTES_PER_MODEL_STEP * float(stats["nst"].sum()) / args.steps,
                     "note": "k_solve_models: LU (2/3 n^3 per factorisation) + triangular solves (2 n^2 per "
                             "Newton iteration) counted by the device, over the step time, against the measured "
                             "dense bf16 peak (the LU's trailing update runs on the tensor cores); the kernel is "
                             "latency-bound (one CTA per model, barrier-separated phases), hence the small "
                             "fraction; traffic = DRAM bytes per model-step from one ncu capture x model-steps"},
        "cpu_baseline": cpu,
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def lu_kernel(args):
    """Batched Newton-matrix LU alone (ucl_lu_factor_device): --models
    matrices of the network's size (I - c*J-like, random), FP32 and FP64,
    timed with CUDA events; prints one line per precision."""
    import torch
    from uclchem_gb300 import _lib, network
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    n, B = ctx.neq, args.models
    rng = np.random.default_rng(SEED)
    for prec, dt in ((_lib.PREC_MIXED, torch.float32), (_lib.PREC_FP64, torch.float64)):
        A = (torch.eye(n, dtype=torch.float64)[None] -
             torch.from_numpy(rng.standard_normal((B, n, n)) * 10.0 ** rng.uniform(-3, 1, (B, 1, n)))).to(dt).cuda()
        m = torch.empty_like(A)
        perm = torch.empty((B, n), dtype=torch.int32, device="cuda")
        info = torch.empty(B, dtype=torch.int32, device="cuda")
        ts = []
        for it in range(args.warmup + args.steps):
            m.copy_(A)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.lu_factor_device(B, n, prec, m.data_ptr(), perm.data_ptr(), info.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            stream.synchronize()
            if it >= args.warmup:
                ts.append(e0.elapsed_time(e1))
        ms = float(np.median(ts))
        flop = 2.0 / 3.0 * n ** 3 * B
        print(json.dumps({"kernel": "k_lu_batch", "precision": "fp32" if prec == _lib.PREC_MIXED else "fp64",
                          "n": n, "matrices": B, "ms": ms, "us_per_matrix_wave": ms * 1e3 / max(1, -(-B // 152)),
                          "tflops": flop / (ms * 1e-3) / 1e12, "info_max": int(info.max())}), flush=True)
    ctx.close()


def serve_requests(n: int, seed: int = SEED):
    """The serving mix: 70% static CLOUD, 30% freefall collapse 1e2 -> 1e6
    cm^-3, finalTime 10^U(4,7) yr, other parameters drawn as in the grid."""
    from uclchem_gb300.params import grid_params
    rng = np.random.default_rng(seed + 5)
    reqs = grid_params(n, seed=seed + 7, final_time=1e6)
    for d in reqs:
        d["finalTime"] = float(10 ** rng.uniform(4, 7))
        if rng.uniform() < 0.3:
            d.update({"freefall": True, "initialDens": 1e2, "finalDens": 1e6})
    return reqs


def serve_arm(args):
    """Poisson request stream through ucl_serve_models_device: requests are
    admitted on the device at their arrival times; p50/p99 latency (arrival
    to completion) and completed models/s."""
    import torch
    from uclchem_gb300 import _lib, network
    from uclchem_gb300.params import make_param_array
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    n, rows = args.serve, 160
    reqs = serve_requests(n)
    params = make_param_array(reqs)
    rng = np.random.default_rng(SEED + 11)
    arrival = np.cumsum(rng.exponential(1.0 / args.rate, n))
    dev = torch.device("cuda", 0)
    p_d = torch.from_numpy(params.view(np.uint8).reshape(n, -1).copy()).to(dev)
    a_d = torch.from_numpy(arrival).to(dev)
    ph = torch.empty((n, rows, 8), dtype=torch.float64, device=dev)
    ab = torch.empty((n, rows, ctx.nspec), dtype=torch.float64, device=dev)
    nr = torch.empty(n, dtype=torch.int32, device=dev)
    fl = torch.empty(n, dtype=torch.int32, device=dev)
    sd = torch.empty((n, _lib.STATS_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.serve_models_device(n, p_d.data_ptr(), a_d.data_ptr(), None, rows, ph.data_ptr(), ab.data_ptr(),
                            nr.data_ptr(), fl.data_ptr(), sd.data_ptr(), _lib.PREC_MIXED, 0, stream.cuda_stream)
    e1.record(stream)
    stream.synchronize()
    ms = e0.elapsed_time(e1)
    st = sd.cpu().numpy().view(_lib.STATS_DTYPE).reshape(n)
    flags = fl.cpu().numpy()
    lat = st["latency_ms"]
    print(json.dumps({"mode": "serving", "requests": n, "arrival_rate_per_s": args.rate,
                      "mix": "70% static CLOUD, 30% freefall 1e2->1e6; finalTime 10^U(4,7) yr",
                      "models_per_s": n / (ms / 1e3), "wall_ms": ms,
                      "p50_latency_ms": float(np.percentile(lat, 50)), "p99_latency_ms": float(np.percentile(lat, 99)),
                      "p50_queue_ms": float(np.percentile(st["queue_ms"], 50)),
                      "p99_queue_ms": float(np.percentile(st["queue_ms"], 99)),
                      "failed": int((flags != 0).sum()), "slots": ctx.slots(_lib.PREC_MIXED)}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.serve > 0:
        serve_arm(args)
        return
    if args.kernel == "lu":
        lu_kernel(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()
