"""Benchmark: models/s of the batched mixed-precision CLOUD-grid solve on one
GB300, against the plain-FP64 GPU path, with p50/p99 per-model latency.

Workload: the 4096-point static CLOUD grid (seeded: density 10^U(2,7) cm^-3,
temperature U(10,50) K, zeta and radfield 10^U(0,3); 1e6 yr; default
335-species network; reltol 1e-8) with 501 output rows per model, the
reference's TIMEPOINTS=500 (src/uclchem/constants.py:22).

A step is 1/K of the grid (K = --steps, default 16, so 256 models a step).
The K steps of the timed region are admitted together into one persistent
launch: a model's cost spans three orders of magnitude (0.1 s to ~100 s), so
back-to-back launches per step would each wait for their slowest model,
while one launch lets the heavy tail of one step overlap the others.
ms_per_step = (timed region) / K.

  value         models/s, mixed path, inputs and outputs resident in HBM
  e2e           the same grid through ucl_solve_models with host buffers
                (params copied in, every output row copied out, inside the
                timed region)
  fp64          the plain-FP64 path and the mixed path on the same
                stratified sample of the grid, to 1e6 yr: makespan and
                per-model device-time ratios, and the max |dex| between them
  cpu_baseline  the CPU oracle (C restatement of the reference solver) on all
                host cores, one model per process, on a seeded sample of the
                grid stratified over density, each model capped at 180 CPU s
                (an upper bound on the CPU's grid models/s)

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
SEED = 20261203
ROWS = 501          # TIMEPOINTS + 1 (src/uclchem/constants.py:22)
# DRAM bytes (read + write) of the mixed solver per model-step, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the 152-model,
# 1e4-yr grid launch: 161.2 GB over 152 x 4187.6 model-steps.  Traffic scales
# with model-steps once the slots' working set exceeds L2.
DRAM_BYTES_PER_MODEL_STEP = 2.53e5
FALLBACK_BF16_TFLOPS = 1900.0


def workload(models: int, final_time: float) -> str:
    return (f"{models}-point static CLOUD grid (seeded), default network (335 species, 3203 reactions), "
            f"{final_time:g} yr, reltol 1e-8, {ROWS} output rows per model")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16, help="the grid is split into this many steps")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--models", type=int, default=4096)
    ap.add_argument("--final-time", type=float, default=1e6, help="finalTime (yr) of the grid models")
    ap.add_argument("--subset", type=int, default=64, help="models in the FP64-vs-mixed sample")
    ap.add_argument("--warmup-models", type=int, default=152, help="models per warm-up step")
    ap.add_argument("--warmup-final-time", type=float, default=1e3, help="finalTime (yr) of warm-up models")
    ap.add_argument("--cpu-sample", type=int, default=32, help="grid models in the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer run")
    ap.add_argument("--dump", default="", help="write per-model parameters, flags and device stats of the "
                                                "timed grid (and of the FP64 sample) to this .npz")
    ap.add_argument("--serve", type=int, default=0, help="serving run: number of Poisson-arriving requests")
    ap.add_argument("--rate", type=float, default=20.0, help="serving arrival rate (requests/s)")
    ap.add_argument("--serve-capacity", type=int, default=4096, help="request/output records of the server")
    ap.add_argument("--synthetic", type=int, default=0,
                    help="synthetic-network run: systems per network size (N = 64, 128, 256, 512), one launch")
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


def job_models_per_s(models_per_rank: int, world: int, ms: float) -> float:
    """Whole-job throughput: every rank integrates its own grid."""
    return models_per_rank * world / (ms / 1e3)


def lu_solve_tflops(n: int, nlu: float, nni: float, ms: float) -> float:
    """LU (2/3 n^3 per factorisation) + triangular-solve (2 n^2 per Newton
    iteration) flops counted by the device over `ms` of kernel time."""
    return (2.0 / 3.0 * n ** 3 * nlu + 2.0 * n * n * nni) / (ms / 1e3) / 1e12


def element_drift(tot: np.ndarray, nrows: np.ndarray, flags: np.ndarray) -> float:
    """Largest |total(row)/total(row 0) - 1| over the rows of successful
    models; tot [models, rows, elements]."""
    worst = 0.0
    for m in np.nonzero(flags == 0)[0]:
        r = int(nrows[m])
        if r < 2:
            continue
        t0 = tot[m, 0]
        ok = t0 > 0
        worst = max(worst, float(np.abs(tot[m, 1:r][:, ok] / t0[ok] - 1.0).max()))
    return worst


def full_grid_conservation(ab_d, nrows, flags, dev):
    """Largest relative drift of the network's conserved element totals (He,
    C, N, O, S, Si, Mg, Cl: every element each reaction conserves; H is not,
    some freeze-outs hydrogenate) over every output row of every successful
    model (totals formed on the device)."""
    import torch
    from uclchem_gb300 import network
    E = network.load_default().invariants().T
    Ed = torch.from_numpy(E.astype(np.float64)).to(dev)
    tot = np.concatenate([torch.matmul(ab_d[i:i + 256], Ed).cpu().numpy() for i in range(0, ab_d.shape[0], 256)])
    return element_drift(tot, nrows, flags)


def max_dex(a_ab, a_nr, a_fl, b_ab, b_nr, b_fl, floor=1e-14):
    """Per-model max |log10 a - log10 b| over species above `floor` in either,
    for models that succeed in both with the same rows (NaN otherwise)."""
    out = np.full(len(a_nr), np.nan)
    for k in range(len(a_nr)):
        if a_fl[k] != 0 or b_fl[k] != 0 or a_nr[k] != b_nr[k]:
            continue
        r = int(a_nr[k])
        a, b = a_ab[k, :r], b_ab[k, :r]
        sel = (a > floor) | (b > floor)
        d = np.abs(np.log10(np.maximum(a, 1e-300)) - np.log10(np.maximum(b, 1e-300)))
        out[k] = float(np.where(sel, d, 0.0).max()) if sel.any() else 0.0
    return out


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
# CPU baseline: the oracle, one model per spawned worker process
_ORACLE = None
CPU_CAP_S = 180.0


def _cpu_one(task):
    """One model on the oracle in a worker process, stopped at `cap` CPU
    seconds; returns (CPU seconds used, whether the cap stopped it)."""
    global _ORACLE
    d, cap = task
    if _ORACLE is None:
        from oracle.oracle import Oracle
        _ORACLE = Oracle()
    _ORACLE.set_cpu_limit(cap)
    t = time.process_time()
    flag = _ORACLE.cloud(d, max_rows=ROWS)[2]
    return time.process_time() - t, flag == _ORACLE.CPU_LIMIT_FLAG


def cpu_sample_run(dicts, idx, procs: int, cap: float):
    """Run the grid models `idx` on `procs` worker processes (spawned, one
    model per process at a time, as the reference's grid script runs its
    models), each stopped at `cap` CPU seconds.  Returns (wall seconds,
    per-model CPU seconds, per-model capped)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        pool.map(_cpu_one, [({"initialDens": 1e4, "finalTime": 1.0}, 0.0)] * procs, chunksize=1)  # start-up
        t0 = time.time()
        # longest-expected (densest) first, so the sample's tail does not start last
        order = sorted(idx, key=lambda i: -dicts[i]["initialDens"])
        res = pool.map(_cpu_one, [(dicts[i], cap) for i in order], chunksize=1)
        wall = time.time() - t0
    return wall, np.array([r[0] for r in res]), np.array([r[1] for r in res])


def cpu_estimate(dicts, size: int, procs: int, cap: float = CPU_CAP_S):
    """The CPU's models/s on the whole grid, estimated from a seeded
    density-stratified sample: with every core busy on a 4096-model grid the
    cores finish models at procs / (mean CPU seconds per model).  Models
    stopped at the cap count as `cap` seconds, so the figure is an upper
    bound on the CPU's throughput (it favours the CPU)."""
    from uclchem_gb300.params import stratified_sample
    idx = stratified_sample(dicts, size, seed=SEED)
    wall, cpu_s, capped = cpu_sample_run(dicts, idx, procs, cap)
    value = procs * len(idx) / float(cpu_s.sum())
    return {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{len(idx)} grid models stratified over density (one per stratum, seeded), {ROWS} rows; "
                      f"each on one of {procs} worker processes, stopped at {cap:g} CPU s; value = cores x models / "
                      f"total CPU s ({int(capped.sum())} of {len(idx)} models hit the cap and count as {cap:g} s, "
                      f"so this is an upper bound on the CPU's models/s); median {np.median(cpu_s):.1f} CPU s",
            "capped": int(capped.sum()), "wall_s": wall}


def reference_arm(args):
    """The reference's CPU path (the oracle port: the reference's Fortran
    cannot be compiled in this image) on all host cores.  The K steps are K
    slices of a seeded density-stratified sample of the grid, all queued to
    one process pool, like the GPU arm's one launch; value as cpu_estimate."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from uclchem_gb300.params import grid_params
    dicts = grid_params(args.models, seed=SEED, final_time=args.final_time)
    procs = os.cpu_count() or 1
    cb = cpu_estimate(dicts, max(args.cpu_sample, args.steps), procs)
    v = cb["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * cb["wall_s"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded parameter grid; default UCLCHEM network)",
            "config": {"workload": workload(args.models, args.final_time), "models": args.models, "seed": SEED,
                       "steps": f"{args.steps} slices of the CPU sample, queued to one pool"},
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
    from uclchem_gb300.params import grid_params, make_param_array, stratified_sample

    ctx = _lib.Context(network.DEFAULT_BLOB, device=local)
    nspec, neq = ctx.nspec, ctx.neq
    M, K = args.models, max(1, args.steps)
    dicts = grid_params(M, seed=SEED + rank, final_time=args.final_time)
    params = make_param_array(dicts)
    dev = torch.device("cuda", local)
    p_d = torch.from_numpy(params.view(np.uint8).reshape(M, -1).copy()).to(dev)
    phys_d = torch.empty((M, ROWS, 8), dtype=torch.float64, device=dev)
    ab_d = torch.empty((M, ROWS, nspec), dtype=torch.float64, device=dev)
    nr_d = torch.empty(M, dtype=torch.int32, device=dev)
    fl_d = torch.empty(M, dtype=torch.int32, device=dev)
    st_d = torch.empty((M, _lib.STATS_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    # a dedicated stream: the C ABI maps a NULL stream handle (torch's default
    # stream) to the context's own stream, which the events would not bracket
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)

    def solve(n, prec):
        ctx.solve_models_device(n, p_d.data_ptr(), None, ROWS, phys_d.data_ptr(), ab_d.data_ptr(),
                                nr_d.data_ptr(), fl_d.data_ptr(), st_d.data_ptr(), prec, 0, stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def upload(arr):
        p_d[: arr.size].copy_(torch.from_numpy(arr.view(np.uint8).reshape(arr.size, -1).copy()))

    def timed(n, prec):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solve(n, prec)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1)

    # warm-up steps: the same kernels on the first grid points, to a short time
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
    solve(M, _lib.PREC_MIXED)  # all K steps in one persistent launch
    ev1.record(stream)
    barrier()
    wall = time.time() - t0
    clocks = clk.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dev, world)
    value = job_models_per_s(M, world, ms)
    stats = st_d.cpu().numpy().view(_lib.STATS_DTYPE).reshape(M)
    flags = fl_d.cpu().numpy()
    nrows = nr_d.cpu().numpy()
    lat = stats["solve_ms"]
    conservation = full_grid_conservation(ab_d, nrows, flags, dev)
    mat_tflops = lu_solve_tflops(neq, float(stats["nlu"].sum()), float(stats["nni"].sum()), ms)
    dump = {"params": params, "flags": flags, "nrows": nrows, "stats": stats}

    # plain FP64 vs mixed on the same stratified sample of the grid
    S = min(args.subset, M)
    sub = stratified_sample(dicts, S, seed=SEED + 2)
    upload(params[sub])
    fp64_ms = timed(S, _lib.PREC_FP64)
    f_st = st_d[:S].cpu().numpy().view(_lib.STATS_DTYPE).reshape(S).copy()
    f_ab, f_nr, f_fl = ab_d[:S].cpu().numpy(), nr_d[:S].cpu().numpy(), fl_d[:S].cpu().numpy()
    mix_ms = timed(S, _lib.PREC_MIXED)
    m_st = st_d[:S].cpu().numpy().view(_lib.STATS_DTYPE).reshape(S).copy()
    m_ab, m_nr, m_fl = ab_d[:S].cpu().numpy(), nr_d[:S].cpu().numpy(), fl_d[:S].cpu().numpy()
    dex = max_dex(m_ab, m_nr, m_fl, f_ab, f_nr, f_fl)
    both = ~np.isnan(dex)
    dump.update(sub=np.array(sub), fp64_stats=f_st, fp64_flags=f_fl, sub_mixed_stats=m_st, sub_dex=dex)
    del f_ab, m_ab

    # end to end through the host-buffer C ABI (copies inside the timed region)
    e2e = None
    if not args.no_e2e:
        t0 = time.time()
        phys_h, ab_h, nr_h, fl_h, st_h = ctx.solve_models(params, ROWS, precision=_lib.PREC_MIXED)
        e2e_s = time.time() - t0
        h2d = params.nbytes
        d2h = phys_h.nbytes + ab_h.nbytes + nr_h.nbytes + fl_h.nbytes + st_h.nbytes
        e2e = {"value": M * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d // K),
               "d2h_bytes_per_step": int(d2h // K),
               "note": "the whole grid (all K steps) in one ucl_solve_models call: params copied in, every "
                       "output row, flag and stat copied out"}
        del phys_h, ab_h

    if args.dump and rank == 0:
        np.savez(args.dump, **dump)
    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("bf16_tflops", FALLBACK_BF16_TFLOPS))
    peak_src = "measured" if "bf16_tflops" in peaks else "fallback"
    cpu = cpu_estimate(dicts, args.cpu_sample, os.cpu_count() or 1) if world == 1 and args.cpu_sample > 0 else None
    nslots = ctx.slots(_lib.PREC_MIXED)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded parameter grid; default UCLCHEM network)",
        "config": {"workload": workload(M, args.final_time), "models": M, "seed": SEED, "rows": ROWS,
                   "precision": "mixed (FP32 LU on tcgen05 3xTF32, FP64 elsewhere)",
                   "step": f"1/{K} of the grid ({M // K} models); the {K} steps are admitted together into one "
                           f"persistent launch of {nslots} model slots",
                   "l2": "inputs larger than L2: 152 resident model slots x ~1.1 MB (J, P, factors, scratch) = "
                         "~167 MB > 129 MB L2, rewritten throughout the launch; 5.5 GB of output rows"},
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "latency": "per-model device time from start to completion (globaltimer)",
        "failed_models": int((flags != 0).sum()),
        "failed_codes": {str(int(c)): int((flags == c).sum()) for c in np.unique(flags[flags != 0])},
        # size-independent parity property over the whole timed grid: element
        # totals (H, He, C, N, O, S) relative to each model's first row
        "max_element_drift": conservation,
        "fp64": {"sample": f"{S} grid models stratified over density (seeded), {args.final_time:g} yr",
                 "fp64_models_per_s": S / (fp64_ms / 1e3), "mixed_models_per_s": S / (mix_ms / 1e3),
                 "speedup_makespan": fp64_ms / mix_ms,
                 "speedup_model_time": float(f_st["solve_ms"].sum() / max(m_st["solve_ms"].sum(), 1e-9)),
                 "fp64_slots": ctx.slots(_lib.PREC_FP64), "mixed_slots": nslots,
                 "max_dex_mixed_vs_fp64": float(np.nanmax(dex)) if both.any() else None,
                 "models_over_0.01_dex": int((dex[both] > 0.01).sum()), "compared": int(both.sum()),
                 "failed_fp64": int((f_fl != 0).sum()), "failed_mixed": int((m_fl != 0).sum())},
        "e2e": e2e,
        # in the timed region: the admission-order sort and the persistent solver
        "gpu_launches": 2 if M > nslots else 1,
        "clocks": clocks,
        "counters": {k: float(stats[k].mean()) for k in ("nst", "nfe", "nje", "nlu", "nni")},
        # device phase timers of the timed grid (globaltimer, per call and share of model time)
        "phase_us_per_call": {
            "rhs": 1e3 * float(stats["t_rhs_ms"].sum() / max(stats["nfe"].sum(), 1)),
            "jacobian": 1e3 * float(stats["t_jac_ms"].sum() / max(stats["nje"].sum(), 1)),
            "lu": 1e3 * float(stats["t_lu_ms"].sum() / max(stats["nlu"].sum(), 1)),
            "solve": 1e3 * float(stats["t_solve_ms"].sum() / max(stats["nni"].sum(), 1))},
        "phase_share": {k: float(stats[f"t_{k}_ms"].sum() / max(stats["solve_ms"].sum(), 1e-30))
                        for k in ("rates", "rhs", "jac", "lu", "solve")},
        "roofline": {"bound": "tensor", "achieved": mat_tflops, "peak": peak, "unit": "TFLOP/s",
                     "frac": mat_tflops / peak,
                     "traffic": DRAM_BYTES_PER_MODEL_STEP * float(stats["nst"].sum()),
                     "peak_source": f"{peak_src} dense bf16 burst (MEASURED_PEAKS.json bf16_tflops"
                                    f"{'' if peak_src == 'measured' else ' absent: recipe fallback'}); no FP32 or "
                                    f"TF32 peak is measured on this pool, and the LU's trailing update runs as "
                                    f"3xTF32 MMAs",
                     "kernel": "k_solve_models<float>, one launch per timed region",
                     "holding_bound": "latency: one 256-thread CTA per model, barrier-separated phases; ncu shows "
                                      "issue active ~14%, no pipe above 15%, DRAM < 1% of peak",
                     "note": "achieved = LU flops (2/3 n^3 per factorisation) + triangular-solve flops (2 n^2 per "
                             "Newton iteration), counted by the device, over the launch's CUDA-event time; "
                             "traffic = DRAM bytes per model-step from one ncu capture x the launch's model-steps"},
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
    """A live serving session (ucl_server_*): the persistent solver is
    launched once; a host thread submits requests at Poisson arrival times
    while it runs (backpressure when the ring is full counts as latency);
    the main thread polls completions and takes each result.  Latency is
    host-observed, from a request's arrival time to the poll that sees it
    done; throughput is completed requests over the session's wall time."""
    from uclchem_gb300 import _lib, network
    from uclchem_gb300.params import make_param_array
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    n, rows = args.serve, 160
    params = make_param_array(serve_requests(n))
    rng = np.random.default_rng(SEED + 11)
    arrival = np.cumsum(rng.exponential(1.0 / args.rate, n))
    srv = _lib.Server(ctx, capacity=args.serve_capacity, max_rows=rows, precision=_lib.PREC_MIXED)
    t_arr = np.zeros(n)
    t_done = np.full(n, np.nan)
    flags = np.zeros(n, dtype=np.int32)
    solve_ms = np.zeros(n)
    submitted = [0]

    def submitter():
        for k in range(n):
            due = t0 + arrival[k]
            while time.perf_counter() < due:
                time.sleep(min(0.002, max(0.0, due - time.perf_counter())))
            t_arr[k] = due
            while srv.submit(params[k]) is None:  # ring full: wait for takes
                time.sleep(0.0005)
            submitted[0] = k + 1

    t0 = time.perf_counter()
    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    done = 0
    nxt = 0
    pending = []
    while done < n:
        while nxt < submitted[0]:
            pending.append(nxt)
            nxt += 1
        still = []
        for k in pending:
            if srv.poll(k):
                t_done[k] = time.perf_counter()
                _, _, _, fl, st = srv.take(k)
                flags[k] = fl
                solve_ms[k] = st["solve_ms"]
                done += 1
            else:
                still.append(k)
        pending = still
        time.sleep(0.001)
    wall = time.perf_counter() - t0
    th.join()
    srv.close()
    lat = (t_done - t_arr) * 1e3
    print(json.dumps({"mode": "serving", "requests": n, "arrival_rate_per_s": args.rate,
                      "mix": "70% static CLOUD, 30% freefall 1e2->1e6; finalTime 10^U(4,7) yr",
                      "server": f"live request ring of {srv.capacity} records, {rows} rows each, mixed precision",
                      "models_per_s": n / wall, "wall_s": wall,
                      "p50_latency_ms": float(np.percentile(lat, 50)), "p99_latency_ms": float(np.percentile(lat, 99)),
                      "p50_solve_ms": float(np.percentile(solve_ms, 50)),
                      "p99_solve_ms": float(np.percentile(solve_ms, 99)),
                      "latency": "host-observed: Poisson arrival time to the poll that sees the request done",
                      "failed": int((flags != 0).sum()),
                      "failed_codes": {str(int(c)): int((flags == c).sum()) for c in np.unique(flags[flags != 0])},
                      "arrivals_s": float(arrival[-1]),
                      "slots": ctx.slots(_lib.PREC_MIXED)}), flush=True)
    ctx.close()


def synthetic_arm(args):
    """Synthetic mass-action networks of four sizes (N = 64, 128, 256, 512,
    10 N reactions), --synthetic systems each, all in one launch of a
    multi-network context (mixed precision: FP64 state, FP32 LU), to 1e6 yr:
    models/s, p50/p99 per-model time, and element/charge conservation."""
    import tempfile
    import torch
    from uclchem_gb300 import _lib
    from uclchem_gb300 import synthetic as S
    per = args.synthetic
    nets = [S.make_network(n) for n in S.SIZES]
    with tempfile.TemporaryDirectory() as d:
        paths = [S.write_blob(net, os.path.join(d, f"syn{net.nspec}.uclnet")) for net in nets]
        ctx = _lib.Context(paths, device=0)
    net_of = np.repeat(np.arange(len(nets), dtype=np.int32), per)
    starts = np.zeros((len(net_of), ctx.neq))
    for k, net in enumerate(nets):
        starts[k * per:(k + 1) * per, : net.nspec + 1] = S.start_vectors(net, per)
    from uclchem_gb300.params import make_param_array
    params = make_param_array([{"initialDens": nets[k].density, "finalTime": 1e6} for k in net_of])
    M, rows = len(net_of), 64
    dev = torch.device("cuda", 0)
    p_d = torch.from_numpy(params.view(np.uint8).reshape(M, -1).copy()).to(dev)
    s_d = torch.from_numpy(starts).to(dev)
    n_d = torch.from_numpy(net_of).to(dev)
    ph = torch.zeros((M, rows, 8), dtype=torch.float64, device=dev)
    ab = torch.zeros((M, rows, ctx.nspec), dtype=torch.float64, device=dev)
    nr = torch.zeros(M, dtype=torch.int32, device=dev)
    fl = torch.zeros(M, dtype=torch.int32, device=dev)
    st = torch.zeros((M, _lib.STATS_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ctx.solve_models_nets_device(M, n_d.data_ptr(), p_d.data_ptr(), s_d.data_ptr(), rows, ph.data_ptr(),
                                 ab.data_ptr(), nr.data_ptr(), fl.data_ptr(), st.data_ptr(), _lib.PREC_MIXED, 0,
                                 stream.cuda_stream)
    e1.record(stream)
    stream.synchronize()
    ms = e0.elapsed_time(e1)
    stats = st.cpu().numpy().view(_lib.STATS_DTYPE).reshape(M)
    flags, nrows, abund = fl.cpu().numpy(), nr.cpu().numpy(), ab.cpu().numpy()
    drift = 0.0
    per_size = {}
    for k, net in enumerate(nets):
        E = net.conserved().astype(float)
        sel = np.nonzero((net_of == k) & (flags == 0))[0]
        for i in sel:
            y = abund[i, : nrows[i], : net.nspec]
            tot = y @ E.T
            drift = max(drift, float((np.abs(tot - tot[0]) / (np.abs(y[0]) @ np.abs(E).T)).max()))
        per_size[str(net.nspec)] = {"p50_ms": float(np.percentile(stats["solve_ms"][net_of == k], 50)),
                                    "failed": int((flags[net_of == k] != 0).sum())}
    print(json.dumps({"mode": "synthetic", "sizes": list(S.SIZES), "systems_per_size": per, "models": M,
                      "final_time_yr": 1e6, "models_per_s": M / (ms / 1e3), "ms": ms,
                      "p50_ms": float(np.percentile(stats["solve_ms"], 50)),
                      "p99_ms": float(np.percentile(stats["solve_ms"], 99)),
                      "failed": int((flags != 0).sum()), "per_size": per_size,
                      "max_conservation_drift": drift,
                      "conservation": "element (H, C, O, N) and charge totals per row, relative to the sum of "
                                      "their terms' magnitudes",
                      "slots": ctx.slots(_lib.PREC_MIXED)}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.serve > 0:
        serve_arm(args)
        return
    if args.synthetic > 0:
        synthetic_arm(args)
        return
    if args.kernel == "lu":
        lu_kernel(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()
