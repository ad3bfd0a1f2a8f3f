"""Generate the grid-parity fixture: the oracle (the CPU restatement of the
reference's rates + GETYDOT + DVODE MF=22 path) on a seeded sample of the
4096-point static CLOUD grid, to 1e6 yr with the reference's 501 output rows.

* grid_sample_1e6yr.npz  64 grid points stratified over density, at the
  reference's tolerances (reltol 1e-8, abstol_factor 1e-14): per model the
  flag, rows, DVODE counters, output times and every row's log10 abundances
  (int16 milli-dex, clamped at -16 dex: only species above 1e-14 are
  compared), and the oracle's CPU time; plus, for every 8th model of the
  sample, the same model at reltol 1e-12 (mxstep 100000) as the "truth" for
  the mixed-precision error statement.  `--add-truth I [I ...]` appends
  truth runs for more sample points (the parity outliers) to the file.

The runs take the oracle tens of CPU-minutes per slow model; they run in a
process pool, each capped in CPU time (2400 s at the reference's tolerance,
1200 s for a truth run, 3600 s for an appended one): a capped run is stored
with the oracle's cap flag (-99) and no rows, and the tests skip it.
Usage: python tests/golden/make_grid_sample.py [--procs N] [--add-truth I ...]
"""
import argparse
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SEED = 20261203
SAMPLE = 64
CAP_S = {False: 2400.0, True: 1200.0}
ADD_TRUTH_CAP_S = 3600.0
ROWS = 501
FLOOR_MDEX = -16000


def quantize(ab):
    """log10 abundances in milli-dex as int16, clamped at -16 dex."""
    q = np.round(1000.0 * np.log10(np.maximum(ab, 1e-30)))
    return np.clip(q, FLOOR_MDEX, 32000).astype(np.int16)


_ORC = None


def run(task):
    global _ORC
    i, d, tight = task[:3]
    cap = task[3] if len(task) > 3 else CAP_S[tight]
    if _ORC is None:
        from oracle.oracle import Oracle
        _ORC = Oracle()
    from uclchem_gb300.params import make_params
    p = make_params(d)
    if tight:
        p["reltol"] = 1e-12
        p["mxstep"] = 100000
    _ORC.set_cpu_limit(cap)
    t = time.process_time()
    phys, ab, flag, cnt = _ORC.cloud(p, max_rows=ROWS)
    return i, tight, int(flag), len(phys), cnt, phys[:, 0].copy(), quantize(ab), time.process_time() - t


def _pack(res, order):
    """Fixture arrays of a list of run() results, in the order of `order`."""
    rr = sorted(res, key=lambda r: order.index(r[0]))
    m = len(rr)
    q = np.full((m, ROWS, 335), FLOOR_MDEX, dtype=np.int16)
    tyr = np.zeros((m, ROWS))
    for k, r in enumerate(rr):
        q[k, : r[3]] = r[6]
        tyr[k, : r[3]] = r[5]
    return {"index": np.array([r[0] for r in rr], dtype=np.int32),
            "flag": np.array([r[2] for r in rr], dtype=np.int32),
            "nrows": np.array([r[3] for r in rr], dtype=np.int32),
            "counters": np.array([r[4] for r in rr], dtype=np.int64),
            "tyears": tyr, "log10_mdex": q, "cpu_s": np.array([r[7] for r in rr])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--add-truth", type=int, nargs="+", default=None)
    args = ap.parse_args()
    from uclchem_gb300.params import grid_params, stratified_sample
    dicts = grid_params(4096, seed=SEED, final_time=1e6)
    path = os.path.join(HERE, "grid_sample_1e6yr.npz")
    if args.add_truth:
        old = dict(np.load(path))
        extra = [i for i in args.add_truth if i in set(old["index"].tolist()) and i not in set(old["tight_index"].tolist())]
        with mp.get_context("spawn").Pool(min(args.procs, max(1, len(extra)))) as pool:
            res = pool.map(run, [(i, dicts[i], True, ADD_TRUTH_CAP_S) for i in extra], chunksize=1)
        new = _pack(res, extra)
        for k, v in new.items():
            old["tight_" + k] = np.concatenate([old["tight_" + k], v])
        np.savez_compressed(path, **old)
        print("appended truth runs", extra, "flags", new["flag"], "cpu_s", new["cpu_s"].round())
        return
    idx = stratified_sample(dicts, SAMPLE, seed=SEED + 3)
    tight = idx[::8]
    tasks = [(i, dicts[i], False) for i in idx] + [(i, dicts[i], True) for i in tight]
    # longest-expected (densest) first
    tasks.sort(key=lambda t: -t[1]["initialDens"] * (4 if t[2] else 1))
    with mp.get_context("spawn").Pool(args.procs) as pool:
        res = pool.map(run, tasks, chunksize=1)
    out = {}
    for tag, sel, order in (("", False, idx), ("tight_", True, tight)):
        for k, v in _pack([r for r in res if r[1] == sel], order).items():
            out[tag + k] = v
    np.savez_compressed(path, seed=SEED, **out)
    print("wrote", path)
    for k in range(len(out["index"])):
        print(out["index"][k], "%.3g" % dicts[out["index"][k]]["initialDens"], out["flag"][k], out["nrows"][k],
              out["counters"][k][:4], "%.1f s" % out["cpu_s"][k])


if __name__ == "__main__":
    main()
