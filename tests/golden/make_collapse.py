"""Generate the collapse fixture: the oracle (the CPU restatement of the
reference's rates + GETYDOT + DVODE MF=22 path with the collapse.f90
physics module) on the four collapse modes with the reference's default
parameters:

* BE1.1 and BE4 to their own end time (0.97 maxTime: 1.14e6 and 1.80e5 yr);
* filament and ambipolar to 1e5 yr.

Stored per mode: flag, rows, DVODE counters, output times, density and Av
of every row (float64), and every row's log10 abundances as int16 milli-dex
clamped at -16 dex (only species above 1e-14 are compared).  The collapse
module has no output file in the reference's examples, so this fixture
pins the device to the oracle's restatement of collapse.f90, not to the
reference's own output.
Usage: python tests/golden/make_collapse.py
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

MODES = {"BE1.1": (1, {}), "BE4": (2, {}), "filament": (3, {"finalTime": 1e5}),
         "ambipolar": (4, {"finalTime": 1e5})}
ROWS = 1300
FLOOR_MDEX = -16000


def run(name):
    from oracle.oracle import Oracle
    from uclchem_gb300.params import make_params
    mode, extra = MODES[name]
    p = make_params(extra)
    p["collapse"] = mode
    phys, ab, flag, cnt = Oracle().cloud(p, max_rows=ROWS)
    q = np.clip(np.round(1000.0 * np.log10(np.maximum(ab, 1e-30))), FLOOR_MDEX, 32000).astype(np.int16)
    return name, int(flag), phys, q, cnt


def main():
    names = list(MODES)
    with mp.get_context("spawn").Pool(len(names)) as pool:
        res = pool.map(run, names, chunksize=1)
    out = {"names": np.array(names), "modes": np.array([MODES[n][0] for n in names], dtype=np.int32)}
    m = len(res)
    out["flag"] = np.array([r[1] for r in res], dtype=np.int32)
    out["nrows"] = np.array([len(r[2]) for r in res], dtype=np.int32)
    out["counters"] = np.array([r[4] for r in res], dtype=np.int64)
    out["tyears"] = np.zeros((m, ROWS))
    out["density"] = np.zeros((m, ROWS))
    out["av"] = np.zeros((m, ROWS))
    out["log10_mdex"] = np.full((m, ROWS, 335), FLOOR_MDEX, dtype=np.int16)
    for k, r in enumerate(res):
        n = len(r[2])
        out["tyears"][k, :n] = r[2][:, 0]
        out["density"][k, :n] = r[2][:, 1]
        out["av"][k, :n] = r[2][:, 4]
        out["log10_mdex"][k, :n] = r[3]
    path = os.path.join(HERE, "collapse_modes.npz")
    np.savez_compressed(path, final_time_filament=1e5, **out)
    for k, n in enumerate(names):
        print(n, out["flag"][k], out["nrows"][k], out["counters"][k][:4])
    print("wrote", path)


if __name__ == "__main__":
    main()
