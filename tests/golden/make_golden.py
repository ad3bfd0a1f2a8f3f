"""Generate the golden fixtures from the reference's own example outputs.

Reads UCLCHEM's shipped example outputs (produced by
scripts/run_uclchem_tests.py of the reference) and stores the rows the parity
tests use as compact .npz files next to this script:

* static_cloud.npz   examples/example-output/static-full.dat, rows with
                     t <= 1e6 yr (the single static CLOUD model: 1e4 cm^-3,
                     10 K, zeta=1, radfield=1, reltol 1e-8)
* freefall_cloud.npz examples/example-output/phase1-full.dat (freefall
                     collapse 1e2 -> 1e5 cm^-3, endAtFinalDensity)

Usage: python tests/golden/make_golden.py <uclchem_root>
       (or UCLCHEM_REFERENCE_ROOT=<uclchem_root> python tests/golden/make_golden.py)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_full(path):
    with open(path) as f:
        header = [h.strip() for h in f.readline().split(",")]
    data = np.genfromtxt(path, delimiter=",", skip_header=1)
    return header, data


def main(ref_root):
    out = os.path.join(ref_root, "examples", "example-output")
    h, d = load_full(os.path.join(out, "static-full.dat"))
    keep = d[:, 0] <= 1.0e6
    np.savez_compressed(os.path.join(HERE, "static_cloud.npz"), phys=d[keep, :8], abund=d[keep, 8:],
                        species=np.array(h[8:]),
                        params=np.array(["initialDens=1e4", "initialTemp=10.0", "finalTime=1e6"]))
    h, d = load_full(os.path.join(out, "phase1-full.dat"))
    np.savez_compressed(os.path.join(HERE, "freefall_cloud.npz"), phys=d[:, :8], abund=d[:, 8:],
                        species=np.array(h[8:]),
                        params=np.array(["initialDens=1e2", "initialTemp=10.0", "finalTime=5e6",
                                         "freefall=True", "endAtFinalDensity=True", "finalDens=1e5"]))
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("UCLCHEM_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <uclchem_root>  (or set UCLCHEM_REFERENCE_ROOT)")
    main(root)
