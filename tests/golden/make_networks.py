"""Generate the other-network fixtures: two MakeRates networks besides the
default one, compiled by this repository's table compiler
(uclchem_gb300.network) and run by the oracle.

* small_chemistry: the reference's minimal test network
  (Makerates/data/small_chemistry: its species file, the UMIST22 gas-phase
  database and its grain reactions);
* photo_on_grain: the default species and grain network with
  add_crp_photo_to_grain (the reference's tests/test_photo_on_grain.py).

The network files come from the reference's own MakeRates code, imported
from the given reference tree (its io_functions.write_odes_f90 /
write_network_file, the writers of network.f90 and odes.f90 at
io_functions.py:231-284), into a scratch folder that is removed afterwards.
The reference package's __init__ imports its compiled Fortran wrapper and
pandas, and run_makerates reads YAML; none of them is on this path, so the
package is entered as a plain namespace and the settings are given here.
(Run on the default settings, this path reproduces the reference's
src/fortran_src/network.f90 and odes.f90 byte for byte.)

Outputs: tests/golden/networks/{name}.npz and .uclnet (the compiled
tables) and tests/golden/networks_oracle.npz: per network and model (the
small network: a static cloud and a freefall stage 1; photo-on-grain: a
static cloud at two tolerances), the oracle's flag, rows, counters,
output times and every row's log10 abundances (int16 milli-dex clamped at
-16 dex).
Usage: python tests/golden/make_networks.py <uclchem reference root>
"""
import os
import shutil
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "networks")
ROWS = 501
FLOOR_MDEX = -16000
# models per network: (name, parameter dictionary)
MODELS = {
    "small_chemistry": [
        ("static", {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e6}),
        ("stage1", {"initialDens": 1e2, "initialTemp": 10.0, "freefall": True, "endAtFinalDensity": True,
                    "finalDens": 1e5, "finalTime": 5e6}),
    ],
    # a static cloud at the reference's tolerances, and at the looser ones of
    # the reference's own photo-on-grain test (reltol 1e-5, abstol_min 1e-15)
    "photo_on_grain": [
        ("static", {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e5}),
        ("static_loose", {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e6,
                          "abstol_min": 1e-15, "reltol": 1e-5}),
    ],
}


def makerates(ref_root, name, scratch):
    """network.f90 and odes.f90 of network `name` into `scratch`."""
    if "uclchem" not in sys.modules:
        pkg = types.ModuleType("uclchem")
        pkg.__path__ = [os.path.join(ref_root, "src", "uclchem")]
        sys.modules["uclchem"] = pkg
        # makerates.py imports yaml for run_makerates' settings file only
        sys.modules.setdefault("yaml", types.ModuleType("yaml"))
    from uclchem.makerates import io_functions as io
    from uclchem.makerates.makerates import _get_network_from_files
    data = os.path.join(ref_root, "Makerates", "data")
    if name == "small_chemistry":
        species, grain, photo = "small_chemistry/species.csv", "small_chemistry/grain_reactions.csv", False
    else:
        species, grain, photo = "default/default_species.csv", "default/default_grain_network.csv", True
    net, _ = _get_network_from_files(
        species_file=os.path.join(data, species),
        reaction_files=[os.path.join(data, "databases", "umist22.csv"), os.path.join(data, grain)],
        reaction_types=["UMIST", "UCL"], gas_phase_extrapolation=False, add_crp_photo_to_grain=photo)
    io.write_odes_f90(os.path.join(scratch, "odes.f90"), net.get_species_list(), net.get_reaction_list(),
                      rates_to_disk=False)
    io.write_network_file(os.path.join(scratch, "network.f90"), net, rates_to_disk=False, gar_database=None)


def main():
    ref_root = sys.argv[1]
    from uclchem_gb300 import network
    from oracle.oracle import Oracle
    from uclchem_gb300.params import make_params
    os.makedirs(OUT, exist_ok=True)
    out = {}
    for name, models in MODELS.items():
        scratch = os.path.join(OUT, "_makerates_" + name)
        os.makedirs(scratch, exist_ok=True)
        try:
            makerates(ref_root, name, scratch)
            net = network.compile_network(os.path.join(scratch, "network.f90"), os.path.join(scratch, "odes.f90"))
        finally:
            shutil.rmtree(scratch)
        blob = os.path.join(OUT, name + ".uclnet")
        network.write_compiled(net, os.path.join(OUT, name + ".npz"), blob)
        print(name, net.nspec, "species", net.nreac, "reactions", flush=True)
        orc = Oracle(blob)
        for mname, pd in models:
            phys, ab, flag, cnt = orc.cloud(make_params(pd), max_rows=ROWS)
            q = np.full((ROWS, net.nspec), FLOOR_MDEX, dtype=np.int16)
            q[: len(ab)] = np.clip(np.round(1000.0 * np.log10(np.maximum(ab, 1e-30))), FLOOR_MDEX, 32000)
            t = np.zeros(ROWS)
            t[: len(ab)] = phys[:, 0]
            key = f"{name}/{mname}/"
            out[key + "flag"] = np.int32(flag)
            out[key + "nrows"] = np.int32(len(ab))
            out[key + "counters"] = cnt
            out[key + "tyears"] = t
            out[key + "log10_mdex"] = q
            print(" ", mname, flag, len(ab), cnt[:4], flush=True)
    np.savez_compressed(os.path.join(HERE, "networks_oracle.npz"), **out)


if __name__ == "__main__":
    main()
