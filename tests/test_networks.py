"""Other MakeRates networks (CPU): the reference's small_chemistry network
and the default network with add_crp_photo_to_grain, compiled by
uclchem_gb300.network (tests/golden/networks/, made by
tests/golden/make_networks.py from the reference's own MakeRates writers).
The blobs load through the C ABI with the tables' sizes; every invariant
is conserved by every reaction's stoichiometry; and the oracle reproduces
the fixture's small-network runs."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN

NETS = os.path.join(GOLDEN, "networks")
NAMES = ("small_chemistry", "photo_on_grain")


@pytest.mark.parametrize("name", NAMES)
def test_blob_loads_through_the_c_abi(name):
    from uclchem_gb300 import _lib, network
    net = network.Network.load_npz(os.path.join(NETS, name + ".npz"))
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ucl_network_load(os.path.join(NETS, name + ".uclnet").encode(), ctypes.byref(h)) == 0
    try:
        assert lib.ucl_network_nspec(h) == net.nspec
        assert lib.ucl_network_nreac(h) == net.nreac
    finally:
        lib.ucl_network_free(h)


@pytest.mark.parametrize("name", NAMES)
def test_invariants_are_exact(name):
    from uclchem_gb300 import network
    net = network.Network.load_npz(os.path.join(NETS, name + ".npz"))
    S = np.zeros((net.nspec, net.nreac), dtype=np.int64)
    for i in range(net.nspec):
        for e in range(net.stoich_ptr[i], net.stoich_ptr[i + 1]):
            S[i, net.stoich_rx[e]] += net.stoich_coef[e]
    inv = net.invariants()
    assert inv.shape[0] >= 4 and not (inv @ S).any()


def test_oracle_reproduces_the_small_network_fixture():
    from oracle.oracle import Oracle
    from uclchem_gb300.params import make_params
    fx = np.load(os.path.join(GOLDEN, "networks_oracle.npz"))
    o = Oracle(os.path.join(NETS, "small_chemistry.uclnet"))
    runs = {"static": {"initialDens": 1e4, "initialTemp": 10.0, "finalTime": 1e6},
            "stage1": {"initialDens": 1e2, "initialTemp": 10.0, "freefall": True, "endAtFinalDensity": True,
                       "finalDens": 1e5, "finalTime": 5e6}}
    for mname, pd in runs.items():
        phys, ab, flag, cnt = o.cloud(make_params(pd), max_rows=501)
        key = f"small_chemistry/{mname}/"
        r = int(fx[key + "nrows"])
        assert flag == int(fx[key + "flag"]) and len(ab) == r
        q = np.clip(np.round(1000.0 * np.log10(np.maximum(ab, 1e-30))), -16000, 32000).astype(np.int16)
        assert np.array_equal(q, fx[key + "log10_mdex"][:r])
        assert np.array_equal(cnt, fx[key + "counters"])
