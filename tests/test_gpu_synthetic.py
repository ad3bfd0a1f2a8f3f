"""Synthetic mass-action networks of four sizes (N = 64, 128, 256, 512
species, 10 N reactions each) integrated in ONE device launch through a
multi-network context (ucl_ctx_create_multi + ucl_solve_models_nets_device),
checked model by model against the oracle's integration of the same network
(orc_ma_cloud: the same CLOUD schedule, retry and clamp logic on a
constant-rate RHS), with element and charge conservation."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from conftest import dex_error
from uclchem_gb300 import synthetic as S
from uclchem_gb300.params import make_param_array

pytestmark = pytest.mark.gpu

PER_SIZE = {64: 6, 128: 6, 256: 4, 512: 3}
ROWS = 64


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    from oracle.oracle import MassActionOracle
    from uclchem_gb300 import _lib
    d = tmp_path_factory.mktemp("syn")
    nets = [S.make_network(n) for n in S.SIZES]
    paths = [S.write_blob(net, str(d / f"syn{net.nspec}.uclnet")) for net in nets]
    ctx = _lib.Context(paths, device=0)
    net_of, starts = [], []
    for k, net in enumerate(nets):
        sv = S.start_vectors(net, PER_SIZE[net.nspec])
        for v in sv:
            row = np.zeros(ctx.neq)
            row[: net.nspec + 1] = v
            starts.append(row)
            net_of.append(k)
    net_of = np.array(net_of, dtype=np.int32)
    starts = np.array(starts)
    dicts = [{"initialDens": nets[k].density, "initialTemp": 10.0, "finalTime": 1e6} for k in net_of]
    oracles = [MassActionOracle(net) for net in nets]

    def one(i):
        net = nets[net_of[i]]
        return oracles[net_of[i]].cloud(starts[i, : net.nspec + 1], final_time_yr=1e6, max_rows=ROWS)

    with ThreadPoolExecutor(max_workers=8) as ex:
        ref = list(ex.map(one, range(len(net_of))))
    yield ctx, nets, net_of, starts, make_param_array(dicts), ref
    ctx.close()


def _solve(ctx, net_of, starts, params, precision):
    import torch
    from uclchem_gb300 import _lib
    M = len(net_of)
    dev = torch.device("cuda", 0)
    p_d = torch.from_numpy(params.view(np.uint8).reshape(M, -1).copy()).to(dev)
    s_d = torch.from_numpy(starts).to(dev)
    n_d = torch.from_numpy(net_of).to(dev)
    ph = torch.zeros((M, ROWS, 8), dtype=torch.float64, device=dev)
    ab = torch.zeros((M, ROWS, ctx.nspec), dtype=torch.float64, device=dev)
    nr = torch.zeros(M, dtype=torch.int32, device=dev)
    fl = torch.zeros(M, dtype=torch.int32, device=dev)
    st = torch.zeros((M, _lib.STATS_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    stream.wait_stream(torch.cuda.current_stream(dev))
    ctx.solve_models_nets_device(M, n_d.data_ptr(), p_d.data_ptr(), s_d.data_ptr(), ROWS, ph.data_ptr(),
                                 ab.data_ptr(), nr.data_ptr(), fl.data_ptr(), st.data_ptr(), precision, 0,
                                 stream.cuda_stream)
    stream.synchronize()
    return ph.cpu().numpy(), ab.cpu().numpy(), nr.cpu().numpy(), fl.cpu().numpy()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_four_network_sizes_in_one_launch_match_oracle(setup, precision):
    ctx, nets, net_of, starts, params, ref = setup
    ph, ab, nr, fl = _solve(ctx, net_of, starts, params, precision)
    worst_dex, worst_drift = 0.0, 0.0
    for i, k in enumerate(net_of):
        net = nets[k]
        tyr, yo, oflag, _ = ref[i]
        r = int(nr[i])
        assert fl[i] == 0 and oflag == 0, (i, fl[i], oflag)
        assert r == len(tyr), (i, r, len(tyr))
        np.testing.assert_allclose(ph[i, :r, 0], tyr, rtol=1e-12)
        y = ab[i, :r, : net.nspec]
        assert not ab[i, :r, net.nspec:].any()  # columns past the network's species stay untouched
        worst_dex = max(worst_dex, dex_error(y, yo))
        # element and charge totals, relative to the sum of their terms' magnitudes
        E = net.conserved().astype(float)
        tot = y @ E.T
        scale = np.abs(y[0]) @ np.abs(E).T
        worst_drift = max(worst_drift, float((np.abs(tot - tot[0]) / scale).max()))
    assert worst_dex < 0.01, worst_dex
    # FP64: the DVODE iteration as is; mixed: projected onto the invariants
    assert worst_drift < (1e-9 if precision == 0 else 1e-10), worst_drift
