"""Grid parity at the benchmark's configuration: a seeded sample of 64
points of the 4096-point static CLOUD grid, density-stratified, integrated
to 1e6 yr with the reference's 501 output rows, in both precisions (the two
runs share the GPU, one launch each), against the oracle's run of the same
points at the reference's tolerances (tests/golden/grid_sample_1e6yr.npz,
made by tests/golden/make_grid_sample.py).  Per model: the same flag and
rows, every species above 1e-14 within 0.01 dex at every row, a DVODE step
count within a band of the oracle's, element totals conserved; and the
mixed path's error against a reltol-1e-12 oracle run ("truth") on every 8th
point is no larger than the reltol-1e-8 oracle's own error plus 0.01 dex."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, dex_error
from uclchem_gb300.params import grid_params, make_param_array

pytestmark = pytest.mark.gpu

FIX = os.path.join(GOLDEN, "grid_sample_1e6yr.npz")
ROWS = 501
# Grid points whose result at the reference's tolerance is set by the
# integration path rather than by the arithmetic: index -> reason.  They
# must still end with the oracle's flag; their dex bound is not applied.
OUTLIERS = {}
CAPPED = -99  # the oracle's run hit its CPU-time cap when the fixture was made: no reference result


@pytest.fixture(scope="module")
def runs():
    """Both precisions over the sample's points that have an oracle result
    (the CPU-capped ones are not run), one launch each on its own stream;
    results scattered back to the fixture's order, capped points flagged
    CAPPED with no rows."""
    import torch
    from uclchem_gb300 import _lib, network
    if not os.path.exists(FIX):
        pytest.fail(f"fixture missing: {FIX}")
    fx = np.load(FIX)
    keep = np.nonzero(fx["flag"] != CAPPED)[0]
    dicts = grid_params(4096, seed=int(fx["seed"]), final_time=1e6)
    params = make_param_array([dicts[i] for i in fx["index"][keep]])
    M, K = len(fx["index"]), len(keep)
    dev = torch.device("cuda", 0)
    ctxs = {p: _lib.Context(network.DEFAULT_BLOB, device=0) for p in (0, 1)}
    streams = {p: torch.cuda.Stream(device=dev) for p in (0, 1)}
    p_d = torch.from_numpy(params.view(np.uint8).reshape(K, -1).copy()).to(dev)
    bufs = {}
    for p in (0, 1):
        bufs[p] = (torch.zeros((K, ROWS, 8), dtype=torch.float64, device=dev),
                   torch.zeros((K, ROWS, 335), dtype=torch.float64, device=dev),
                   torch.zeros(K, dtype=torch.int32, device=dev), torch.zeros(K, dtype=torch.int32, device=dev),
                   torch.zeros((K, _lib.STATS_DTYPE.itemsize), dtype=torch.uint8, device=dev))
    torch.cuda.synchronize()
    for p in (0, 1):  # FP64 and mixed run side by side, K models each
        ph, ab, nr, fl, st = bufs[p]
        ctxs[p].solve_models_device(K, p_d.data_ptr(), None, ROWS, ph.data_ptr(), ab.data_ptr(), nr.data_ptr(),
                                    fl.data_ptr(), st.data_ptr(), p, K, streams[p].cuda_stream)
    out = {}
    for p in (0, 1):
        streams[p].synchronize()
        ph, ab, nr, fl, st = (b.cpu().numpy() for b in bufs[p])
        full = (np.zeros((M, ROWS, 8)), np.zeros((M, ROWS, 335)), np.zeros(M, dtype=np.int32),
                np.full(M, CAPPED, dtype=np.int32), np.zeros(M, dtype=_lib.STATS_DTYPE))
        full[0][keep], full[1][keep], full[2][keep], full[3][keep] = ph, ab, nr, fl
        full[4][keep] = st.view(_lib.STATS_DTYPE).reshape(K)
        out[p] = full
        ctxs[p].close()
    return fx, out


def _oracle_rows(fx, k, tag=""):
    r = int(fx[tag + "nrows"][k])
    return 10.0 ** (fx[tag + "log10_mdex"][k, :r].astype(np.float64) / 1000.0), fx[tag + "tyears"][k, :r]


def _schedule(fx):
    """The output times of the static CLOUD schedule (cloud.f90:39-51): the
    rows of the sample's shortest successful run.  A run writes a row at
    each of them, plus one wherever DVODE stops at MXSTEP before its target
    (a time that depends on the step sequence, so it is not compared)."""
    ok = np.nonzero(fx["flag"] == 0)[0]
    k = ok[np.argmin(fx["nrows"][ok])]
    return fx["tyears"][k, : fx["nrows"][k]]


def _rows_at(t, times):
    """Row index of each schedule time in `times` (-1 where absent)."""
    out = np.full(len(times), -1)
    for j, s in enumerate(times):
        hit = np.nonzero(np.abs(t - s) <= 1e-12 * max(abs(s), 1.0))[0]
        if hit.size:
            out[j] = hit[0]
    return out


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_grid_sample_matches_oracle(runs, precision):
    """Per point: the oracle's flag; a row at every schedule time the oracle
    reached; at those rows every species above 1e-14 within 0.01 dex."""
    fx, out = runs
    ph, ab, nr, fl, st = out[precision]
    sched = _schedule(fx)
    flags, missing, bad = [], [], []
    for k, i in enumerate(fx["index"]):
        if fx["flag"][k] == CAPPED:
            continue
        if fl[k] != fx["flag"][k]:
            flags.append((int(i), int(fl[k]), int(fx["flag"][k])))
            continue
        oab, otyr = _oracle_rows(fx, k)
        r = int(nr[k])
        o_at = _rows_at(otyr, sched)
        g_at = _rows_at(ph[k, :r, 0], sched)
        want = o_at >= 0
        if (g_at[want] < 0).any():
            missing.append((int(i), int((g_at[want] < 0).sum())))
            continue
        if int(i) in OUTLIERS:
            continue
        # the fixture holds milli-dex, clamped at 1e-16: compare above 1e-14
        d = dex_error(ab[k, g_at[want]], oab[o_at[want]])
        if d >= 0.01:
            bad.append((int(i), round(d, 4)))
    assert not flags and not missing and not bad, (flags, missing, bad)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_grid_sample_step_counts_follow_the_oracle(runs, precision):
    """The device takes DVODE's decisions; with the analytic Jacobian (and the
    FP32 factorisation on the mixed path) the step counts stay within a
    band of the oracle's finite-difference-Jacobian counts."""
    fx, out = runs
    st, fl = out[precision][4], out[precision][3]
    ok = (fl == 0) & (fx["flag"] == 0)
    ratio = st["nst"][ok] / fx["counters"][ok, 0]
    assert 0.95 <= np.median(ratio) <= 1.1, np.median(ratio)
    assert ratio.min() > 0.5 and ratio.max() < 2.0, (ratio.min(), ratio.max())


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_grid_sample_conserves_elements(runs, net, precision):
    """The network's conserved elements (He, C, N, O, S, Si, Mg, Cl) to 1e-10
    relative at every row of every successful model."""
    fx, out = runs
    ph, ab, nr, fl, st = out[precision]
    E = net.invariants().T
    worst = 0.0
    for k in np.nonzero(fl == 0)[0]:
        tot = ab[k, : nr[k]] @ E
        worst = max(worst, float(np.abs(tot / tot[0] - 1.0).max()))
    assert worst < 1e-10, worst


def test_mixed_error_against_tight_tolerance_truth(runs):
    """Configuration 3's error statement: on every 8th sample point, the
    mixed path's max |dex| against the oracle at reltol 1e-12 is at most the
    reference-tolerance oracle's own |dex| against it plus 0.01."""
    fx, out = runs
    ph, ab, nr, fl, st = out[1]
    pos = {int(i): k for k, i in enumerate(fx["index"])}
    for j, i in enumerate(fx["tight_index"]):
        k = pos[int(i)]
        if fx["tight_flag"][j] != 0 or fl[k] != 0 or fx["flag"][k] != 0:
            continue
        truth, ttyr = _oracle_rows(fx, j, "tight_")
        ref, rtyr = _oracle_rows(fx, k)
        r = min(len(ttyr), int(nr[k]), len(rtyr))
        if not (np.allclose(ttyr[:r], ph[k, :r, 0], rtol=1e-12) and np.allclose(rtyr[:r], ttyr[:r], rtol=1e-12)):
            continue  # retries changed the output times: rows are not comparable
        e_mixed = dex_error(ab[k, :r], truth[:r])
        e_ref = dex_error(ref[:r], truth[:r])
        assert e_mixed <= e_ref + 0.01, (int(i), e_mixed, e_ref)
