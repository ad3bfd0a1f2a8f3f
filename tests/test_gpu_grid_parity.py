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
# integration path rather than by the arithmetic: index -> reason.  Each
# has a reltol-1e-12 oracle run in the fixture; the device must end with the
# oracle's flag and be at least as close to that truth as the oracle at the
# reference's tolerance is (test_outliers_are_no_further_from_the_truth).
OUTLIERS = {3767: "late-time S2 and N-ice chemistry (n = 4.7e4, T = 39 K, G = 582) that no tolerance "
                  "settles: at 1e6 yr the oracle at reltol 1e-8 is 0.69 dex from its reltol-1e-12 run, and its "
                  "reltol-1e-10 run 0.29 dex; the device is 0.34 (FP64) / 0.30 (mixed) dex from it"}
# Grid points where the oracle ends with -5 (integration failure after the
# retries of updateChemistry) and the device completes: in each, the
# oracle's Newton iteration with DVODE's finite-difference Jacobian fails on
# more than 5% of its steps, the device's with the analytic Jacobian on
# under 1% (checked below).
FD_JACOBIAN_FAILURES = {1558: "oracle: 23145 Newton failures in 319958 steps",
                        2535: "oracle: 29615 Newton failures in 275244 steps"}
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
            cnt = fx["counters"][k]
            if (int(i) in FD_JACOBIAN_FAILURES and fx["flag"][k] == -5 and fl[k] == 0
                    and cnt[5] > 0.05 * cnt[0] and st["ncfn"][k] < 0.01 * st["nst"][k]):
                continue
            flags.append((int(i), int(fl[k]), int(fx["flag"][k])))
            continue
        if fl[k] != 0:
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
    """The device takes DVODE's decisions, so its step counts follow the
    oracle's: median ratio 0.95-1.1, none above 2x.  The exception is where
    the oracle's Newton iteration with DVODE's finite-difference Jacobian
    keeps failing (Newton plus error-test failures on 5% of its steps or
    more, each failure shrinking the step): there the analytic Jacobian,
    whose Newton iteration fails on under 1% of the device's steps, needs
    fewer steps, down to a few percent of the oracle's."""
    fx, out = runs
    st, fl = out[precision][4], out[precision][3]
    ok = np.nonzero((fl == 0) & (fx["flag"] == 0))[0]
    cnt = fx["counters"][ok]
    ratio = st["nst"][ok] / cnt[:, 0]
    assert 0.95 <= np.median(ratio) <= 1.1, np.median(ratio)
    assert ratio.max() < 2.0, [(int(fx["index"][k]), r) for k, r in zip(ok, ratio) if r >= 2.0]
    low = ratio < 0.5
    fd_fail = (cnt[:, 5] + cnt[:, 6]) >= 0.05 * cnt[:, 0]
    dev_ok = st["ncfn"][ok] < 0.01 * st["nst"][ok]
    odd = low & ~(fd_fail & dev_ok)
    assert not odd.any(), [(int(fx["index"][k]), round(float(r), 3), [int(x) for x in c[:7]])
                           for k, r, c in zip(ok[odd], ratio[odd], cnt[odd])]


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


def _truth_errors(fx, out, precision, k, j, sched):
    """(device, oracle) max |dex| against the truth run j of sample point k,
    at the schedule times all three reached."""
    ph, ab, nr, fl, st = out[precision]
    truth, ttyr = _oracle_rows(fx, j, "tight_")
    ref, rtyr = _oracle_rows(fx, k)
    t_at, r_at = _rows_at(ttyr, sched), _rows_at(rtyr, sched)
    g_at = _rows_at(ph[k, : nr[k], 0], sched)
    m = (t_at >= 0) & (r_at >= 0) & (g_at >= 0)
    return dex_error(ab[k, g_at[m]], truth[t_at[m]]), dex_error(ref[r_at[m]], truth[t_at[m]])


def test_mixed_error_against_tight_tolerance_truth(runs):
    """Configuration 3's error statement: on every 8th sample point, the
    mixed path's max |dex| against the oracle at reltol 1e-12 is at most the
    reference-tolerance oracle's own |dex| against it plus 0.01."""
    fx, out = runs
    fl = out[1][3]
    sched = _schedule(fx)
    pos = {int(i): k for k, i in enumerate(fx["index"])}
    checked = 0
    for j, i in enumerate(fx["tight_index"]):
        k = pos[int(i)]
        if int(i) in OUTLIERS or fx["tight_flag"][j] != 0 or fl[k] != 0 or fx["flag"][k] != 0:
            continue
        e_mixed, e_ref = _truth_errors(fx, out, 1, k, j, sched)
        assert e_mixed <= e_ref + 0.01, (int(i), e_mixed, e_ref)
        checked += 1
    assert checked >= 5, checked


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_outliers_are_no_further_from_the_truth(runs, precision):
    """Every parity outlier: the device's max |dex| against the oracle's
    reltol-1e-12 run is at most the reltol-1e-8 oracle's own plus 0.01."""
    fx, out = runs
    fl = out[precision][3]
    sched = _schedule(fx)
    pos = {int(i): k for k, i in enumerate(fx["index"])}
    tpos = {int(i): j for j, i in enumerate(fx["tight_index"])}
    for i in OUTLIERS:
        k, j = pos[i], tpos[i]
        assert fx["tight_flag"][j] == 0 and fl[k] == fx["flag"][k] == 0, (i, int(fl[k]))
        e_dev, e_ref = _truth_errors(fx, out, precision, k, j, sched)
        assert e_dev <= e_ref + 0.01, (i, e_dev, e_ref)
