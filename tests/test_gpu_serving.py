"""Serving path (ucl_serve_models_device): requests admitted on the device at
their arrival times, static and freefall models mixed.  Results must equal
the batch path's, and queue/latency times must be consistent."""
import numpy as np
import pytest

from uclchem_gb300.params import make_param_array

pytestmark = pytest.mark.gpu


def _requests():
    rng = np.random.default_rng(5)
    reqs = []
    for k in range(12):
        d = {"initialDens": float(10 ** rng.uniform(2, 5)), "initialTemp": float(rng.uniform(10, 30)),
             "finalTime": float(10 ** rng.uniform(2, 3.5))}
        if k % 3 == 2:  # the freefall share of the serving mix
            d.update({"initialDens": 1e2, "freefall": True, "finalDens": 1e6})
        reqs.append(d)
    return reqs


def test_serving_matches_batch_and_times_are_consistent():
    import torch
    from uclchem_gb300 import _lib, network
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    dev = torch.device("cuda", 0)
    st = torch.cuda.Stream(device=dev)
    reqs = _requests()
    n, rows, nspec = len(reqs), 64, ctx.nspec
    params = make_param_array(reqs)
    arrival = np.arange(n) * 0.02  # seconds after launch
    p_d = torch.from_numpy(params.view(np.uint8).reshape(n, -1).copy()).to(dev)
    a_d = torch.from_numpy(arrival).to(dev)
    out = {}
    for mode in ("batch", "serve"):
        ph = torch.zeros((n, rows, 8), dtype=torch.float64, device=dev)
        ab = torch.zeros((n, rows, nspec), dtype=torch.float64, device=dev)
        nr = torch.zeros(n, dtype=torch.int32, device=dev)
        fl = torch.zeros(n, dtype=torch.int32, device=dev)
        sd = torch.zeros((n, _lib.STATS_DTYPE.itemsize), dtype=torch.uint8, device=dev)
        st.wait_stream(torch.cuda.current_stream(dev))
        args = (ph.data_ptr(), ab.data_ptr(), nr.data_ptr(), fl.data_ptr(), sd.data_ptr(), _lib.PREC_MIXED, 4,
                st.cuda_stream)
        if mode == "batch":
            ctx.solve_models_device(n, p_d.data_ptr(), None, rows, *args)
        else:
            ctx.serve_models_device(n, p_d.data_ptr(), a_d.data_ptr(), None, rows, *args)
        st.synchronize()
        out[mode] = (ph.cpu().numpy(), ab.cpu().numpy(), nr.cpu().numpy(), fl.cpu().numpy(),
                     sd.cpu().numpy().view(_lib.STATS_DTYPE).reshape(n))
    bph, bab, bnr, bfl, _ = out["batch"]
    sph, sab, snr, sfl, sst = out["serve"]
    assert (bfl == 0).all() and (sfl == 0).all()
    np.testing.assert_array_equal(bnr, snr)
    for k in range(n):
        r = int(bnr[k])
        np.testing.assert_array_equal(bab[k, :r], sab[k, :r])
        np.testing.assert_array_equal(bph[k, :r], sph[k, :r])
    # batch admission is longest-expected first: the max_ctas highest-key
    # models (log10 n + 0.05 T) start at once
    bst = out["batch"][4]
    key = np.log10(params["initialDens"]) + 0.05 * params["initialTemp"]
    first = np.argsort(-key.astype(np.float32), kind="stable")[:4]
    assert (bst["queue_ms"][first] < 5.0).all()
    # latency = queueing + service; requests start no earlier than arrival
    assert (sst["queue_ms"] >= 0).all()
    np.testing.assert_allclose(sst["latency_ms"], sst["queue_ms"] + sst["solve_ms"], atol=0.5)
    assert (sst["latency_ms"] >= sst["solve_ms"] - 1e-6).all()
    ctx.close()


def test_live_server_serves_requests_submitted_while_it_runs():
    """ucl_server_*: the persistent solver is launched first; requests are
    appended afterwards, one at a time with pauses, through the pinned
    request ring.  Each result equals the batch path's bit for bit; a ring
    with every record holding an untaken result refuses a new request
    (UCL_E_AGAIN) until one is taken; closing ends the launch cleanly."""
    import time
    from uclchem_gb300 import _lib, network
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    reqs = _requests()[:6]
    params = make_param_array(reqs)
    rows = 64
    bph, bab, bnr, bfl, _ = ctx.solve_models(params, rows, precision=_lib.PREC_MIXED)
    srv = _lib.Server(ctx, capacity=4, max_rows=rows, precision=_lib.PREC_MIXED, max_ctas=3, idle_timeout_s=60.0)
    try:
        assert srv.capacity == 4
        time.sleep(0.5)  # the solver is idle, polling the empty ring
        ids = []
        for k in range(4):
            ids.append(srv.submit(params[k]))
            time.sleep(0.05)
        assert ids == [0, 1, 2, 3]
        assert srv.submit(params[4]) is None  # every record is taken by a request
        got = {}
        t0 = time.time()
        while len(got) < 4 and time.time() - t0 < 300:
            for k in ids:
                if k not in got and srv.poll(k):
                    got[k] = srv.take(k)
            time.sleep(0.01)
        assert sorted(got) == ids
        for k in (4, 5):  # records are free again
            assert srv.submit(params[k]) == k
        t0 = time.time()
        while len(got) < 6 and time.time() - t0 < 300:
            for k in (4, 5):
                if k not in got and srv.poll(k):
                    got[k] = srv.take(k)
            time.sleep(0.01)
        for k in range(6):
            phys, ab, nr, fl, st = got[k]
            assert fl == 0 == bfl[k] and nr == bnr[k]
            np.testing.assert_array_equal(ab[:nr], bab[k, :nr])
            np.testing.assert_array_equal(phys[:nr], bph[k, :nr])
    finally:
        srv.close()
    ctx.close()
