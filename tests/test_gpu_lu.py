"""Batched LU (the Newton-matrix factorisation) against numpy, on the GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_batched_lu_reconstructs(precision):
    import torch
    from uclchem_gb300 import _lib, network
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    rng = np.random.default_rng(1)
    n, nsys = 336, 6
    # Newton-like matrices I - c*J with a wide spread of scales
    A = np.eye(n)[None] - rng.standard_normal((nsys, n, n)) * 10.0 ** rng.uniform(-3, 1, (nsys, 1, n))
    dt = torch.float32 if precision == 1 else torch.float64
    m = torch.tensor(A, dtype=dt, device="cuda")
    perm = torch.empty((nsys, n), dtype=torch.int32, device="cuda")
    info = torch.empty(nsys, dtype=torch.int32, device="cuda")
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    ctx.lu_factor_device(nsys, n, precision, m.data_ptr(), perm.data_ptr(), info.data_ptr(), st.cuda_stream)
    st.synchronize()
    LU, p, inf = m.double().cpu().numpy(), perm.cpu().numpy(), info.cpu().numpy()
    assert (inf == 0).all()
    tol = 1e-4 if precision == 1 else 1e-12
    for s in range(nsys):
        L = np.tril(LU[s], -1) + np.eye(n)
        U = np.triu(LU[s])
        assert sorted(p[s]) == list(range(n))
        err = np.abs(L @ U - A[s][p[s]]).max() / np.abs(A[s]).max()
        assert err < tol, (s, err)
        # pivots chosen as in partial pivoting: |L| <= 1
        assert np.abs(np.tril(LU[s], -1)).max() <= 1.0 + 1e-6
    ctx.close()


def test_autotuner_picks_the_faster_lu_update(monkeypatch):
    """The context's autotuner times the FP32 LU's tensor-core and CUDA-core
    trailing updates for the network's size and keeps the faster;
    UCL_AUTOTUNE=0 skips the timing and keeps the tensor cores."""
    from uclchem_gb300 import _lib, network
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    tc, us_tc, us_cc = ctx.lu_variant(0)
    assert us_tc > 0 and us_cc > 0
    assert tc == (us_tc <= us_cc)
    ctx.close()
    monkeypatch.setenv("UCL_AUTOTUNE", "0")
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    assert ctx.lu_variant(0) == (True, 0.0, 0.0)
    ctx.close()
