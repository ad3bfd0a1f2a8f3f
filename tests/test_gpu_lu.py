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
