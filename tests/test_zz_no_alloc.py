"""The allocation-free batched LU entry point (ucl_lu_factor_device_static)
against the context-based one, through the C ABI.  Collected last so it also
runs after every other test in the same process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [1, 0], ids=["fp32", "fp64"])
def test_static_scratch_lu_matches_context_lu(precision):
    import torch
    from uclchem_gb300 import _lib, network
    lib = _lib.load()
    ctx = _lib.Context(network.DEFAULT_BLOB, device=0)
    torch.cuda.set_device(0)
    rng = np.random.default_rng(7 + precision)
    n = 336
    # more matrices than the static scratch holds at once, so CTAs take turns
    cap = (16 << 20) // (2 * (32 if precision == 1 else 16) * n * (4 if precision == 1 else 8))
    nsys = cap + 37
    A = np.eye(n)[None] - rng.standard_normal((nsys, n, n)) * 10.0 ** rng.uniform(-3, 1, (nsys, 1, n))
    dt = torch.float32 if precision == 1 else torch.float64
    src = torch.tensor(A, dtype=dt, device="cuda")
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    ref = src.clone()
    p_ref = torch.empty((nsys, n), dtype=torch.int32, device="cuda")
    i_ref = torch.empty(nsys, dtype=torch.int32, device="cuda")
    ctx.lu_factor_device(nsys, n, precision, ref.data_ptr(), p_ref.data_ptr(), i_ref.data_ptr(), st.cuda_stream)
    outs = []
    for _ in range(2):  # two calls in a row share the same scratch
        m = src.clone()
        p = torch.empty((nsys, n), dtype=torch.int32, device="cuda")
        info = torch.full((nsys,), -7, dtype=torch.int32, device="cuda")
        st.wait_stream(torch.cuda.current_stream())
        rc = lib.ucl_lu_factor_device_static(nsys, n, precision, ctypes.c_void_p(m.data_ptr()),
                                             ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(info.data_ptr()),
                                             ctypes.c_void_p(st.cuda_stream))
        assert rc == 0
        st.synchronize()
        outs.append((m.cpu().numpy(), p.cpu().numpy(), info.cpu().numpy()))
    st.synchronize()
    ref_m, ref_p, ref_i = ref.cpu().numpy(), p_ref.cpu().numpy(), i_ref.cpu().numpy()
    tol = 1e-5 if precision == 1 else 1e-13
    for m, p, info in outs:
        assert (info == 0).all() and (ref_i == 0).all()
        np.testing.assert_array_equal(p, ref_p)
        scale = np.abs(ref_m).max(axis=(1, 2), keepdims=True)
        assert (np.abs(m - ref_m) / scale).max() <= tol
    # sizes beyond the supported range are rejected, nothing is launched
    assert lib.ucl_lu_factor_device_static(1, 522, precision, ctypes.c_void_p(src.data_ptr()),
                                           ctypes.c_void_p(p_ref.data_ptr()), ctypes.c_void_p(i_ref.data_ptr()),
                                           ctypes.c_void_p(st.cuda_stream)) == -101  # UCL_E_ARG
    ctx.close()
