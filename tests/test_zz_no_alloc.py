"""The allocation-free batched LU entry point (ucl_lu_factor_device_static)
against the context-based one, through the C ABI.  It is for callers that
cannot allocate device memory: a framework whose caching allocator owns all
of the GPU's memory, or a serving loop that has given its whole HBM budget
to resident model state and must not pay an allocation's implicit device
synchronisation.  Collected last so it also runs after every other test in
the same process; it passes alone in a fresh process too."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_lu(lib, nsys, n, precision, m, p, info, stream):
    return lib.ucl_lu_factor_device_static(nsys, n, precision, ctypes.c_void_p(m.data_ptr()),
                                           ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(info.data_ptr()),
                                           ctypes.c_void_p(stream.cuda_stream))


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
    A[5, :, 17] = 0.0  # singular: a zero column, so info reports a zero pivot
    dt = torch.float32 if precision == 1 else torch.float64
    src = torch.tensor(A, dtype=dt, device="cuda")
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    ref = src.clone()
    p_ref = torch.empty((nsys, n), dtype=torch.int32, device="cuda")
    i_ref = torch.empty(nsys, dtype=torch.int32, device="cuda")
    ctx.lu_factor_device(nsys, n, precision, ref.data_ptr(), p_ref.data_ptr(), i_ref.data_ptr(), st.cuda_stream)
    # every buffer the static calls touch exists before the first of them
    ms = [src.clone() for _ in range(2)]
    ps = [torch.empty((nsys, n), dtype=torch.int32, device="cuda") for _ in range(2)]
    infos = [torch.full((nsys,), -7, dtype=torch.int32, device="cuda") for _ in range(2)]
    st.wait_stream(torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert _static_lu(lib, nsys, n, precision, ms[0], ps[0], infos[0], st) == 0  # first call: per-device set-up
    st.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    ms[0].copy_(src)
    st.wait_stream(torch.cuda.current_stream())
    outs = []
    for k in range(2):  # two calls in a row share the same scratch
        assert _static_lu(lib, nsys, n, precision, ms[k], ps[k], infos[k], st) == 0
        st.synchronize()
        # nothing was allocated on the device by the call
        assert torch.cuda.mem_get_info()[0] == free0
        outs.append((ms[k].cpu().numpy(), ps[k].cpu().numpy(), infos[k].cpu().numpy()))
    ref_m, ref_p, ref_i = ref.cpu().numpy(), p_ref.cpu().numpy(), i_ref.cpu().numpy()
    tol = 1e-5 if precision == 1 else 1e-13
    ok = np.arange(nsys) != 5
    assert ref_i[5] > 0 and (ref_i[ok] == 0).all()
    for m, p, info in outs:
        np.testing.assert_array_equal(info, ref_i)
        np.testing.assert_array_equal(p[ok], ref_p[ok])
        scale = np.abs(ref_m[ok]).max(axis=(1, 2), keepdims=True)
        assert (np.abs(m[ok] - ref_m[ok]) / scale).max() <= tol
    # sizes beyond the supported range are rejected, nothing is launched
    assert lib.ucl_lu_factor_device_static(1, 522, precision, ctypes.c_void_p(src.data_ptr()),
                                           ctypes.c_void_p(p_ref.data_ptr()), ctypes.c_void_p(i_ref.data_ptr()),
                                           ctypes.c_void_p(st.cuda_stream)) == -101  # UCL_E_ARG
    ctx.close()
