"""vxg_factor_static: refactorization for callers that cannot allocate.

Callers inside allocation-free hooks (framework custom calls, real-time
loops, hosts whose device allocator belongs to another runtime) cannot
provide vxg_factor's workspace. vxg_factor_static keeps the Schur scratch in
a fixed 8 MiB array inside libvxg.so instead. This file checks, through the
C ABI, that two calls in a row give the same factors as vxg_factor with a
caller workspace (same kernels, same order: equal solves within the factor
tests' tolerance), and that an oversized batch is rejected with
VXG_ERR_TOO_LARGE before anything runs.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup(precision):
    from voltax_gb300 import _lib as L
    from voltax_gb300 import sparse, symbolic, workloads
    from voltax_gb300.runtime import engine_for
    c = workloads.power_grid(12, seed=11)
    st = symbolic.structure(c)
    eng = engine_for(st, c)
    B = 3
    z = torch.rand((B, st.size), dtype=torch.float64, device="cuda")
    data = sparse.jacobian(c, z, 0.0, structure=st, gmin=1e-12).contiguous()
    return L, sparse, st, eng, B, data, L.VXG_F32 if precision == "f32" else L.VXG_F64


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_static_scratch_factor_equals_workspace_factor(precision):
    L, sparse, st, eng, B, data, p = _setup(precision)
    ref = sparse.factor(st, data, precision)
    stream = torch.cuda.current_stream().cuda_stream
    rhs = torch.randn((B, st.size), dtype=torch.float64, device="cuda")
    x_ref = sparse.solve(st, ref, rhs)
    for _ in range(2):  # two calls in a row share the static scratch
        buf = eng.factor_buffer(B, p)
        buf.fill_(0xFF)
        L.check(eng.lib.vxg_factor_static(eng.handle, B, p, data.data_ptr(), buf.data_ptr(),
                                          stream), "vxg_factor_static")
        torch.cuda.synchronize()
        fac = sparse.Factors(eng, p, B, buf, data)
        x = sparse.solve(st, fac, rhs)
        np.testing.assert_allclose(x.cpu().numpy(), x_ref.cpu().numpy(), rtol=1e-8,
                                   atol=1e-10 * float(x_ref.abs().max()))
        assert torch.equal(buf, ref.buffer)  # same kernels and order: same bits


def test_static_scratch_rejects_oversized_batch():
    L, sparse, st, eng, B, data, p = _setup("f64")
    need_per_instance = 8 * int(max(lv.schur_len for lv in st.plan.levels))
    too_many = (8 << 20) // max(need_per_instance, 1) + 1
    # buffers sized for `too_many` instances, so the call is in bounds either way
    big = data[:1].expand(too_many, -1).contiguous()
    buf = eng.factor_buffer(too_many, p)
    status = eng.lib.vxg_factor_static(eng.handle, too_many, p, big.data_ptr(),
                                       C.c_void_p(buf.data_ptr()).value,
                                       torch.cuda.current_stream().cuda_stream)
    assert status == L.VXG_ERR_TOO_LARGE
    assert b"static array" in eng.lib.vxg_last_error()
