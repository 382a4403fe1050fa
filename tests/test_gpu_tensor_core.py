"""The tcgen05 tensor-core product (vxg_gemm_tf32x3): C = A B in FP32 from
three TF32 products per term, checked against float64 matmul. The bound is
FP32-class: |C - C_ref| <= 4e-6 (|A| |B|) elementwise plus a small absolute
floor, which one TF32 product (10-bit mantissas, errors ~1e-3) cannot meet;
edge tiles (M, N, K not multiples of 128, 64, 32) and 1 x 1 x 1 included."""

import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 64, 32), (300, 200, 250), (97, 33, 7), (1, 1, 1),
                                   (256, 128, 512)])
def test_tf32x3_product_matches_float64(M, N, K):
    from voltax_gb300 import _lib as L
    lib = L.load()
    g = torch.Generator(device="cpu").manual_seed(M * 1000 + N * 10 + K)
    A = torch.randn(M, K, generator=g, dtype=torch.float32).cuda()
    B = torch.randn(K, N, generator=g, dtype=torch.float32).cuda()
    Cm = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    for _ in range(2):  # a second call reuses nothing from the first
        L.check(lib.vxg_gemm_tf32x3(M, N, K, A.data_ptr(), K, B.data_ptr(), N, Cm.data_ptr(), N,
                                    status.data_ptr(), torch.cuda.current_stream().cuda_stream),
                "vxg_gemm_tf32x3")
        torch.cuda.synchronize()
        assert int(status) == 0
        ref = A.double() @ B.double()
        scale = A.double().abs() @ B.double().abs()
        err = (Cm.double() - ref).abs()
        assert bool((err <= 4e-6 * scale + 1e-30).all()), float((err / scale).max())
