// Dense FP32 product on the fifth-generation tensor cores: C = A B with
// three TF32 products per slab (the panel-update primitive of wide
// supernodes, tc::product_3xtf32), exposed as vxg_gemm_tf32x3.

#include "internal.cuh"
#include "tc.cuh"

namespace vxg {

// One 128 x 64 tile of C per CTA (grid: M tiles x N tiles), 128 threads.
__global__ void __launch_bounds__(128)
    gemm_tf32x3_kernel(int M, int N, int K, const float* __restrict__ A, int lda,
                       const float* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                       int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tmem_slot;
  tc::ProductState st;
  tc::product_begin(st, smem, &tmem_slot);
  const int m0 = blockIdx.x * tc::kTileM, n0 = blockIdx.y * tc::kTileN;
  const int mt = min(tc::kTileM, M - m0), nt = min(tc::kTileN, N - n0);
  tc::product_3xtf32<128>(
      st, mt, nt, K, [&](int m, int k) { return A[(long long)(m0 + m) * lda + k]; },
      [&](int k, int n) { return B[(long long)k * ldb + n0 + n]; },
      [&](int m, int n, float v) { C[(long long)(m0 + m) * ldc + n0 + n] = v; });
  tc::product_end(st);
  if (!st.ok && threadIdx.x == 0) atomicExch(status, 1);
}

}  // namespace vxg

using namespace vxg;

extern "C" int vxg_gemm_tf32x3(int32_t M, int32_t N, int32_t K, const float* A, int32_t lda,
                               const float* B, int32_t ldb, float* C, int32_t ldc,
                               int32_t* status, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !C || !status || lda < K || ldb < N ||
      ldc < N)
    return VXG_ERR_INVALID;
  const size_t smem = tc::kProductSmem + 1024;  // + alignment slack of the dynamic base
  VXG_CUDA_TRY(cudaFuncSetAttribute(gemm_tf32x3_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)((M + tc::kTileM - 1) / tc::kTileM),
            (unsigned)((N + tc::kTileN - 1) / tc::kTileN));
  gemm_tf32x3_kernel<<<grid, 128, smem, (cudaStream_t)stream>>>(M, N, K, A, lda, B, ldb, C,
                                                                   ldc, status);
  VXG_LAUNCHED();
  return VXG_OK;
}
