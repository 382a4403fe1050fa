// Learned Newton warm start: the kernels of a small MLP that maps an
// instance's parameter vector to its DC node voltages (no counterpart in
// voltax, whose Newton always starts from the caller's guess or zeros,
// voltax/analysis.py:410-431).
//
// Layers are y = act(x W^T + b) with W stored [out, in] in BF16, bias in
// FP32, activations in BF16 and every product accumulated in FP32 on the
// fifth-generation tensor cores (tcgen05.mma kind::f16, accumulators in
// tensor memory, tc::product_bf16). One GEMM kernel serves the forward pass
// and both backward products; it reads its two operands through (outer,
// reduction) strides, so no operand is ever transposed in memory:
//
//   forward   Y[m,n]  = sum_k X[m,k]  W[n,k]      A = X,    B = W
//   data grad dX[m,k] = sum_n dY[m,n] W[n,k]      A = dY,   B = W^T (strides)
//   weight    dW[n,k] = sum_m dY[m,n] X[m,k]      A = dY^T, B = X^T (strides)
//
// The tensor core's accumulation order is fixed and every other reduction
// here runs in a fixed order: the kernels are bitwise reproducible run to
// run.

#include <cuda_bf16.h>

#include "internal.cuh"
#include "tc.cuh"

namespace vxg {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int BM = 64, BN = 64;  // tile sizes of the launch-size checks

// Element (o, r) of an operand is p[o * so + r * sr].
struct Operand {
  const bf16* p;
  long long so, sr;
};

__device__ __forceinline__ float gelu(float v) {
  return 0.5f * v * (1.f + erff(v * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float v) {
  // d/dv [v Phi(v)] = Phi(v) + v phi(v)
  return 0.5f * (1.f + erff(v * 0.70710678118654752f)) +
         v * 0.39894228040143268f * expf(-0.5f * v * v);
}

// C[o1, o2] = sum_r A(o1, r) B(o2, r) on the fifth-generation tensor cores: BF16 operands from
// the strided views, FP32 accumulation in tensor memory (tc::product_bf16),
// 128 x 64 output tiles, 128 threads; every output goes through `epi`.
template <class Epi>
__global__ void __launch_bounds__(128) gemm_tc_kernel(long long M1, int M2, int R, Operand a,
                                                      Operand b, Epi epi) {
  extern __shared__ __align__(1024) unsigned char smem_tc[];
  __shared__ uint32_t tmem_slot;
  tc::ProductState ps;
  tc::product_begin(ps, smem_tc, &tmem_slot);
  tc::product_bf16<128>(
      ps, M1, M2, R,
      [&](long long o, int r) { return __bfloat16_as_ushort(a.p[o * a.so + r * a.sr]); },
      [&](long long o, int r) { return __bfloat16_as_ushort(b.p[o * b.so + r * b.sr]); },
      [&](long long m, int n, float v) { epi(m, n, v); });
  tc::product_end(ps);
}

template <class Epi>
int launch_gemm(long long M1, int M2, int R, const Operand& a, const Operand& b, const Epi& epi,
                cudaStream_t s) {
  const size_t smem = tc::kProductSmem + 1024;
  VXG_CUDA_TRY(cudaFuncSetAttribute(gemm_tc_kernel<Epi>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const dim3 grid((unsigned)((M1 + tc::kTileM - 1) / tc::kTileM),
                  (unsigned)((M2 + tc::kTileN - 1) / tc::kTileN));
  gemm_tc_kernel<Epi><<<grid, 128, smem, s>>>(M1, M2, R, a, b, epi);
  VXG_LAUNCHED();
  return VXG_OK;
}

// y = act(acc + bias): pre-activation (FP32), activation (BF16), raw output
// (FP32) and/or the de-normalised output written into a state vector.
struct FwdEpi {
  long long M;
  int N, act;
  const float* bias;
  float* pre;
  bf16* y;
  float* yf;
  const float *scale, *shift;
  double* z;
  long long ldz;
  __device__ __forceinline__ void operator()(long long m, int n, float v) const {
    if (m >= M || n >= N) return;
    v += bias ? bias[n] : 0.f;
    const long long o = m * N + n;
    if (pre) pre[o] = v;
    if (act == VXG_ACT_GELU) v = gelu(v);
    if (y) y[o] = __float2bfloat16_rn(v);
    if (yf) yf[o] = v;
    if (z) z[m * ldz + n] = (double)v * (double)scale[n] + (double)shift[n];
  }
};

// dx = acc * gelu'(pre) (or acc where the input had no activation).
struct DxEpi {
  long long M;
  int K;
  const float* pre;
  bf16* dx;
  __device__ __forceinline__ void operator()(long long m, int k, float v) const {
    if (m >= M || k >= K) return;
    const long long o = m * K + k;
    if (pre) v *= gelu_grad(pre[o]);
    dx[o] = __float2bfloat16_rn(v);
  }
};

struct DwEpi {
  int N, K;
  float* dw;
  __device__ __forceinline__ void operator()(long long n, int k, float v) const {
    if (n >= N || k >= K) return;
    dw[n * K + k] = v;
  }
};

// db[n] = sum_m dy[m, n], m ascending.
__global__ void colsum_kernel(long long M, int N, const bf16* dy, float* db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float acc = 0.f;
  for (long long m = 0; m < M; ++m) acc += __bfloat162float(dy[m * N + n]);
  db[n] = acc;
}

// x_bf16[m, k] = bf16((x[rows[m], k] - mean[k]) * inv_std[k])
__global__ void normalize_kernel(long long M, int K, const double* x, long long ldx,
                                 const long long* rows, const float* mean,
                                 const float* inv_std, bf16* out) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M * K) return;
  const long long m = e / K;
  const int k = (int)(e % K);
  const long long src = rows ? rows[m] : m;
  const float v = (float)x[src * ldx + k];
  out[e] = __float2bfloat16_rn((v - mean[k]) * inv_std[k]);
}

constexpr int kMseBlocks = 256, kMseThreads = 256;

// Squared error against target rows (gathered through `rows`), the output
// gradient dy = 2 (y - t) / (M N) in BF16, and one partial loss per block
// (thread-strided elements, then a fixed tree).
__global__ void __launch_bounds__(kMseThreads) mse_kernel(long long M, int N, const float* y,
                                                          const float* t, const long long* rows,
                                                          bf16* dy, float* partial) {
  __shared__ float red[kMseThreads];
  const float inv = 1.f / ((float)M * (float)N);
  float acc = 0.f;
  const long long total = M * N;
  for (long long e = (long long)blockIdx.x * kMseThreads + threadIdx.x; e < total;
       e += (long long)kMseBlocks * kMseThreads) {
    const long long m = e / N;
    const int n = (int)(e % N);
    const long long tr = rows ? rows[m] : m;
    const float d = y[e] - t[tr * N + n];
    acc += d * d;
    dy[e] = __float2bfloat16_rn(2.f * d * inv);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kMseThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0] * inv;
}

__global__ void __launch_bounds__(kMseBlocks) sum_partials_kernel(const float* partial,
                                                                  float* loss) {
  __shared__ float red[kMseBlocks];
  red[threadIdx.x] = partial[threadIdx.x];
  __syncthreads();
  for (int s = kMseBlocks / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = red[0];
}

// Adam on FP32 master weights; the BF16 copy the GEMMs read is rewritten.
__global__ void adam_kernel(long long n, float* w, bf16* wb, const float* g, float* m,
                            float* v, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16_rn(wi);
}

__global__ void cast_kernel(long long n, const float* w, bf16* wb) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

inline unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

inline bool grid_ok(long long m_tiles, long long n_tiles) {
  return m_tiles > 0 && m_tiles < (1LL << 31) && n_tiles > 0 && n_tiles <= 65535;
}

}  // namespace
}  // namespace vxg

using namespace vxg;

extern "C" int vxg_mlp_normalize(int64_t M, int32_t K, const double* x, int64_t ldx,
                                 const int64_t* rows, const float* mean, const float* inv_std,
                                 void* x_bf16, void* stream) {
  if (M <= 0 || K <= 0 || ldx < K || !x || !mean || !inv_std || !x_bf16) return VXG_ERR_INVALID;
  normalize_kernel<<<blocks_for(M * K, 256), 256, 0, (cudaStream_t)stream>>>(
      M, K, x, ldx, (const long long*)rows, mean, inv_std, (bf16*)x_bf16);
  VXG_LAUNCHED();
  return VXG_OK;
}

extern "C" int vxg_mlp_linear(int64_t M, int32_t N, int32_t K, const void* x_bf16,
                              const void* w_bf16, const float* bias, int32_t act, float* pre,
                              void* y_bf16, float* y_f32, const float* scale,
                              const float* shift, double* z, int64_t ldz, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || !x_bf16 || !w_bf16) return VXG_ERR_INVALID;
  if (act != VXG_ACT_NONE && act != VXG_ACT_GELU) return VXG_ERR_INVALID;
  if (z && (!scale || !shift || ldz < N)) return VXG_ERR_INVALID;
  const long long mt = (M + BM - 1) / BM, nt = (N + BN - 1) / BN;
  if (!grid_ok(mt, nt)) return VXG_ERR_TOO_LARGE;
  FwdEpi epi{M, N, act, bias, pre, (bf16*)y_bf16, y_f32, scale, shift, z, ldz};
  Operand a{(const bf16*)x_bf16, K, 1}, b{(const bf16*)w_bf16, K, 1};
  return launch_gemm(M, N, K, a, b, epi, (cudaStream_t)stream);
}

extern "C" int vxg_mlp_linear_dx(int64_t M, int32_t N, int32_t K, const void* dy_bf16,
                                 const void* w_bf16, const float* pre, void* dx_bf16,
                                 void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || !dy_bf16 || !w_bf16 || !dx_bf16) return VXG_ERR_INVALID;
  const long long mt = (M + BM - 1) / BM, kt = (K + BN - 1) / BN;
  if (!grid_ok(mt, kt)) return VXG_ERR_TOO_LARGE;
  // dX[m, k] = sum_n dY[m, n] W[n, k]: A(m, n) = dy[m*N + n], B(k, n) = w[n*K + k]
  Operand a{(const bf16*)dy_bf16, N, 1}, b{(const bf16*)w_bf16, 1, K};
  DxEpi epi{M, K, pre, (bf16*)dx_bf16};
  return launch_gemm(M, K, N, a, b, epi, (cudaStream_t)stream);
}

extern "C" int vxg_mlp_linear_dw(int64_t M, int32_t N, int32_t K, const void* dy_bf16,
                                 const void* x_bf16, float* dw, float* db, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || !dy_bf16 || !x_bf16 || !dw) return VXG_ERR_INVALID;
  if (M > INT32_MAX) return VXG_ERR_TOO_LARGE;
  const long long nt = (N + BM - 1) / BM, kt = (K + BN - 1) / BN;
  if (!grid_ok(nt, kt)) return VXG_ERR_TOO_LARGE;
  // dW[n, k] = sum_m dY[m, n] X[m, k]: A(n, m) = dy[m*N + n], B(k, m) = x[m*K + k]
  Operand a{(const bf16*)dy_bf16, 1, N}, b{(const bf16*)x_bf16, 1, K};
  DwEpi epi{N, K, dw};
  cudaStream_t s = (cudaStream_t)stream;
  const int st = launch_gemm(N, K, (int)M, a, b, epi, s);
  if (st != VXG_OK) return st;
  if (db) {
    colsum_kernel<<<blocks_for(N, 128), 128, 0, s>>>(M, N, (const bf16*)dy_bf16, db);
    VXG_LAUNCHED();
  }
  return VXG_OK;
}

extern "C" int vxg_mlp_mse(int64_t M, int32_t N, const float* y, const float* target,
                           const int64_t* rows, void* dy_bf16, float* loss, float* scratch,
                           void* stream) {
  if (M <= 0 || N <= 0 || !y || !target || !dy_bf16 || !loss || !scratch)
    return VXG_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  mse_kernel<<<kMseBlocks, kMseThreads, 0, s>>>(M, N, y, target, (const long long*)rows,
                                                (bf16*)dy_bf16, scratch);
  VXG_LAUNCHED();
  sum_partials_kernel<<<1, kMseBlocks, 0, s>>>(scratch, loss);
  VXG_LAUNCHED();
  return VXG_OK;
}

extern "C" int vxg_mlp_adam(int64_t n, float* w, void* w_bf16, const float* grad, float* m,
                            float* v, float lr, float beta1, float beta2, float eps,
                            int32_t step, void* stream) {
  if (n <= 0 || !w) return VXG_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (step == 0) {  // no update: refresh the BF16 copy only
    if (!w_bf16) return VXG_ERR_INVALID;
    cast_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, w, (bf16*)w_bf16);
    VXG_LAUNCHED();
    return VXG_OK;
  }
  if (step < 0 || !grad || !m || !v) return VXG_ERR_INVALID;
  const float c1 = 1.f / (1.f - powf(beta1, (float)step));
  const float c2 = 1.f / (1.f - powf(beta2, (float)step));
  adam_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, w, (bf16*)w_bf16, grad, m, v, lr, beta1,
                                                 beta2, eps, c1, c2);
  VXG_LAUNCHED();
  return VXG_OK;
}
