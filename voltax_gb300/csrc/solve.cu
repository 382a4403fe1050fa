// Level-scheduled block triangular solves with the supernodal factors, and
// the FP64 sparse matrix-vector products used for refinement.
//
// Forward, per level (voltax/sparse.py:583-589): y = x[piv];
// x[piv] = W y (W^T y); border contributions c = Lb y (Ub^T y) go to the
// level scratch and a second launch applies x[border] -= sum(c) with one
// thread per target unknown, sources in ascending order (deterministic).
// Backward, per level in reverse (voltax/sparse.py:590-594):
// x[piv] -= Ub x[border] (Lb^T x[border]).
// Row dot products use a warp per row (lane-strided, coalesced); transposed
// products use a thread per output column (coalesced across the warp).

#include "cplx.cuh"
#include "internal.cuh"

namespace vxg {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int off = 16; off > 0; off >>= 1) v += shfl_xor(v, off);
  return v;
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT)
    solve_fwd_kernel(const int* __restrict__ lv_sn, const long long* __restrict__ bord_off,
                     const int* __restrict__ sn_k, const int* __restrict__ sn_r,
                     const long long* __restrict__ sn_panel,
                     const long long* __restrict__ sn_piv_ptr, const int* __restrict__ sn_piv,
                     const T* __restrict__ fac, long long fstride, T* __restrict__ x, int S,
                     T* __restrict__ contrib, long long cstride, int transpose) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = lv_sn[blockIdx.x];
  const int b = blockIdx.y;
  const int k = sn_k[j], r = sn_r[j];
  const T* W = fac + (long long)b * fstride + sn_panel[j];
  const T* Ub = W + (long long)k * k;
  const T* Lb = Ub + (long long)k * r;
  const int* piv = sn_piv + sn_piv_ptr[j];
  T* xb = x + (long long)b * S;
  T* cb = contrib + (long long)b * cstride + bord_off[blockIdx.x];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* ys = reinterpret_cast<T*>(smem_raw);
  for (int l = threadIdx.x; l < k; l += NT) ys[l] = xb[piv[l]];
  __syncthreads();
  if (!transpose) {
    for (int i = warp; i < k; i += NW) {
      T acc = T(0);
      for (int l = lane; l < k; l += 32) acc += W[(long long)i * k + l] * ys[l];
      acc = warp_sum(acc);
      if (lane == 0) xb[piv[i]] = acc;
    }
    for (int a = warp; a < r; a += NW) {
      T acc = T(0);
      for (int l = lane; l < k; l += 32) acc += Lb[(long long)a * k + l] * ys[l];
      acc = warp_sum(acc);
      if (lane == 0) cb[a] = acc;
    }
  } else {
    for (int i = threadIdx.x; i < k; i += NT) {
      T acc = T(0);
      for (int l = 0; l < k; ++l) acc += W[(long long)l * k + i] * ys[l];
      xb[piv[i]] = acc;
    }
    for (int a = threadIdx.x; a < r; a += NT) {
      T acc = T(0);
      for (int l = 0; l < k; ++l) acc += Ub[(long long)l * r + a] * ys[l];
      cb[a] = acc;
    }
  }
}

template <typename T>
__global__ void border_apply_kernel(int B, long long ntgt, const int* __restrict__ tgt,
                                    const long long* __restrict__ ptr,
                                    const long long* __restrict__ src,
                                    const T* __restrict__ contrib, long long cstride,
                                    T* __restrict__ x, int S) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * ntgt) return;
  const int b = (int)(gid / ntgt);
  const long long t = gid - (long long)b * ntgt;
  const T* c = contrib + (long long)b * cstride;
  T acc = T(0);
  for (long long p = ptr[t]; p < ptr[t + 1]; ++p) acc += c[src[p]];
  x[(long long)b * S + tgt[t]] -= acc;
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT)
    solve_bwd_kernel(const int* __restrict__ lv_sn, const int* __restrict__ sn_k,
                     const int* __restrict__ sn_r, const long long* __restrict__ sn_panel,
                     const long long* __restrict__ sn_piv_ptr, const int* __restrict__ sn_piv,
                     const long long* __restrict__ sn_bord_ptr,
                     const int* __restrict__ sn_bord, const T* __restrict__ fac,
                     long long fstride, T* __restrict__ x, int S, int transpose) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = lv_sn[blockIdx.x];
  const int b = blockIdx.y;
  const int k = sn_k[j], r = sn_r[j];
  if (r == 0) return;
  const T* W = fac + (long long)b * fstride + sn_panel[j];
  const T* Ub = W + (long long)k * k;
  const T* Lb = Ub + (long long)k * r;
  const int* piv = sn_piv + sn_piv_ptr[j];
  const int* brd = sn_bord + sn_bord_ptr[j];
  T* xb = x + (long long)b * S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* xs = reinterpret_cast<T*>(smem_raw);
  for (int a = threadIdx.x; a < r; a += NT) xs[a] = xb[brd[a]];
  __syncthreads();
  if (!transpose) {
    for (int i = warp; i < k; i += NW) {
      T acc = T(0);
      for (int a = lane; a < r; a += 32) acc += Ub[(long long)i * r + a] * xs[a];
      acc = warp_sum(acc);
      if (lane == 0) xb[piv[i]] -= acc;
    }
  } else {
    for (int i = threadIdx.x; i < k; i += NT) {
      T acc = T(0);
      for (int a = 0; a < r; ++a) acc += Lb[(long long)a * k + i] * xs[a];
      xb[piv[i]] -= acc;
    }
  }
}

// ---------------------------------------------------------------- helpers
template <typename A, typename Bt>
__global__ void cast_kernel(long long n, const A* __restrict__ in, Bt* __restrict__ out) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (Bt)in[i];
}

__global__ void add_cast_kernel(long long n, const float* __restrict__ in,
                                double* __restrict__ out) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] += (double)in[i];
}

__global__ void spmv_kernel(int B, int S, const long long* __restrict__ indptr,
                            const int* __restrict__ indices, long long nnz,
                            const double* __restrict__ data, const double* __restrict__ x,
                            double* __restrict__ y) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * S) return;
  const int b = (int)(gid / S);
  const int i = (int)(gid - (long long)b * S);
  const double* d = data + (long long)b * nnz;
  const double* xb = x + (long long)b * S;
  double acc = 0.0;
  for (long long e = indptr[i]; e < indptr[i + 1]; ++e) acc += d[e] * xb[indices[e]];
  y[gid] = acc;
}

__global__ void spmv_t_kernel(int B, int S, const long long* __restrict__ tptr,
                              const long long* __restrict__ tent, const int* __restrict__ rows,
                              long long nnz, const double* __restrict__ data,
                              const double* __restrict__ x, double* __restrict__ y) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * S) return;
  const int b = (int)(gid / S);
  const int j = (int)(gid - (long long)b * S);
  const double* d = data + (long long)b * nnz;
  const double* xb = x + (long long)b * S;
  double acc = 0.0;
  for (long long p = tptr[j]; p < tptr[j + 1]; ++p) {
    const long long e = tent[p];
    acc += d[e] * xb[rows[e]];
  }
  y[gid] = acc;
}

// r = b - y
__global__ void sub_kernel(long long n, const double* __restrict__ b,
                           const double* __restrict__ y, double* __restrict__ r) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) r[i] = b[i] - y[i];
}

static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int launch_spmv(const Topo& t, int B, const double* data, const double* x, double* y,
                int transpose, cudaStream_t s) {
  const long long n = (long long)B * t.S;
  if (!n) return VXG_OK;
  if (!transpose)
    spmv_kernel<<<nblk(n, 256), 256, 0, s>>>(B, t.S, t.indptr, t.indices, t.nnz, data, x, y);
  else
    spmv_t_kernel<<<nblk(n, 256), 256, 0, s>>>(B, t.S, t.tptr, t.tent, t.rows, t.nnz, data, x,
                                                y);
  VXG_LAUNCHED();
  return VXG_OK;
}

// In-place solve of x (T, B x S) with factors fac.
template <typename T>
static int solve_levels(const Topo& t, int B, const T* fac, T* x, T* contrib, int transpose,
                        cudaStream_t s) {
  const long long fs = t.work, cs = t.max_bord;
  for (int L = 0; L < t.n_levels; ++L) {
    const long long lo = t.h_lv_ptr[L], hi = t.h_lv_ptr[L + 1];
    if (hi == lo) continue;
    dim3 grid((unsigned)(hi - lo), (unsigned)B);
    const size_t smem = sizeof(T) * (size_t)max(t.h_lv_kmax[L], 1);
    solve_fwd_kernel<T, 128><<<grid, 128, smem, s>>>(t.lv_sn + lo, t.lv_bord_off + lo, t.sn_k,
                                                     t.sn_r, t.sn_panel, t.sn_piv_ptr,
                                                     t.sn_piv, fac, fs, x, t.S, contrib, cs,
                                                     transpose);
    VXG_LAUNCHED();
    const long long tlo = t.h_lv_bt_ptr[L], thi = t.h_lv_bt_ptr[L + 1];
    const long long nt = (long long)B * (thi - tlo);
    if (nt) {
      border_apply_kernel<T><<<nblk(nt, 256), 256, 0, s>>>(B, thi - tlo, t.bt_tgt + tlo,
                                                           t.bt_ptr + tlo, t.bt_src, contrib,
                                                           cs, x, t.S);
      VXG_LAUNCHED();
    }
  }
  for (int L = t.n_levels - 1; L >= 0; --L) {
    const long long lo = t.h_lv_ptr[L], hi = t.h_lv_ptr[L + 1];
    if (hi == lo || t.h_lv_rmax[L] == 0) continue;
    dim3 grid((unsigned)(hi - lo), (unsigned)B);
    const size_t smem = sizeof(T) * (size_t)t.h_lv_rmax[L];
    solve_bwd_kernel<T, 128><<<grid, 128, smem, s>>>(t.lv_sn + lo, t.sn_k, t.sn_r, t.sn_panel,
                                                     t.sn_piv_ptr, t.sn_piv, t.sn_bord_ptr,
                                                     t.sn_bord, fac, fs, x, t.S, transpose);
    VXG_LAUNCHED();
  }
  return VXG_OK;
}

// x = A^-1 b for the complex factors of every frequency; b shared by all
// frequencies when b_stride is 0 (interleaved re, im).
__global__ void bcast_cplx_kernel(long long n, int S, const cplx* __restrict__ b,
                                  long long b_stride, cplx* __restrict__ x) {
  const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= n) return;
  const long long f = gid / S, i = gid - f * S;
  x[gid] = b[f * b_stride + i];
}

int launch_solve_ac(const Topo& t, int B, const void* factors, const double* b,
                    long long b_stride, double* x, void* scratch, cudaStream_t s) {
  const long long n = (long long)B * t.S;
  if (!n) return VXG_OK;
  bcast_cplx_kernel<<<nblk(n, 256), 256, 0, s>>>(n, t.S, (const cplx*)b, b_stride, (cplx*)x);
  VXG_LAUNCHED();
  return solve_levels<cplx>(t, B, (const cplx*)factors, (cplx*)x, (cplx*)scratch, 0, s);
}

int launch_solve(const Topo& t, int B, int precision, const void* factors, const double* data,
                 const double* b, double* x, int transpose, int refine, void* vec_t,
                 void* scratch, double* r64, cudaStream_t s) {
  const long long n = (long long)B * t.S;
  if (!n) return VXG_OK;
  if (precision == VXG_F64) {
    if (x != b) VXG_CUDA_TRY(cudaMemcpyAsync(x, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    return solve_levels<double>(t, B, (const double*)factors, x, (double*)scratch, transpose, s);
  }
  if (precision != VXG_F32) return VXG_ERR_INVALID;
  // r64 holds 2*B*S doubles: [copy of b | residual]
  double* bcopy = r64;
  double* res = r64 + n;
  float* xt = (float*)vec_t;
  VXG_CUDA_TRY(cudaMemcpyAsync(bcopy, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  cast_kernel<double, float><<<nblk(n, 256), 256, 0, s>>>(n, bcopy, xt);
  VXG_LAUNCHED();
  int st = solve_levels<float>(t, B, (const float*)factors, xt, (float*)scratch, transpose, s);
  if (st) return st;
  cast_kernel<float, double><<<nblk(n, 256), 256, 0, s>>>(n, xt, x);
  VXG_LAUNCHED();
  if (!data) refine = 0;
  for (int it = 0; it < refine; ++it) {
    st = launch_spmv(t, B, data, x, res, transpose, s);
    if (st) return st;
    sub_kernel<<<nblk(n, 256), 256, 0, s>>>(n, bcopy, res, res);
    VXG_LAUNCHED();
    cast_kernel<double, float><<<nblk(n, 256), 256, 0, s>>>(n, res, xt);
    VXG_LAUNCHED();
    st = solve_levels<float>(t, B, (const float*)factors, xt, (float*)scratch, transpose, s);
    if (st) return st;
    add_cast_kernel<<<nblk(n, 256), 256, 0, s>>>(n, xt, x);
    VXG_LAUNCHED();
  }
  return VXG_OK;
}

}  // namespace vxg
