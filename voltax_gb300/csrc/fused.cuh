// The fused persistent Newton kernel (included by fused.cu and the
// per-instantiation units fused_<type>_<threads>.cu).
#pragma once

// Fused persistent Newton kernel for small circuits.
//
// One CTA owns one circuit instance at a time (grid-stride over the batch)
// and runs the whole analysis in shared memory: the DC operating point with
// the gmin-stepping fallback (voltax/analysis.py:236-266), then every
// backward-Euler or trapezoidal time step (voltax/analysis.py:434-480), each
// a damped Newton solve (voltax/analysis.py:208-233) of
//   device evaluation -> deterministic stamping -> supernodal refactorization
//   -> level-scheduled solves (+ FP64 refinement) -> damped update.
// Nothing but parameters, time points and the output states touches global
// memory; the topology tables are read through L1.
//
// Each level's supernodes are factored one per thread (many tiny ones),
// one per warp (several, k <= 32) or by the whole CTA (a lone supernode, or
// any with k > 32, up to 128): Gauss-Jordan with partial pivoting in shared
// memory, then Ub, the Schur block and Lb. Schur and border updates of a
// level are applied by a second pass with one thread per target slot
// summing its sources in a fixed order, so results are bitwise
// reproducible.

#include <algorithm>
#include <cstring>

#include "devices.cuh"

namespace vxg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kCtaK = 128;    // widest supernode the whole-CTA factorization takes
constexpr int kMaxWarps = 16;  // largest CTA: 512 threads

struct FusedArgs {
  GroupTable gt;
  int S, nv, nnz, n_res, n_jac, work, n_levels, max_scr;
  const long long *res_ptr, *res_src, *jac_ptr, *jac_src, *a_pos, *indptr;
  const int *indices, *rows;
  const int *sn_k, *sn_r, *sn_piv, *sn_bord;
  const long long *sn_panel, *sn_piv_ptr, *sn_bord_ptr;
  const long long* lv_ptr;
  const int* lv_kmax;  // largest supernode of each level
  const int* lv_sn;
  const long long *lv_schur_off, *lv_bord_off;
  const long long *lv_st_ptr, *st_tgt, *st_ptr, *st_src;
  const long long* lv_bt_ptr;
  const int* bt_tgt;
  const long long *bt_ptr, *bt_src;
  const unsigned short* blob;  // 16-bit tables (global), staged into shared memory
  Blob bo;
  int first_global;  // sections from this one on stay in global memory
  int staged;        // table elements copied to shared memory (a multiple of 8)
  int B, mode, n_t, max_steps, refine, dc_first, gmin_steps, direct_steps;
  double rtol, atol, max_dv, gmin;
  const double* ts;
  const double* gmins;
  const double* z0;
  double* z_out;
  int* conv;
  int* iters;
  // DC sweep (vxg_fused_sweep; sweep_vals null otherwise): before point n,
  // instance b writes sweep_vals[n] to sweep_slot[b * sweep_stride], its
  // own copy of the swept parameter, then solves DC at sweep_t from point
  // n-1's solution
  const double* sweep_vals;
  double* sweep_slot;
  long long sweep_stride;
  double sweep_t;
  // phase timing (a diagnostic, normally null): SM clock cycles of each CTA
  // per phase, summed over CTAs -- eval, assemble, factor, solve, update,
  // and the whole kernel -- see vxg_fused_set_profile
  long long* phase_clk;
};

enum { PH_EVAL = 0, PH_ASSEMBLE, PH_FACTOR, PH_SOLVE, PH_UPDATE, PH_TOTAL, PH_COUNT = 8 };

__host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline int sbuf_values(int nw) { return 64 * nw > 2 * kCtaK ? 64 * nw : 2 * kCtaK; }
__host__ __device__ inline int sbuf_records(int nw) { return 32 * nw > kCtaK ? 32 * nw : kCtaK; }

// Shared-memory layout of one instance.
struct FusedLayout {
  size_t blob, z, fp, qp, f, q, rhs, dz, data, cf, cq, cj, work, scr, xt, red, prof, sbuf, total;
};

// The chosen form (FP32 panels) evaluates its devices in two passes -- FP64
// currents and charges, then the FP32 local Jacobians -- so its Jacobian
// contributions reuse the storage of the current and charge contributions.
template <typename T>
__host__ __device__ constexpr bool split_eval() {
  return sizeof(T) == sizeof(float);
}

// Shared memory of one instance; a warp-owned instance (warp_group) needs
// only one warp's column/row buffers and pivot records.
__host__ __device__ inline int inst_sbuf_values(int nw, bool warp_group) {
  return warp_group ? 64 : sbuf_values(nw);
}
__host__ __device__ inline int inst_sbuf_records(int nw, bool warp_group) {
  return warp_group ? 32 : sbuf_records(nw);
}

template <typename T>
__host__ __device__ inline FusedLayout fused_layout(int S, int nnz, int n_res, int n_jac,
                                                    int work, int max_scr, int blob_len,
                                                    int nw, bool warp_group = false) {
  // T is the panel type; the Jacobian contributions use the same type
  FusedLayout L;
  size_t o = 0;
  L.blob = o;
  o = a16(o + sizeof(unsigned short) * (size_t)blob_len);
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = a16(o + bytes);
    return at;
  };
  const size_t d = sizeof(double);
  L.z = take(d * S);
  L.fp = take(d * S);
  L.qp = take(d * S);
  L.f = take(d * S);
  L.q = take(d * S);
  L.rhs = take(d * S);
  L.dz = take(d * S);
  L.data = take(sizeof(T) * nnz);
  // The device contributions (written by the evaluation, read by the
  // assembly) and the panels, Schur scratch and solve vector (written after
  // the assembly, read until the solve ends) are never live at the same
  // time, so they share one region; so do the current/charge and the
  // Jacobian contributions when they are evaluated in two passes.
  const size_t shared_at = o;
  L.cf = take(d * n_res);
  L.cq = take(d * n_res);
  size_t contrib_end = o;
  if (split_eval<T>()) o = shared_at;
  L.cj = take(sizeof(T) * n_jac);
  if (o > contrib_end) contrib_end = o;
  o = shared_at;
  L.work = take(sizeof(T) * work);
  L.scr = take(sizeof(T) * (max_scr > 0 ? max_scr : 1));
  L.xt = take(sizeof(T) * S);
  if (o < contrib_end) o = contrib_end;
  L.red = take(64 * sizeof(double));
  L.prof = take(PH_COUNT * sizeof(long long));
  // per-warp column/row buffers (64 values) and pivot records (32) of nw
  // warps, or the whole CTA's (2 kCtaK values, kCtaK records)
  L.sbuf = take(sizeof(T) * inst_sbuf_values(nw, warp_group) +
                sizeof(int) * inst_sbuf_records(nw, warp_group));
  L.total = o;
  return L;
}

template <typename T>
__device__ __forceinline__ T tabs_(T x) {
  return x < T(0) ? -x : x;
}

// ------------------------------------------------------------ block helpers
template <int NT>
__device__ double block_max_nan(double v, int nan_flag, double* red, int* nan_out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int off = 16; off > 0; off >>= 1) {
    v = fmax(v, __shfl_xor_sync(kFull, v, off));
    nan_flag |= __shfl_xor_sync(kFull, nan_flag, off);
  }
  int* redi = reinterpret_cast<int*>(red + 32);
  __syncthreads();
  if (lane == 0) {
    red[warp] = v;
    redi[warp] = nan_flag;
  }
  __syncthreads();
  double m = 0.0;
  int nf = 0;
  for (int w = 0; w < NT / 32; ++w) {
    m = fmax(m, red[w]);
    nf |= redi[w];
  }
  *nan_out = nf;
  return m;
}

template <int NT>
__device__ int block_all(int ok, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ok = __all_sync(kFull, ok);
  int* redi = reinterpret_cast<int*>(red + 32);
  __syncthreads();
  if (lane == 0) redi[warp] = ok;
  __syncthreads();
  int all = 1;
  for (int w = 0; w < NT / 32; ++w) all &= redi[w];
  return all;
}

// ------------------------------------------------------- supernode LDU
// One supernode's block LDU by a group of threads: one warp (CTA = false,
// the supernodes of a wide level in parallel, k <= 32) or the whole CTA
// (CTA = true, the lone supernodes of the top levels, k <= kCtaK).
//   W  = F11^-1 by Gauss-Jordan with partial pivoting: for k <= 32 by one
//        warp with the rows in registers (warp_gj; in a CTA group the other
//        warps wait), for wider blocks by the whole CTA in shared memory
//        with two barriers per pivot step, lane l owning columns l, l + 32,
//        ... (row swaps recorded, undone as column swaps);
//   Ub = W F12 in place (one column per warp, the column held in registers
//        and broadcast by shuffles);
//   S  = F21 Ub into Sout;  Lb = F21 W in place (one row per warp).
template <bool CTA, int NT>
__device__ __forceinline__ void group_sync() {
  if (CTA)
    __syncthreads();
  else
    __syncwarp();
}

// Warp argmax of |a| over the lanes in `valid` (ties to the lowest lane);
// -1 when no lane is valid. One warp-wide integer max reduction on the bit
// pattern (a non-negative float orders like its bits), not five shuffle
// rounds; doubles compare their high word first and, only between lanes
// that tie on it, the low word.
__device__ __forceinline__ int warp_argmax_abs(float a, bool valid) {
  const unsigned key = valid ? __float_as_uint(fabsf(a)) + 1u : 0u;
  const unsigned m = __reduce_max_sync(kFull, key);
  if (m == 0u) return -1;
  return __ffs(__ballot_sync(kFull, key == m)) - 1;
}
__device__ __forceinline__ int warp_argmax_abs(double a, bool valid) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(fabs(a));
  const unsigned hi = valid ? (unsigned)(bits >> 32) + 1u : 0u;
  const unsigned mh = __reduce_max_sync(kFull, hi);
  if (mh == 0u) return -1;
  unsigned cand = __ballot_sync(kFull, hi == mh);
  if (__popc(cand) > 1) {
    const bool in = (cand >> (threadIdx.x & 31)) & 1u;
    const unsigned lo = in ? (unsigned)bits : 0u;
    const unsigned ml = __reduce_max_sync(kFull, lo);
    cand = __ballot_sync(kFull, in && lo == ml);
  }
  return __ffs(cand) - 1;
}

// Gauss-Jordan inverse of the k x k block A (row-major in shared memory,
// k <= K <= 32) by one warp, one matrix row per lane in registers, with
// partial pivoting (largest |a| in the column among rows not yet used,
// ties to the lower row). Rows never move: step c exchanges the pivot row
// p_c with column c in place (the exchange operator: the pivot row becomes
// x_c in terms of the right-hand side, the other rows are eliminated), so
// the result is the inverse with its rows in pivot-row order and its
// columns in pivot-step order; the write-back puts row p_c into row c and
// column c into column p_c. The pivot row is staged in `prow` (one
// division per lane per step); perm[c] = p_c.
template <typename T, int K>
__device__ __forceinline__ T reg_at(const T (&row)[K], int c) {
  T x = T(0);
#pragma unroll
  for (int j = 0; j < K; ++j)
    if (j == c) x = row[j];
  return x;
}

template <typename T, int K>
__device__ __forceinline__ void warp_gj(T* A, int k, T* prow, int* perm) {
  const int lane = threadIdx.x & 31;
  T row[K];
#pragma unroll
  for (int j = 0; j < K; ++j) row[j] = (lane < k && j < k) ? A[lane * k + j] : T(0);
  const unsigned rows_k = k >= 32 ? kFull : ((1u << k) - 1u);
  unsigned used = 0u;
  int my_step = 0;  // the step at which this lane's row is the pivot
#pragma unroll 1
  for (int c = 0; c < k; ++c) {
    const T a = reg_at(row, c);
    const bool free_row = ((rows_k & ~used) >> lane) & 1u;
    int p = warp_argmax_abs(a, free_row && a == a);
    if (p < 0) p = __ffs(rows_k & ~used) - 1;  // every candidate NaN
    used |= 1u << p;
    if (lane == 0) perm[c] = p;
    if (lane == p) {
      my_step = c;
#pragma unroll
      for (int j = 0; j < K; ++j)
        if (j < k) prow[j] = row[j];
    }
    __syncwarp();
    const T d = __shfl_sync(kFull, a, p);
    if (lane < k) prow[lane] = ((lane == c) ? T(1) : prow[lane]) / d;
    __syncwarp();
    const T f = a;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (j < k) {
        const T rj = prow[j];
        row[j] = (lane == p) ? rj : ((j == c) ? T(0) : row[j]) - f * rj;
      }
    }
    __syncwarp();  // prow is rewritten by the next step
  }
  // row p_c holds row c of the inverse with column c' at perm[c']
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const int col = perm[j < k ? j : 0];
    if (j < k && lane < k) A[my_step * k + col] = row[j];
  }
  __syncwarp();
}

template <typename T, bool CTA, int NT, int KQ>  // KQ: columns per lane (k <= 32 KQ)
__device__ void sn_factor(T* P, int k, int r, T* Sout, T* colb, T* rowb, int* perm) {
  constexpr int GW = CTA ? NT / 32 : 1;  // warps in the group
  const int lane = threadIdx.x & 31;
  const int gw = CTA ? (threadIdx.x >> 5) : 0;  // warp index inside the group
  T* A = P;
  T* F12 = P + k * k;
  T* F21 = F12 + k * r;
  if (!CTA || k <= 32) {  // one warp (k <= 32): rows in registers
    if (!CTA || gw == 0) {
      if (k <= 8)
        warp_gj<T, 8>(A, k, rowb, perm);
      else if (k <= 16)
        warp_gj<T, 16>(A, k, rowb, perm);
      else
        warp_gj<T, 32>(A, k, rowb, perm);
    }
    group_sync<CTA, NT>();
  } else {  // the whole CTA (k > 32): shared-memory Gauss-Jordan, rows over warps
  for (int c = 0; c < k; ++c) {
    if (gw == 0) {
      // pivot: largest |A[i][c]| over i >= c, ties to the lower row
      T v = T(-1);
      int bi = k;
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        const int i = lane + 32 * q;
        if (i >= c && i < k) {
          const T a = tabs_(A[i * k + c]);
          if (a > v) {
            v = a;
            bi = i;
          }
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const T ov = __shfl_down_sync(kFull, v, off);
        const int oi = __shfl_down_sync(kFull, bi, off);
        if (ov > v || (ov == v && oi < bi)) {
          v = ov;
          bi = oi;
        }
      }
      int p = __shfl_sync(kFull, bi, 0);
      if (p < c || p >= k) p = c;
      if (lane == 0) perm[c] = p;
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        const int j = lane + 32 * q;
        if (p != c && j < k) {
          const T tmp = A[p * k + j];
          A[p * k + j] = A[c * k + j];
          A[c * k + j] = tmp;
        }
      }
      __syncwarp();
      const T d = A[c * k + c];
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        const int j = lane + 32 * q;
        if (j < k) {
          rowb[j] = ((j == c) ? T(1) : A[c * k + j]) / d;
          colb[j] = (j == c) ? T(0) : A[j * k + c];
        }
      }
    }
    group_sync<CTA, NT>();
    T rj[KQ];  // this lane's entries of the scaled pivot row
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int j = lane + 32 * q;
      rj[q] = j < k ? rowb[j] : T(0);
    }
#pragma unroll 4
    for (int i = gw; i < k; i += GW) {
      const T ci = colb[i];
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        const int j = lane + 32 * q;
        if (j < k) {
          if (i == c) {
            A[c * k + j] = rj[q];
          } else {
            const T a = (j == c) ? T(0) : A[i * k + j];
            A[i * k + j] = a - ci * rj[q];
          }
        }
      }
    }
    group_sync<CTA, NT>();
  }
  // undo the row swaps as column swaps; one thread per row
  for (int i = CTA ? threadIdx.x : lane; i < k; i += CTA ? NT : 32)
    for (int c = k - 1; c >= 0; --c) {
      const int p = perm[c];
      if (p != c) {
        const T tmp = A[i * k + c];
        A[i * k + c] = A[i * k + p];
        A[i * k + p] = tmp;
      }
    }
  group_sync<CTA, NT>();
  }
  if (r == 0) return;
  // Ub = W F12: warp-strided columns; lane l holds F12[l + 32q][col]
  for (int col = gw; col < r; col += GW) {
    T v[KQ], acc[KQ];
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int i = lane + 32 * q;
      v[q] = i < k ? F12[i * r + col] : T(0);
      acc[q] = T(0);
    }
#pragma unroll
    for (int qs = 0; qs < KQ; ++qs) {
      const int l1 = min(32, k - 32 * qs);
      for (int ll = 0; ll < l1; ++ll) {
        const int l = 32 * qs + ll;
        const T x = __shfl_sync(kFull, v[qs], ll);
#pragma unroll
        for (int q = 0; q < KQ; ++q) {
          const int i = lane + 32 * q;
          if (i < k) acc[q] += A[i * k + l] * x;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int i = lane + 32 * q;
      if (i < k) F12[i * r + col] = acc[q];
    }
  }
  group_sync<CTA, NT>();
  // S = F21 Ub
  for (int a = gw; a < r; a += GW)
    for (int b = lane; b < r; b += 32) {
      T acc = T(0);
      for (int l = 0; l < k; ++l) acc += F21[a * k + l] * F12[l * r + b];
      Sout[a * r + b] = acc;
    }
  group_sync<CTA, NT>();
  // Lb = F21 W, one row per warp
  for (int a = gw; a < r; a += GW) {
    T acc[KQ];
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int j = lane + 32 * q;
      acc[q] = T(0);
      if (j < k)
        for (int l = 0; l < k; ++l) acc[q] += F21[a * k + l] * A[l * k + j];
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < KQ; ++q) {
      const int j = lane + 32 * q;
      if (j < k) F21[a * k + j] = acc[q];
    }
    __syncwarp();
  }
  group_sync<CTA, NT>();
}

// ---------------------------------------------- tiny supernodes (k <= 4)
// One thread per supernode: closed loops over k <= 4 with the same
// Gauss-Jordan / Ub / S / Lb steps as sn_factor.
constexpr int kTiny = 4;

template <typename T>
__device__ void tiny_factor(T* P, int k, int r, T* Sout) {
  T* A = P;
  T* F12 = P + k * k;
  T* F21 = F12 + k * r;
  int perm[kTiny];
#pragma unroll
  for (int c = 0; c < kTiny; ++c) {
    if (c >= k) break;
    int p = c;
    T best = tabs_(A[c * k + c]);
    for (int i = c + 1; i < k; ++i) {
      const T v = tabs_(A[i * k + c]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    perm[c] = p;
    if (p != c)
      for (int j = 0; j < k; ++j) {
        const T t = A[p * k + j];
        A[p * k + j] = A[c * k + j];
        A[c * k + j] = t;
      }
    const T d = A[c * k + c];
    A[c * k + c] = T(1);
    for (int j = 0; j < k; ++j) A[c * k + j] = A[c * k + j] / d;
    for (int i = 0; i < k; ++i) {
      if (i == c) continue;
      const T f = A[i * k + c];
      A[i * k + c] = T(0);
      for (int j = 0; j < k; ++j) A[i * k + j] -= f * A[c * k + j];
    }
  }
#pragma unroll
  for (int c = kTiny - 1; c >= 0; --c) {
    if (c >= k) continue;
    const int p = perm[c];
    if (p != c)
      for (int i = 0; i < k; ++i) {
        const T t = A[i * k + c];
        A[i * k + c] = A[i * k + p];
        A[i * k + p] = t;
      }
  }
  if (r == 0) return;
  for (int col = 0; col < r; ++col) {  // Ub = W F12
    T x[kTiny];
#pragma unroll
    for (int l = 0; l < kTiny; ++l) x[l] = l < k ? F12[l * r + col] : T(0);
#pragma unroll
    for (int i = 0; i < kTiny; ++i) {
      if (i >= k) break;
      T acc = T(0);
#pragma unroll
      for (int l = 0; l < kTiny; ++l)
        if (l < k) acc += A[i * k + l] * x[l];
      F12[i * r + col] = acc;
    }
  }
  for (int a = 0; a < r; ++a) {  // S = F21 Ub, then Lb = F21 W (row a)
    T f[kTiny];
#pragma unroll
    for (int l = 0; l < kTiny; ++l) f[l] = l < k ? F21[a * k + l] : T(0);
    for (int b = 0; b < r; ++b) {
      T acc = T(0);
#pragma unroll
      for (int l = 0; l < kTiny; ++l)
        if (l < k) acc += f[l] * F12[l * r + b];
      Sout[a * r + b] = acc;
    }
#pragma unroll
    for (int j = 0; j < kTiny; ++j) {
      if (j >= k) break;
      T acc = T(0);
#pragma unroll
      for (int l = 0; l < kTiny; ++l)
        if (l < k) acc += f[l] * A[l * k + j];
      F21[a * k + j] = acc;
    }
  }
}

// ------------------------------------------------------------- one instance
typedef unsigned short u16;

// One instance worked on by a group of threads: the whole CTA (kWarp false,
// NT threads) or one warp (kWarp true; the CTA then holds NT / 32 instances,
// one per warp, sharing the staged tables). tid() / wid() are the thread and
// warp index inside the group, GT / GW its thread and warp counts, sync()
// its barrier.
template <typename T, int NT, bool kWarp = false>
struct Instance {
  static constexpr int GT = kWarp ? 32 : NT;
  static constexpr int GW = kWarp ? 1 : NT / 32;
  __device__ __forceinline__ static int tid() {
    return kWarp ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
  }
  __device__ __forceinline__ static int wid() { return kWarp ? 0 : (int)(threadIdx.x >> 5); }
  __device__ __forceinline__ static void sync() {
    if (kWarp)
      __syncwarp();
    else
      __syncthreads();
  }

  const FusedArgs& A;
  int b;
  double *z, *fp, *qp, *f, *q, *rhs, *dz, *cf, *cq, *red;
  T *data, *cj, *work, *scr, *xt, *sbuf;
  int* ibuf;
  long long* prof;  // per-instance phase cycles (shared memory), used when A.phase_clk
  const u16* tb;  // shared-memory tables

  // The group's thread 0 adds the cycles since *t0 to phase p; every phase
  // ends with the group's barrier, so that thread's clock is the group's.
  __device__ __forceinline__ void mark(int p, long long* t0) const {
    if (A.phase_clk && tid() == 0) {
      const long long t = clock64();
      prof[p] += t - *t0;
      *t0 = t;
    }
  }

  // a staged table section (shared memory; the Schur gather sections may
  // instead stay in global memory, see apply_schur)
  __device__ __forceinline__ const u16* sec(int k) const { return tb + A.bo.off[k]; }

  // work[tgt] -= (sum of the level's Schur block entries aimed at it), one
  // thread per target, sources in a fixed order
  __device__ __forceinline__ void apply_schur(int t0, int t1, const u16* st_tgt,
                                              const u16* st_ptr, const u16* st_src) {
    for (int t = t0 + tid(); t < t1; t += GT) {
      T acc = T(0);
      const int p1 = st_ptr[t + 1];
      for (int p = st_ptr[t]; p < p1; ++p) acc += scr[st_src[p]];
      work[st_tgt[t]] -= acc;
    }
  }

  // How a level's supernodes are factored and solved: one thread each
  // (many tiny supernodes with short borders), one warp each (several
  // supernodes), or the whole CTA (a lone supernode, supernodes wider than
  // 32, or a few with wide borders whose Schur blocks need more than a warp).
  // A warp-owned instance (kWarp) has no CTA mode: its warp takes the
  // supernodes one after the other, or its lanes take tiny ones in parallel
  // (its topologies have no supernode wider than 32).
  enum { LV_TINY = 0, LV_WARP = 1, LV_CTA = 2 };
  __device__ __forceinline__ int level_mode(int L) const {
    const u16* lv_ptr = sec(B_LV_PTR);
    const int n = lv_ptr[L + 1] - lv_ptr[L];
    const int kmax = sec(B_LV_KMAX)[L], rmax = sec(B_LV_RMAX)[L];
    if (kWarp) return (kmax <= kTiny && rmax <= 8 && n >= 4) ? LV_TINY : LV_WARP;
    if (kmax > 32) return LV_CTA;
    if (kmax <= kTiny && n >= GW && rmax <= 8) return LV_TINY;
    if (n >= 2 && (2 * n >= GW || rmax <= 16)) return LV_WARP;
    return LV_CTA;
  }

  // devices -> contribution slots (structure of arrays per group)
  __device__ void eval(const double* zz, double t, double cfc, double cqc, bool wf, bool wq,
                       bool wj) {
    const GroupTable& gt = A.gt;
    const u16* nodes = sec(B_NODES);
    for (int flat = tid(); flat < gt.n_dev; flat += GT) {
      int gi = 0;
      while (gi + 1 < gt.n_groups && gt.g[gi + 1].dev_base <= flat) ++gi;
      const GroupDev& g = gt.g[gi];
      const int d = flat - (int)g.dev_base;
      const u16* nd = nodes + A.bo.node_off[gi] + d * g.T;
      double u[kFusedMaxM];
#pragma unroll
      for (int i = 0; i < kFusedMaxM; ++i) {
        if (i < g.T) {
          const u16 node = nd[i];
          u[i] = node != 0xFFFF ? zz[node] : 0.0;
        } else if (i < g.m) {
          u[i] = zz[g.int_offset + d * g.K + (i - g.T)];
        } else {
          u[i] = 0.0;
        }
      }
      eval_soa<T>(g, b, d, u, t, cfc, cqc, wf, wq, wj, cf + g.res_base, cq + g.res_base,
                  cj + g.jac_base, zz);
    }
  }

  // Sum of vals[src[p]] over p in [p0, p1): one thread in order for short
  // lists; lists longer than 32 are summed by a whole warp -- lane l adds
  // p0 + l, p0 + l + 32, ... in order, then a fixed butterfly combines the
  // lanes -- so a node with hundreds of contributions (a supply rail) is not
  // one long serial chain. Both orders are fixed: bitwise reproducible.
  template <typename V>
  __device__ __forceinline__ V warp_list_sum(const V* vals, const u16* src, int p0, int p1) {
    const int lane = threadIdx.x & 31;
    V acc = V(0);
    for (int p = p0 + lane; p < p1; p += 32) acc += vals[src[p]];
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(kFull, acc, off);
    return acc;
  }

  __device__ void assemble_res(double* fo, double* qo) {
    const u16* ptr = sec(B_RES_PTR);
    const u16* src = sec(B_RES_SRC);
    for (int i = tid(); i < A.S; i += GT) {
      const int p0 = ptr[i], p1 = ptr[i + 1];
      if (p1 - p0 > 32) continue;  // long rows: below
      if (fo) {
        double acc = 0.0;
        for (int p = p0; p < p1; ++p) acc += cf[src[p]];
        fo[i] = acc;
      }
      if (qo) {
        double acc = 0.0;
        for (int p = p0; p < p1; ++p) acc += cq[src[p]];
        qo[i] = acc;
      }
    }
    const u16* longs = sec(B_LONG_RES);
    const int n_long = A.bo.off[B_LONG_RES + 1] - A.bo.off[B_LONG_RES];
    const int lane = threadIdx.x & 31, warp = wid();
    for (int li = warp; li < n_long; li += GW) {
      const int i = longs[li];
      const int p0 = ptr[i], p1 = ptr[i + 1];
      if (fo) {
        const double v = warp_list_sum<double>(cf, src, p0, p1);
        if (lane == 0) fo[i] = v;
      }
      if (qo) {
        const double v = warp_list_sum<double>(cq, src, p0, p1);
        if (lane == 0) qo[i] = v;
      }
    }
  }

  // The Jacobian contributions alone (the chosen form's second pass): EKV
  // devices from FP32 intermediates, the other kinds from their ordinary
  // evaluation with the value outputs switched off.
  __device__ void eval_jac(const double* zz, double t, double cfc, double cqc) {
    const GroupTable& gt = A.gt;
    const u16* nodes = sec(B_NODES);
    for (int flat = tid(); flat < gt.n_dev; flat += GT) {
      int gi = 0;
      while (gi + 1 < gt.n_groups && gt.g[gi + 1].dev_base <= flat) ++gi;
      const GroupDev& g = gt.g[gi];
      const int d = flat - (int)g.dev_base;
      const u16* nd = nodes + A.bo.node_off[gi] + d * g.T;
      double u[kFusedMaxM];
#pragma unroll
      for (int i = 0; i < kFusedMaxM; ++i) {
        if (i < g.T) {
          const u16 node = nd[i];
          u[i] = node != 0xFFFF ? zz[node] : 0.0;
        } else if (i < g.m) {
          u[i] = zz[g.int_offset + d * g.K + (i - g.T)];
        } else {
          u[i] = 0.0;
        }
      }
      if constexpr (sizeof(T) == sizeof(float)) {
        if (g.kind == VXG_KIND_EKV) {
          ekv_jac_f32(g, b, d, u, cfc, cqc, cj + g.jac_base);
          continue;
        }
      }
      eval_soa<T>(g, b, d, u, t, cfc, cqc, false, false, true, nullptr, nullptr,
                  cj + g.jac_base, zz);
    }
  }

  // Residual rows f (and q), the captured q(z_prev) and rhs = -r. On the
  // first iteration of a time step the state is still z_prev, so q(z_prev)
  // is taken from this evaluation instead of a separate one.
  __device__ void assemble_residual(int mode, double gmin, double h, bool first) {
    assemble_res(f, mode == VXG_MODE_DC ? nullptr : q);
    sync();
    for (int i = tid(); i < A.S; i += GT) {
      if (first && mode != VXG_MODE_DC) qp[i] = q[i];
      const double gm = i < A.nv ? gmin * z[i] : 0.0;
      double r;
      if (mode == VXG_MODE_DC)
        r = f[i] + gm;
      else if (mode == VXG_MODE_BE)
        r = (q[i] - qp[i]) / h + f[i] + gm;
      else
        r = (q[i] - qp[i]) / h + 0.5 * (f[i] + fp[i]) + gm;
      rhs[i] = -r;
    }
    sync();
  }

  // CSR values (+gmin) and the panels. Jacobian values in the panel type:
  // FP64 in the plain form; FP32 in the chosen form, where they feed the
  // FP32 factorization and the FP64 refinement residual rhs - J dz
  // (accumulated in FP64).
  __device__ void assemble_jacobian(double gmin) {
    const u16* jptr = sec(B_JAC_PTR);
    const u16* jsrc = sec(B_JAC_SRC);
    const u16* rows = sec(B_ROWS);
    const u16* cols = sec(B_INDICES);
    for (int e = tid(); e < A.nnz; e += GT) {
      const int p0 = jptr[e], p1 = jptr[e + 1];
      if (p1 - p0 > 32) continue;  // long entries: below
      T acc = T(0);
      for (int p = p0; p < p1; ++p) acc += cj[jsrc[p]];
      const int r = rows[e];
      if (r < A.nv && cols[e] == r) acc += (T)gmin;
      data[e] = acc;
    }
    {
      const u16* longs = sec(B_LONG_JAC);
      const int n_long = A.bo.off[B_LONG_JAC + 1] - A.bo.off[B_LONG_JAC];
      const int lane = threadIdx.x & 31, warp = wid();
      for (int li = warp; li < n_long; li += GW) {
        const int e = longs[li];
        T acc = warp_list_sum<T>(cj, jsrc, jptr[e], jptr[e + 1]);
        const int r = rows[e];
        if (r < A.nv && cols[e] == r) acc += (T)gmin;
        if (lane == 0) data[e] = acc;
      }
    }
    sync();
    // the panels overlay the contributions consumed above
    for (int i = tid(); i < A.work; i += GT) work[i] = T(0);
    sync();
    const u16* apos = sec(B_APOS);
    for (int e = tid(); e < A.nnz; e += GT) work[apos[e]] = data[e];
    sync();
  }

  __device__ void factor() {
    constexpr int NW = GW;
    const int warp = wid();
    T* colb = sbuf + warp * 64;
    T* rowb = colb + 32;
    int* perm = ibuf + warp * 32;
    const u16 *lv_ptr = sec(B_LV_PTR), *lv_sn = sec(B_LV_SN);
    const u16 *sch_off = sec(B_LV_SCHUR_OFF), *sn_k = sec(B_SN_K), *sn_r = sec(B_SN_R);
    const u16 *sn_panel = sec(B_SN_PANEL), *st_lv = sec(B_LV_ST_PTR);
    for (int L = 0; L < A.n_levels; ++L) {
      const int lo = lv_ptr[L], hi = lv_ptr[L + 1];
      const int mode = level_mode(L);
      if (mode == LV_TINY) {
        for (int p = lo + tid(); p < hi; p += GT) {
          const int j = lv_sn[p];
          tiny_factor<T>(work + sn_panel[j], sn_k[j], sn_r[j], scr + sch_off[p]);
        }
      } else if (mode == LV_WARP) {
        for (int p = lo + warp; p < hi; p += NW) {
          const int j = lv_sn[p];
          sn_factor<T, false, NT, 1>(work + sn_panel[j], sn_k[j], sn_r[j], scr + sch_off[p], colb,
                                  rowb, perm);
        }
      } else if constexpr (!kWarp) {
        for (int p = lo; p < hi; ++p) {
          const int j = lv_sn[p];
          if (sn_k[j] <= 32)
            sn_factor<T, true, NT, 1>(work + sn_panel[j], sn_k[j], sn_r[j], scr + sch_off[p],
                                      sbuf, sbuf + kCtaK, ibuf);
          else
            sn_factor<T, true, NT, kCtaK / 32>(work + sn_panel[j], sn_k[j], sn_r[j],
                                               scr + sch_off[p], sbuf, sbuf + kCtaK, ibuf);
        }
      }
      sync();
      if (A.first_global > B_ST_TGT)  // tables in shared memory
        apply_schur(st_lv[L], st_lv[L + 1], sec(B_ST_TGT), sec(B_ST_PTR), sec(B_ST_SRC));
      else
        apply_schur(st_lv[L], st_lv[L + 1], A.blob + A.bo.off[B_ST_TGT],
                    A.blob + A.bo.off[B_ST_PTR], A.blob + A.bo.off[B_ST_SRC]);
      sync();
    }
  }

  // in-place solve of xt
  __device__ void solve_t() {
    const int lane = threadIdx.x & 31, warp = wid();
    const u16 *lv_ptr = sec(B_LV_PTR), *lv_sn = sec(B_LV_SN);
    const u16 *bord_off = sec(B_LV_BORD_OFF), *sn_k = sec(B_SN_K), *sn_r = sec(B_SN_R);
    const u16 *sn_panel = sec(B_SN_PANEL), *piv_ptr = sec(B_SN_PIV_PTR), *pivs = sec(B_SN_PIV);
    const u16 *bord_ptr = sec(B_SN_BORD_PTR), *bords = sec(B_SN_BORD);
    const u16 *bt_lv = sec(B_LV_BT_PTR), *bt_tgt = sec(B_BT_TGT), *bt_ptr = sec(B_BT_PTR);
    const u16* bt_src = sec(B_BT_SRC);
    for (int L = 0; L < A.n_levels; ++L) {
      const int lo = lv_ptr[L], hi = lv_ptr[L + 1];
      if (level_mode(L) == LV_TINY) {
        for (int p = lo + tid(); p < hi; p += GT) {
          const int j = lv_sn[p];
          const int k = sn_k[j], r = sn_r[j];
          const T* W = work + sn_panel[j];
          const T* Lb = W + k * k + k * r;
          const u16* piv = pivs + piv_ptr[j];
          T* cb = scr + bord_off[p];
          T y[kTiny];
#pragma unroll
          for (int l = 0; l < kTiny; ++l) y[l] = l < k ? xt[piv[l]] : T(0);
          for (int a = 0; a < r; ++a) {
            T c = T(0);
#pragma unroll
            for (int l = 0; l < kTiny; ++l)
              if (l < k) c += Lb[a * k + l] * y[l];
            cb[a] = c;
          }
#pragma unroll
          for (int i = 0; i < kTiny; ++i) {
            if (i >= k) break;
            T acc = T(0);
#pragma unroll
            for (int l = 0; l < kTiny; ++l)
              if (l < k) acc += W[i * k + l] * y[l];
            xt[piv[i]] = acc;
          }
        }
      } else if (sec(B_LV_KMAX)[L] > 32) {  // wide supernodes: the whole CTA on each
        for (int p = lo; p < hi; ++p) {
          const int j = lv_sn[p];
          const int k = sn_k[j], r = sn_r[j];
          const T* W = work + sn_panel[j];
          const T* Lb = W + k * k + k * r;
          const u16* piv = pivs + piv_ptr[j];
          T* cb = scr + bord_off[p];
          T* y = sbuf;
          for (int l = tid(); l < k; l += GT) y[l] = xt[piv[l]];
          sync();
          for (int i = tid(); i < k + r; i += GT) {
            T acc = T(0);
            if (i < k) {
              for (int l = 0; l < k; ++l) acc += W[i * k + l] * y[l];
              xt[piv[i]] = acc;
            } else {
              for (int l = 0; l < k; ++l) acc += Lb[(i - k) * k + l] * y[l];
              cb[i - k] = acc;
            }
          }
          sync();
        }
      } else {
        for (int p = lo + warp; p < hi; p += GW) {
          const int j = lv_sn[p];
          const int k = sn_k[j], r = sn_r[j];
          const T* W = work + sn_panel[j];
          const T* Lb = W + k * k + k * r;
          const u16* piv = pivs + piv_ptr[j];
          const T y = lane < k ? xt[piv[lane]] : T(0);
          T acc = T(0);
          T* cb = scr + bord_off[p];
          for (int l = 0; l < k; ++l) {
            const T yl = __shfl_sync(kFull, y, l);
            if (lane < k) acc += W[lane * k + l] * yl;
          }
          for (int a0 = 0; a0 < r; a0 += 32) {
            const int a = a0 + lane;
            T c = T(0);
            for (int l = 0; l < k; ++l) {
              const T yl = __shfl_sync(kFull, y, l);
              if (a < r) c += Lb[a * k + l] * yl;
            }
            if (a < r) cb[a] = c;
          }
          if (lane < k) xt[piv[lane]] = acc;
        }
      }
      sync();
      for (int t = bt_lv[L] + tid(); t < bt_lv[L + 1]; t += GT) {
        T acc = T(0);
        const int p1 = bt_ptr[t + 1];
        for (int p = bt_ptr[t]; p < p1; ++p) acc += scr[bt_src[p]];
        xt[bt_tgt[t]] -= acc;
      }
      sync();
    }
    for (int L = A.n_levels - 1; L >= 0; --L) {
      const int lo = lv_ptr[L], hi = lv_ptr[L + 1];
      if (level_mode(L) == LV_TINY) {
        for (int p = lo + tid(); p < hi; p += GT) {
          const int j = lv_sn[p];
          const int k = sn_k[j], r = sn_r[j];
          const T* Ub = work + sn_panel[j] + k * k;
          const u16* piv = pivs + piv_ptr[j];
          const u16* brd = bords + bord_ptr[j];
          for (int i = 0; i < k; ++i) {
            T acc = T(0);
            for (int a = 0; a < r; ++a) acc += Ub[i * r + a] * xt[brd[a]];
            xt[piv[i]] -= acc;
          }
        }
      } else if (sec(B_LV_KMAX)[L] > 32) {
        for (int p = lo; p < hi; ++p) {
          const int j = lv_sn[p];
          const int k = sn_k[j], r = sn_r[j];
          if (r == 0) continue;
          const T* Ub = work + sn_panel[j] + k * k;
          const u16* piv = pivs + piv_ptr[j];
          const u16* brd = bords + bord_ptr[j];
          for (int i = tid(); i < k; i += GT) {
            T acc = T(0);
            for (int a = 0; a < r; ++a) acc += Ub[i * r + a] * xt[brd[a]];
            xt[piv[i]] -= acc;
          }
        }
      } else {
        for (int p = lo + warp; p < hi; p += GW) {
          const int j = lv_sn[p];
          const int k = sn_k[j], r = sn_r[j];
          if (r == 0) continue;
          const T* Ub = work + sn_panel[j] + k * k;
          const u16* piv = pivs + piv_ptr[j];
          const u16* brd = bords + bord_ptr[j];
          if (lane < k) {
            T acc = T(0);
            for (int a = 0; a < r; ++a) acc += Ub[lane * r + a] * xt[brd[a]];
            xt[piv[lane]] -= acc;
          }
        }
      }
      sync();
    }
  }

  // dz = J^-1 rhs with FP64 refinement
  __device__ void solve(int refine) {
    for (int i = tid(); i < A.S; i += GT) xt[i] = (T)rhs[i];
    sync();
    solve_t();
    for (int i = tid(); i < A.S; i += GT) dz[i] = (double)xt[i];
    sync();
    const u16* indptr = sec(B_INDPTR);
    const u16* cols = sec(B_INDICES);
    const u16* longs = sec(B_LONG_ROW);
    const int n_long = A.bo.off[B_LONG_ROW + 1] - A.bo.off[B_LONG_ROW];
    const int lane = threadIdx.x & 31, warp = wid();
    for (int it = 0; it < refine; ++it) {
      for (int i = tid(); i < A.S; i += GT) {
        const int e0 = indptr[i], e1 = indptr[i + 1];
        if (e1 - e0 > 32) continue;  // long rows: a warp each, below
        double acc = 0.0;
        for (int e = e0; e < e1; ++e) acc += (double)data[e] * dz[cols[e]];
        xt[i] = (T)(rhs[i] - acc);
      }
      for (int li = warp; li < n_long; li += GW) {
        const int i = longs[li];
        double acc = 0.0;
        for (int e = indptr[i] + lane; e < indptr[i + 1]; e += 32)
          acc += (double)data[e] * dz[cols[e]];
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(kFull, acc, off);
        if (lane == 0) xt[i] = (T)(rhs[i] - acc);
      }
      sync();
      solve_t();
      for (int i = tid(); i < A.S; i += GT) dz[i] += (double)xt[i];
      sync();
    }
  }

  // damped update; returns converged (uniform across the group)
  __device__ int update() {
    double m = 0.0;
    int nanf = 0;
    for (int i = tid(); i < A.nv; i += GT) {
      const double v = fabs(dz[i]);
      if (isnan(v)) nanf = 1;
      else m = fmax(m, v);
    }
    int any_nan = 0;
    if constexpr (kWarp) {
      for (int off = 16; off > 0; off >>= 1) {
        m = fmax(m, __shfl_xor_sync(kFull, m, off));
        nanf |= __shfl_xor_sync(kFull, nanf, off);
      }
      any_nan = nanf;
    } else {
      m = block_max_nan<NT>(m, nanf, red, &any_nan);
    }
    const double dv_max = any_nan ? nan("") : m;
    const double qd = A.max_dv / (dv_max + 1e-300);
    const double scale = isnan(qd) ? qd : fmin(1.0, qd);
    int ok = 1;
    for (int i = tid(); i < A.S; i += GT) {
      const double d = dz[i];
      const double zn = z[i] + scale * d;
      if (!(fabs(d) <= A.atol + A.rtol * fabs(zn))) ok = 0;
      if (!isfinite(zn)) ok = 0;
      z[i] = zn;
    }
    if constexpr (kWarp)
      ok = __all_sync(kFull, ok);
    else
      ok = block_all<NT>(ok, red);
    return ok && scale == 1.0;
  }

  // DC at time t from the current state (voltax/analysis.py:236-266): the
  // direct attempt, then on failure the gmin stages restarted from `restart`.
  __device__ __forceinline__ int dc_solve(double t, const double* restart, int* iters_out) {
    const int direct = A.gmin_steps > 0 ? A.direct_steps : A.max_steps;
    int it = 0;
    int ok = newton(VXG_MODE_DC, t, 0.0, A.gmin, direct, &it);
    if (!ok && A.gmin_steps > 0) {
      for (int i = tid(); i < A.S; i += GT) z[i] = restart[i];
      sync();
      for (int s = 1; s <= A.gmin_steps; ++s) {
        int its = 0;
        ok = newton(VXG_MODE_DC, t, 0.0, A.gmins[s], A.max_steps, &its);
        it += its;
      }
    }
    *iters_out = it;
    return ok;
  }

  __device__ int newton(int mode, double t, double t_prev, double gmin, int max_steps,
                        int* iters_out) {
    const bool dc = mode == VXG_MODE_DC;
    const double cfc = mode == VXG_MODE_TRAP ? 0.5 : 1.0;
    const double cqc = dc ? 0.0 : 1.0 / (t - t_prev);
    const double h = t - t_prev;
    int done = 0, it = 0;
    long long t0 = A.phase_clk ? clock64() : 0;
    while (it < max_steps && !done) {
      if constexpr (split_eval<T>()) {  // FP64 values, then the FP32 Jacobian
        eval(z, t, cfc, cqc, true, !dc, false);
        sync();
        mark(PH_EVAL, &t0);
        assemble_residual(mode, gmin, h, it == 0);
        mark(PH_ASSEMBLE, &t0);
        eval_jac(z, t, cfc, cqc);
        sync();
        mark(PH_EVAL, &t0);
      } else {
        eval(z, t, cfc, cqc, true, !dc, true);
        sync();
        mark(PH_EVAL, &t0);
        assemble_residual(mode, gmin, h, it == 0);
      }
      assemble_jacobian(gmin);
      mark(PH_ASSEMBLE, &t0);
      factor();
      mark(PH_FACTOR, &t0);
      solve(sizeof(T) == sizeof(float) ? A.refine : 0);
      mark(PH_SOLVE, &t0);
      done = update();
      mark(PH_UPDATE, &t0);
      ++it;
    }
    *iters_out = it;
    return done;
  }
};

// Resident CTAs per SM the register allocation is sized for. FP32 with
// 128-thread CTAs: six (80 registers a thread; on the 4096-instance adder
// 2.63 M solves/s against 2.57 M with five and 2.14 M with four, the extra
// spills of the smaller budget notwithstanding). FP64, whose spills grow
// faster, and larger blocks: 640 threads per SM (five 128-thread CTAs, two
// 256-thread CTAs at 128 registers, one 512-thread CTA).
#ifndef VXG_FUSED_THREADS_PER_SM
#define VXG_FUSED_THREADS_PER_SM 640
#endif
#ifndef VXG_FUSED_CTAS_128
#define VXG_FUSED_CTAS_128 6
#endif
template <typename T, int NT>
constexpr int fused_ctas_per_sm() {
  return (NT == 128 && sizeof(T) == 4) ? VXG_FUSED_CTAS_128 : VXG_FUSED_THREADS_PER_SM / NT;
}

// Point an instance's buffers into its shared-memory region `base`.
template <typename T, int NT, bool kWarp>
__device__ __forceinline__ void bind(Instance<T, NT, kWarp>& I, unsigned char* base,
                                     const FusedLayout& L, const u16* tables) {
  I.tb = tables;
  I.z = reinterpret_cast<double*>(base + L.z);
  I.fp = reinterpret_cast<double*>(base + L.fp);
  I.qp = reinterpret_cast<double*>(base + L.qp);
  I.f = reinterpret_cast<double*>(base + L.f);
  I.q = reinterpret_cast<double*>(base + L.q);
  I.rhs = reinterpret_cast<double*>(base + L.rhs);
  I.dz = reinterpret_cast<double*>(base + L.dz);
  I.data = reinterpret_cast<T*>(base + L.data);
  I.cf = reinterpret_cast<double*>(base + L.cf);
  I.cq = reinterpret_cast<double*>(base + L.cq);
  I.cj = reinterpret_cast<T*>(base + L.cj);
  I.work = reinterpret_cast<T*>(base + L.work);
  I.scr = reinterpret_cast<T*>(base + L.scr);
  I.xt = reinterpret_cast<T*>(base + L.xt);
  I.red = reinterpret_cast<double*>(base + L.red);
  I.prof = reinterpret_cast<long long*>(base + L.prof);
  I.sbuf = reinterpret_cast<T*>(base + L.sbuf);
  I.ibuf = reinterpret_cast<int*>(base + L.sbuf +
                                  sizeof(T) * inst_sbuf_values(NT / 32, kWarp));
}

// The whole analysis of instances first, first + stride, ... by one group:
// the DC operating point (direct attempt, then gmin stepping restarting from
// z0), then one Newton solve per time point.
template <typename T, int NT, bool kWarp>
__device__ __forceinline__ void run_instances(const FusedArgs& A, Instance<T, NT, kWarp>& I,
                                              int first, int stride) {
  using G = Instance<T, NT, kWarp>;
  const long long BS = (long long)A.B * A.S;
  for (int b = first; b < A.B; b += stride) {
    I.b = b;
    for (int i = G::tid(); i < A.S; i += G::GT) I.z[i] = A.z0[(long long)b * A.S + i];
    G::sync();
    // Point n is a DC solve (every point of a sweep; point 0 of a transient
    // when dc_first) or a time step; one call site each, so that the Newton
    // body is inlined at three places only.
    const bool sweep = A.sweep_vals != nullptr;
    for (int n = 0; n < A.n_t; ++n) {
      int ok = 1, it = 0;
      if (sweep || n == 0) {
        if (sweep) {
          if (G::tid() == 0) A.sweep_slot[(long long)b * A.sweep_stride] = A.sweep_vals[n];
          G::sync();  // the group's evaluations read the value after this barrier
        }
        if (sweep || A.dc_first)
          ok = I.dc_solve(sweep ? A.sweep_t : A.ts[0],
                          n == 0 ? A.z0 + (long long)b * A.S
                                 : A.z_out + (long long)(n - 1) * BS + (long long)b * A.S,
                          &it);
      } else {
        const double tp = A.ts[n - 1], t = A.ts[n];
        if (A.mode == VXG_MODE_TRAP) {  // f(z_prev, t_prev); q(z_prev) comes from iteration 0
          I.eval(I.z, tp, 1.0, 0.0, true, false, false);
          G::sync();
          I.assemble_res(I.fp, nullptr);
          G::sync();
        }
        ok = I.newton(A.mode, t, tp, A.gmin, A.max_steps, &it);
      }
      for (int i = G::tid(); i < A.S; i += G::GT)
        A.z_out[(long long)n * BS + (long long)b * A.S + i] = I.z[i];
      if (G::tid() == 0) {
        A.conv[(long long)n * A.B + b] = ok;
        A.iters[(long long)n * A.B + b] = it;
      }
    }
    G::sync();
  }
}

// Thread 0 of a group adds its phase cycles to the global counters.
template <typename T, int NT, bool kWarp>
__device__ __forceinline__ void flush_profile(const FusedArgs& A, Instance<T, NT, kWarp>& I,
                                              long long k_start) {
  if (A.phase_clk && Instance<T, NT, kWarp>::tid() == 0) {
    I.prof[PH_TOTAL] = clock64() - k_start;
    for (int p = 0; p < PH_COUNT; ++p)
      atomicAdd(reinterpret_cast<unsigned long long*>(A.phase_clk + p),
                (unsigned long long)I.prof[p]);
  }
}

// Copy the first A.staged 16-bit table elements into shared memory.
__device__ __forceinline__ void stage_tables(const FusedArgs& A, unsigned char* dst_bytes) {
  const uint4* src = reinterpret_cast<const uint4*>(A.blob);
  uint4* dst = reinterpret_cast<uint4*>(dst_bytes);
  for (int i = threadIdx.x; i < A.staged / 8; i += blockDim.x) dst[i] = src[i];
}

// One CTA per instance (grid-stride over the batch).
template <typename T, int NT>
__global__ void __launch_bounds__(NT, fused_ctas_per_sm<T, NT>())
    fused_kernel(const __grid_constant__ FusedArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const FusedLayout L =
      fused_layout<T>(A.S, A.nnz, A.n_res, A.n_jac, A.work, A.max_scr, A.staged, NT / 32);
  stage_tables(A, smem + L.blob);
  Instance<T, NT> I{A, 0};
  bind(I, smem, L, reinterpret_cast<const u16*>(smem + L.blob));
  const long long k_start = clock64();
  if (A.phase_clk && threadIdx.x < PH_COUNT) I.prof[threadIdx.x] = 0;
  __syncthreads();
  run_instances(A, I, blockIdx.x, gridDim.x);
  flush_profile(A, I, k_start);
}

// Shared-memory bytes of the warp-per-instance kernel: the staged tables
// once, then one instance region per warp.
template <typename T>
__host__ __device__ inline size_t warp_table_bytes(const FusedArgs& A) {
  return a16(sizeof(u16) * (size_t)A.staged);
}
template <typename T>
__host__ __device__ inline FusedLayout warp_instance_layout(const FusedArgs& A) {
  return fused_layout<T>(A.S, A.nnz, A.n_res, A.n_jac, A.work, A.max_scr, 0, 1, true);
}

// One warp per instance, WPC instances per CTA sharing the staged tables
// (grid-stride over the batch). No CTA barrier after the tables are staged:
// each warp runs its instances with warp barriers only, so one instance's
// latency-bound factorization overlaps other warps' device evaluation.
#ifndef VXG_FUSED_WARPS_PER_SM
#define VXG_FUSED_WARPS_PER_SM 16  // register budget: 128 per thread
#endif

template <typename T, int WPC>
__global__ void __launch_bounds__(32 * WPC, VXG_FUSED_WARPS_PER_SM / WPC)
    fused_warp_kernel(const __grid_constant__ FusedArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const size_t tab = warp_table_bytes<T>(A);
  const FusedLayout L = warp_instance_layout<T>(A);
  stage_tables(A, smem);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Instance<T, 32 * WPC, true> I{A, 0};
  bind(I, smem + tab + (size_t)w * L.total, L, reinterpret_cast<const u16*>(smem));
  const long long k_start = clock64();
  if (A.phase_clk && lane < PH_COUNT) I.prof[lane] = 0;
  __syncwarp();
  run_instances(A, I, blockIdx.x * WPC + w, gridDim.x * WPC);
  flush_profile(A, I, k_start);
}

template <typename T, int NT>
int launch_fused(const FusedArgs& a, cudaStream_t s) {
  auto kern = fused_kernel<T, NT>;
  const size_t smem = fused_layout<T>(a.S, a.nnz, a.n_res, a.n_jac, a.work, a.max_scr, a.staged,
                                      NT / 32).total;
  VXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int dev = 0, sms = 0, per_sm = 0, smem_sm = 0;
  VXG_CUDA_TRY(cudaGetDevice(&dev));
  VXG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  VXG_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  // Carve out only the shared memory the resident CTAs need; the rest of the
  // SM's unified L1/shared storage stays L1, where the topology tables (stamp
  // gathers, plan and level tables) that every CTA walks every iteration live.
  cudaFuncAttributes fa;
  VXG_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
  const int by_regs = std::max(1, 65536 / std::max(1, fa.numRegs * NT));
  const int resident = std::max(1, std::min(by_regs, (a.B + sms - 1) / sms));
  const size_t need = (smem + 1024) * (size_t)resident;
  const int pct = (int)std::min<size_t>(100, (need * 100 + smem_sm - 1) / smem_sm);
  VXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
  VXG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem));
  const int grid = std::max(1, std::min(a.B, sms * std::max(per_sm, 1)));
  kern<<<grid, NT, smem, s>>>(a);
  VXG_LAUNCHED();
  return VXG_OK;
}


// Shared memory of the warp-per-instance kernel with WPC warps per CTA.
template <typename T>
inline size_t warp_kernel_smem(const FusedArgs& a, int wpc) {
  return warp_table_bytes<T>(a) + (size_t)wpc * warp_instance_layout<T>(a).total;
}

template <typename T, int WPC>
int launch_fused_warp(const FusedArgs& a, cudaStream_t s) {
  auto kern = fused_warp_kernel<T, WPC>;
  const size_t smem = warp_kernel_smem<T>(a, WPC);
  VXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  VXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int dev = 0, sms = 0, per_sm = 0;
  VXG_CUDA_TRY(cudaGetDevice(&dev));
  VXG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  VXG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * WPC, smem));
  const int ctas = (a.B + WPC - 1) / WPC;
  const int grid = std::max(1, std::min(ctas, sms * std::max(per_sm, 1)));
  kern<<<grid, 32 * WPC, smem, s>>>(a);
  VXG_LAUNCHED();
  return VXG_OK;
}

// One translation unit per instantiation (fused_<type>_<threads>.cu and
// fused_warp_<type>.cu), so that the kernels compile in parallel.
extern template int launch_fused<float, 64>(const FusedArgs&, cudaStream_t);
extern template int launch_fused<float, 128>(const FusedArgs&, cudaStream_t);
extern template int launch_fused<float, 256>(const FusedArgs&, cudaStream_t);
extern template int launch_fused<float, 512>(const FusedArgs&, cudaStream_t);
extern template int launch_fused<double, 64>(const FusedArgs&, cudaStream_t);
extern template int launch_fused<double, 128>(const FusedArgs&, cudaStream_t);
extern template int launch_fused<double, 256>(const FusedArgs&, cudaStream_t);
extern template int launch_fused<double, 512>(const FusedArgs&, cudaStream_t);
extern template int launch_fused_warp<float, 2>(const FusedArgs&, cudaStream_t);
extern template int launch_fused_warp<float, 4>(const FusedArgs&, cudaStream_t);
extern template int launch_fused_warp<float, 8>(const FusedArgs&, cudaStream_t);
extern template int launch_fused_warp<double, 2>(const FusedArgs&, cudaStream_t);
extern template int launch_fused_warp<double, 4>(const FusedArgs&, cudaStream_t);
extern template int launch_fused_warp<double, 8>(const FusedArgs&, cudaStream_t);

}  // namespace vxg
