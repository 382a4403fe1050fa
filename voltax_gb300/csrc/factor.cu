// Supernodal block-LDU refactorization under a fixed plan.
//
// Panels: every supernode j owns F11 (k x k) | F12 (k x r) | F21 (r x k),
// row-major and unpadded. One launch per elimination level; one CTA per
// (supernode of the level, instance). A CTA keeps F11 in shared memory and
//   1. inverts it by Gauss-Jordan with partial pivoting inside the block
//      (voltax/sparse.py:543-546 uses LAPACK LU + inverse: same W up to
//      rounding), writing W over F11;
//   2. Ub = W F12 over F12 (column tiles staged in shared memory);
//   3. the Schur block S = F21 Ub into the level scratch (r x r);
//   4. Lb = F21 W over F21 (row tiles staged in shared memory).
// A second launch applies the level's Schur blocks to the ancestors' panels:
// one thread per target slot sums its sources in ascending order
// (deterministic, no atomics): work[t] -= sum(S[src]).
// (voltax/sparse.py:549-572)
//
// Wide supernodes (F11 larger than a CTA's shared memory: k above ~141 in
// FP64, ~211 in FP32, ~104 in the complex AC factorization; up to ~437 /
// ~870 / ~424) run the same kernel with F11 left in place in its panel
// (`Wide`): the Gauss-Jordan steps read and write global memory, which the
// CTA's own barriers order exactly as they order shared memory, and only the
// pivot row and column and the 32-wide (complex: 16-wide) tiles are staged
// on chip. Every arithmetic operation and its order are unchanged.

#include <type_traits>

#include "cplx.cuh"
#include "internal.cuh"
#include "tc.cuh"

namespace vxg {

// Width of the staged F12 column tiles and F21 row tiles: 32 values, 16
// for the complex (AC) factorization, whose 16-byte values would otherwise
// leave too little shared memory for wide supernodes.
__host__ __device__ constexpr int tile_width(size_t es) { return es > 8 ? 16 : 32; }

template <typename T>
__global__ void fill_panels_kernel(int B, long long nnz, const long long* __restrict__ a_pos,
                                   const double* __restrict__ data, T* __restrict__ work,
                                   long long work_stride) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * nnz) return;
  const int b = (int)(gid / nnz);
  const long long e = gid - (long long)b * nnz;
  work[(long long)b * work_stride + a_pos[e]] = (T)data[gid];
}

template <typename T>
__device__ __forceinline__ T tabs(T x) {
  return x < T(0) ? -x : x;
}

// C[a][j] = sum_l X[a*ldx + l] * Y[l*ldy + j] for a < nr, j < nc <= 32 (lane
// = column), handed to store(a, j, value). Each warp carries four rows at a
// time in independent accumulators (one Y load per four FMAs); every sum
// runs over l in ascending order.
template <typename T, int NT, typename Store>
__device__ __forceinline__ void tile_product(int nr, int nc, int k, const T* X, int ldx,
                                             const T* Y, int ldy, Store store) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane >= nc) return;
  for (int a0 = warp; a0 < nr; a0 += 4 * NW) {
    const int na = min(4, (nr - a0 + NW - 1) / NW);
    T acc[4] = {T(0), T(0), T(0), T(0)};
    for (int l = 0; l < k; ++l) {
      const T y = Y[l * ldy + lane];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q < na) acc[q] += X[(a0 + q * NW) * ldx + l] * y;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (q < na) store(a0 + q * NW, lane, acc[q]);
  }
}

// Supernodes at least this wide, with borders at least this long, take
// their Schur product S = F21 Ub (r x k times k x r) on the tensor cores in
// the FP32 form (3xTF32, tc::product_3xtf32); narrower products would be
// mostly padding of the 128 x 64 tensor-core tile.
constexpr int kTcMinK = 64, kTcMinR = 64;

template <typename T, int NT, bool Wide, bool TC = false>
__global__ void __launch_bounds__(NT)
    factor_level_kernel(const int* __restrict__ lv_sn, const long long* __restrict__ schur_off,
                        const int* __restrict__ sn_k, const int* __restrict__ sn_r,
                        const long long* __restrict__ sn_panel, T* __restrict__ work,
                        long long work_stride, T* __restrict__ scratch,
                        long long scratch_stride) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = lv_sn[blockIdx.x];
  const int b = blockIdx.y;
  const int k = sn_k[j], r = sn_r[j];
  T* F11 = work + (long long)b * work_stride + sn_panel[j];
  T* F12 = F11 + (long long)k * k;
  T* F21 = F12 + (long long)k * r;
  T* Sout = scratch + (long long)b * scratch_stride + schur_off[blockIdx.x];

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* const base = reinterpret_cast<T*>(smem_raw);
  T* A = Wide ? F11 : base;               // k*k (on chip unless wide)
  T* col = Wide ? base : base + k * k;    // k: pivot column
  T* rowb = col + k;                      // k: scaled pivot row
  constexpr int kTile = tile_width(sizeof(T));
  T* tA = rowb + k;                       // kTile*k
  T* tB = tA + kTile * k;                 // k*kTile
  int* perm = reinterpret_cast<int*>(tB + k * kTile);

  if (!Wide)
    for (int i = threadIdx.x; i < k * k; i += NT) A[i] = F11[i];
  __syncthreads();

  // ---- Gauss-Jordan inverse with partial pivoting (row swaps recorded).
  // Warp 0 picks the pivot, swaps the rows and stages the pivot column and
  // the scaled pivot row; then every warp updates its rows: two barriers
  // per pivot step.
  for (int c = 0; c < k; ++c) {
    if (warp == 0) {
      using M = decltype(pmag(T()));
      M best = M(-1);
      int bi = c;
      for (int i = c + lane; i < k; i += 32) {
        const M v = pmag(A[i * k + c]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const M ov = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      const int p = __shfl_sync(0xffffffffu, bi, 0);
      if (lane == 0) perm[c] = p;
      if (p != c)
        for (int jj = lane; jj < k; jj += 32) {
          const T tmp = A[p * k + jj];
          A[p * k + jj] = A[c * k + jj];
          A[c * k + jj] = tmp;
        }
      __syncwarp();
      const T d = A[c * k + c];
      for (int jj = lane; jj < k; jj += 32) {
        rowb[jj] = ((jj == c) ? T(1) : A[c * k + jj]) / d;
        col[jj] = (jj == c) ? T(0) : A[jj * k + c];
      }
    }
    __syncthreads();
    for (int i = warp; i < k; i += NW) {
      const T f = col[i];
      for (int jj = lane; jj < k; jj += 32) {
        if (i == c) {
          A[c * k + jj] = rowb[jj];
        } else {
          const T a = (jj == c) ? T(0) : A[i * k + jj];
          A[i * k + jj] = a - f * rowb[jj];
        }
      }
    }
    __syncthreads();
  }
  // undo the row swaps as column swaps: one thread per row, all swaps in order
  for (int i = threadIdx.x; i < k; i += NT)
    for (int c = k - 1; c >= 0; --c) {
      const int p = perm[c];
      if (p != c) {
        const T tmp = A[i * k + c];
        A[i * k + c] = A[i * k + p];
        A[i * k + p] = tmp;
      }
    }
  __syncthreads();
  if (!Wide)
    for (int i = threadIdx.x; i < k * k; i += NT) F11[i] = A[i];
  if (r == 0) return;

  // ---- Ub = W F12 (in place, column tiles)
  for (int c0 = 0; c0 < r; c0 += kTile) {
    const int tw = min(kTile, r - c0);
    for (int i = warp; i < k; i += NW)
      for (int jj = lane; jj < tw; jj += 32) tB[i * kTile + jj] = F12[(long long)i * r + c0 + jj];
    __syncthreads();
    tile_product<T, NT>(k, tw, k, A, k, tB, kTile, [&](int i, int jj, T v) {
      F12[(long long)i * r + c0 + jj] = v;
    });
    __syncthreads();
  }

  // ---- S = F21 Ub on the tensor cores (FP32 form, k >= kTcMinK): every
  // row at once, before Lb overwrites F21. A wait that gives up leaves NaN in
  // the Schur block, so the factorization reports non-finite values.
  bool schur_done = false;
  if constexpr (TC) {
    if (k >= kTcMinK && r >= kTcMinR) {
      __shared__ uint32_t tmem_slot;
      const uint32_t used = tc::smem_u32(perm + k);
      unsigned char* tcbuf = reinterpret_cast<unsigned char*>(perm + k) +
                             (((used + 1023u) & ~1023u) - used);
      tc::ProductState ps;
      tc::product_begin(ps, tcbuf, &tmem_slot);
      tc::product_3xtf32<NT>(
          ps, r, r, k, [&](int a, int l) { return (float)F21[(long long)a * k + l]; },
          [&](int l, int c) { return (float)F12[(long long)l * r + c]; },
          [&](int a, int c, float v) { Sout[(long long)a * r + c] = (T)v; });
      tc::product_end(ps);
      if (!ps.ok)
        for (long long i = threadIdx.x; i < (long long)r * r; i += NT) Sout[i] = (T)NAN;
      __syncthreads();
      schur_done = true;
    }
  }

  // ---- per row tile of F21: Schur rows S = F21 Ub, then Lb = F21 W
  for (int a0 = 0; a0 < r; a0 += kTile) {
    const int tr = min(kTile, r - a0);
    for (int a = warp; a < tr; a += NW)
      for (int l = lane; l < k; l += 32) tA[a * k + l] = F21[(long long)(a0 + a) * k + l];
    __syncthreads();
    for (int c0 = 0; c0 < r && !schur_done; c0 += kTile) {
      const int tw = min(kTile, r - c0);
      for (int i = warp; i < k; i += NW)
        for (int jj = lane; jj < tw; jj += 32)
          tB[i * kTile + jj] = F12[(long long)i * r + c0 + jj];
      __syncthreads();
      tile_product<T, NT>(tr, tw, k, tA, k, tB, kTile, [&](int a, int jj, T v) {
        Sout[(long long)(a0 + a) * r + c0 + jj] = v;
      });
      __syncthreads();
    }
    for (int j0 = 0; j0 < k; j0 += 32)
      tile_product<T, NT>(tr, min(32, k - j0), k, tA, k, A + j0, k, [&](int a, int jj, T v) {
        F21[(long long)(a0 + a) * k + j0 + jj] = v;
      });
    __syncthreads();
  }
}

template <typename T>
__global__ void schur_apply_kernel(int B, long long ntgt, const long long* __restrict__ tgt,
                                   const long long* __restrict__ ptr,
                                   const long long* __restrict__ src,
                                   const T* __restrict__ scratch, long long scratch_stride,
                                   T* __restrict__ work, long long work_stride) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * ntgt) return;
  const int b = (int)(gid / ntgt);
  const long long t = gid - (long long)b * ntgt;
  const T* S = scratch + (long long)b * scratch_stride;
  T acc = T(0);
  for (long long p = ptr[t]; p < ptr[t + 1]; ++p) acc += S[src[p]];
  work[(long long)b * work_stride + tgt[t]] -= acc;
}

size_t factor_smem_bytes(int k, size_t es, bool wide = false, bool tc = false) {
  const size_t a = wide ? 0 : (size_t)k * k;
  const size_t base =
      (a + 2 * (size_t)k + 2 * (size_t)tile_width(es) * k) * es + (size_t)k * sizeof(int) + 16;
  return tc ? base + 1024 + tc::kProductSmem : base;  // + the tensor-core tiles, 1 KB aligned
}

template <typename T, int NT, bool Wide, bool TC = false>
static int launch_level(dim3 grid, size_t smem, const Topo& t, long long lo, T* work,
                        long long ws, T* scratch, long long ss, cudaStream_t s) {
  auto kern = factor_level_kernel<T, NT, Wide, TC>;
  VXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, NT, smem, s>>>(t.lv_sn + lo, t.lv_schur_off + lo, t.sn_k, t.sn_r, t.sn_panel, work,
                              ws, scratch, ss);
  VXG_LAUNCHED();
  return VXG_OK;
}

template <typename T>
static int factor_levels(const Topo& t, int B, T* work, T* scratch, cudaStream_t s);

// CTA width of level L's factor kernel (levels whose F11 fits in shared
// memory and whose Schur product stays on the CUDA cores): the width
// vxg_tune_factor measured fastest, else the size rule.
template <typename T>
static int level_width(const Topo& t, int L) {
  if constexpr (!std::is_same<T, cplx>::value) {
    const int* tw = t.h_lv_nt[std::is_same<T, float>::value ? 1 : 0];
    if (tw && tw[L]) return tw[L];
  }
  const int kmax = t.h_lv_kmax[L];
  return kmax > 80 ? 512 : kmax > 48 ? 256 : 128;
}

template <typename T>
static int launch_width(int nt, dim3 grid, size_t smem, const Topo& t, long long lo, T* work,
                        long long ws, T* scratch, long long ss, cudaStream_t s) {
  if (nt == 512) return launch_level<T, 512, false>(grid, smem, t, lo, work, ws, scratch, ss, s);
  if (nt == 256) return launch_level<T, 256, false>(grid, smem, t, lo, work, ws, scratch, ss, s);
  return launch_level<T, 128, false>(grid, smem, t, lo, work, ws, scratch, ss, s);
}

template <typename T>
static int factor_impl(const Topo& t, int B, const double* data, T* work, T* scratch,
                       cudaStream_t s) {
  const long long ws = t.work;
  VXG_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(T) * (size_t)B * ws, s));
  const long long n = (long long)B * t.nnz;
  if (n)
    fill_panels_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(B, t.nnz, t.a_pos, data,
                                                                        work, ws);
  VXG_LAUNCHED();
  return factor_levels<T>(t, B, work, scratch, s);
}

// Panels of A = G + j omega[b] C for every frequency b (AC small-signal).
__global__ void fill_panels_ac_kernel(int B, long long nnz, const long long* __restrict__ a_pos,
                                      const double* __restrict__ G,
                                      const double* __restrict__ C,
                                      const double* __restrict__ omega, cplx* __restrict__ work,
                                      long long work_stride) {
  const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * nnz) return;
  const int b = (int)(gid / nnz);
  const long long e = gid - (long long)b * nnz;
  work[(long long)b * work_stride + a_pos[e]] = cplx(G[e], omega[b] * C[e]);
}

static int max_optin_smem() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return -1;
  return v;
}

// Level L's factor kernel, one launch: the tensor-core Schur products (FP32,
// k and r at least 64), the wide kernel (F11 left in its panel) when F11
// does not fit in shared memory, else the tuned or size-rule CTA width.
template <typename T>
static int factor_level_once(const Topo& t, int L, int B, T* work, T* scratch, int max_optin,
                             cudaStream_t s) {
  const long long ws = t.work, ss = t.max_schur;
  const long long lo = t.h_lv_ptr[L], hi = t.h_lv_ptr[L + 1];
  const int kmax = t.h_lv_kmax[L];
  const dim3 grid((unsigned)(hi - lo), (unsigned)B);
  size_t smem = factor_smem_bytes(kmax, sizeof(T));
  if constexpr (std::is_same<T, float>::value) {
    if (kmax >= kTcMinK && t.h_lv_rmax[L] >= kTcMinR) {  // Schur products on the tensor cores
      const bool wide = factor_smem_bytes(kmax, 4, false, true) > (size_t)max_optin;
      smem = factor_smem_bytes(kmax, 4, wide, true);
      if (smem > (size_t)max_optin) return VXG_ERR_TOO_LARGE;
      return wide ? launch_level<T, 512, true, true>(grid, smem, t, lo, work, ws, scratch, ss, s)
                  : launch_level<T, 512, false, true>(grid, smem, t, lo, work, ws, scratch, ss,
                                                      s);
    }
  }
  if (smem > (size_t)max_optin) {  // F11 stays in the panel
    smem = factor_smem_bytes(kmax, sizeof(T), true);
    if (smem > (size_t)max_optin) return VXG_ERR_TOO_LARGE;
    return launch_level<T, 512, true>(grid, smem, t, lo, work, ws, scratch, ss, s);
  }
  return launch_width<T>(level_width<T>(t, L), grid, smem, t, lo, work, ws, scratch, ss, s);
}

// work[t] -= sum of level L's Schur block entries aimed at t.
template <typename T>
static int apply_level_schur(const Topo& t, int L, int B, T* work, T* scratch, cudaStream_t s) {
  const long long tlo = t.h_lv_st_ptr[L], thi = t.h_lv_st_ptr[L + 1];
  const long long nt = (long long)B * (thi - tlo);
  if (nt) {
    schur_apply_kernel<T><<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(
        B, thi - tlo, t.st_tgt + tlo, t.st_ptr + tlo, t.st_src, scratch, t.max_schur, work,
        t.work);
    VXG_LAUNCHED();
  }
  return VXG_OK;
}

template <typename T>
static int factor_levels(const Topo& t, int B, T* work, T* scratch, cudaStream_t s) {
  const int max_optin = max_optin_smem();
  if (max_optin < 0) return VXG_ERR_CUDA;
  for (int L = 0; L < t.n_levels; ++L) {
    if (t.h_lv_ptr[L + 1] == t.h_lv_ptr[L]) continue;
    int st = factor_level_once<T>(t, L, B, work, scratch, max_optin, s);
    if (st == VXG_OK) st = apply_level_schur<T>(t, L, B, work, scratch, s);
    if (st != VXG_OK) return st;
  }
  return VXG_OK;
}

int launch_factor_ac(const Topo& t, int B, const double* G, const double* C,
                     const double* omega, void* factors, void* scratch, cudaStream_t s) {
  cplx* work = (cplx*)factors;
  VXG_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(cplx) * (size_t)B * t.work, s));
  const long long n = (long long)B * t.nnz;
  if (n)
    fill_panels_ac_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(B, t.nnz, t.a_pos, G, C,
                                                                      omega, work, t.work);
  VXG_LAUNCHED();
  return factor_levels<cplx>(t, B, work, (cplx*)scratch, s);
}

// Each tunable level's kernel timed at 128, 256 and 512 threads (the best of
// three launches each, CUDA events on the stream) on the panels of `data`,
// then its Schur block applied, level by level as a factorization runs.
// The repeated in-place launches leave the panels meaningless, which changes
// no launch's work: the kernels' control flow and addresses depend on the
// plan alone. widths[L] = the fastest width, or 0 for a level with a fixed
// shape (wide, or tensor-core Schur products).
template <typename T>
static int tune_levels(const Topo& t, int B, const double* data, T* work, T* scratch,
                       int* widths, cudaStream_t s) {
  const long long ws = t.work, ss = t.max_schur;
  VXG_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(T) * (size_t)B * ws, s));
  const long long n = (long long)B * t.nnz;
  if (n)
    fill_panels_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(B, t.nnz, t.a_pos, data,
                                                                        work, ws);
  VXG_LAUNCHED();
  const int max_optin = max_optin_smem();
  if (max_optin < 0) return VXG_ERR_CUDA;
  cudaEvent_t e[2] = {nullptr, nullptr};
  int st = VXG_OK;
  for (int q = 0; q < 2 && st == VXG_OK; ++q)
    if (cudaEventCreate(&e[q]) != cudaSuccess) st = VXG_ERR_CUDA;
  for (int L = 0; L < t.n_levels && st == VXG_OK; ++L) {
    widths[L] = 0;
    const long long lo = t.h_lv_ptr[L], hi = t.h_lv_ptr[L + 1];
    if (hi == lo) continue;
    const int kmax = t.h_lv_kmax[L];
    const dim3 grid((unsigned)(hi - lo), (unsigned)B);
    const size_t smem = factor_smem_bytes(kmax, sizeof(T));
    const bool tc = std::is_same<T, float>::value && kmax >= kTcMinK && t.h_lv_rmax[L] >= kTcMinR;
    if (tc || smem > (size_t)max_optin) {
      st = factor_level_once<T>(t, L, B, work, scratch, max_optin, s);
    } else {
      float best = 0.f;
      for (int nt : {128, 256, 512}) {
        float tmin = 0.f;
        for (int rep = 0; rep < 3 && st == VXG_OK; ++rep) {
          float ms = 0.f;
          if (cudaEventRecord(e[0], s) != cudaSuccess) st = VXG_ERR_CUDA;
          if (st == VXG_OK) st = launch_width<T>(nt, grid, smem, t, lo, work, ws, scratch, ss, s);
          if (st == VXG_OK && (cudaEventRecord(e[1], s) != cudaSuccess ||
                               cudaEventSynchronize(e[1]) != cudaSuccess ||
                               cudaEventElapsedTime(&ms, e[0], e[1]) != cudaSuccess))
            st = VXG_ERR_CUDA;
          if (rep == 0 || ms < tmin) tmin = ms;
        }
        if (st == VXG_OK && (widths[L] == 0 || tmin < best)) {
          best = tmin;
          widths[L] = nt;
        }
      }
    }
    if (st == VXG_OK) st = apply_level_schur<T>(t, L, B, work, scratch, s);
  }
  for (cudaEvent_t x : e)
    if (x) cudaEventDestroy(x);
  if (st == VXG_OK) VXG_CUDA_TRY(cudaStreamSynchronize(s));
  return st;
}

int tune_factor(const Topo& t, int B, int precision, const double* data, void* factors,
                void* scratch, int* widths, cudaStream_t s) {
  if (precision == VXG_F64)
    return tune_levels<double>(t, B, data, (double*)factors, (double*)scratch, widths, s);
  if (precision == VXG_F32)
    return tune_levels<float>(t, B, data, (float*)factors, (float*)scratch, widths, s);
  return VXG_ERR_INVALID;
}

int launch_factor(const Topo& t, int B, int precision, const double* data, void* factors,
                  void* scratch, cudaStream_t s) {
  if (precision == VXG_F64)
    return factor_impl<double>(t, B, data, (double*)factors, (double*)scratch, s);
  if (precision == VXG_F32)
    return factor_impl<float>(t, B, data, (float*)factors, (float*)scratch, s);
  return VXG_ERR_INVALID;
}

}  // namespace vxg
