// Fifth-generation tensor core primitives (tcgen05, sm_103a), inline PTX:
// tensor-memory allocation, the shared-memory operand and instruction
// descriptors of tcgen05.mma, MMA issue and completion through an mbarrier
// (with bounded waits), and tensor-memory loads.
//
// Operand layout used throughout (K-major, no swizzle): a tile of R rows and
// 32 reduction elements of 4 bytes is stored as 8-row x 16-byte "core
// matrices"; element (r, k) lives at byte
//     (r / 8) * kSbo + (k / 4) * kLbo + (r % 8) * 16 + (k % 4) * 4,
// kLbo = 128 (core matrices adjacent along the reduction dimension are
// contiguous) and kSbo = 1024 (one 8-row group holds the 8 core matrices of
// a 32-element slab). One tf32 MMA consumes 8 reduction elements (two core
// matrices along K), so the descriptor of step s starts 256 * s bytes in.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vxg {
namespace tc {

constexpr uint32_t kLbo = 128;
constexpr uint32_t kSbo = 1024;
constexpr int kSlab = 32;  // reduction elements staged per round

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) of a staged K-major tile.
__device__ __forceinline__ uint32_t tile_offset(int r, int k) {
  return (uint32_t)(r >> 3) * kSbo + (uint32_t)(k >> 2) * kLbo + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
}

// Shared-memory matrix descriptor of a K-major tile without swizzle.
__device__ __forceinline__ uint64_t smem_desc(const void* tile) {
  uint64_t d = (uint64_t)((smem_u32(tile) >> 4) & 0x3FFFu);
  d |= (uint64_t)((kLbo >> 4) & 0x3FFFu) << 16;  // leading (reduction) dimension
  d |= (uint64_t)((kSbo >> 4) & 0x3FFFu) << 32;  // stride (row-group) dimension
  d |= (uint64_t)1 << 46;                        // tcgen05 descriptor version
  return d;                                      // base offset 0, no swizzle
}

// Instruction descriptor of kind::tf32 with FP32 accumulation, both
// operands K-major, an M x N tile.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                           // D: FP32
         | (2u << 7)                         // A: TF32
         | (2u << 10)                        // B: TF32
         | ((uint32_t)(N >> 3) << 17)        // N / 8
         | ((uint32_t)(M >> 4) << 24);       // M / 16
}

// Round to TF32 (10 explicit mantissa bits), nearest with ties away.
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ---- tensor memory (warp-wide calls)
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// ---- ordering
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core's reads
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Wait for the phase of `parity` to complete; false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ---- MMA (one issuing thread)
// D[tmem] = (accumulate ? D : 0) + A B^T, A: M x K, B: N x K, kind::tf32.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive once on `bar` when every MMA this thread issued so far completes.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// ---- tensor memory -> registers: lane (row) of this thread, 16 columns
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace vxg

namespace vxg {
namespace tc {

// Shared memory of one product tile set: A hi/lo (128 x 32 FP32 each),
// B hi/lo (64 x 32 each), the mbarrier and the TMEM address slot.
constexpr int kTileM = 128, kTileN = 64;
constexpr size_t kProductSmem = 2 * kTileM * kSlab * 4 + 2 * kTileN * kSlab * 4 + 16;

struct ProductState {
  float *a_hi, *a_lo, *b_hi, *b_lo;
  uint64_t* bar;
  uint32_t tmem;    // 64 FP32 columns x 128 lanes
  uint32_t phase;   // parity of the mbarrier phase in progress
  int ok;           // 0 once a wait gave up
};

// Carve the product buffers out of `smem` (1024-byte aligned), allocate 64
// TMEM columns (warp 0) and initialise the mbarrier. Every thread of the
// CTA calls this, with no thread having exited.
__device__ __forceinline__ void product_begin(ProductState& s, unsigned char* smem,
                                              uint32_t* tmem_slot) {
  s.a_hi = reinterpret_cast<float*>(smem);
  s.a_lo = s.a_hi + kTileM * kSlab;
  s.b_hi = s.a_lo + kTileM * kSlab;
  s.b_lo = s.b_hi + kTileN * kSlab;
  s.bar = reinterpret_cast<uint64_t*>(s.b_lo + kTileN * kSlab);
  if (threadIdx.x < 32) {
    tmem_alloc(tmem_slot, 64);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) mbar_init(s.bar, 1);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  s.tmem = *tmem_slot;
  s.phase = 0;
  s.ok = 1;
}

// Free the TMEM columns (every thread calls; warp 0 frees). After a wait
// that gave up, first wait (bounded) once more for the MMAs still in flight.
__device__ __forceinline__ void product_end(ProductState& s, int limit = 1 << 20) {
  if (!s.ok) mbar_wait(s.bar, s.phase ^ 1u, limit);
  fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tmem_dealloc(s.tmem, 64);
}

// C = A B in FP32 from three TF32 tensor-core products per slab,
// A_hi B_hi + A_hi B_lo + A_lo B_hi (x = x_hi + x_lo, each part rounded to
// TF32), accumulated in FP32 in tensor memory: for an M x K A and a K x N B
// given by element functions la(m, k) and lb(k, n), every C element handed
// to st(m, n, value). 128 x 64 output tiles; the CTA's NT threads (a
// multiple of 128) stage the operands, thread 0 issues the MMAs, and the
// tile is read out of tensor memory by all warps. Waits on the MMAs are
// bounded (`limit` polls); after a timeout s.ok is 0, the remaining work is
// skipped and the caller must report the failure.
template <int NT, class LA, class LB, class ST>
__device__ void product_3xtf32(ProductState& s, int M, int N, int K, LA la, LB lb, ST st,
                               int limit = 1 << 20) {
  static_assert(NT % 128 == 0, "product_3xtf32 needs a multiple of 4 warps");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr uint32_t idesc = idesc_tf32(kTileM, kTileN);
  unsigned char* ah = reinterpret_cast<unsigned char*>(s.a_hi);
  unsigned char* al = reinterpret_cast<unsigned char*>(s.a_lo);
  unsigned char* bh = reinterpret_cast<unsigned char*>(s.b_hi);
  unsigned char* bl = reinterpret_cast<unsigned char*>(s.b_lo);
  for (int m0 = 0; m0 < M && s.ok; m0 += kTileM)
    for (int n0 = 0; n0 < N && s.ok; n0 += kTileN) {
      for (int k0 = 0; k0 < K && s.ok; k0 += kSlab) {
        for (int e = tid; e < kTileM * kSlab; e += NT) {
          const int r = e / kSlab, k = e - r * kSlab;
          const float x = (m0 + r < M && k0 + k < K) ? la(m0 + r, k0 + k) : 0.0f;
          const float hi = to_tf32(x);
          const uint32_t o = tile_offset(r, k);
          *reinterpret_cast<float*>(ah + o) = hi;
          *reinterpret_cast<float*>(al + o) = to_tf32(x - hi);
        }
        for (int e = tid; e < kTileN * kSlab; e += NT) {
          const int n = e % kTileN, k = e / kTileN;  // consecutive threads: consecutive n
          const float y = (n0 + n < N && k0 + k < K) ? lb(k0 + k, n0 + n) : 0.0f;
          const float hi = to_tf32(y);
          const uint32_t o = tile_offset(n, k);
          *reinterpret_cast<float*>(bh + o) = hi;
          *reinterpret_cast<float*>(bl + o) = to_tf32(y - hi);
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
          fence_after_sync();
#pragma unroll
          for (int step = 0; step < kSlab / 8; ++step) {
            const uint32_t off = 256u * step;
            const uint64_t dah = smem_desc(ah + off), dal = smem_desc(al + off);
            const uint64_t dbh = smem_desc(bh + off), dbl = smem_desc(bl + off);
            mma_tf32(s.tmem, dal, dbh, idesc, (k0 > 0 || step > 0) ? 1u : 0u);
            mma_tf32(s.tmem, dah, dbl, idesc, 1u);
            mma_tf32(s.tmem, dah, dbh, idesc, 1u);
          }
          mma_commit(s.bar);
        }
        // the MMAs read the staged slab: wait before it is overwritten
        if (!mbar_wait(s.bar, s.phase, limit)) s.ok = 0;
        s.phase ^= 1u;
        s.ok = __syncthreads_and(s.ok);
      }
      if (!s.ok) break;
      fence_after_sync();
      for (int chunk = warp >> 2; chunk < kTileN / 16; chunk += NT / 128) {
        float v[16];
        tmem_ld16(s.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 16u * chunk, v);
        const int m = m0 + 32 * (warp & 3) + lane;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int n = n0 + 16 * chunk + i;
          if (m < M && n < N) st(m, n, v[i]);
        }
      }
      fence_before_sync();
      __syncthreads();  // the next tile's first MMA overwrites the accumulator
    }
}

}  // namespace tc
}  // namespace vxg

namespace vxg {
namespace tc {

// kind::f16 with BF16 operands, FP32 accumulation, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                      // D: FP32
         | (1u << 7)                    // A: BF16
         | (1u << 10)                   // B: BF16
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Byte offset of 16-bit element (r, k) of a staged K-major tile whose slab
// holds 64 elements per row: the same core-matrix layout as tile_offset
// (8 elements per 16-byte core-matrix row).
__device__ __forceinline__ uint32_t tile_offset16(int r, int k) {
  return (uint32_t)(r >> 3) * kSbo + (uint32_t)(k >> 3) * kLbo + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k & 7) * 2u;
}

// C = A B with BF16 operands (16-bit patterns from la(m, k), lb(n, k): B is
// given N x K) accumulated in FP32 on the tensor cores: 128 x 64 output
// tiles, 64-element slabs (four K = 16 MMAs each), the same staging, waits
// and read-out as product_3xtf32, in the A-hi / B-hi buffers of `s`.
template <int NT, class LA, class LB, class ST>
__device__ void product_bf16(ProductState& s, long long M, int N, int K, LA la, LB lb, ST st,
                             int limit = 1 << 20) {
  static_assert(NT % 128 == 0, "product_bf16 needs a multiple of 4 warps");
  constexpr int kSlab16 = 64;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr uint32_t idesc = idesc_bf16(kTileM, kTileN);
  unsigned char* at = reinterpret_cast<unsigned char*>(s.a_hi);
  unsigned char* bt = reinterpret_cast<unsigned char*>(s.b_hi);
  for (long long m0 = (long long)blockIdx.x * kTileM; m0 < M && s.ok;
       m0 += (long long)gridDim.x * kTileM)
    for (int n0 = blockIdx.y * kTileN; n0 < N && s.ok; n0 += gridDim.y * kTileN) {
      for (int k0 = 0; k0 < K && s.ok; k0 += kSlab16) {
        for (int e = tid; e < kTileM * kSlab16; e += NT) {
          const int r = e / kSlab16, k = e - r * kSlab16;
          const uint16_t x = (m0 + r < M && k0 + k < K) ? la(m0 + r, k0 + k) : (uint16_t)0;
          *reinterpret_cast<uint16_t*>(at + tile_offset16(r, k)) = x;
        }
        for (int e = tid; e < kTileN * kSlab16; e += NT) {
          const int n = e / kSlab16, k = e - n * kSlab16;
          const uint16_t y = (n0 + n < N && k0 + k < K) ? lb(n0 + n, k0 + k) : (uint16_t)0;
          *reinterpret_cast<uint16_t*>(bt + tile_offset16(n, k)) = y;
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
          fence_after_sync();
#pragma unroll
          for (int step = 0; step < kSlab16 / 16; ++step) {
            const uint32_t off = 256u * step;
            mma_bf16(s.tmem, smem_desc(at + off), smem_desc(bt + off), idesc,
                     (k0 > 0 || step > 0) ? 1u : 0u);
          }
          mma_commit(s.bar);
        }
        if (!mbar_wait(s.bar, s.phase, limit)) s.ok = 0;
        s.phase ^= 1u;
        s.ok = __syncthreads_and(s.ok);
      }
      if (!s.ok) break;
      fence_after_sync();
      for (int chunk = warp >> 2; chunk < kTileN / 16; chunk += NT / 128) {
        float v[16];
        tmem_ld16(s.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 16u * chunk, v);
        const long long m = m0 + 32 * (warp & 3) + lane;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int n = n0 + 16 * chunk + i;
          if (m < M && n < N) st(m, n, v[i]);
        }
      }
      fence_before_sync();
      __syncthreads();
    }
  if (!s.ok)  // a wait gave up: every output of this CTA's tiles becomes NaN
    for (long long m0 = (long long)blockIdx.x * kTileM; m0 < M; m0 += (long long)gridDim.x * kTileM)
      for (int n0 = blockIdx.y * kTileN; n0 < N; n0 += gridDim.y * kTileN)
        for (int e = tid; e < kTileM * kTileN; e += NT) {
          const long long m = m0 + e / kTileN;
          const int n = n0 + e % kTileN;
          if (m < M && n < N) st(m, n, __int_as_float(0x7fc00000));
        }
}

}  // namespace tc
}  // namespace vxg
