// Refactorization without caller-provided scratch: vxg_factor_static.
//
// vxg_factor needs a workspace for the Schur blocks of each elimination
// level, and its callers allocate it (vxg_workspace_size). Some callers
// cannot allocate device memory at the point where they refactor: code
// running inside a framework's custom-call or plugin hook that forbids
// allocation on the execution path, real-time loops that must not touch
// the allocator, or hosts whose allocator belongs to someone else (an XLA
// buffer assignment, a memory pool locked for the duration of a run).
// This entry point serves them: the Schur scratch lives in a fixed-size
// array in this library's own device memory, and the call allocates
// nothing.
//
// Limits and rules (also in include/vxg.h):
//  * the scratch is kScratchBytes (8 MiB). A call whose batch needs more
//    (batch * largest level Schur block set * element size) returns
//    VXG_ERR_TOO_LARGE before launching anything;
//  * every GPU that loads the library holds the 8 MiB until the process
//    exits;
//  * all calls share the one array per device: calls whose kernels overlap
//    on a GPU (different streams or threads) race on it and corrupt each
//    other's factors. Serialise them;
//  * the first call on a device looks up the array's device address once
//    (cudaGetSymbolAddress with that device current) and caches it with the
//    device's current context. Make that first call before any stream
//    capture. After a cudaDeviceReset (or any teardown that gives the device
//    a new primary context) the next call sees a new context and looks the
//    address up again; that call, too, must come before any capture;
//  * nothing in the scratch has to start at zero: every Schur block a level
//    writes is read back only by the same call, after it is written.

#include <cstdio>
#include <mutex>

#include "internal.cuh"

namespace vxg {

constexpr size_t kScratchBytes = size_t(8) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

static std::mutex g_scratch_mu;
static void* g_scratch_ptr[kMaxDevices];
static void* g_scratch_ctx[kMaxDevices];  // the context the address belongs to

// The current driver context (an opaque identity), through the runtime's
// driver entry point so that the library links against libcudart only.
static int current_context(void** ctx) {
  using GetCurrent = int (*)(void**);  // CUresult cuCtxGetCurrent(CUcontext*)
  static GetCurrent fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    VXG_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000,
                                                  cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) return VXG_ERR_CUDA;
    fn = reinterpret_cast<GetCurrent>(p);
  }
  *ctx = nullptr;
  return fn(ctx) == 0 ? VXG_OK : VXG_ERR_CUDA;
}

// Device address of g_static_scratch on the current device, looked up once
// per device and context.
static int static_scratch(void** out) {
  int dev = 0;
  VXG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return VXG_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  void* ctx = nullptr;
  int st = current_context(&ctx);
  if (st) return st;
  if (!g_scratch_ptr[dev] || !ctx || g_scratch_ctx[dev] != ctx) {
    void* p = nullptr;
    VXG_CUDA_TRY(cudaGetSymbolAddress(&p, g_static_scratch));  // makes the context current
    st = current_context(&ctx);
    if (st) return st;
    g_scratch_ptr[dev] = p;
    g_scratch_ctx[dev] = ctx;
  }
  *out = g_scratch_ptr[dev];
  return VXG_OK;
}

}  // namespace vxg

extern "C" int vxg_factor_static(const vxg_handle* h, int32_t batch, int32_t precision,
                                 const double* data, void* factors, void* stream) {
  using namespace vxg;
  if (!h || batch <= 0 || !data || !factors) return VXG_ERR_INVALID;
  if (precision != VXG_F64 && precision != VXG_F32) return VXG_ERR_INVALID;
  const size_t need = elem_size(precision) * (size_t)batch *
                      (size_t)(h->t.max_schur > 0 ? h->t.max_schur : 1);
  if (need > kScratchBytes) {
    std::snprintf(last_error_buffer(), 256,
                  "vxg_factor_static: scratch for %d instances needs %zu bytes, the static "
                  "array holds %zu (use vxg_factor with a workspace)",
                  batch, need, kScratchBytes);
    return VXG_ERR_TOO_LARGE;
  }
  void* scratch = nullptr;
  const int st = static_scratch(&scratch);
  if (st) return st;
  return launch_factor(h->t, batch, precision, data, factors, scratch, (cudaStream_t)stream);
}
