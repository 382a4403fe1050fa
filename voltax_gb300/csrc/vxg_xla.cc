// XLA FFI handlers over the C ABI (libvxg_xla.so): voltax's sparse.jacobian,
// sparse.factor and sparse.solve (voltax/sparse.py:220-249, 543-595) as XLA
// custom calls on the XLA compute stream, so that a jitted vx.dc /
// vx.transient and jax.grad through spsolve's custom_vjp
// (voltax/sparse.py:598-621) and _root's filter_custom_vjp
// (voltax/analysis.py:269-288) run the GB300 kernels unchanged.
//
// Built only where jaxlib's FFI headers exist (jax.ffi.include_dir()); the
// Python side is voltax_gb300/xla.py. Each handler takes the topology
// handle (a vxg_handle* from vxg_create, as an int64 attribute), the batch
// and the numeric format as attributes, device buffers as operands and
// results, and the caller-sized workspace as a result buffer XLA allocates
// (so the handlers allocate nothing). A non-zero vxg status becomes an FFI
// error carrying vxg_last_error().
#include <cuda_runtime.h>

#include <cstdint>

#include "vxg.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status(int st) {
  if (st == VXG_OK) return ffi::Error::Success();
  return ffi::Error(st == VXG_ERR_INVALID ? ffi::ErrorCode::kInvalidArgument
                                          : ffi::ErrorCode::kInternal,
                    vxg_last_error());
}

vxg_handle* as_handle(int64_t h) { return reinterpret_cast<vxg_handle*>(h); }

// Stamping: f (B x S), q (B x S) and the CSR values (B x nnz) at state z and
// time t with Jacobian coefficients (cf, cq) and a scalar gmin; the
// parameter rows of every group are concatenated into one FP64 operand
// whose per-group offsets, row strides and batch strides are attributes.
ffi::Error EvalImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> params, ffi::Buffer<ffi::F64> z,
                    ffi::ResultBuffer<ffi::F64> f, ffi::ResultBuffer<ffi::F64> q,
                    ffi::ResultBuffer<ffi::F64> data, ffi::ResultBuffer<ffi::U8> workspace,
                    int64_t handle, int32_t batch, double t, double cf, double cq, double gmin,
                    ffi::Span<const int64_t> offsets, ffi::Span<const int64_t> row_strides,
                    ffi::Span<const int64_t> batch_strides) {
  const size_t n = offsets.size();
  if (n > VXG_MAX_GROUPS || row_strides.size() != n || batch_strides.size() != n)
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "vxg_eval: group attribute sizes");
  vxg_group_params gp[VXG_MAX_GROUPS];
  for (size_t i = 0; i < n; ++i) {
    gp[i].params = params.typed_data() + offsets[i];
    gp[i].row_stride = row_strides[i];
    gp[i].batch_stride = batch_strides[i];
  }
  return status(vxg_eval(as_handle(handle), batch, gp, z.typed_data(), t, cf, cq, nullptr, gmin,
                         f->typed_data(), q->typed_data(), data->typed_data(),
                         workspace->untyped_data(), stream));
}

// Refactorization of the CSR values into the factor buffer.
ffi::Error FactorImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> data,
                      ffi::ResultBuffer<ffi::U8> factors, ffi::ResultBuffer<ffi::U8> workspace,
                      int64_t handle, int32_t batch, int32_t precision) {
  return status(vxg_factor(as_handle(handle), batch, precision, data.typed_data(),
                           factors->untyped_data(), workspace->untyped_data(), stream));
}

// x = A^-1 b (transpose: A^-T b) with `refine` FP64 refinement sweeps of the
// FP32 form against the CSR values.
ffi::Error SolveImpl(cudaStream_t stream, ffi::Buffer<ffi::U8> factors,
                     ffi::Buffer<ffi::F64> data, ffi::Buffer<ffi::F64> b,
                     ffi::ResultBuffer<ffi::F64> x, ffi::ResultBuffer<ffi::U8> workspace,
                     int64_t handle, int32_t batch, int32_t precision, int32_t transpose,
                     int32_t refine) {
  return status(vxg_solve(as_handle(handle), batch, precision, factors.untyped_data(),
                          data.typed_data(), b.typed_data(), x->typed_data(), transpose, refine,
                          workspace->untyped_data(), stream));
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(vxg_eval_ffi, EvalImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::U8>>()
                                  .Attr<int64_t>("handle")
                                  .Attr<int32_t>("batch")
                                  .Attr<double>("t")
                                  .Attr<double>("cf")
                                  .Attr<double>("cq")
                                  .Attr<double>("gmin")
                                  .Attr<ffi::Span<const int64_t>>("offsets")
                                  .Attr<ffi::Span<const int64_t>>("row_strides")
                                  .Attr<ffi::Span<const int64_t>>("batch_strides"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(vxg_factor_ffi, FactorImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::U8>>()
                                  .Ret<ffi::Buffer<ffi::U8>>()
                                  .Attr<int64_t>("handle")
                                  .Attr<int32_t>("batch")
                                  .Attr<int32_t>("precision"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(vxg_solve_ffi, SolveImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::U8>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::U8>>()
                                  .Attr<int64_t>("handle")
                                  .Attr<int32_t>("batch")
                                  .Attr<int32_t>("precision")
                                  .Attr<int32_t>("transpose")
                                  .Attr<int32_t>("refine"));
