// Fused persistent Newton kernel: eligibility and the C ABI entry points
// (vxg_fused_smem, vxg_fused_run). The kernel itself is in fused.cuh.

#include "fused.cuh"

namespace vxg {

// Shared memory one instance needs with the first `staged` table elements on
// chip. All tables are staged when they fit; otherwise the Schur gather
// tables (the largest, read once per level) stay in global memory.
static int fused_eligible(const Topo& t, int precision, size_t* smem_out,
                          int* first_global = nullptr, int* staged_out = nullptr) {
  if (t.kmax > kCtaK || t.n_seg != 1 || !t.d_blob || t.max_m > kFusedMaxM)
    return VXG_ERR_TOO_LARGE;
  const int max_scr = (int)std::max(t.max_schur, t.max_bord);
  int dev = 0, max_optin = 0;
  VXG_CUDA_TRY(cudaGetDevice(&dev));
  VXG_CUDA_TRY(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int options[2][2] = {{B_COUNT, t.blob.len},
                             {B_ST_TGT, (t.blob.off[B_ST_TGT] + 7) / 8 * 8}};
  for (int o = 0; o < 2; ++o) {
    const int staged = options[o][1];
    // sized for the widest CTA; narrower CTAs need slightly less
    const size_t smem = precision == VXG_F32
                            ? fused_layout<float>(t.S, (int)t.nnz, (int)t.n_res_slots,
                                                  (int)t.n_jac_slots, (int)t.work, max_scr,
                                                  staged, kMaxWarps).total
                            : fused_layout<double>(t.S, (int)t.nnz, (int)t.n_res_slots,
                                                   (int)t.n_jac_slots, (int)t.work, max_scr,
                                                   staged, kMaxWarps).total;
    *smem_out = smem;
    if (smem <= (size_t)max_optin) {
      if (first_global) *first_global = options[o][0];
      if (staged_out) *staged_out = staged;
      return VXG_OK;
    }
  }
  return VXG_ERR_TOO_LARGE;
}

// The warp-per-instance kernel: topologies whose supernodes are at most 32
// wide. Warps per CTA (2, 4 or 8) chosen for the most resident instances per
// SM (ties: more warps, i.e. fewer copies of the staged tables); the Schur
// gather tables stay in global memory when the rest does not fit otherwise.
static int launch_warp_kernel(const Topo& t, FusedArgs& a, bool f32, cudaStream_t s) {
  if (t.kmax > 32) return VXG_ERR_TOO_LARGE;
  int dev = 0, max_optin = 0, smem_sm = 0;
  VXG_CUDA_TRY(cudaGetDevice(&dev));
  VXG_CUDA_TRY(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  VXG_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  const int options[2][2] = {{B_COUNT, t.blob.len},
                             {B_ST_TGT, (t.blob.off[B_ST_TGT] + 7) / 8 * 8}};
  int best_inst = 0, best_wpc = 0, best_opt = 0;
  for (int o = 0; o < 2 && !best_inst; ++o) {
    a.first_global = options[o][0];
    a.staged = options[o][1];
    for (int wpc : {8, 4, 2}) {
      const size_t smem = f32 ? warp_kernel_smem<float>(a, wpc) : warp_kernel_smem<double>(a, wpc);
      if (smem > (size_t)max_optin) continue;
      const int ctas = std::min<int>((int)(smem_sm / (smem + 1024)), VXG_FUSED_WARPS_PER_SM / wpc);
      if (ctas * wpc > best_inst) {
        best_inst = ctas * wpc;
        best_wpc = wpc;
        best_opt = o;
      }
    }
  }
  if (!best_inst) return VXG_ERR_TOO_LARGE;
  a.first_global = options[best_opt][0];
  a.staged = options[best_opt][1];
  switch (best_wpc) {
    case 8: return f32 ? launch_fused_warp<float, 8>(a, s) : launch_fused_warp<double, 8>(a, s);
    case 4: return f32 ? launch_fused_warp<float, 4>(a, s) : launch_fused_warp<double, 4>(a, s);
    default: return f32 ? launch_fused_warp<float, 2>(a, s) : launch_fused_warp<double, 2>(a, s);
  }
}

// Phase-timing target of this thread's vxg_fused_run calls (null: off).
static thread_local long long* t_phase_clk = nullptr;

}  // namespace vxg

using namespace vxg;

extern "C" int vxg_fused_set_profile(int64_t* cycles) {
  t_phase_clk = reinterpret_cast<long long*>(cycles);
  return VXG_OK;
}

extern "C" int vxg_fused_smem(const vxg_handle* h, int32_t precision, size_t* bytes) {
  if (!h || !bytes || (precision != VXG_F64 && precision != VXG_F32)) return VXG_ERR_INVALID;
  return fused_eligible(h->t, precision, bytes);
}

// The persistent launch of vxg_fused_run and vxg_fused_sweep: tables,
// options and the CTA width (the caller's, an autotuned choice, else wider
// CTAs when few instances or few resident CTAs per SM leave warps idle).
static int launch_args(const Topo& t, int batch, const vxg_group_params* params,
                       const vxg_newton_opts* o, FusedArgs& a, cudaStream_t s) {
  size_t smem = 0;
  int first_global = B_COUNT, staged = 0;
  int st = fused_eligible(t, o->precision, &smem, &first_global, &staged);
  if (st) return st;
  a.first_global = first_global;
  a.staged = staged;
  a.gt = make_table(t, params);
  a.S = t.S;
  a.nv = t.nv;
  a.nnz = (int)t.nnz;
  a.n_res = (int)t.n_res_slots;
  a.n_jac = (int)t.n_jac_slots;
  a.work = (int)t.work;
  a.n_levels = t.n_levels;
  a.max_scr = (int)std::max(t.max_schur, t.max_bord);
  a.res_ptr = t.res_ptr;
  a.res_src = t.res_src;
  a.jac_ptr = t.jac_ptr;
  a.jac_src = t.jac_src;
  a.a_pos = t.a_pos;
  a.indptr = t.indptr;
  a.indices = t.indices;
  a.rows = t.rows;
  a.sn_k = t.sn_k;
  a.sn_r = t.sn_r;
  a.sn_piv = t.sn_piv;
  a.sn_bord = t.sn_bord;
  a.sn_panel = t.sn_panel;
  a.sn_piv_ptr = t.sn_piv_ptr;
  a.sn_bord_ptr = t.sn_bord_ptr;
  a.lv_ptr = t.d_lv_ptr;
  a.lv_kmax = t.d_lv_kmax;
  a.lv_sn = t.lv_sn;
  a.lv_schur_off = t.lv_schur_off;
  a.lv_bord_off = t.lv_bord_off;
  a.lv_st_ptr = t.d_lv_st_ptr;
  a.st_tgt = t.st_tgt;
  a.st_ptr = t.st_ptr;
  a.st_src = t.st_src;
  a.lv_bt_ptr = t.d_lv_bt_ptr;
  a.bt_tgt = t.bt_tgt;
  a.bt_ptr = t.bt_ptr;
  a.bt_src = t.bt_src;
  a.blob = t.d_blob;
  a.bo = t.blob;
  a.B = batch;
  a.max_steps = o->max_steps;
  a.refine = o->refine;
  a.rtol = o->rtol;
  a.atol = o->atol;
  a.max_dv = o->max_dv;
  a.phase_clk = t_phase_clk;
  int dev = 0, sms = 0;
  VXG_CUDA_TRY(cudaGetDevice(&dev));
  VXG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int nt = o->block;
  if (nt == 0) {
    int smem_sm = 0;
    VXG_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                        dev));
    const int fit = (int)(smem_sm / (smem + 1024));
    nt = batch < 2 * sms ? 256 : fit <= 1 ? 512 : fit <= 2 ? 256 : 128;
  }
  const bool f32 = o->precision == VXG_F32;
  if (nt == 32) return launch_warp_kernel(t, a, f32, s);
  switch (nt) {
    case 64: return f32 ? launch_fused<float, 64>(a, s) : launch_fused<double, 64>(a, s);
    case 128: return f32 ? launch_fused<float, 128>(a, s) : launch_fused<double, 128>(a, s);
    case 256: return f32 ? launch_fused<float, 256>(a, s) : launch_fused<double, 256>(a, s);
    case 512: return f32 ? launch_fused<float, 512>(a, s) : launch_fused<double, 512>(a, s);
    default: return VXG_ERR_INVALID;
  }
}

static bool opts_ok(const vxg_newton_opts* o) {
  return o && o->max_steps >= 0 && o->refine >= 0 &&
         (o->precision == VXG_F64 || o->precision == VXG_F32);
}

extern "C" int vxg_fused_run(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                             int32_t mode, int32_t n_t, const double* ts, const double* z0,
                             int32_t dc_first, const double* gmins, int32_t gmin_steps,
                             int32_t direct_steps, double gmin, const vxg_newton_opts* o,
                             double* z_out, int32_t* converged, int32_t* iters, void* stream) {
  if (!h || batch <= 0 || !params || n_t <= 0 || !ts || !z0 || !z_out || !converged ||
      !iters || !opts_ok(o) || mode < 0 || mode > 2 || (n_t > 1 && mode == VXG_MODE_DC) ||
      (dc_first && gmin_steps > 0 && !gmins))
    return VXG_ERR_INVALID;
  FusedArgs a;
  std::memset(&a, 0, sizeof(a));
  a.mode = mode;
  a.n_t = n_t;
  a.dc_first = dc_first;
  a.gmin_steps = gmin_steps;
  a.direct_steps = direct_steps;
  a.gmin = gmin;
  a.ts = ts;
  a.gmins = gmins;
  a.z0 = z0;
  a.z_out = z_out;
  a.conv = converged;
  a.iters = iters;
  return launch_args(h->t, batch, params, o, a, (cudaStream_t)stream);
}

extern "C" int vxg_fused_sweep(const vxg_handle* h, int32_t batch,
                               const vxg_group_params* params, int32_t group, int32_t row,
                               int32_t device, int32_t n_points, const double* values, double t,
                               const double* z0, const double* gmins, int32_t gmin_steps,
                               int32_t direct_steps, double gmin, const vxg_newton_opts* o,
                               double* z_out, int32_t* converged, int32_t* iters,
                               void* stream) {
  if (!h || batch <= 0 || !params || n_points <= 0 || !values || !z0 || !z_out ||
      !converged || !iters || !opts_ok(o) || (gmin_steps > 0 && !gmins))
    return VXG_ERR_INVALID;
  const Topo& tp = h->t;
  if (group < 0 || group >= tp.n_groups || row < 0 || row >= tp.groups[group].n_params ||
      device < 0 || device >= tp.groups[group].n || !params[group].params ||
      params[group].batch_stride <= 0)
    return VXG_ERR_INVALID;
  FusedArgs a;
  std::memset(&a, 0, sizeof(a));
  a.mode = VXG_MODE_DC;
  a.n_t = n_points;
  a.dc_first = 1;
  a.gmin_steps = gmin_steps;
  a.direct_steps = direct_steps;
  a.gmin = gmin;
  a.gmins = gmins;
  a.z0 = z0;
  a.z_out = z_out;
  a.conv = converged;
  a.iters = iters;
  a.sweep_vals = values;
  a.sweep_slot = const_cast<double*>(params[group].params) + row * params[group].row_stride +
                 device;
  a.sweep_stride = params[group].batch_stride;
  a.sweep_t = t;
  return launch_args(tp, batch, params, o, a, (cudaStream_t)stream);
}
