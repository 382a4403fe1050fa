// Internal types shared by the vxg kernels and the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vxg.h"

namespace vxg {

constexpr int kMaxM = 6;       // largest local block (transformer, CCVS: 4 + 2)
constexpr int kFusedMaxM = 4;  // largest local block the fused kernel evaluates

// One group as the kernels see it (passed by value in a GroupTable).
struct GroupDev {
  int kind, n, T, K, m, wave, n_params;
  int int_offset;
  long long dev_base;  // flattened device index of device 0
  long long res_base;  // first residual slot (n*m slots per group)
  long long jac_base;  // first Jacobian slot (n*m*m slots per group)
  const int* nodes;    // device copy, n*T
  const double* params;
  long long row_stride, batch_stride;
};

struct GroupTable {
  int n_groups;
  long long n_dev;  // devices over all groups
  GroupDev g[VXG_MAX_GROUPS];
};

// 16-bit copy of every table the fused kernel walks each Newton iteration,
// staged into shared memory once per CTA. Section k starts at off[k]
// (elements); node tables hold 0xFFFF for ground.
enum BlobSection {
  B_RES_PTR, B_RES_SRC, B_JAC_PTR, B_JAC_SRC, B_ROWS, B_INDICES, B_INDPTR, B_APOS,
  B_SN_K, B_SN_R, B_SN_PANEL, B_SN_PIV_PTR, B_SN_PIV, B_SN_BORD_PTR, B_SN_BORD,
  B_LV_PTR, B_LV_KMAX, B_LV_RMAX, B_LV_SN, B_LV_SCHUR_OFF, B_LV_BORD_OFF,
  B_LV_ST_PTR, B_LV_BT_PTR, B_BT_TGT, B_BT_PTR, B_BT_SRC,
  B_NODES, B_LONG_RES, B_LONG_JAC, B_LONG_ROW,
  B_ST_TGT, B_ST_PTR, B_ST_SRC,  // last: left in global memory when shared memory is short
  B_COUNT
};
struct Blob {
  int off[B_COUNT + 1];
  int node_off[VXG_MAX_GROUPS];
  int len;  // elements, a multiple of 8
};

// Device-resident copy of a topology + plan.
struct Topo {
  int S, nv;
  long long nnz;
  long long *indptr, *tptr, *tent, *diag;
  int *indices, *rows;
  int n_groups;
  vxg_group_desc groups[VXG_MAX_GROUPS];  // host copy of the descriptors
  int* group_nodes[VXG_MAX_GROUPS];       // device node arrays
  long long n_res_slots, n_jac_slots, n_dev;
  long long *res_ptr, *res_src, *jac_ptr, *jac_src;
  int n_seg;
  int *seg_ptr, *seg_of, *seg_idx;
  int n_sn;
  int *sn_k, *sn_r, *sn_piv, *sn_bord;
  long long *sn_panel, *sn_piv_ptr, *sn_bord_ptr, *a_pos;
  long long work;
  int n_levels;
  // level tables (host copies for launch sizes, device copies for kernels)
  long long *h_lv_ptr, *h_lv_schur_len, *h_lv_bord_len, *h_lv_st_ptr, *h_lv_bt_ptr;
  int* h_lv_kmax;  // largest k per level
  int* h_lv_rmax;  // largest r per level
  int* lv_sn;
  long long *lv_schur_off, *lv_bord_off;
  long long *d_lv_ptr, *d_lv_st_ptr, *d_lv_bt_ptr;  // device copies of the level pointers
  int* d_lv_kmax;                                   // device copy of h_lv_kmax
  long long *st_tgt, *st_ptr, *st_src;
  int* bt_tgt;
  long long *bt_ptr, *bt_src;
  long long max_schur, max_bord;  // largest per-level scratch
  // CTA width of each level's factor kernel picked by vxg_tune_factor
  // (F64, F32; 0 or a null table: the size rule)
  int* h_lv_nt[2];
  int kmax, rmax;
  int max_m;  // largest local block (terminals + internals) over the groups
  // 16-bit tables of the fused kernel (null when some index does not fit)
  unsigned short* d_blob;
  Blob blob;
};

}  // namespace vxg

namespace vxg {
struct GraphCache;  // instantiated Newton-loop graphs of a handle (capi.cu)
}

struct vxg_handle {
  vxg::Topo t;
  vxg::GraphCache* graphs = nullptr;
};

namespace vxg {
void count_launch();
void count_launches(unsigned long long n);
char* last_error_buffer();
GraphCache* new_graph_cache();
void delete_graph_cache(GraphCache* c);  // this thread's vxg_last_error text (256 bytes)
// Per-level CTA widths of the factor kernels that beat the size rule, timed
// on `data` (writes `factors` and `scratch`; synchronizes `s`).
int tune_factor(const Topo& t, int B, int precision, const double* data, void* factors,
                void* scratch, int* widths, cudaStream_t s);
}

// Count one kernel launch and surface launch errors.
#define VXG_LAUNCHED()                     \
  do {                                     \
    vxg::count_launch();                   \
    VXG_CUDA_TRY(cudaGetLastError());      \
  } while (0)

#define VXG_CUDA_TRY(expr)                 \
  do {                                     \
    cudaError_t _e = (expr);               \
    if (_e != cudaSuccess) {               \
      vxg::set_error(_e);                  \
      return VXG_ERR_CUDA;                 \
    }                                      \
  } while (0)

namespace vxg {
void set_error(cudaError_t e);
GroupTable make_table(const Topo& t, const vxg_group_params* params);

// ---- launchers (kernels in stamp.cu / factor.cu / solve.cu / newton.cu)
int launch_eval(const Topo& t, const GroupTable& gt, int B, const double* z, double t_now,
                double cf, double cq, bool want_f, bool want_q, bool want_j, double* cf_buf,
                double* cq_buf, double* cj_buf, cudaStream_t s);
int launch_gather(const Topo& t, int B, const double* cf_buf, const double* cq_buf,
                  const double* cj_buf, const double* gmin, double gmin_scalar, double* f_out,
                  double* q_out, double* data_out, cudaStream_t s);
int launch_factor_ac(const Topo& t, int B, const double* G, const double* C,
                     const double* omega, void* factors, void* scratch, cudaStream_t s);
int launch_solve_ac(const Topo& t, int B, const void* factors, const double* b,
                    long long b_stride, double* x, void* scratch, cudaStream_t s);
int launch_factor(const Topo& t, int B, int precision, const double* data, void* factors,
                  void* scratch, cudaStream_t s);
int launch_solve(const Topo& t, int B, int precision, const void* factors, const double* data,
                 const double* b, double* x, int transpose, int refine, void* vec_t,
                 void* scratch, double* r64, cudaStream_t s);
int launch_spmv(const Topo& t, int B, const double* data, const double* x, double* y,
                int transpose, cudaStream_t s);

size_t elem_size(int precision);
}  // namespace vxg
