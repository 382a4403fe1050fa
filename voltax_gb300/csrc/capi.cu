// C ABI: handle management, workspace layout and the Newton / transient
// drivers (host code). No exception crosses this boundary.

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "internal.cuh"

namespace vxg {

int launch_compose(const Topo& t, int B, int mode, double h, const double* z, const double* f,
                   const double* q, const double* fp, const double* qp, const double* gmin,
                   double gmin_scalar, double* rhs, cudaStream_t s);
int launch_newton_init(int n, const int* mask, int* active, int* converged, int* iters,
                       cudaStream_t s);
int launch_update(const Topo& t, int B, double* z, const double* dz, int* active,
                  int* converged, int* iters, double max_dv, double rtol, double atol,
                  int* n_active, cudaStream_t s);
int launch_param_vjp(const Topo& t, const GroupTable& gt, int B, const double* z, double t_now,
                     double cf, double cq, const double* lam, double* const* grads,
                     cudaStream_t s);

static thread_local char g_err[256] = "";

void set_error(cudaError_t e) {
  std::snprintf(g_err, sizeof(g_err), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
}

char* last_error_buffer() { return g_err; }

void set_error_text(const char* what) {
  std::snprintf(g_err, sizeof(g_err), "invalid topology descriptor: %s", what);
}

size_t elem_size(int precision) {
  return precision == VXG_F32 ? sizeof(float) : precision == VXG_C128 ? 2 * sizeof(double)
                                                                       : sizeof(double);
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Workspace regions for `B` instances.
struct Layout {
  size_t cf, cq, cj, f, q, fp, qp, rhs, dz, data, r64, fac, scratch, xt, active, cnt, total;
};

static Layout layout(const Topo& t, int B, int precision) {
  Layout L;
  const size_t es = elem_size(precision);
  const size_t nS = (size_t)B * t.S;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = align_up(o + bytes);
    return at;
  };
  L.cf = take(sizeof(double) * (size_t)B * t.n_res_slots);
  L.cq = take(sizeof(double) * (size_t)B * t.n_res_slots);
  L.cj = take(sizeof(double) * (size_t)B * t.n_jac_slots);
  L.f = take(sizeof(double) * nS);
  L.q = take(sizeof(double) * nS);
  L.fp = take(sizeof(double) * nS);
  L.qp = take(sizeof(double) * nS);
  L.rhs = take(sizeof(double) * nS);
  L.dz = take(sizeof(double) * nS);
  L.data = take(sizeof(double) * (size_t)B * t.nnz);
  L.r64 = take(sizeof(double) * 2 * nS);
  L.fac = take(es * (size_t)B * t.work);
  L.scratch = take(es * (size_t)B * std::max<long long>(std::max(t.max_schur, t.max_bord), 1));
  L.xt = take(es * nS);
  L.active = take(sizeof(int) * (size_t)B * t.n_seg);
  L.cnt = take(sizeof(int) * 4);
  L.total = o;
  return L;
}

template <typename P>
static P* at(void* base, size_t off) {
  return reinterpret_cast<P*>(static_cast<char*>(base) + off);
}

// Jacobian contribution slots of a group: an m x m block per device, or for
// the non-local kind a row block of m rows by all n*m group unknowns.
static long long jac_slots(int kind, long long n, long long m) {
  return kind == VXG_KIND_COUPLED_L ? n * m * n * m : n * m * m;
}

GroupTable make_table(const Topo& t, const vxg_group_params* params) {
  GroupTable gt;
  std::memset(&gt, 0, sizeof(gt));
  gt.n_groups = t.n_groups;
  long long dev = 0, res = 0, jac = 0;
  for (int i = 0; i < t.n_groups; ++i) {
    const vxg_group_desc& d = t.groups[i];
    GroupDev& g = gt.g[i];
    g.kind = d.kind;
    g.n = d.n;
    g.T = d.T;
    g.K = d.K;
    g.m = d.T + d.K;
    g.wave = d.wave;
    g.n_params = d.n_params;
    g.int_offset = d.int_offset;
    g.dev_base = dev;
    g.res_base = res;
    g.jac_base = jac;
    g.nodes = t.group_nodes[i];
    if (params) {
      g.params = params[i].params;
      g.row_stride = params[i].row_stride;
      g.batch_stride = params[i].batch_stride;
    }
    dev += d.n;
    res += (long long)d.n * g.m;
    jac += jac_slots(d.kind, d.n, g.m);
  }
  gt.n_dev = dev;
  return gt;
}

template <typename X, typename Y>
static int upload(X** dst, const Y* src, size_t n) {
  static_assert(sizeof(X) == sizeof(Y), "element size mismatch");
  *dst = nullptr;
  const size_t bytes = sizeof(X) * std::max<size_t>(n, 1);
  cudaError_t e = cudaMalloc((void**)dst, bytes);
  if (e != cudaSuccess) {
    set_error(e);
    return VXG_ERR_ALLOC;
  }
  if (n && src) {
    e = cudaMemcpy(*dst, src, sizeof(X) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      set_error(e);
      return VXG_ERR_CUDA;
    }
  } else {
    cudaMemset(*dst, 0, bytes);
  }
  return VXG_OK;
}

static void free_topo(Topo& t) {
  void* ptrs[] = {t.indptr, t.tptr, t.tent, t.diag, t.indices, t.rows, t.res_ptr, t.res_src,
                  t.jac_ptr, t.jac_src, t.seg_ptr, t.seg_of, t.seg_idx, t.sn_k, t.sn_r, t.sn_piv, t.sn_bord,
                  t.sn_panel, t.sn_piv_ptr, t.sn_bord_ptr, t.a_pos, t.lv_sn, t.lv_schur_off,
                  t.lv_bord_off, t.st_tgt, t.st_ptr, t.st_src, t.bt_tgt, t.bt_ptr, t.bt_src,
                  t.d_lv_ptr, t.d_lv_st_ptr, t.d_lv_bt_ptr, t.d_lv_kmax,
                  t.d_blob};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int i = 0; i < t.n_groups; ++i)
    if (t.group_nodes[i]) cudaFree(t.group_nodes[i]);
  delete[] t.h_lv_ptr;
  delete[] t.h_lv_schur_len;
  delete[] t.h_lv_bord_len;
  delete[] t.h_lv_st_ptr;
  delete[] t.h_lv_bt_ptr;
  delete[] t.h_lv_kmax;
  delete[] t.h_lv_rmax;
  delete[] t.h_lv_nt[0];
  delete[] t.h_lv_nt[1];
}

constexpr long long kLongSum = 32;

// Build the 16-bit table blob of the fused kernel; false if a value does not fit.
static bool build_blob(const vxg_topology_desc* d, std::vector<unsigned short>& out, Blob& b) {
  // indptr[S] = nnz is one of the blob's values: a pattern this large can
  // never fit, so skip walking (and allocating for) every table
  if (d->nnz >= 0xFFFF) return false;
  bool ok = true;
  auto push = [&](int sec, const auto* src, long long n, bool nodes = false) {
    b.off[sec] = (int)out.size();
    for (long long i = 0; i < n; ++i) {
      const long long v = (long long)src[i];
      if (nodes && v < 0) {
        out.push_back(0xFFFF);
      } else if (v < 0 || v >= 0xFFFF) {
        ok = false;
        out.push_back(0);
      } else {
        out.push_back((unsigned short)v);
      }
    }
  };
  const long long S = d->size, nnz = d->nnz, nl = d->n_levels, nsn = d->n_sn;
  push(B_RES_PTR, d->res_ptr, S + 1);
  push(B_RES_SRC, d->res_src, d->res_ptr[S]);
  push(B_JAC_PTR, d->jac_ptr, nnz + 1);
  push(B_JAC_SRC, d->jac_src, d->jac_ptr[nnz]);
  push(B_ROWS, d->rows, nnz);
  push(B_INDICES, d->indices, nnz);
  push(B_INDPTR, d->indptr, S + 1);
  push(B_APOS, d->a_pos, nnz);
  push(B_SN_K, d->sn_k, nsn);
  push(B_SN_R, d->sn_r, nsn);
  push(B_SN_PANEL, d->sn_panel, nsn);
  push(B_SN_PIV_PTR, d->sn_piv_ptr, nsn + 1);
  push(B_SN_PIV, d->sn_piv, d->sn_piv_ptr[nsn]);
  push(B_SN_BORD_PTR, d->sn_bord_ptr, nsn + 1);
  push(B_SN_BORD, d->sn_bord, d->sn_bord_ptr[nsn]);
  push(B_LV_PTR, d->lv_ptr, nl + 1);
  std::vector<int> kmax(nl, 0), rmax(nl, 0);
  for (long long L = 0; L < nl; ++L)
    for (long long q = d->lv_ptr[L]; q < d->lv_ptr[L + 1]; ++q) {
      kmax[L] = std::max(kmax[L], d->sn_k[d->lv_sn[q]]);
      rmax[L] = std::max(rmax[L], d->sn_r[d->lv_sn[q]]);
    }
  push(B_LV_KMAX, kmax.data(), nl);
  push(B_LV_RMAX, rmax.data(), nl);
  push(B_LV_SN, d->lv_sn, d->lv_ptr[nl]);
  push(B_LV_SCHUR_OFF, d->lv_schur_off, d->lv_ptr[nl]);
  push(B_LV_BORD_OFF, d->lv_bord_off, d->lv_ptr[nl]);
  const long long nst = d->lv_st_ptr[nl], nbt = d->lv_bt_ptr[nl];
  push(B_LV_ST_PTR, d->lv_st_ptr, nl + 1);
  push(B_LV_BT_PTR, d->lv_bt_ptr, nl + 1);
  push(B_BT_TGT, d->bt_tgt, nbt);
  push(B_BT_PTR, d->bt_ptr, nbt + 1);
  push(B_BT_SRC, d->bt_src, d->bt_ptr[nbt]);
  b.off[B_NODES] = (int)out.size();
  for (int g = 0; g < d->n_groups; ++g) {
    b.node_off[g] = (int)out.size() - b.off[B_NODES];
    const long long cnt = (long long)d->groups[g].n * d->groups[g].T;
    const int32_t* nd = d->groups[g].nodes;
    for (long long i = 0; i < cnt; ++i) {
      const long long v = nd[i];
      if (v < 0) out.push_back(0xFFFF);
      else if (v >= 0xFFFF) { ok = false; out.push_back(0); }
      else out.push_back((unsigned short)v);
    }
  }
  // rows / entries with more than kLongSum contributions: summed by a warp
  std::vector<long long> lr, lj;
  for (long long i = 0; i < S; ++i)
    if (d->res_ptr[i + 1] - d->res_ptr[i] > kLongSum) lr.push_back(i);
  for (long long e = 0; e < nnz; ++e)
    if (d->jac_ptr[e + 1] - d->jac_ptr[e] > kLongSum) lj.push_back(e);
  std::vector<long long> lrow;
  for (long long i = 0; i < S; ++i)
    if (d->indptr[i + 1] - d->indptr[i] > kLongSum) lrow.push_back(i);
  push(B_LONG_RES, lr.data(), (long long)lr.size());
  push(B_LONG_JAC, lj.data(), (long long)lj.size());
  push(B_LONG_ROW, lrow.data(), (long long)lrow.size());
  push(B_ST_TGT, d->st_tgt, nst);
  push(B_ST_PTR, d->st_ptr, nst + 1);
  push(B_ST_SRC, d->st_src, d->st_ptr[nst]);
  b.off[B_COUNT] = (int)out.size();
  while (out.size() % 8) out.push_back(0);  // 16-byte granules for the copy
  b.len = (int)out.size();
  return ok;
}

// Terminals, internals and parameter rows the device kernels use for each
// kind (rows of sources: by waveform).
struct KindShape {
  int T, K, rows;
};
constexpr KindShape kShapes[VXG_KIND_COUPLED_L + 1] = {
    {2, 0, 1},  {2, 0, 1},  {2, 1, -1}, {2, 0, -1}, {4, 0, 13}, {4, 0, 12},
    {2, 0, 4},  {2, 1, 2},  {4, 0, 1},  {3, 0, 10}, {4, 1, 1},  {4, 1, 1},
    {4, 2, 1},  {4, 2, 3},  {3, 1, 0},  {3, 1, 6},  {4, 0, 4},  {2, 1, 3}};
constexpr int kWaveRows[3] = {1, 4, 7};  // constant, step, pulse

// Every index the kernels dereference lies inside its buffer: checked once
// on the host, so that a malformed descriptor is an error status, never an
// out-of-bounds access on the device. Returns the first violation, or null.
const char* validate(const vxg_topology_desc* d) {
  const long long S = d->size, nnz = d->nnz;
  if (S <= 0 || d->n_nodes < 0 || d->n_nodes > S || nnz < S) return "size, n_nodes or nnz";
  if (d->n_groups < 0 || d->n_groups > VXG_MAX_GROUPS || (d->n_groups && !d->groups))
    return "n_groups";
  if (d->n_seg <= 0 || d->n_sn <= 0 || d->n_levels <= 0 || d->work <= 0)
    return "n_seg, n_sn, n_levels or work";
  const void* req[] = {d->indptr, d->indices, d->rows, d->tptr, d->tent, d->diag, d->res_ptr,
                       d->jac_ptr, d->seg_ptr, d->seg_of, d->sn_k, d->sn_r, d->sn_panel,
                       d->sn_piv_ptr, d->sn_piv, d->sn_bord_ptr, d->a_pos, d->lv_ptr, d->lv_sn,
                       d->lv_schur_off, d->lv_bord_off, d->lv_schur_len, d->lv_bord_len,
                       d->lv_st_ptr, d->st_ptr, d->lv_bt_ptr, d->bt_ptr};
  for (const void* p : req)
    if (!p) return "a required array is NULL";
  auto is_ptr = [](const int64_t* p, long long n, long long total) {  // CSR offsets
    if (p[0] != 0 || p[n] != total) return false;
    for (long long i = 0; i < n; ++i)
      if (p[i + 1] < p[i]) return false;
    return true;
  };
  // pattern
  if (!is_ptr(d->indptr, S, nnz) || !is_ptr(d->tptr, S, nnz)) return "indptr or tptr";
  for (long long i = 0; i < S; ++i)
    for (long long e = d->indptr[i]; e < d->indptr[i + 1]; ++e)
      if (d->rows[e] != i || d->indices[e] < 0 || d->indices[e] >= S) return "indices or rows";
  for (long long e = 0; e < nnz; ++e)
    if (d->tent[e] < 0 || d->tent[e] >= nnz) return "tent";
  for (long long i = 0; i < S; ++i) {
    const long long e = d->diag[i];
    if (e < 0 || e >= nnz || d->rows[e] != i || d->indices[e] != i) return "diag";
  }
  // groups and stamping gathers
  long long res = 0, jac = 0;
  for (int i = 0; i < d->n_groups; ++i) {
    const vxg_group_desc& g = d->groups[i];
    if (g.kind < VXG_KIND_CONDUCTANCE || g.kind > VXG_KIND_COUPLED_L || g.n < 0)
      return "group kind or size";
    const KindShape sh = kShapes[g.kind];
    int rows = sh.rows;
    if (rows < 0) {
      if (g.wave < VXG_WAVE_CONSTANT || g.wave > VXG_WAVE_PULSE) return "source waveform";
      rows = kWaveRows[g.wave];
    }
    if (g.T != sh.T || g.K != sh.K) return "group terminals or internals for its kind";
    if (g.n_params < rows || g.n_params > VXG_MAX_PARAM_ROWS) return "group parameter rows";
    if (g.n && g.T && !g.nodes) return "group nodes";
    for (long long q = 0; q < (long long)g.n * g.T; ++q)
      if (g.nodes[q] < -1 || g.nodes[q] >= d->n_nodes) return "group node index";
    if (g.K && (g.int_offset < d->n_nodes || g.int_offset + (long long)g.n * g.K > S))
      return "group internal offset";
    const long long m = g.T + g.K;
    res += g.n * m;
    jac += jac_slots(g.kind, g.n, m);
  }
  if (res != d->n_res_slots || jac != d->n_jac_slots) return "n_res_slots or n_jac_slots";
  if (!is_ptr(d->res_ptr, S, d->res_ptr[S]) || !is_ptr(d->jac_ptr, nnz, d->jac_ptr[nnz]))
    return "res_ptr or jac_ptr";
  if ((d->res_ptr[S] && !d->res_src) || (d->jac_ptr[nnz] && !d->jac_src)) return "res_src or jac_src";
  for (long long q = 0; q < d->res_ptr[S]; ++q)
    if (d->res_src[q] < 0 || d->res_src[q] >= res) return "res_src";
  for (long long q = 0; q < d->jac_ptr[nnz]; ++q)
    if (d->jac_src[q] < 0 || d->jac_src[q] >= jac) return "jac_src";
  // segments
  {
    const int32_t* sp = d->seg_ptr;
    if (sp[0] != 0 || sp[d->n_seg] != S) return "seg_ptr";
    for (int s = 0; s < d->n_seg; ++s) {
      if (sp[s + 1] < sp[s]) return "seg_ptr";
      for (long long q = sp[s]; q < sp[s + 1]; ++q) {
        const long long u = d->seg_idx ? d->seg_idx[q] : q;
        if (u < 0 || u >= S || d->seg_of[u] != s) return "seg_idx or seg_of";
      }
    }
  }
  // supernodes and panels
  const long long nsn = d->n_sn;
  long long piv = 0, bord = 0;
  for (long long j = 0; j < nsn; ++j) {
    const long long k = d->sn_k[j], r = d->sn_r[j];
    if (k < 1 || r < 0 || d->sn_piv_ptr[j] != piv || d->sn_bord_ptr[j] != bord)
      return "sn_k, sn_r or their offsets";
    piv += k;
    bord += r;
    if (d->sn_panel[j] < 0 || d->sn_panel[j] + k * k + 2 * k * r > d->work) return "sn_panel";
  }
  if (piv != S || d->sn_piv_ptr[nsn] != S || d->sn_bord_ptr[nsn] != bord) return "sn_piv_ptr";
  if (bord && !d->sn_bord) return "sn_bord";
  for (long long q = 0; q < S; ++q)
    if (d->sn_piv[q] < 0 || d->sn_piv[q] >= S) return "sn_piv";
  for (long long q = 0; q < bord; ++q)
    if (d->sn_bord[q] < 0 || d->sn_bord[q] >= S) return "sn_bord";
  for (long long e = 0; e < nnz; ++e)
    if (d->a_pos[e] < 0 || d->a_pos[e] >= d->work) return "a_pos";
  // levels and their gathers
  const long long nl = d->n_levels;
  if (!is_ptr(d->lv_ptr, nl, nsn)) return "lv_ptr";
  const long long nst = d->lv_st_ptr[nl], nbt = d->lv_bt_ptr[nl];
  if (!is_ptr(d->lv_st_ptr, nl, nst) || !is_ptr(d->lv_bt_ptr, nl, nbt)) return "lv_st_ptr or lv_bt_ptr";
  if (!is_ptr(d->st_ptr, nst, d->st_ptr[nst]) || !is_ptr(d->bt_ptr, nbt, d->bt_ptr[nbt]))
    return "st_ptr or bt_ptr";
  if ((nst && (!d->st_tgt || !d->st_src)) || (nbt && (!d->bt_tgt || !d->bt_src)))
    return "st_tgt, st_src, bt_tgt or bt_src";
  for (long long L = 0; L < nl; ++L) {
    const long long slen = d->lv_schur_len[L], blen = d->lv_bord_len[L];
    if (slen < 0 || blen < 0) return "lv_schur_len or lv_bord_len";
    for (long long q = d->lv_ptr[L]; q < d->lv_ptr[L + 1]; ++q) {
      const long long j = d->lv_sn[q];
      if (j < 0 || j >= nsn) return "lv_sn";
      const long long r = d->sn_r[j];
      if (d->lv_schur_off[q] < 0 || d->lv_schur_off[q] + r * r > slen) return "lv_schur_off";
      if (d->lv_bord_off[q] < 0 || d->lv_bord_off[q] + r > blen) return "lv_bord_off";
    }
    for (long long t = d->lv_st_ptr[L]; t < d->lv_st_ptr[L + 1]; ++t) {
      if (d->st_tgt[t] < 0 || d->st_tgt[t] >= d->work) return "st_tgt";
      for (long long p = d->st_ptr[t]; p < d->st_ptr[t + 1]; ++p)
        if (d->st_src[p] < 0 || d->st_src[p] >= slen) return "st_src";
    }
    for (long long t = d->lv_bt_ptr[L]; t < d->lv_bt_ptr[L + 1]; ++t) {
      if (d->bt_tgt[t] < 0 || d->bt_tgt[t] >= S) return "bt_tgt";
      for (long long p = d->bt_ptr[t]; p < d->bt_ptr[t + 1]; ++p)
        if (d->bt_src[p] < 0 || d->bt_src[p] >= blen) return "bt_src";
    }
  }
  return nullptr;
}

}  // namespace vxg

using namespace vxg;

extern "C" {

const char* vxg_last_error(void) { return g_err; }

int vxg_create(const vxg_topology_desc* d, vxg_handle** out) {
  if (!d || !out) return VXG_ERR_INVALID;
  if (const char* why = validate(d)) {
    set_error_text(why);
    return VXG_ERR_INVALID;
  }
  *out = nullptr;
  vxg_handle* h = new (std::nothrow) vxg_handle;
  if (!h) return VXG_ERR_ALLOC;
  std::memset(&h->t, 0, sizeof(Topo));
  Topo& t = h->t;
  t.S = d->size;
  t.nv = d->n_nodes;
  t.nnz = d->nnz;
  t.n_groups = d->n_groups;
  t.max_m = 0;
  for (int i = 0; i < d->n_groups; ++i)
    t.max_m = std::max(t.max_m, d->groups[i].T + d->groups[i].K);
  t.n_res_slots = d->n_res_slots;
  t.n_jac_slots = d->n_jac_slots;
  t.n_seg = d->n_seg;
  t.n_sn = d->n_sn;
  t.work = d->work;
  t.n_levels = d->n_levels;
  int st = VXG_OK;
#define UP(field, src, n) \
  if (st == VXG_OK) st = upload(&t.field, src, (size_t)(n))
  const long long S = d->size, nnz = d->nnz;
  UP(indptr, d->indptr, S + 1);
  UP(indices, d->indices, nnz);
  UP(rows, d->rows, nnz);
  UP(tptr, d->tptr, S + 1);
  UP(tent, d->tent, nnz);
  UP(diag, d->diag, S);
  UP(res_ptr, d->res_ptr, S + 1);
  UP(res_src, d->res_src, d->res_ptr[S]);
  UP(jac_ptr, d->jac_ptr, nnz + 1);
  UP(jac_src, d->jac_src, d->jac_ptr[nnz]);
  UP(seg_ptr, d->seg_ptr, d->n_seg + 1);
  UP(seg_of, d->seg_of, S);
  {
    std::vector<int32_t> ident;
    const int32_t* idx = d->seg_idx;
    if (!idx) {
      ident.resize((size_t)S);
      for (long long i = 0; i < S; ++i) ident[(size_t)i] = (int32_t)i;
      idx = ident.data();
    }
    UP(seg_idx, idx, S);
  }
  UP(sn_k, d->sn_k, d->n_sn);
  UP(sn_r, d->sn_r, d->n_sn);
  UP(sn_panel, d->sn_panel, d->n_sn);
  UP(sn_piv_ptr, d->sn_piv_ptr, d->n_sn + 1);
  UP(sn_piv, d->sn_piv, d->sn_piv_ptr[d->n_sn]);
  UP(sn_bord_ptr, d->sn_bord_ptr, d->n_sn + 1);
  UP(sn_bord, d->sn_bord, d->sn_bord_ptr[d->n_sn]);
  UP(a_pos, d->a_pos, nnz);
  const long long nl = d->n_levels;
  const long long n_lv_sn = d->lv_ptr[nl];
  UP(lv_sn, d->lv_sn, n_lv_sn);
  UP(lv_schur_off, d->lv_schur_off, n_lv_sn);
  UP(lv_bord_off, d->lv_bord_off, n_lv_sn);
  const long long nst = d->lv_st_ptr[nl], nbt = d->lv_bt_ptr[nl];
  UP(st_tgt, d->st_tgt, nst);
  UP(st_ptr, d->st_ptr, nst + 1);
  UP(st_src, d->st_src, d->st_ptr[nst]);
  UP(bt_tgt, d->bt_tgt, nbt);
  UP(bt_ptr, d->bt_ptr, nbt + 1);
  UP(bt_src, d->bt_src, d->bt_ptr[nbt]);
  UP(d_lv_ptr, d->lv_ptr, nl + 1);
  UP(d_lv_st_ptr, d->lv_st_ptr, nl + 1);
  UP(d_lv_bt_ptr, d->lv_bt_ptr, nl + 1);
  for (int i = 0; i < d->n_groups && st == VXG_OK; ++i) {
    t.groups[i] = d->groups[i];
    st = upload(&t.group_nodes[i], d->groups[i].nodes, (size_t)d->groups[i].n * d->groups[i].T);
  }
#undef UP
  if (st == VXG_OK) {
    t.h_lv_ptr = new long long[nl + 1];
    t.h_lv_schur_len = new long long[nl + 1];
    t.h_lv_bord_len = new long long[nl + 1];
    t.h_lv_st_ptr = new long long[nl + 1];
    t.h_lv_bt_ptr = new long long[nl + 1];
    t.h_lv_kmax = new int[nl + 1];
    t.h_lv_rmax = new int[nl + 1];
    t.max_schur = t.max_bord = 0;
    t.kmax = t.rmax = 0;
    for (long long L = 0; L <= nl; ++L) {
      t.h_lv_ptr[L] = d->lv_ptr[L];
      t.h_lv_st_ptr[L] = d->lv_st_ptr[L];
      t.h_lv_bt_ptr[L] = d->lv_bt_ptr[L];
      t.h_lv_kmax[L] = t.h_lv_rmax[L] = 0;
      if (L < nl) {
        t.h_lv_schur_len[L] = d->lv_schur_len[L];
        t.h_lv_bord_len[L] = d->lv_bord_len[L];
        t.max_schur = std::max(t.max_schur, (long long)d->lv_schur_len[L]);
        t.max_bord = std::max(t.max_bord, (long long)d->lv_bord_len[L]);
        for (long long p = d->lv_ptr[L]; p < d->lv_ptr[L + 1]; ++p) {
          const int j = d->lv_sn[p];
          t.h_lv_kmax[L] = std::max(t.h_lv_kmax[L], d->sn_k[j]);
          t.h_lv_rmax[L] = std::max(t.h_lv_rmax[L], d->sn_r[j]);
        }
        t.kmax = std::max(t.kmax, t.h_lv_kmax[L]);
        t.rmax = std::max(t.rmax, t.h_lv_rmax[L]);
      }
    }
    st = upload(&t.d_lv_kmax, t.h_lv_kmax, (size_t)nl);
  }
  if (st == VXG_OK) {
    std::vector<unsigned short> blob;
    if (build_blob(d, blob, t.blob)) st = upload(&t.d_blob, blob.data(), blob.size());
  }
  if (st == VXG_OK) h->graphs = new_graph_cache();
  if (st != VXG_OK) {
    free_topo(t);
    delete h;
    return st;
  }
  *out = h;
  return VXG_OK;
}

int vxg_destroy(vxg_handle* h) {
  if (!h) return VXG_ERR_INVALID;
  delete_graph_cache(h->graphs);
  free_topo(h->t);
  delete h;
  return VXG_OK;
}

int vxg_workspace_size(const vxg_handle* h, int32_t batch, int32_t precision, size_t* bytes) {
  if (!h || !bytes || batch <= 0 ||
      (precision != VXG_F64 && precision != VXG_F32 && precision != VXG_C128))
    return VXG_ERR_INVALID;
  *bytes = layout(h->t, batch, precision).total;
  return VXG_OK;
}

int vxg_factor_size(const vxg_handle* h, int32_t batch, int32_t precision, size_t* bytes) {
  if (!h || !bytes || batch <= 0 ||
      (precision != VXG_F64 && precision != VXG_F32 && precision != VXG_C128))
    return VXG_ERR_INVALID;
  *bytes = elem_size(precision) * (size_t)batch * h->t.work;
  return VXG_OK;
}

int vxg_ac_factor(const vxg_handle* h, int32_t n_freq, const double* G, const double* C,
                  const double* omega, void* factors, void* workspace, void* stream) {
  if (!h || n_freq <= 0 || !G || !C || !omega || !factors || !workspace) return VXG_ERR_INVALID;
  const Layout L = layout(h->t, n_freq, VXG_C128);
  return launch_factor_ac(h->t, n_freq, G, C, omega, factors, at<char>(workspace, L.scratch),
                          (cudaStream_t)stream);
}

int vxg_ac_solve(const vxg_handle* h, int32_t n_freq, const void* factors, const double* b,
                 int64_t b_stride, double* x, void* workspace, void* stream) {
  if (!h || n_freq <= 0 || !factors || !b || !x || !workspace || b_stride < 0)
    return VXG_ERR_INVALID;
  const Layout L = layout(h->t, n_freq, VXG_C128);
  return launch_solve_ac(h->t, n_freq, factors, b, b_stride, x, at<char>(workspace, L.scratch),
                         (cudaStream_t)stream);
}

int vxg_eval(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
             const double* z, double t_now, double cf, double cq, const double* gmin,
             double gmin_scalar, double* f_out, double* q_out, double* data_out,
             void* workspace, void* stream) {
  if (!h || batch <= 0 || !params || !z || !workspace) return VXG_ERR_INVALID;
  const Topo& t = h->t;
  cudaStream_t s = (cudaStream_t)stream;
  Layout L = layout(t, batch, VXG_F64);
  GroupTable gt = make_table(t, params);
  double* cfb = at<double>(workspace, L.cf);
  double* cqb = at<double>(workspace, L.cq);
  double* cjb = at<double>(workspace, L.cj);
  int st = launch_eval(t, gt, batch, z, t_now, cf, cq, f_out != nullptr, q_out != nullptr,
                       data_out != nullptr, cfb, cqb, cjb, s);
  if (st) return st;
  return launch_gather(t, batch, cfb, cqb, cjb, gmin, gmin_scalar, f_out, q_out, data_out, s);
}

int vxg_factor(const vxg_handle* h, int32_t batch, int32_t precision, const double* data,
               void* factors, void* workspace, void* stream) {
  if (!h || batch <= 0 || !data || !factors || !workspace) return VXG_ERR_INVALID;
  if (precision != VXG_F64 && precision != VXG_F32) return VXG_ERR_INVALID;
  Layout L = layout(h->t, batch, precision);
  return launch_factor(h->t, batch, precision, data, factors,
                       at<void>(workspace, L.scratch), (cudaStream_t)stream);
}

int vxg_solve(const vxg_handle* h, int32_t batch, int32_t precision, const void* factors,
              const double* data, const double* b, double* x, int32_t transpose,
              int32_t refine, void* workspace, void* stream) {
  if (!h || batch <= 0 || !factors || !b || !x || !workspace || refine < 0)
    return VXG_ERR_INVALID;
  if (precision != VXG_F64 && precision != VXG_F32) return VXG_ERR_INVALID;
  Layout L = layout(h->t, batch, precision);
  return launch_solve(h->t, batch, precision, factors, data, b, x, transpose, refine,
                      at<void>(workspace, L.xt), at<void>(workspace, L.scratch),
                      at<double>(workspace, L.r64), (cudaStream_t)stream);
}

int vxg_level_count(const vxg_handle* h, int32_t* n_levels) {
  if (!h || !n_levels) return VXG_ERR_INVALID;
  *n_levels = h->t.n_levels;
  return VXG_OK;
}

int vxg_set_factor_shapes(vxg_handle* h, int32_t precision, const int32_t* widths) {
  if (!h || (precision != VXG_F64 && precision != VXG_F32)) return VXG_ERR_INVALID;
  Topo& t = h->t;
  const int nl = t.n_levels;
  if (widths)
    for (int L = 0; L < nl; ++L)
      if (widths[L] != 0 && widths[L] != 128 && widths[L] != 256 && widths[L] != 512)
        return VXG_ERR_INVALID;
  int*& tab = t.h_lv_nt[precision == VXG_F32 ? 1 : 0];
  if (!widths) {
    delete[] tab;
    tab = nullptr;
  } else {
    if (!tab) tab = new (std::nothrow) int[nl];
    if (!tab) return VXG_ERR_ALLOC;
    for (int L = 0; L < nl; ++L) tab[L] = widths[L];
  }
  // the cached Newton graphs baked in the previous widths
  delete_graph_cache(h->graphs);
  h->graphs = new_graph_cache();
  return h->graphs ? VXG_OK : VXG_ERR_ALLOC;
}

int vxg_tune_factor(vxg_handle* h, int32_t batch, int32_t precision, const double* data,
                    void* factors, void* workspace, int32_t* widths, void* stream) {
  if (!h || batch <= 0 || !data || !factors || !workspace) return VXG_ERR_INVALID;
  if (precision != VXG_F64 && precision != VXG_F32) return VXG_ERR_INVALID;
  const Layout L = layout(h->t, batch, precision);
  std::vector<int> w((size_t)std::max(h->t.n_levels, 1), 0);
  const int st = tune_factor(h->t, batch, precision, data, factors, at<void>(workspace, L.scratch),
                             w.data(), (cudaStream_t)stream);
  if (st != VXG_OK) return st;
  if (widths)
    for (int i = 0; i < h->t.n_levels; ++i) widths[i] = w[(size_t)i];
  return vxg_set_factor_shapes(h, precision, w.data());
}

int vxg_spmv(const vxg_handle* h, int32_t batch, const double* data, const double* x,
             double* y, int32_t transpose, void* stream) {
  if (!h || batch <= 0 || !data || !x || !y) return VXG_ERR_INVALID;
  return launch_spmv(h->t, batch, data, x, y, transpose, (cudaStream_t)stream);
}

}  // extern "C"

namespace vxg {
__global__ void gdata_kernel(int B, long long nnz, int S, const int* __restrict__ rows,
                             const int* __restrict__ indices, const double* __restrict__ g,
                             const double* __restrict__ x, double* __restrict__ gd) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * nnz) return;
  const int b = (int)(gid / nnz);
  const long long e = gid - (long long)b * nnz;
  gd[gid] = -g[(long long)b * S + rows[e]] * x[(long long)b * S + indices[e]];
}

// ---------------------------------------------------------------------------
// Device-resident Newton loop (voltax/analysis.py:208-233, a lax.while_loop
// there). One Newton solve is one CUDA graph:
//   prologue   per-instance flags; for BE / TRAP, f and q at the previous
//              state; the iteration counter reset;
//   WHILE node one Newton iteration -- evaluation and stamping, residual,
//              refactorization, solve (+ refinement), damped update with the
//              count of still-active instances -- ending in a one-thread
//              kernel that counts the iteration and sets the loop condition:
//              some instance active and the limit not reached;
//   epilogue   (adjoint only) the factors of the Jacobian at the result.
// The host launches the graph on the caller's stream and returns; no host
// round trip per iteration. Counters live in the caller's workspace, so
// calls on different workspaces and streams are independent. Graphs are
// instantiated once per distinct argument set and cached on the handle.
__global__ void fill_int_kernel(int* p, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void newton_continue_kernel(cudaGraphConditionalHandle h, const int* n_active,
                                       int* iter, int max_steps) {
  const int n = ++iter[0];
  cudaGraphSetConditional(h, (n_active[0] != 0 && n < max_steps) ? 1u : 0u);
}

struct NewtonCall {
  const vxg_handle* h;
  int B;
  const vxg_group_params* params;
  int mode;
  double t_now, t_prev;
  const double* z_prev;
  const double* gmin;
  double gmin_scalar;
  const vxg_newton_opts* o;
  double* z;
  int* converged;
  int* iters;
  void* factors_out;
  void* ws;
  const int* mask;
};

struct GraphEntry {
  std::vector<unsigned char> key;
  cudaGraphExec_t exec;
  unsigned long long kernels;  // kernels of one launch, the loop body counted once
  unsigned long long used;
};

struct GraphCache {
  std::mutex mu;
  std::vector<GraphEntry> entries;
  unsigned long long tick = 0;
};

constexpr size_t kGraphCacheEntries = 16;

GraphCache* new_graph_cache() { return new (std::nothrow) GraphCache(); }

void delete_graph_cache(GraphCache* c) {
  if (!c) return;
  for (GraphEntry& e : c->entries) cudaGraphExecDestroy(e.exec);  // freed once idle
  delete c;
}

// Every argument the graph bakes in, byte by byte.
static std::vector<unsigned char> newton_key(const NewtonCall& a) {
  std::vector<unsigned char> k;
  auto put = [&](const auto& x) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&x);
    k.insert(k.end(), p, p + sizeof(x));
  };
  put(a.B);
  put(a.mode);
  put(a.t_now);
  put(a.t_prev);
  put(a.z_prev);
  put(a.gmin);
  put(a.gmin_scalar);
  put(a.o->max_steps);
  put(a.o->rtol);
  put(a.o->atol);
  put(a.o->max_dv);
  put(a.o->precision);
  put(a.o->refine);
  for (int i = 0; i < a.h->t.n_groups; ++i) {
    put(a.params[i].params);
    put(a.params[i].row_stride);
    put(a.params[i].batch_stride);
  }
  put(a.z);
  put(a.converged);
  put(a.iters);
  put(a.factors_out);
  put(a.ws);
  put(a.mask);
  return k;
}

// A private stream per thread and device to record the graphs on (the
// caller's stream may be the legacy default stream, which cannot capture).
static cudaStream_t capture_stream() {
  thread_local std::vector<std::pair<int, cudaStream_t>> streams;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  for (auto& p : streams)
    if (p.first == dev) return p.second;
  cudaStream_t cs = nullptr;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  streams.emplace_back(dev, cs);
  return cs;
}

static thread_local int t_capturing = 0;
static thread_local unsigned long long t_captured = 0;

// Record what `body` enqueues on `cs` into a new graph (*out) or into the
// existing graph `into` (a conditional node's body).
template <class F>
static int record(cudaStream_t cs, cudaGraph_t into, cudaGraph_t* out, unsigned long long* n,
                  F&& body) {
  cudaError_t e = into ? cudaStreamBeginCaptureToGraph(cs, into, nullptr, nullptr, 0,
                                                       cudaStreamCaptureModeRelaxed)
                       : cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    set_error(e);
    return VXG_ERR_CUDA;
  }
  ++t_capturing;
  t_captured = 0;
  int st = body(cs);
  --t_capturing;
  *n = t_captured;
  cudaGraph_t got = nullptr;
  e = cudaStreamEndCapture(cs, &got);
  if (st == VXG_OK && e != cudaSuccess) {
    set_error(e);
    st = VXG_ERR_CUDA;
  }
  if (st != VXG_OK) {
    if (got && !into) cudaGraphDestroy(got);
    return st;
  }
  if (out) *out = got;
  return VXG_OK;
}

static int build_newton_graph(const NewtonCall& a, cudaGraphExec_t* exec,
                              unsigned long long* kernels) {
  const Topo& t = a.h->t;
  const int B = a.B, prec = a.o->precision, mode = a.mode;
  const Layout L = layout(t, B, prec);
  const GroupTable gt = make_table(t, a.params);
  void* ws = a.ws;
  double* cfb = at<double>(ws, L.cf);
  double* cqb = at<double>(ws, L.cq);
  double* cjb = at<double>(ws, L.cj);
  double* f = at<double>(ws, L.f);
  double* q = at<double>(ws, L.q);
  double* fp = at<double>(ws, L.fp);
  double* qp = at<double>(ws, L.qp);
  double* rhs = at<double>(ws, L.rhs);
  double* dz = at<double>(ws, L.dz);
  double* data = at<double>(ws, L.data);
  void* fac = at<void>(ws, L.fac);
  void* scratch = at<void>(ws, L.scratch);
  void* xt = at<void>(ws, L.xt);
  double* r64 = at<double>(ws, L.r64);
  int* active = at<int>(ws, L.active);
  int* cnt = at<int>(ws, L.cnt);  // [0] active instances, [1] iterations done
  const bool dc = mode == VXG_MODE_DC;
  const double cf = mode == VXG_MODE_TRAP ? 0.5 : 1.0;
  const double cq = dc ? 0.0 : 1.0 / (a.t_now - a.t_prev);
  const double hstep = a.t_now - a.t_prev;
  cudaStream_t cs = capture_stream();
  if (!cs) {
    set_error(cudaErrorUnknown);
    return VXG_ERR_CUDA;
  }
  cudaGraph_t g = nullptr;
  VXG_CUDA_TRY(cudaGraphCreate(&g, 0));
  unsigned long long n_pro = 0, n_body = 0, n_epi = 0;
  cudaGraph_t pro = nullptr;
  int st = record(cs, nullptr, &pro, &n_pro, [&](cudaStream_t s) -> int {
    int r = launch_newton_init(B * t.n_seg, a.mask, active, a.converged, a.iters, s);
    if (r) return r;
    VXG_CUDA_TRY(cudaMemsetAsync(cnt + 1, 0, sizeof(int), s));
    if (dc) return VXG_OK;
    r = launch_eval(t, gt, B, a.z_prev, a.t_prev, 1.0, 0.0, mode == VXG_MODE_TRAP, true, false,
                    cfb, cqb, cjb, s);
    if (r) return r;
    return launch_gather(t, B, cfb, cqb, cjb, nullptr, 0.0,
                         mode == VXG_MODE_TRAP ? fp : nullptr, qp, nullptr, s);
  });
  cudaGraphNode_t n0 = nullptr, n1 = nullptr, n2 = nullptr;
  cudaGraphConditionalHandle hc = 0;
  union ZeroedParams {  // the struct's reserved bytes must be zero
    cudaGraphNodeParams p;
    unsigned char raw[sizeof(cudaGraphNodeParams)];
    ZeroedParams() { std::memset(raw, 0, sizeof(raw)); }
  } params_buf;
  cudaGraphNodeParams& cp = params_buf.p;
  auto cuda_ok = [&](cudaError_t e) {
    if (e == cudaSuccess) return true;
    set_error(e);
    st = VXG_ERR_CUDA;
    return false;
  };
  if (st == VXG_OK && cuda_ok(cudaGraphAddChildGraphNode(&n0, g, nullptr, 0, pro)) &&
      cuda_ok(cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault))) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = hc;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cuda_ok(cudaGraphAddNode(&n1, g, &n0, nullptr, 1, &cp));
  }
  if (pro) cudaGraphDestroy(pro);  // the child node holds a copy
  if (st == VXG_OK) {
    const int max_steps = a.o->max_steps;
    st = record(cs, cp.conditional.phGraph_out[0], nullptr, &n_body, [&](cudaStream_t s) -> int {
      int r = launch_eval(t, gt, B, a.z, a.t_now, cf, cq, true, !dc, true, cfb, cqb, cjb, s);
      if (r) return r;
      r = launch_gather(t, B, cfb, cqb, cjb, a.gmin, a.gmin_scalar, f, dc ? nullptr : q, data,
                        s);
      if (r) return r;
      r = launch_compose(t, B, mode, hstep, a.z, f, q, fp, qp, a.gmin, a.gmin_scalar, rhs, s);
      if (r) return r;
      r = launch_factor(t, B, prec, data, fac, scratch, s);
      if (r) return r;
      r = launch_solve(t, B, prec, fac, data, rhs, dz, 0, prec == VXG_F32 ? a.o->refine : 0,
                       xt, scratch, r64, s);
      if (r) return r;
      VXG_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int), s));
      r = launch_update(t, B, a.z, dz, active, a.converged, a.iters, a.o->max_dv, a.o->rtol,
                        a.o->atol, cnt, s);
      if (r) return r;
      newton_continue_kernel<<<1, 1, 0, s>>>(hc, cnt, cnt + 1, max_steps);
      VXG_LAUNCHED();
      return VXG_OK;
    });
  }
  if (st == VXG_OK && a.factors_out) {  // factors of the Jacobian at the returned state
    cudaGraph_t epi = nullptr;
    st = record(cs, nullptr, &epi, &n_epi, [&](cudaStream_t s) -> int {
      int r = launch_eval(t, gt, B, a.z, a.t_now, cf, cq, false, false, true, cfb, cqb, cjb, s);
      if (r) return r;
      r = launch_gather(t, B, cfb, cqb, cjb, a.gmin, a.gmin_scalar, nullptr, nullptr, data, s);
      if (r) return r;
      return launch_factor(t, B, prec, data, a.factors_out, scratch, s);
    });
    if (st == VXG_OK) {
      cuda_ok(cudaGraphAddChildGraphNode(&n2, g, &n1, 1, epi));
      cudaGraphDestroy(epi);
    }
  }
  if (st == VXG_OK) cuda_ok(cudaGraphInstantiate(exec, g, 0));
  cudaGraphDestroy(g);
  *kernels = n_pro + n_body + n_epi;
  return st;
}

static int newton_core(const NewtonCall& a, cudaStream_t s, bool cache) {
  const Topo& t = a.h->t;
  if (a.o->max_steps == 0) {  // no iteration: flags, and the factors if asked
    const Layout L = layout(t, a.B, a.o->precision);
    int st = launch_newton_init(a.B * t.n_seg, a.mask, at<int>(a.ws, L.active), a.converged,
                                a.iters, s);
    if (st || !a.factors_out) return st;
    const GroupTable gt = make_table(t, a.params);
    const bool dc = a.mode == VXG_MODE_DC;
    const double cf = a.mode == VXG_MODE_TRAP ? 0.5 : 1.0;
    const double cq = dc ? 0.0 : 1.0 / (a.t_now - a.t_prev);
    st = launch_eval(t, gt, a.B, a.z, a.t_now, cf, cq, false, false, true,
                     at<double>(a.ws, L.cf), at<double>(a.ws, L.cq), at<double>(a.ws, L.cj), s);
    if (st) return st;
    st = launch_gather(t, a.B, at<double>(a.ws, L.cf), at<double>(a.ws, L.cq),
                       at<double>(a.ws, L.cj), a.gmin, a.gmin_scalar, nullptr, nullptr,
                       at<double>(a.ws, L.data), s);
    if (st) return st;
    return launch_factor(t, a.B, a.o->precision, at<double>(a.ws, L.data), a.factors_out,
                         at<void>(a.ws, L.scratch), s);
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  VXG_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) {  // a graph with a loop cannot be nested
    std::snprintf(last_error_buffer(), 256,
                  "vxg_newton: the caller's stream is being captured; the Newton loop is "
                  "itself a graph with a conditional node and cannot be nested");
    return VXG_ERR_INVALID;
  }
  GraphCache* gc = a.h->graphs;
  if (!cache || !gc) {
    cudaGraphExec_t exec = nullptr;
    unsigned long long kernels = 0;
    int st = build_newton_graph(a, &exec, &kernels);
    if (st) return st;
    const cudaError_t e = cudaGraphLaunch(exec, s);
    cudaGraphExecDestroy(exec);  // freed once the launch completes
    if (e != cudaSuccess) {
      set_error(e);
      return VXG_ERR_CUDA;
    }
    count_launches(kernels);
    return VXG_OK;
  }
  std::vector<unsigned char> key = newton_key(a);
  std::lock_guard<std::mutex> lock(gc->mu);
  GraphEntry* hit = nullptr;
  for (GraphEntry& e : gc->entries)
    if (e.key == key) hit = &e;
  if (!hit) {
    GraphEntry e{std::move(key), nullptr, 0, 0};
    int st = build_newton_graph(a, &e.exec, &e.kernels);
    if (st) return st;
    if (gc->entries.size() >= kGraphCacheEntries) {  // evict the least recently used
      auto old = std::min_element(gc->entries.begin(), gc->entries.end(),
                                  [](const GraphEntry& x, const GraphEntry& y) {
                                    return x.used < y.used;
                                  });
      cudaGraphExecDestroy(old->exec);
      gc->entries.erase(old);
    }
    gc->entries.push_back(std::move(e));
    hit = &gc->entries.back();
  }
  hit->used = ++gc->tick;
  VXG_CUDA_TRY(cudaGraphLaunch(hit->exec, s));
  count_launches(hit->kernels);
  return VXG_OK;
}

}  // namespace vxg

extern "C" {

int vxg_spsolve_gdata(const vxg_handle* h, int32_t batch, const double* g, const double* x,
                      double* gdata, void* stream) {
  if (!h || batch <= 0 || !g || !x || !gdata) return VXG_ERR_INVALID;
  const long long n = (long long)batch * h->t.nnz;
  if (!n) return VXG_OK;
  gdata_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      batch, h->t.nnz, h->t.S, h->t.rows, h->t.indices, g, x, gdata);
  VXG_LAUNCHED();
  return VXG_OK;
}

static bool opts_ok(const vxg_newton_opts* o) {
  return o && o->max_steps >= 0 && (o->precision == VXG_F64 || o->precision == VXG_F32) &&
         o->refine >= 0;
}

int vxg_newton(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
               int32_t mode, double t_now, double t_prev, const double* z_prev,
               const double* gmin, double gmin_scalar, const vxg_newton_opts* opts, double* z,
               int32_t* converged, int32_t* iters, void* factors, void* workspace,
               void* stream) {
  if (!h || batch <= 0 || !params || !z || !converged || !iters || !workspace ||
      !opts_ok(opts) || mode < 0 || mode > 2 || (mode != VXG_MODE_DC && !z_prev))
    return VXG_ERR_INVALID;
  const NewtonCall a{h, batch, params, mode, t_now, t_prev, z_prev, gmin, gmin_scalar, opts,
                     z, converged, iters, factors, workspace, nullptr};
  return newton_core(a, (cudaStream_t)stream, true);
}

int vxg_newton_masked(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                      int32_t mode, double t_now, double t_prev, const double* z_prev,
                      const double* gmin, double gmin_scalar, const vxg_newton_opts* opts,
                      double* z, int32_t* converged, int32_t* iters, const int32_t* mask,
                      void* workspace, void* stream) {
  if (!h || batch <= 0 || !params || !z || !converged || !iters || !workspace ||
      !opts_ok(opts) || mode < 0 || mode > 2 || (mode != VXG_MODE_DC && !z_prev))
    return VXG_ERR_INVALID;
  const NewtonCall a{h, batch, params, mode, t_now, t_prev, z_prev, gmin, gmin_scalar, opts,
                     z, converged, iters, nullptr, workspace, mask};
  return newton_core(a, (cudaStream_t)stream, true);
}

int vxg_transient(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                  int32_t mode, int32_t n_t, const double* ts, const double* z0,
                  double gmin_scalar, const vxg_newton_opts* opts, double* z_out,
                  int32_t* converged, int32_t* iters, void* workspace, void* stream) {
  if (!h || batch <= 0 || !params || n_t <= 0 || !ts || !z0 || !z_out || !converged ||
      !iters || !workspace || !opts_ok(opts) || (mode != VXG_MODE_BE && mode != VXG_MODE_TRAP))
    return VXG_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nS = (size_t)batch * h->t.S;
  const int ninst = batch * h->t.n_seg;
  VXG_CUDA_TRY(cudaMemcpyAsync(z_out, z0, sizeof(double) * nS, cudaMemcpyDeviceToDevice, s));
  // row 0 is the initial state: converged, no iterations
  fill_int_kernel<<<(ninst + 255) / 256, 256, 0, s>>>(converged, ninst, 1);
  VXG_LAUNCHED();
  VXG_CUDA_TRY(cudaMemsetAsync(iters, 0, sizeof(int) * ninst, s));
  for (int n = 1; n < n_t; ++n) {
    double* prev = z_out + (size_t)(n - 1) * nS;
    double* cur = z_out + (size_t)n * nS;
    VXG_CUDA_TRY(cudaMemcpyAsync(cur, prev, sizeof(double) * nS, cudaMemcpyDeviceToDevice, s));
    const NewtonCall a{h, batch, params, mode, ts[n], ts[n - 1], prev, nullptr, gmin_scalar,
                       opts, cur, converged + (size_t)n * ninst, iters + (size_t)n * ninst,
                       nullptr, workspace, nullptr};
    int st = newton_core(a, s, false);  // one graph per step, not cached
    if (st) return st;
  }
  return VXG_OK;
}

int vxg_param_vjp(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                  const double* z, double t_now, double cf, double cq, const double* lam,
                  double* const* grads, void* stream) {
  if (!h || batch <= 0 || !params || !z || !lam || !grads) return VXG_ERR_INVALID;
  GroupTable gt = make_table(h->t, params);
  return launch_param_vjp(h->t, gt, batch, z, t_now, cf, cq, lam, grads, (cudaStream_t)stream);
}

}  // extern "C"

namespace vxg {
static std::atomic<unsigned long long> g_launches{0};
// Launches recorded into a graph are counted when the graph is launched.
void count_launch() {
  if (t_capturing)
    ++t_captured;
  else
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace vxg

extern "C" uint64_t vxg_launch_count(void) { return vxg::g_launches.load(); }
