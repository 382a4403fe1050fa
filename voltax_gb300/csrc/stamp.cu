// Device evaluation and deterministic stamping.
//
// Phase 1 (eval_kernel): one thread per (instance, device) gathers the
// device's local unknowns, evaluates its physics (devices.cuh) and writes
// its residual contributions and its local Jacobian block to contribution
// slots, laid out structure-of-arrays per group (slot (i, j) of device d at
// (i*m + j)*n + d) so that neighbouring threads store to neighbouring words.
//
// Phase 2 (gather_kernel): one thread per (instance, CSR entry) or
// (instance, row) sums its contribution slots in the canonical order
// (group, device, local row, local column; the host sorts each source list
// by that key) -- then adds
// gmin on node diagonals. The same inputs therefore always give the same
// bits, and they equal the oracle's ordered np.add.at assembly bit for bit.
// No atomics anywhere.

#include "devices.cuh"

namespace vxg {

__global__ void eval_kernel(GroupTable gt, int B, const double* __restrict__ z, int S, int nv,
                            double t, double cf, double cq, int want_f, int want_q,
                            int want_j, long long n_res_slots, long long n_jac_slots,
                            double* __restrict__ cf_buf, double* __restrict__ cq_buf,
                            double* __restrict__ cj_buf) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * gt.n_dev) return;
  const int b = (int)(gid / gt.n_dev);
  const long long flat = gid - (long long)b * gt.n_dev;
  int gi = 0;
  while (gi + 1 < gt.n_groups && gt.g[gi + 1].dev_base <= flat) ++gi;
  const GroupDev& g = gt.g[gi];
  const int d = (int)(flat - g.dev_base);
  double u[kMaxM];
  const double* zb = z + (long long)b * S;
  gather_u(g, d, zb, u);
  eval_soa<double>(g, b, d, u, t, cf, cq, want_f, want_q, want_j,
                   cf_buf + (long long)b * n_res_slots + g.res_base,
                   cq_buf + (long long)b * n_res_slots + g.res_base,
                   cj_buf + (long long)b * n_jac_slots + g.jac_base, zb);
}

// data[e] = sum of Jacobian slots of entry e (+ gmin on node diagonals)
__global__ void gather_jac_kernel(int B, long long nnz, const long long* __restrict__ ptr,
                                  const long long* __restrict__ src, long long n_jac_slots,
                                  const double* __restrict__ cj, const int* __restrict__ rows,
                                  const int* __restrict__ indices, int nv,
                                  const int* __restrict__ seg_of, int n_seg,
                                  const double* __restrict__ gmin, double gmin_scalar,
                                  double* __restrict__ data) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * nnz) return;
  const int b = (int)(gid / nnz);
  const long long e = gid - (long long)b * nnz;
  const double* c = cj + (long long)b * n_jac_slots;
  double acc = 0.0;
  for (long long p = ptr[e]; p < ptr[e + 1]; ++p) acc += c[src[p]];
  const int r = rows[e];
  if (r < nv && indices[e] == r) {
    const double gm = gmin ? gmin[(long long)b * n_seg + seg_of[r]] : gmin_scalar;
    acc += gm;
  }
  data[gid] = acc;
}

// f[i] / q[i] = sum of residual slots of row i
__global__ void gather_res_kernel(int B, int S, const long long* __restrict__ ptr,
                                  const long long* __restrict__ src, long long n_res_slots,
                                  const double* __restrict__ cf_buf,
                                  const double* __restrict__ cq_buf, double* __restrict__ f_out,
                                  double* __restrict__ q_out) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * S) return;
  const int b = (int)(gid / S);
  const int i = (int)(gid - (long long)b * S);
  const long long base = (long long)b * n_res_slots;
  if (f_out) {
    double acc = 0.0;
    for (long long p = ptr[i]; p < ptr[i + 1]; ++p) acc += cf_buf[base + src[p]];
    f_out[gid] = acc;
  }
  if (q_out) {
    double acc = 0.0;
    for (long long p = ptr[i]; p < ptr[i + 1]; ++p) acc += cq_buf[base + src[p]];
    q_out[gid] = acc;
  }
}

static inline unsigned blocks_for(long long n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

int launch_eval(const Topo& t, const GroupTable& gt, int B, const double* z, double t_now,
                double cf, double cq, bool want_f, bool want_q, bool want_j, double* cf_buf,
                double* cq_buf, double* cj_buf, cudaStream_t s) {
  const long long n = (long long)B * gt.n_dev;
  if (n == 0) return VXG_OK;
  eval_kernel<<<blocks_for(n, 128), 128, 0, s>>>(gt, B, z, t.S, t.nv, t_now, cf, cq, want_f,
                                                 want_q, want_j, t.n_res_slots, t.n_jac_slots,
                                                 cf_buf, cq_buf, cj_buf);
  VXG_LAUNCHED();
  return VXG_OK;
}

int launch_gather(const Topo& t, int B, const double* cf_buf, const double* cq_buf,
                  const double* cj_buf, const double* gmin, double gmin_scalar, double* f_out,
                  double* q_out, double* data_out, cudaStream_t s) {
  if (data_out) {
    const long long n = (long long)B * t.nnz;
    gather_jac_kernel<<<blocks_for(n, 256), 256, 0, s>>>(
        B, t.nnz, t.jac_ptr, t.jac_src, t.n_jac_slots, cj_buf, t.rows, t.indices, t.nv,
        t.seg_of, t.n_seg, gmin, gmin_scalar, data_out);
    VXG_LAUNCHED();
  }
  if (f_out || q_out) {
    const long long n = (long long)B * t.S;
    gather_res_kernel<<<blocks_for(n, 256), 256, 0, s>>>(B, t.S, t.res_ptr, t.res_src,
                                                          t.n_res_slots, cf_buf, cq_buf,
                                                          f_out, q_out);
    VXG_LAUNCHED();
  }
  return VXG_OK;
}

}  // namespace vxg
