// Newton kernels: residual composition, damped update with the convergence
// test, and the parameter VJP of the residual.
//
//   residuals      voltax/analysis.py:325-350
//   damped update  voltax/analysis.py:221-230
//   parameter VJP  voltax/analysis.py:282-288 (eqx.filter_vjp of the residual)

#include <math.h>

#include "devices.cuh"

namespace vxg {

__global__ void compose_kernel(int B, int S, int nv, int mode, double h,
                               const double* __restrict__ z, const double* __restrict__ f,
                               const double* __restrict__ q, const double* __restrict__ fp,
                               const double* __restrict__ qp, const double* __restrict__ gmin,
                               double gmin_scalar, const int* __restrict__ seg_of, int n_seg,
                               double* __restrict__ rhs) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * S) return;
  const int b = (int)(gid / S);
  const int i = (int)(gid - (long long)b * S);
  double gm = 0.0;
  if (i < nv) {
    const double g = gmin ? gmin[(long long)b * n_seg + seg_of[i]] : gmin_scalar;
    gm = g * z[gid];
  }
  double r;
  if (mode == VXG_MODE_DC) {
    r = f[gid] + gm;
  } else if (mode == VXG_MODE_BE) {
    r = (q[gid] - qp[gid]) / h + f[gid] + gm;
  } else {
    r = (q[gid] - qp[gid]) / h + 0.5 * (f[gid] + fp[gid]) + gm;
  }
  rhs[gid] = -r;
}

__global__ void newton_init_kernel(int n, const int* __restrict__ mask, int* __restrict__ active,
                                   int* __restrict__ converged, int* __restrict__ iters) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int on = mask ? (mask[i] != 0) : 1;
  active[i] = on;
  if (on) {
    converged[i] = 0;
    iters[i] = 0;
  }
}

template <int NT>
__global__ void __launch_bounds__(NT)
    newton_update_kernel(int S, int nv, int n_seg, const int* __restrict__ seg_ptr,
                         const int* __restrict__ seg_idx, double* __restrict__ z, const double* __restrict__ dz,
                         int* __restrict__ active, int* __restrict__ converged,
                         int* __restrict__ iters, double max_dv, double rtol, double atol,
                         int* __restrict__ n_active) {
  const int inst = blockIdx.x;
  if (!active[inst]) return;
  const int b = inst / n_seg, sg = inst - b * n_seg;
  const int lo = seg_ptr[sg], hi = seg_ptr[sg + 1];
  double* zb = z + (long long)b * S;
  const double* db = dz + (long long)b * S;
  __shared__ double s_red[NT / 32];
  __shared__ int s_flag[NT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // max |dz| over node voltages; NaN propagates as in jnp.max
  double m = 0.0;
  int has_nan = 0;
  for (int q = lo + threadIdx.x; q < hi; q += NT) {
    const int i = seg_idx[q];
    if (i >= nv) continue;  // node voltages only
    const double v = fabs(db[i]);
    if (isnan(v)) has_nan = 1;
    else m = fmax(m, v);
  }
  for (int off = 16; off > 0; off >>= 1) {
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    has_nan |= __shfl_xor_sync(0xffffffffu, has_nan, off);
  }
  if (lane == 0) {
    s_red[warp] = m;
    s_flag[warp] = has_nan;
  }
  __syncthreads();
  m = 0.0;
  has_nan = 0;
  for (int w = 0; w < NT / 32; ++w) {
    m = fmax(m, s_red[w]);
    has_nan |= s_flag[w];
  }
  __syncthreads();
  const double dv_max = has_nan ? nan("") : m;
  const double qd = max_dv / (dv_max + 1e-300);
  const double scale = isnan(qd) ? qd : fmin(1.0, qd);
  int ok = 1;
  for (int q = lo + threadIdx.x; q < hi; q += NT) {
    const int i = seg_idx[q];
    const double d = db[i];
    const double zn = zb[i] + scale * d;
    if (!(fabs(d) <= atol + rtol * fabs(zn))) ok = 0;
    if (!isfinite(zn)) ok = 0;
    zb[i] = zn;
  }
  ok = __all_sync(0xffffffffu, ok);
  if (lane == 0) s_flag[warp] = ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int all = 1;
    for (int w = 0; w < NT / 32; ++w) all &= s_flag[w];
    const int done = all && scale == 1.0;
    iters[inst] += 1;
    if (done) {
      converged[inst] = 1;
      active[inst] = 0;
    } else {
      atomicAdd(n_active, 1);
    }
  }
}

// ------------------------------------------------------------ dual numbers
struct Dual {
  double v, d;
};
__device__ __forceinline__ Dual mk(double v) { return {v, 0.0}; }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) {
  return {a.v * b.v, a.d * b.v + a.v * b.d};
}
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)};
}
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ Dual dexp(Dual a) {
  const double e = exp(a.v);
  return {e, e * a.d};
}
__device__ __forceinline__ Dual dsqrt(Dual a) {
  const double s = sqrt(a.v);
  return {s, a.d / (2.0 * s)};
}
__device__ __forceinline__ Dual dsoftplus(Dual a) {
  double sp, sg;
  softplus_and_sigmoid(a.v, &sp, &sg);
  return {sp, sg * a.d};
}
__device__ __forceinline__ Dual dclamp01(Dual a) {
  if (a.v <= 0.0) return {0.0, 0.0};
  if (a.v >= 1.0) return {1.0, 0.0};
  return a;
}
__device__ __forceinline__ Dual dmin(Dual a, Dual b) { return a.v <= b.v ? a : b; }
__device__ __forceinline__ Dual dpymod(Dual x, Dual y) {
  const double r = py_mod(x.v, y.v);
  const double k = (x.v - r) / y.v;  // integer quotient
  return {r, x.d - k * y.d};
}

__device__ Dual dwave(int wave, const Dual* p, double t) {
  switch (wave) {
    case VXG_WAVE_CONSTANT:
      return p[0];
    case VXG_WAVE_STEP: {
      const Dual frac = dclamp01((mk(t) - p[2]) / p[3]);
      return p[0] + (p[1] - p[0]) * frac;
    }
    case VXG_WAVE_PULSE: {
      const Dual tc = dpymod(mk(t) - p[2], p[6]);
      const Dual up = dclamp01(tc / (p[3] + mk(1e-30)));
      const Dual tfe = p[3] + p[5] + p[4];
      const Dual down = dclamp01((tfe - tc) / (p[4] + mk(1e-30)));
      const Dual value = p[0] + (p[1] - p[0]) * dmin(up, down);
      return t < p[2].v ? p[0] : value;
    }
  }
  return mk(0.0);
}

// Outputs (cf I + cq Q) of one device with dual parameters.
// max / min with the derivative split 1/2 : 1/2 at a tie (jnp.maximum)
__device__ __forceinline__ Dual dmax_tie(Dual a, Dual b) {
  if (a.v > b.v) return a;
  if (a.v < b.v) return b;
  return {a.v, 0.5 * (a.d + b.d)};
}
__device__ __forceinline__ Dual dmin_tie(Dual a, Dual b) {
  if (a.v < b.v) return a;
  if (a.v > b.v) return b;
  return {a.v, 0.5 * (a.d + b.d)};
}

// Level 1 threshold and one side of the drain current in parameter duals
// (voltax/elements/mosfet.py:229-247)
__device__ Dual l1_dual_vt(double vsb, Dual vt0, Dual gamma, Dual phi) {
  if (gamma.v == 0.0 && gamma.d == 0.0) return vt0;
  const Dual sphi = dsqrt(phi);
  const Dual root = vsb >= 0.0 ? dsqrt(phi + mk(fmax(vsb, 0.0)))
                               : dmax_tie(sphi + mk(fmin(vsb, 0.0)) / (2.0 * sphi), mk(0.0));
  return vt0 + gamma * (root - sphi);
}
__device__ Dual l1_dual_side(Dual vgs, Dual vds, Dual vt, Dual k, Dual lam, double s) {
  const Dual vov = s > 0.0 ? s * dsoftplus((vgs - vt) / mk(s)) : dmax_tie(vgs - vt, mk(0.0));
  const Dual vde = dmin_tie(vds, vov);
  return k * (vov - 0.5 * vde) * vde * (1.0 + lam * vds);
}

__device__ void dual_outputs(const GroupDev& g, const Dual* p, const double* u, double t,
                             double cf, double cq, Dual* out) {
  for (int i = 0; i < g.m; ++i) out[i] = mk(0.0);
  switch (g.kind) {
    case VXG_KIND_CONDUCTANCE: {
      const Dual i = mk(u[0] - u[1]) * p[0];
      out[0] = cf * i;
      out[1] = cf * (-i);
      break;
    }
    case VXG_KIND_CAPACITOR: {
      const Dual q = p[0] * mk(u[0] - u[1]);
      out[0] = cq * q;
      out[1] = cq * (-q);
      break;
    }
    case VXG_KIND_VSOURCE:
      out[2] = cf * (mk(u[0] - u[1]) - dwave(g.wave, p, t));
      break;
    case VXG_KIND_ISOURCE: {
      const Dual i = dwave(g.wave, p, t);
      out[0] = cf * i;
      out[1] = cf * (-i);
      break;
    }
    case VXG_KIND_EKV: {
      const double sign = p[0].v;
      const Dual i_spec = p[1], vth = p[2], dvth = p[3], n = p[4], vt = p[5], lam = p[6];
      const Dual c_ox = p[7], cov_w = p[8];
      const Dual vd = mk(sign * u[0]), vg = mk(sign * u[1]), vs = mk(sign * u[2]),
                 vb = mk(sign * u[3]);
      const Dual two_vt = 2.0 * vt;
      const Dual vp = (vg - vb - vth - dvth) / n;
      const Dual sf = dsoftplus((vp - (vs - vb)) / two_vt);
      const Dual sr = dsoftplus((vp - (vd - vb)) / two_vt);
      const Dual i_f = sf * sf, i_r = sr * sr;
      if (cf != 0.0) {
        const double vds = vd.v - vs.v;
        const double sabs = sqrt(vds * vds + 1e-3 * 1e-3) - 1e-3;
        const Dual ids = i_spec * (i_f - i_r) * (1.0 + lam * mk(sabs));
        out[0] = cf * (sign * ids);
        out[2] = cf * (sign * (-ids));
      }
      if (cq != 0.0) {
        const Dual xf = dsqrt(0.25 + i_f), xr = dsqrt(0.25 + i_r);
        const Dual scale = c_ox * n * vt;
        const Dual s = xf + xr;
        const Dual s2 = s * s;
        const double c415 = 4.0 / 15.0;
        const Dual nd = 3.0 * xr * xr * xr + 6.0 * xr * xr * xf + 4.0 * xr * xf * xf +
                        2.0 * xf * xf * xf;
        const Dual ns = 3.0 * xf * xf * xf + 6.0 * xf * xf * xr + 4.0 * xf * xr * xr +
                        2.0 * xr * xr * xr;
        const Dual q_d = -(scale * (c415 * nd / s2 - mk(0.5)));
        const Dual q_s = -(scale * (c415 * ns / s2 - mk(0.5)));
        const Dual q_i = q_d + q_s;
        const Dual kb = -(n - mk(1.0)) / n;
        const Dual q_b = kb * (c_ox * (vg - vb) + q_i);
        const Dual q_g = -(q_i + q_b);
        const Dual q_gs = cov_w * (vg - vs), q_gd = cov_w * (vg - vd);
        out[0] = out[0] + cq * (sign * (q_d - q_gd));
        out[1] = out[1] + cq * (sign * (q_g + (q_gs + q_gd)));
        out[2] = out[2] + cq * (sign * (q_s - q_gs));
        out[3] = out[3] + cq * (sign * q_b);
      }
      break;
    }
    case VXG_KIND_DIODE: {
      const Dual i_s = p[0], inv_nvt = p[1], tt = p[2], cj = p[3];
      const double v = u[0] - u[1];
      const Dual x = mk(v) * inv_nvt;
      const Dual e = dexp(x.v > 40.0 ? mk(40.0) : x);
      const Dual ex = x.v > 40.0 ? e * (1.0 + (x - mk(40.0))) : e;
      const Dual i = i_s * (ex - mk(1.0));
      out[0] = cf * i;
      out[1] = cf * (-i);
      if (cq != 0.0) {
        const Dual q = tt * i + cj * mk(v);
        out[0] = out[0] + cq * q;
        out[1] = out[1] + cq * (-q);
      }
      break;
    }
    case VXG_KIND_INDUCTOR:
      out[2] = cf * (p[1] * mk(u[2])) + cq * (p[0] * mk(u[2]));
      break;
    case VXG_KIND_BJT: {
      const double sg = p[0].v;
      const Dual i_s = p[1], inv_vt = p[2], ibf = p[3], ibr = p[4], ivaf = p[5];
      const Dual tf = p[6], tr = p[7], cje = p[8], cjc = p[9];
      const double vbe = sg * (u[1] - u[2]), vbc = sg * (u[1] - u[0]);
      const Dual xf = mk(vbe) * inv_vt, xr = mk(vbc) * inv_vt;
      const Dual ef = dexp(xf.v > 40.0 ? mk(40.0) : xf), er = dexp(xr.v > 40.0 ? mk(40.0) : xr);
      const Dual exf = xf.v > 40.0 ? ef * (1.0 + (xf - mk(40.0))) : ef;
      const Dual exr = xr.v > 40.0 ? er * (1.0 + (xr - mk(40.0))) : er;
      const Dual i_f = i_s * (exf - mk(1.0)), i_r = i_s * (exr - mk(1.0));
      const Dual early = 1.0 + mk(vbe - vbc) * ivaf;
      const Dual ic = (i_f - i_r) * early - i_r * ibr;
      const Dual ib = i_f * ibf + i_r * ibr;
      out[0] = cf * (sg * ic);
      out[1] = cf * (sg * ib);
      out[2] = cf * (sg * (-(ic + ib)));
      if (cq != 0.0) {
        const Dual q_be = tf * i_f + cje * mk(vbe), q_bc = tr * i_r + cjc * mk(vbc);
        out[0] = out[0] + cq * (sg * (-q_bc));
        out[1] = out[1] + cq * (sg * (q_be + q_bc));
        out[2] = out[2] + cq * (sg * (-q_be));
      }
      break;
    }
    case VXG_KIND_OPAMP: {
      const Dual a0 = p[0], grout = p[1], tau = p[2], mid = p[3], half = p[4];
      const Dual arg = (a0 * mk(u[0] - u[1]) - mid) / half;
      const double th = tanh(arg.v);
      const Dual clip = mid + half * Dual{th, (1.0 - th * th) * arg.d};
      out[2] = cf * (mk(u[2] - u[3]) * grout);
      out[3] = cf * (mk(u[3]) - clip) + cq * (tau * mk(u[3]));
      break;
    }
    case VXG_KIND_SWITCH: {
      const Dual on_arg = (mk(u[2] - u[3]) - p[2]) * p[3];
      double sp, sg;
      softplus_and_sigmoid(on_arg.v, &sp, &sg);
      const Dual on = {sg, sg * (1.0 - sg) * on_arg.d};
      const Dual gg = dexp(on * p[1] - p[0]);
      const Dual i = gg * mk(u[0] - u[1]);
      out[0] = cf * i;
      out[1] = cf * (-i);
      break;
    }
    case VXG_KIND_VCVS:
      out[4] = cf * (mk(u[0] - u[1]) - p[0] * mk(u[2] - u[3]));
      break;
    case VXG_KIND_CCCS:
      out[0] = cf * (p[0] * mk(u[4]));
      out[1] = cf * (-(p[0] * mk(u[4])));
      break;
    case VXG_KIND_CCVS:
      out[4] = cf * (mk(u[0] - u[1]) - p[0] * mk(u[5]));
      break;
    case VXG_KIND_XFMR:
      out[4] = cq * (p[0] * mk(u[4]) + p[2] * mk(u[5]));
      out[5] = cq * (p[2] * mk(u[4]) + p[1] * mk(u[5]));
      break;
    case VXG_KIND_VCCS: {
      const Dual i = p[0] * mk(u[2] - u[3]);
      out[0] = cf * i;
      out[1] = cf * (-i);
      break;
    }
    case VXG_KIND_L1: {
      const double sign = p[0].v;
      const Dual k = p[1], vt0 = p[2] + p[3], lam = p[4], gamma = p[5], phi = p[6];
      const double s = p[7].v;
      const Dual cov_w = p[8];
      const double vd = sign * u[0], vg = sign * u[1], vs = sign * u[2], vb = sign * u[3];
      if (cf != 0.0) {
        const Dual vds = mk(vd - vs);
        const Dual f = l1_dual_side(mk(vg - vs), dmax_tie(vds, mk(0.0)),
                                    l1_dual_vt(vs - vb, vt0, gamma, phi), k, lam, s);
        const Dual r = l1_dual_side(mk(vg - vd), dmax_tie(-vds, mk(0.0)),
                                    l1_dual_vt(vd - vb, vt0, gamma, phi), k, lam, s);
        const Dual ids = f - r;
        out[0] = cf * (sign * ids);
        out[2] = cf * (sign * (-ids));
      }
      if (cq != 0.0) {
        const Dual q_gs = cov_w * mk(u[1] - u[2]), q_gd = cov_w * mk(u[1] - u[0]);
        out[0] = out[0] + cq * (-q_gd);
        out[1] = out[1] + cq * (q_gs + q_gd);
        out[2] = out[2] + cq * (-q_gs);
      }
      break;
    }
  }
}

constexpr int kMaxParams = 13;

struct GradPtrs {
  double* p[VXG_MAX_GROUPS];
};

__global__ void param_vjp_kernel(GroupTable gt, int B, const double* __restrict__ z, int S,
                                 double t, double cf, double cq, const double* __restrict__ lam,
                                 GradPtrs grads) {
  long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gid >= (long long)B * gt.n_dev) return;
  const int b = (int)(gid / gt.n_dev);
  const long long flat = gid - (long long)b * gt.n_dev;
  int gi = 0;
  while (gi + 1 < gt.n_groups && gt.g[gi + 1].dev_base <= flat) ++gi;
  const GroupDev& g = gt.g[gi];
  const int d = (int)(flat - g.dev_base);
  const double* zb = z + (long long)b * S;
  const double* lb = lam + (long long)b * S;
  double u[kMaxM], l[kMaxM];
  for (int i = 0; i < g.T; ++i) {
    const int node = g.nodes[d * g.T + i];
    u[i] = node >= 0 ? zb[node] : 0.0;
    l[i] = node >= 0 ? lb[node] : 0.0;
  }
  for (int i = 0; i < g.K; ++i) {
    u[g.T + i] = zb[g.int_offset + d * g.K + i];
    l[g.T + i] = lb[g.int_offset + d * g.K + i];
  }
  double* out = grads.p[gi];
  if (g.kind == VXG_KIND_COUPLED_L) {
    // Device e's rows (l, sqrt l, k) enter the flux rows of every device:
    // q_d = l_d i_d + k_d s_d sum_{e != d} s_e i_e (s = sqrt l), scaled by cq.
    const int e = d, n = g.n;
    const double* ib = zb + g.int_offset;
    const double* lmb = lb + g.int_offset;
    const double se = prm(g, 1, b, e);
    double others = 0.0, cross = 0.0;  // sum_{e' != e} s_e' i_e'; sum_{d != e} lam_d k_d s_d
    for (int q = 0; q < n; ++q) {
      if (q == e) continue;
      const double sq = prm(g, 1, b, q);
      others += sq * ib[q];
      cross += lmb[q] * prm(g, 2, b, q) * sq;
    }
    const double ke = prm(g, 2, b, e);
    out[((long long)0 * B + b) * n + e] = -cq * lmb[e] * ib[e];
    out[((long long)1 * B + b) * n + e] = -cq * (lmb[e] * ke * others + cross * ib[e]);
    out[((long long)2 * B + b) * n + e] = -cq * lmb[e] * se * others;
    return;
  }
  Dual p[kMaxParams];
  for (int r = 0; r < g.n_params; ++r) p[r] = mk(prm(g, r, b, d));
  for (int r = 0; r < g.n_params; ++r) {
    p[r].d = 1.0;
    Dual o[kMaxM];
    dual_outputs(g, p, u, t, cf, cq, o);
    double acc = 0.0;
    for (int i = 0; i < g.m; ++i) acc += l[i] * o[i].d;
    p[r].d = 0.0;
    out[((long long)r * B + b) * g.n + d] = -acc;
  }
}

int launch_param_vjp(const Topo& t, const GroupTable& gt, int B, const double* z, double t_now,
                     double cf, double cq, const double* lam, double* const* grads,
                     cudaStream_t s) {
  const long long n = (long long)B * gt.n_dev;
  if (!n) return VXG_OK;
  GradPtrs gp;
  for (int i = 0; i < VXG_MAX_GROUPS; ++i) gp.p[i] = i < gt.n_groups ? grads[i] : nullptr;
  param_vjp_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(gt, B, z, t.S, t_now, cf, cq,
                                                                 lam, gp);
  VXG_LAUNCHED();
  return VXG_OK;
}

int launch_compose(const Topo& t, int B, int mode, double h, const double* z, const double* f,
                   const double* q, const double* fp, const double* qp, const double* gmin,
                   double gmin_scalar, double* rhs, cudaStream_t s) {
  const long long n = (long long)B * t.S;
  if (!n) return VXG_OK;
  compose_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      B, t.S, t.nv, mode, h, z, f, q, fp, qp, gmin, gmin_scalar, t.seg_of, t.n_seg, rhs);
  VXG_LAUNCHED();
  return VXG_OK;
}

int launch_newton_init(int n, const int* mask, int* active, int* converged, int* iters,
                       cudaStream_t s) {
  if (!n) return VXG_OK;
  newton_init_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, mask, active, converged, iters);
  VXG_LAUNCHED();
  return VXG_OK;
}

int launch_update(const Topo& t, int B, double* z, const double* dz, int* active,
                  int* converged, int* iters, double max_dv, double rtol, double atol,
                  int* n_active, cudaStream_t s) {
  const int n = B * t.n_seg;
  if (!n) return VXG_OK;
  newton_update_kernel<256><<<n, 256, 0, s>>>(t.S, t.nv, t.n_seg, t.seg_ptr, t.seg_idx, z, dz,
                                              active,
                                              converged, iters, max_dv, rtol, atol, n_active);
  VXG_LAUNCHED();
  return VXG_OK;
}

}  // namespace vxg
