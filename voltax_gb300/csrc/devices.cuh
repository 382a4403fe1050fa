// Device physics with analytic local Jacobians, FP64.
//
// Each device maps its local unknowns u (terminal voltages, then internal
// unknowns) to
//   I[i] : resistive contribution (currents into the device / internal eqs)
//   Q[i] : reactive contribution (charges / fluxes)
//   J[i*m+j] = cf dI[i]/du[j] + cq dQ[i]/du[j]
// following voltax's element equations:
//   conductance  voltax/elements/passive.py:37-38, behavioral.py:98-99
//   capacitor    voltax/elements/passive.py:58-59
//   V source     voltax/elements/sources.py:85-87
//   I source     voltax/elements/sources.py:110-112
//   EKV MOSFET   voltax/elements/mosfet.py:127-205
//   Level 1      voltax/elements/mosfet.py:208-257
//   diode, BJT   voltax/elements/semiconductor.py:17-135
//   inductor     voltax/elements/passive.py:62-87
//   VCCS         voltax/elements/controlled.py:46-60
//   waveforms    voltax/signals.py:58-114
// voltax differentiates these by forward-mode AD; the derivatives below are
// the same chain rule written out by hand.
#pragma once

#include "internal.cuh"

namespace vxg {

__device__ __forceinline__ double prm(const GroupDev& g, int row, int b, int d) {
  return g.params[row * g.row_stride + (long long)b * g.batch_stride + d];
}

// Python-style float remainder, as jnp.remainder: fmod, then shift into
// the divisor's sign.
__device__ __forceinline__ double py_mod(double x, double y) {
  double r = fmod(x, y);
  if (r != 0.0 && ((r < 0.0) != (y < 0.0))) r += y;
  return r;
}

__device__ __forceinline__ double clamp01(double x) { return fmin(fmax(x, 0.0), 1.0); }

__device__ inline double wave_value(const GroupDev& g, int b, int d, double t) {
  switch (g.wave) {
    case VXG_WAVE_CONSTANT:
      return prm(g, 0, b, d);
    case VXG_WAVE_STEP: {
      double v0 = prm(g, 0, b, d), v1 = prm(g, 1, b, d);
      double delay = prm(g, 2, b, d), rise = prm(g, 3, b, d);
      double frac = clamp01((t - delay) / rise);
      return v0 + (v1 - v0) * frac;
    }
    case VXG_WAVE_PULSE: {
      double v1 = prm(g, 0, b, d), v2 = prm(g, 1, b, d), delay = prm(g, 2, b, d);
      double rise = prm(g, 3, b, d), fall = prm(g, 4, b, d), width = prm(g, 5, b, d);
      double period = prm(g, 6, b, d);
      double tc = py_mod(t - delay, period);
      double up = clamp01(tc / (rise + 1e-30));
      double t_fall_end = rise + width + fall;
      double down = clamp01((t_fall_end - tc) / (fall + 1e-30));
      double value = v1 + (v2 - v1) * fmin(up, down);
      return t < delay ? v1 : value;
    }
  }
  return 0.0;
}

// softplus(x) = logaddexp(x, 0) = max(x, 0) + log1p(exp(-|x|)); sigmoid is
// its derivative.
__device__ __forceinline__ void softplus_and_sigmoid(double x, double* sp, double* sg) {
  double e = exp(-fabs(x));
  *sp = fmax(x, 0.0) + log1p(e);
  *sg = x >= 0.0 ? 1.0 / (1.0 + e) : e / (1.0 + e);
}

}  // namespace vxg

namespace vxg {

// --------------------------------------------------------------------------
// Structure-of-arrays evaluation. Slot (i, d) of a group's residual block is
// res[i * n + d]; slot (i, j, d) of its Jacobian block is jac[(i * m + j) * n
// + d]. Consecutive devices therefore write consecutive addresses. Values
// (currents, charges) are FP64; Jacobian entries are computed and stored in
// JT (double for the plain form, float for the FP32-factor form, whose
// Jacobian only feeds the FP32 factorization and the refinement matrix).
// --------------------------------------------------------------------------
// The quantities the EKV local Jacobian is built from, in the Jacobian's
// type: derivatives of the forward/reverse arguments, the softplus values
// and sigmoids, the drain-current factors, and the charge-sheet terms.
template <typename JT>
struct EkvTerms {
  JT af_g, af_s, af_b;  // d af / d (vg, vs, vb); ar has the same with vd for vs
  JT dif, dir;          // d i_f / d af, d i_r / d ar
  JT isp, mf, dI, dsa, lam;
  JT xf, xr, s, nd, ns, sc, kb, cox, cw;
};

// Local Jacobian of one EKV device (voltax/elements/mosfet.py:171-205 by
// the chain rule), J[i][j] = cf dI_i/du_j + cq dQ_i/du_j in the device's
// mirrored n-frame; the sign flips of a PMOS cancel in J.
template <typename JT>
__device__ __forceinline__ void ekv_jac_write(const EkvTerms<JT>& e, double cf, double cq,
                                              bool need_i, bool need_q, int n, int d, JT* jo) {
  JT ji[4] = {JT(0), JT(0), JT(0), JT(0)};
  if (need_i && cf != 0.0) {
    ji[0] = e.isp * ((-e.dir * e.af_s) * e.mf + e.dI * e.lam * e.dsa);
    ji[1] = e.isp * ((e.dif - e.dir) * e.af_g * e.mf);
    ji[2] = e.isp * ((e.dif * e.af_s) * e.mf - e.dI * e.lam * e.dsa);
    ji[3] = e.isp * ((e.dif - e.dir) * e.af_b * e.mf);
  }
  JT dq0[4] = {JT(0), JT(0), JT(0), JT(0)}, dq1[4] = {JT(0), JT(0), JT(0), JT(0)};
  JT dq2[4] = {JT(0), JT(0), JT(0), JT(0)}, dq3[4] = {JT(0), JT(0), JT(0), JT(0)};
  if (need_q && cq != 0.0) {
    const JT fx = e.xf, rx = e.xr, ss = e.s, s3 = ss * ss * ss;
    const JT gd_f = ((JT(6) * rx * rx + JT(8) * rx * fx + JT(6) * fx * fx) * ss - JT(2) * e.nd) / s3;
    const JT gd_r = ((JT(9) * rx * rx + JT(12) * rx * fx + JT(4) * fx * fx) * ss - JT(2) * e.nd) / s3;
    const JT gs_f = ((JT(9) * fx * fx + JT(12) * fx * rx + JT(4) * rx * rx) * ss - JT(2) * e.ns) / s3;
    const JT gs_r = ((JT(6) * fx * fx + JT(8) * fx * rx + JT(6) * rx * rx) * ss - JT(2) * e.ns) / s3;
    const JT dxf_da = e.dif / (JT(2) * fx), dxr_da = e.dir / (JT(2) * rx);
    const JT c415 = JT(4) / JT(15);
    const JT dafk[4] = {JT(0), e.af_g, e.af_s, e.af_b};
    const JT dark[4] = {e.af_s, e.af_g, JT(0), e.af_b};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const JT dxf = dxf_da * dafk[k], dxr = dxr_da * dark[k];
      const JT dqd = -e.sc * c415 * (gd_f * dxf + gd_r * dxr);
      const JT dqs = -e.sc * c415 * (gs_f * dxf + gs_r * dxr);
      const JT dqi = dqd + dqs;
      const JT dvgb = (k == 1 ? JT(1) : JT(0)) - (k == 3 ? JT(1) : JT(0));
      const JT dqb = e.kb * (e.cox * dvgb + dqi);
      const JT dqg = -(dqi + dqb);
      const JT dgs = e.cw * ((k == 1 ? JT(1) : JT(0)) - (k == 2 ? JT(1) : JT(0)));
      const JT dgd = e.cw * ((k == 1 ? JT(1) : JT(0)) - (k == 0 ? JT(1) : JT(0)));
      dq0[k] = dqd - dgd;
      dq1[k] = dqg + (dgs + dgd);
      dq2[k] = dqs - dgs;
      dq3[k] = dqb;
    }
  }
  const JT cfj = (JT)cf, cqj = (JT)cq;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    JT r0 = cf != 0.0 ? cfj * ji[j] : JT(0);
    JT r2 = cf != 0.0 ? cfj * -ji[j] : JT(0);
    JT r1 = JT(0), r3 = JT(0);
    if (cq != 0.0) {
      r0 = r0 + cqj * dq0[j];
      r1 = r1 + cqj * dq1[j];
      r2 = r2 + cqj * dq2[j];
      r3 = r3 + cqj * dq3[j];
    }
    jo[(0 * 4 + j) * n + d] = r0;
    jo[(1 * 4 + j) * n + d] = r1;
    jo[(2 * 4 + j) * n + d] = r2;
    jo[(3 * 4 + j) * n + d] = r3;
  }
}

// Charge-sheet terms of the EKV charges from the normalised currents.
template <typename X>
__device__ __forceinline__ void ekv_charge_terms(X i_f, X i_r, X* xf, X* xr, X* s, X* nd,
                                                 X* ns) {
  *xf = sqrt(X(0.25) + i_f);
  *xr = sqrt(X(0.25) + i_r);
  *s = *xf + *xr;
  const X xf2 = *xf * *xf, xr2 = *xr * *xr;
  *nd = xr2 * (X(3) * *xr + X(6) * *xf) + xf2 * (X(4) * *xr + X(2) * *xf);
  *ns = xf2 * (X(3) * *xf + X(6) * *xr) + xr2 * (X(4) * *xf + X(2) * *xr);
}

template <typename JT>
__device__ __forceinline__ void ekv_soa(const GroupDev& g, int b, int d, const double* u,
                                        double cf, double cq, bool wf, bool wq, bool wj,
                                        double* fo, double* qo, JT* jo) {
  const int n = g.n;
  const bool neg = prm(g, 0, b, d) < 0.0;  // PMOS: evaluate in the mirrored n-frame
  const double i_spec = prm(g, 1, b, d), vth = prm(g, 2, b, d), dvth = prm(g, 3, b, d);
  const double lam = prm(g, 6, b, d), c_ox = prm(g, 7, b, d);
  const double cov_w = prm(g, 8, b, d), inv_n = prm(g, 9, b, d), inv_2vt = prm(g, 10, b, d);
  const double scale = prm(g, 11, b, d), kb = prm(g, 12, b, d);
  const double vd = neg ? -u[0] : u[0], vg = neg ? -u[1] : u[1];
  const double vs = neg ? -u[2] : u[2], vb = neg ? -u[3] : u[3];
  const double vp = (vg - vb - vth - dvth) * inv_n;
  const double af = (vp - (vs - vb)) * inv_2vt;
  const double ar = (vp - (vd - vb)) * inv_2vt;
  // softplus(x) = max(x, 0) + log1p(exp(-|x|)), exp kept for the sigmoid
  const double ef = exp(-fabs(af)), er = exp(-fabs(ar));
  const double spf = fmax(af, 0.0) + log1p(ef), spr = fmax(ar, 0.0) + log1p(er);
  const double i_f = spf * spf, i_r = spr * spr;
  const bool need_i = wf || (wj && cf != 0.0);
  const bool need_q = wq || (wj && cq != 0.0);
  const double vds = vd - vs;
  double root = 0.0, mfac = 0.0;
  if (need_i) {
    root = sqrt(vds * vds + 1e-3 * 1e-3);
    mfac = 1.0 + lam * (root - 1e-3);
  }
  if (wf) {
    const double ids = i_spec * (i_f - i_r) * mfac;
    fo[0 * n + d] = neg ? -ids : ids;
    fo[1 * n + d] = 0.0;
    fo[2 * n + d] = neg ? ids : -ids;
    fo[3 * n + d] = 0.0;
  }
  double xf = 0.0, xr = 0.0, s = 1.0, nd = 0.0, ns = 0.0;
  if (need_q) ekv_charge_terms(i_f, i_r, &xf, &xr, &s, &nd, &ns);
  if (wq) {
    const double w415 = (4.0 / 15.0) / (s * s);
    const double q_d = -scale * (w415 * nd - 0.5);
    const double q_s = -scale * (w415 * ns - 0.5);
    const double q_i = q_d + q_s;
    const double q_b = kb * (c_ox * (vg - vb) + q_i);
    const double q_g = -(q_i + q_b);
    const double q_gs = cov_w * (vg - vs), q_gd = cov_w * (vg - vd);
    const double o0 = q_d - q_gd, o1 = q_g + (q_gs + q_gd), o2 = q_s - q_gs;
    qo[0 * n + d] = neg ? -o0 : o0;
    qo[1 * n + d] = neg ? -o1 : o1;
    qo[2 * n + d] = neg ? -o2 : o2;
    qo[3 * n + d] = neg ? -q_b : q_b;
  }
  if (!wj) return;
  EkvTerms<JT> e;
  const JT tv2 = (JT)inv_2vt, g1 = (JT)inv_n;
  e.af_g = g1 * tv2;
  e.af_s = -tv2;
  e.af_b = (JT(1) - g1) * tv2;
  const JT sgf = af >= 0.0 ? JT(1) / (JT(1) + (JT)ef) : (JT)ef / (JT(1) + (JT)ef);
  const JT sgr = ar >= 0.0 ? JT(1) / (JT(1) + (JT)er) : (JT)er / (JT(1) + (JT)er);
  e.dif = JT(2) * (JT)spf * sgf;
  e.dir = JT(2) * (JT)spr * sgr;
  e.isp = (JT)i_spec;
  e.mf = (JT)mfac;
  e.dI = (JT)(i_f - i_r);
  e.dsa = need_i ? (JT)vds / (JT)root : JT(0);
  e.lam = (JT)lam;
  e.xf = (JT)xf;
  e.xr = (JT)xr;
  e.s = (JT)s;
  e.nd = (JT)nd;
  e.ns = (JT)ns;
  e.sc = (JT)scale;
  e.kb = (JT)kb;
  e.cox = (JT)c_ox;
  e.cw = (JT)cov_w;
  ekv_jac_write(e, cf, cq, need_i, need_q, n, d, jo);
}

// The EKV local Jacobian alone, from FP32 intermediates: the chosen form's
// second evaluation pass (its FP64 currents and charges come from ekv_soa
// with wj = false). Only the bias differences are formed in FP64; the
// exponentials, logarithms and roots run on the FP32 pipes. The Jacobian
// only steers Newton (the residual stays FP64), so its FP32 rounding changes
// at most the convergence rate, which the FP32 factorization already sets.
__device__ __forceinline__ void ekv_jac_f32(const GroupDev& g, int b, int d, const double* u,
                                            double cf, double cq, float* jo) {
  const int n = g.n;
  const bool neg = prm(g, 0, b, d) < 0.0;
  const double vd = neg ? -u[0] : u[0], vg = neg ? -u[1] : u[1];
  const double vs = neg ? -u[2] : u[2], vb = neg ? -u[3] : u[3];
  const double inv_n = prm(g, 9, b, d), inv_2vt = prm(g, 10, b, d);
  const double vp = (vg - vb - prm(g, 2, b, d) - prm(g, 3, b, d)) * inv_n;
  const float af = (float)((vp - (vs - vb)) * inv_2vt);
  const float ar = (float)((vp - (vd - vb)) * inv_2vt);
  const float vds = (float)(vd - vs);
  const bool need_i = cf != 0.0, need_q = cq != 0.0;
  const float ef = __expf(-fabsf(af)), er = __expf(-fabsf(ar));
  const float spf = fmaxf(af, 0.0f) + log1pf(ef), spr = fmaxf(ar, 0.0f) + log1pf(er);
  const float i_f = spf * spf, i_r = spr * spr;
  EkvTerms<float> e;
  const float tv2 = (float)inv_2vt, g1 = (float)inv_n;
  e.af_g = g1 * tv2;
  e.af_s = -tv2;
  e.af_b = (1.0f - g1) * tv2;
  const float sgf = af >= 0.0f ? 1.0f / (1.0f + ef) : ef / (1.0f + ef);
  const float sgr = ar >= 0.0f ? 1.0f / (1.0f + er) : er / (1.0f + er);
  e.dif = 2.0f * spf * sgf;
  e.dir = 2.0f * spr * sgr;
  e.isp = (float)prm(g, 1, b, d);
  e.lam = (float)prm(g, 6, b, d);
  const float root = sqrtf(vds * vds + 1e-6f);
  e.mf = 1.0f + e.lam * (root - 1e-3f);
  e.dI = i_f - i_r;
  e.dsa = vds / root;
  e.xf = e.xr = e.s = 1.0f;
  e.nd = e.ns = 0.0f;
  if (need_q) ekv_charge_terms(i_f, i_r, &e.xf, &e.xr, &e.s, &e.nd, &e.ns);
  e.sc = (float)prm(g, 11, b, d);
  e.kb = (float)prm(g, 12, b, d);
  e.cox = (float)prm(g, 7, b, d);
  e.cw = (float)prm(g, 8, b, d);
  ekv_jac_write(e, cf, cq, need_i, need_q, n, d, jo);
}

// Level 1 (Shichman-Hodges) MOSFET, smoothed (voltax/elements/mosfet.py:208-257):
// I = F(vg - vs, max(vds, 0), vt(vs - vb)) - F(vg - vd, max(-vds, 0), vt(vd - vb)),
// F = k (vov - vde/2) vde (1 + lam vds), vov = s softplus((vgs - vt)/s) (or
// max(vgs - vt, 0) when s = 0), vde = min(vds, vov); vt with the body effect
// linearised for a forward-biased bulk; overlap charges only. Like
// jnp.maximum / jnp.minimum, max and min split the derivative 1/2 : 1/2 at
// a tie (vds = 0 is a tie at every symmetric bias point).
__device__ __forceinline__ double tie_gt(double a, double b) {  // d max(a, b) / da
  return a > b ? 1.0 : (a == b ? 0.5 : 0.0);
}

// threshold and d threshold / d vsb
__device__ __forceinline__ void l1_vt(double vsb, double vt0, double gamma, double phi,
                                     double sphi, double inv2sphi, double* vt, double* dvt) {
  if (gamma == 0.0) {
    *vt = vt0;
    *dvt = 0.0;
    return;
  }
  double root, droot;
  if (vsb >= 0.0) {
    root = sqrt(phi + fmax(vsb, 0.0));
    droot = tie_gt(vsb, 0.0) * 0.5 / root;
  } else {
    const double lin = sphi + vsb * inv2sphi;
    root = fmax(lin, 0.0);
    droot = tie_gt(lin, 0.0) * inv2sphi;
  }
  *vt = vt0 + gamma * (root - sphi);
  *dvt = gamma * droot;
}

// F and its partials in (vgs, vds) (d/dvt = -d/dvgs)
__device__ __forceinline__ void l1_side(double vgs, double vds, double vt, double k, double lam,
                                       double s, double inv_s, double* f, double* fgs,
                                       double* fds) {
  const double x = vgs - vt;
  double vov, dvov;
  if (s > 0.0) {
    double sp, sg;
    softplus_and_sigmoid(x * inv_s, &sp, &sg);
    vov = s * sp;
    dvov = sg;
  } else {
    vov = fmax(x, 0.0);
    dvov = tie_gt(x, 0.0);
  }
  const double vde = fmin(vds, vov);
  const double dde_ds = tie_gt(vov, vds), dde_dov = tie_gt(vds, vov);
  const double m = 1.0 + lam * vds;
  *f = k * (vov - 0.5 * vde) * vde * m;
  const double df_ov = k * vde * m, df_de = k * (vov - vde) * m;
  *fgs = (df_ov + df_de * dde_dov) * dvov;
  *fds = k * (vov - 0.5 * vde) * vde * lam + df_de * dde_ds;
}

template <typename JT>
__device__ __forceinline__ void l1_soa(const GroupDev& g, int b, int d, const double* u,
                                       double cf, double cq, bool wf, bool wq, bool wj,
                                       double* fo, double* qo, JT* jo) {
  const int n = g.n;
  const bool neg = prm(g, 0, b, d) < 0.0;
  const double cov_w = prm(g, 8, b, d);
  const bool need_i = wf || (wj && cf != 0.0);
  double I = 0.0, gd = 0.0, gg = 0.0, gs = 0.0, gb = 0.0;
  if (need_i) {
    const double k = prm(g, 1, b, d), vt0 = prm(g, 2, b, d) + prm(g, 3, b, d);
    const double lam = prm(g, 4, b, d), gamma = prm(g, 5, b, d), phi = prm(g, 6, b, d);
    const double sm = prm(g, 7, b, d), sphi = prm(g, 9, b, d), inv2sphi = prm(g, 10, b, d);
    const double inv_s = prm(g, 11, b, d);
    const double vd = neg ? -u[0] : u[0], vg = neg ? -u[1] : u[1];
    const double vs = neg ? -u[2] : u[2], vb = neg ? -u[3] : u[3];
    const double vds = vd - vs;
    const double dp = tie_gt(vds, 0.0), dn = tie_gt(-vds, 0.0);
    double vtf, dvtf, vtr, dvtr, F, Fgs, Fds, R, Rgs, Rds;
    l1_vt(vs - vb, vt0, gamma, phi, sphi, inv2sphi, &vtf, &dvtf);
    l1_vt(vd - vb, vt0, gamma, phi, sphi, inv2sphi, &vtr, &dvtr);
    l1_side(vg - vs, fmax(vds, 0.0), vtf, k, lam, sm, inv_s, &F, &Fgs, &Fds);
    l1_side(vg - vd, fmax(-vds, 0.0), vtr, k, lam, sm, inv_s, &R, &Rgs, &Rds);
    I = F - R;
    gd = Fds * dp + Rgs + Rds * dn + Rgs * dvtr;
    gg = Fgs - Rgs;
    gs = -Fgs - Fds * dp - Fgs * dvtf - Rds * dn;
    gb = Fgs * dvtf - Rgs * dvtr;
  }
  if (wf) {
    fo[0 * n + d] = neg ? -I : I;
    fo[1 * n + d] = 0.0;
    fo[2 * n + d] = neg ? I : -I;
    fo[3 * n + d] = 0.0;
  }
  if (wq) {
    const double q_gs = cov_w * (u[1] - u[2]), q_gd = cov_w * (u[1] - u[0]);
    qo[0 * n + d] = -q_gd;
    qo[1 * n + d] = q_gs + q_gd;
    qo[2 * n + d] = -q_gs;
    qo[3 * n + d] = 0.0;
  }
  if (!wj) return;
  const JT ji[4] = {(JT)gd, (JT)gg, (JT)gs, (JT)gb};
  const JT cw = (JT)cov_w;
  const JT dq0[4] = {cw, -cw, JT(0), JT(0)};
  const JT dq1[4] = {-cw, JT(2) * cw, -cw, JT(0)};
  const JT dq2[4] = {JT(0), -cw, cw, JT(0)};
  const JT cfj = (JT)cf, cqj = (JT)cq;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    JT r0 = cf != 0.0 ? cfj * ji[j] : JT(0);
    JT r2 = cf != 0.0 ? cfj * -ji[j] : JT(0);
    JT r1 = JT(0);
    if (cq != 0.0) {
      r0 = r0 + cqj * dq0[j];
      r1 = r1 + cqj * dq1[j];
      r2 = r2 + cqj * dq2[j];
    }
    jo[(0 * 4 + j) * n + d] = r0;
    jo[(1 * 4 + j) * n + d] = r1;
    jo[(2 * 4 + j) * n + d] = r2;
    jo[(3 * 4 + j) * n + d] = JT(0);
  }
}

// Evaluate device d of group g (instance b) reading state zz; write its slots.
// fo/qo/jo point at the group's first slot in each contribution array.
// u: the device's local unknowns (terminal voltages, then internals).
// zz: the instance's state, read by the non-local kind for the other
// devices' unknowns.
template <typename JT>
__device__ __forceinline__ void eval_soa(const GroupDev& g, int b, int d, const double* u,
                                         double t, double cf, double cq, bool wf, bool wq,
                                         bool wj, double* fo, double* qo, JT* jo,
                                         const double* zz) {
  const int n = g.n;
  switch (g.kind) {
    case VXG_KIND_COUPLED_L: {  // u = (vp, vn, i); flux sum_e M_de i_e over the group
      const double ld = prm(g, 0, b, d), sd = prm(g, 1, b, d), kc = prm(g, 2, b, d);
      if (wf) {
        fo[d] = u[2];
        fo[n + d] = -u[2];
        fo[2 * n + d] = -(u[0] - u[1]);
      }
      if (wq) {
        double acc = 0.0;
        for (int e = 0; e < n; ++e)
          acc += (e == d ? ld : kc * (sd * prm(g, 1, b, e))) * zz[g.int_offset + e];
        qo[d] = 0.0;
        qo[n + d] = 0.0;
        qo[2 * n + d] = acc;
      }
      if (wj) {  // rows (p, n, i) of device d; columns (vp, vn, i) of every device e
        const long long W = 3LL * n;
        for (long long c = 0; c < 3 * W; ++c) jo[c * n + d] = JT(0);
        jo[(0 * W + 3 * d + 2) * n + d] = (JT)cf;
        jo[(1 * W + 3 * d + 2) * n + d] = (JT)(-cf);
        jo[(2 * W + 3 * d + 0) * n + d] = (JT)(-cf);
        jo[(2 * W + 3 * d + 1) * n + d] = (JT)cf;
        if (cq != 0.0)
          for (int e = 0; e < n; ++e)
            jo[(2 * W + 3 * e + 2) * n + d] =
                (JT)(cq * (e == d ? ld : kc * (sd * prm(g, 1, b, e))));
      }
      break;
    }
    case VXG_KIND_CONDUCTANCE: {
      const double gg = prm(g, 0, b, d);
      const double i = (u[0] - u[1]) * gg;
      if (wf) {
        fo[d] = i;
        fo[n + d] = -i;
      }
      if (wq) {
        qo[d] = 0.0;
        qo[n + d] = 0.0;
      }
      if (wj) {
        const JT a = cf != 0.0 ? (JT)(cf * gg) : JT(0);
        jo[d] = a;
        jo[n + d] = -a;
        jo[2 * n + d] = -a;
        jo[3 * n + d] = a;
      }
      break;
    }
    case VXG_KIND_CAPACITOR: {
      const double c = prm(g, 0, b, d);
      const double q = c * (u[0] - u[1]);
      if (wf) {
        fo[d] = 0.0;
        fo[n + d] = 0.0;
      }
      if (wq) {
        qo[d] = q;
        qo[n + d] = -q;
      }
      if (wj) {
        const JT a = cq != 0.0 ? (JT)(cq * c) : JT(0);
        jo[d] = a;
        jo[n + d] = -a;
        jo[2 * n + d] = -a;
        jo[3 * n + d] = a;
      }
      break;
    }
    case VXG_KIND_VSOURCE: {
      if (wf) {
        fo[d] = u[2];
        fo[n + d] = -u[2];
        fo[2 * n + d] = (u[0] - u[1]) - wave_value(g, b, d, t);
      }
      if (wq) {
        qo[d] = 0.0;
        qo[n + d] = 0.0;
        qo[2 * n + d] = 0.0;
      }
      if (wj) {  // rows (p, n, eq), cols (vp, vn, i)
        const JT a = (JT)cf;
#pragma unroll
        for (int e = 0; e < 9; ++e) jo[e * n + d] = JT(0);
        if (cf != 0.0) {
          jo[2 * n + d] = a;
          jo[5 * n + d] = -a;
          jo[6 * n + d] = a;
          jo[7 * n + d] = -a;
        }
      }
      break;
    }
    case VXG_KIND_ISOURCE: {
      if (wf) {
        const double i = wave_value(g, b, d, t);
        fo[d] = i;
        fo[n + d] = -i;
      }
      if (wq) {
        qo[d] = 0.0;
        qo[n + d] = 0.0;
      }
      if (wj) {
#pragma unroll
        for (int e = 0; e < 4; ++e) jo[e * n + d] = JT(0);
      }
      break;
    }
    case VXG_KIND_EKV:
      ekv_soa<JT>(g, b, d, u, cf, cq, wf, wq, wj, fo, qo, jo);
      break;
    case VXG_KIND_L1:
      l1_soa<JT>(g, b, d, u, cf, cq, wf, wq, wj, fo, qo, jo);
      break;
    case VXG_KIND_DIODE: {  // voltax/elements/semiconductor.py:17-70
      const double i_s = prm(g, 0, b, d), inv_nvt = prm(g, 1, b, d);
      const double tt = prm(g, 2, b, d), cj = prm(g, 3, b, d);
      const double v = u[0] - u[1], x = v * inv_nvt;
      const double e = exp(fmin(x, 40.0));
      // explin and its derivative (min splits 1/2 : 1/2 at x = 40, as jnp does)
      const double ex = x > 40.0 ? e * (1.0 + x - 40.0) : e;
      const double dex = x > 40.0 ? e : (x == 40.0 ? 0.5 * e : e);
      const double i = i_s * (ex - 1.0);
      const double q = tt * i + cj * v;
      if (wf) {
        fo[d] = i;
        fo[n + d] = -i;
      }
      if (wq) {
        qo[d] = q;
        qo[n + d] = -q;
      }
      if (wj) {
        const double gi = i_s * dex * inv_nvt;
        const JT a = (JT)(cf * gi + cq * (tt * gi + cj));
        jo[d] = a;
        jo[n + d] = -a;
        jo[2 * n + d] = -a;
        jo[3 * n + d] = a;
      }
      break;
    }
    case VXG_KIND_INDUCTOR: {  // voltax/elements/passive.py:62-87; u = (vp, vn, i)
      const double l = prm(g, 0, b, d), rs = prm(g, 1, b, d);
      if (wf) {
        fo[d] = u[2];
        fo[n + d] = -u[2];
        fo[2 * n + d] = rs * u[2] - (u[0] - u[1]);
      }
      if (wq) {
        qo[d] = 0.0;
        qo[n + d] = 0.0;
        qo[2 * n + d] = l * u[2];
      }
      if (wj) {  // rows (p, n, branch), cols (vp, vn, i)
        const JT a = (JT)cf;
        jo[0 * n + d] = JT(0);
        jo[1 * n + d] = JT(0);
        jo[2 * n + d] = a;
        jo[3 * n + d] = JT(0);
        jo[4 * n + d] = JT(0);
        jo[5 * n + d] = -a;
        jo[6 * n + d] = -a;
        jo[7 * n + d] = a;
        jo[8 * n + d] = (JT)(cf * rs + cq * l);
      }
      break;
    }
    case VXG_KIND_BJT: {  // voltax/elements/semiconductor.py:73-135, u = (vc, vb, ve)
      const double sg = prm(g, 0, b, d), i_s = prm(g, 1, b, d), inv_vt = prm(g, 2, b, d);
      const double ibf = prm(g, 3, b, d), ibr = prm(g, 4, b, d), ivaf = prm(g, 5, b, d);
      const double tf = prm(g, 6, b, d), tr = prm(g, 7, b, d);
      const double cje = prm(g, 8, b, d), cjc = prm(g, 9, b, d);
      const double vc = sg * u[0], vb = sg * u[1], ve = sg * u[2];
      const double vbe = vb - ve, vbc = vb - vc;
      const double xf = vbe * inv_vt, xr = vbc * inv_vt;
      const double ef = exp(fmin(xf, 40.0)), er = exp(fmin(xr, 40.0));
      const double exf = xf > 40.0 ? ef * (1.0 + xf - 40.0) : ef;
      const double exr = xr > 40.0 ? er * (1.0 + xr - 40.0) : er;
      const double i_f = i_s * (exf - 1.0), i_r = i_s * (exr - 1.0);
      const double early = 1.0 + (vbe - vbc) * ivaf;
      const double ic = (i_f - i_r) * early - i_r * ibr;
      const double ib = i_f * ibf + i_r * ibr;
      if (wf) {
        fo[d] = sg * ic;
        fo[n + d] = sg * ib;
        fo[2 * n + d] = sg * (-ic - ib);
      }
      const double q_be = tf * i_f + cje * vbe, q_bc = tr * i_r + cjc * vbc;
      if (wq) {
        qo[d] = sg * -q_bc;
        qo[n + d] = sg * (q_be + q_bc);
        qo[2 * n + d] = sg * -q_be;
      }
      if (wj) {
        const double gf = i_s * (xf == 40.0 ? 0.5 * ef : ef) * inv_vt;
        const double gr = i_s * (xr == 40.0 ? 0.5 * er : er) * inv_vt;
        const double dbe[3] = {0.0, 1.0, -1.0}, dbc[3] = {-1.0, 1.0, 0.0};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double dic = (gf * dbe[k] - gr * dbc[k]) * early +
                             (i_f - i_r) * ivaf * (dbe[k] - dbc[k]) - gr * ibr * dbc[k];
          const double dib = gf * ibf * dbe[k] + gr * ibr * dbc[k];
          const double dqbe = (tf * gf + cje) * dbe[k], dqbc = (tr * gr + cjc) * dbc[k];
          jo[(0 * 3 + k) * n + d] = (JT)(cf * dic + cq * -dqbc);
          jo[(1 * 3 + k) * n + d] = (JT)(cf * dib + cq * (dqbe + dqbc));
          jo[(2 * 3 + k) * n + d] = (JT)(cf * (-dic - dib) + cq * -dqbe);
        }
      }
      break;
    }
    case VXG_KIND_VCVS:   // voltax/elements/controlled.py:27-43, u = (p, n, cp, cn, i)
    case VXG_KIND_CCCS:   // controlled.py:63-79, u = (p, n, cp, cn, i_sense)
    case VXG_KIND_CCVS:   // controlled.py:82-98, u = (p, n, cp, cn, i, i_sense)
    case VXG_KIND_XFMR: {  // passive.py:90-129, u = (p1, n1, p2, n2, i1, i2)
      const int m = g.m;
      double I[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0};
      double J[36];  // cf dI/du + cq dQ/du, linear devices
#pragma unroll
      for (int e = 0; e < 36; ++e) J[e] = 0.0;
      const double p0 = prm(g, 0, b, d);
      if (g.kind == VXG_KIND_VCVS) {
        I[0] = u[4];
        I[1] = -u[4];
        I[4] = (u[0] - u[1]) - p0 * (u[2] - u[3]);
        J[0 * 5 + 4] = cf;
        J[1 * 5 + 4] = -cf;
        J[4 * 5 + 0] = cf;
        J[4 * 5 + 1] = -cf;
        J[4 * 5 + 2] = -cf * p0;
        J[4 * 5 + 3] = cf * p0;
      } else if (g.kind == VXG_KIND_CCCS) {
        I[0] = p0 * u[4];
        I[1] = -p0 * u[4];
        I[2] = u[4];
        I[3] = -u[4];
        I[4] = u[2] - u[3];
        J[0 * 5 + 4] = cf * p0;
        J[1 * 5 + 4] = -cf * p0;
        J[2 * 5 + 4] = cf;
        J[3 * 5 + 4] = -cf;
        J[4 * 5 + 2] = cf;
        J[4 * 5 + 3] = -cf;
      } else if (g.kind == VXG_KIND_CCVS) {
        I[0] = u[4];
        I[1] = -u[4];
        I[2] = u[5];
        I[3] = -u[5];
        I[4] = (u[0] - u[1]) - p0 * u[5];
        I[5] = u[2] - u[3];
        J[0 * 6 + 4] = cf;
        J[1 * 6 + 4] = -cf;
        J[2 * 6 + 5] = cf;
        J[3 * 6 + 5] = -cf;
        J[4 * 6 + 0] = cf;
        J[4 * 6 + 1] = -cf;
        J[4 * 6 + 5] = -cf * p0;
        J[5 * 6 + 2] = cf;
        J[5 * 6 + 3] = -cf;
      } else {  // transformer: rows [l1, l2, m]
        const double l2 = prm(g, 1, b, d), mm = prm(g, 2, b, d);
        I[0] = u[4];
        I[1] = -u[4];
        I[2] = u[5];
        I[3] = -u[5];
        I[4] = -(u[0] - u[1]);
        I[5] = -(u[2] - u[3]);
        Q[4] = p0 * u[4] + mm * u[5];
        Q[5] = mm * u[4] + l2 * u[5];
        J[0 * 6 + 4] = cf;
        J[1 * 6 + 4] = -cf;
        J[2 * 6 + 5] = cf;
        J[3 * 6 + 5] = -cf;
        J[4 * 6 + 0] = -cf;
        J[4 * 6 + 1] = cf;
        J[5 * 6 + 2] = -cf;
        J[5 * 6 + 3] = cf;
        J[4 * 6 + 4] = cq * p0;
        J[4 * 6 + 5] = cq * mm;
        J[5 * 6 + 4] = cq * mm;
        J[5 * 6 + 5] = cq * l2;
      }
      for (int i = 0; i < m; ++i) {
        if (wf) fo[i * n + d] = I[i];
        if (wq) qo[i * n + d] = Q[i];
      }
      if (wj)
        for (int e = 0; e < m * m; ++e) jo[e * n + d] = (JT)J[e];
      break;
    }
    case VXG_KIND_IDEAL_OPAMP: {  // voltax/elements/opamp.py:13-32, u = (inp, inn, out, i)
      if (wf) {
        fo[d] = 0.0;
        fo[n + d] = 0.0;
        fo[2 * n + d] = -u[3];
        fo[3 * n + d] = u[0] - u[1];
      }
      if (wq) {
#pragma unroll
        for (int e = 0; e < 4; ++e) qo[e * n + d] = 0.0;
      }
      if (wj) {
#pragma unroll
        for (int e = 0; e < 16; ++e) jo[e * n + d] = JT(0);
        jo[(2 * 4 + 3) * n + d] = (JT)(-cf);
        jo[(3 * 4 + 0) * n + d] = (JT)cf;
        jo[(3 * 4 + 1) * n + d] = (JT)(-cf);
      }
      break;
    }
    case VXG_KIND_OPAMP: {  // voltax/elements/opamp.py:35-103, u = (inp, inn, out, x)
      const double a0 = prm(g, 0, b, d), grout = prm(g, 1, b, d), tau = prm(g, 2, b, d);
      const double mid = prm(g, 3, b, d), half = prm(g, 4, b, d), ihalf = prm(g, 5, b, d);
      const double th = tanh((a0 * (u[0] - u[1]) - mid) * ihalf);
      if (wf) {
        fo[d] = 0.0;
        fo[n + d] = 0.0;
        fo[2 * n + d] = (u[2] - u[3]) * grout;
        fo[3 * n + d] = u[3] - (mid + half * th);
      }
      if (wq) {
        qo[d] = 0.0;
        qo[n + d] = 0.0;
        qo[2 * n + d] = 0.0;
        qo[3 * n + d] = tau * u[3];
      }
      if (wj) {
        const double ds = a0 * (1.0 - th * th);  // d clip(a0 vd) / d vd
#pragma unroll
        for (int e = 0; e < 16; ++e) jo[e * n + d] = JT(0);
        jo[(2 * 4 + 2) * n + d] = (JT)(cf * grout);
        jo[(2 * 4 + 3) * n + d] = (JT)(-cf * grout);
        jo[(3 * 4 + 0) * n + d] = (JT)(-cf * ds);
        jo[(3 * 4 + 1) * n + d] = (JT)(cf * ds);
        jo[(3 * 4 + 3) * n + d] = (JT)(cf + cq * tau);
      }
      break;
    }
    case VXG_KIND_SWITCH: {  // voltax/elements/switch.py:14-50, u = (p, n, cp, cn)
      const double lroff = prm(g, 0, b, d), lratio = prm(g, 1, b, d);
      const double vth = prm(g, 2, b, d), iw = prm(g, 3, b, d);
      double sp, on;
      softplus_and_sigmoid((u[2] - u[3] - vth) * iw, &sp, &on);
      const double gg = exp(-lroff + on * lratio);
      const double vpn = u[0] - u[1];
      const double i = gg * vpn;
      if (wf) {
        fo[d] = i;
        fo[n + d] = -i;
        fo[2 * n + d] = 0.0;
        fo[3 * n + d] = 0.0;
      }
      if (wq) {
#pragma unroll
        for (int e = 0; e < 4; ++e) qo[e * n + d] = 0.0;
      }
      if (wj) {
        const double dgc = gg * lratio * on * (1.0 - on) * iw * vpn;  // d i / d v_ctrl
#pragma unroll
        for (int e = 0; e < 16; ++e) jo[e * n + d] = JT(0);
        const double a = cf * gg, c = cf * dgc;
        jo[0 * n + d] = (JT)a;
        jo[1 * n + d] = (JT)(-a);
        jo[2 * n + d] = (JT)c;
        jo[3 * n + d] = (JT)(-c);
        jo[4 * n + d] = (JT)(-a);
        jo[5 * n + d] = (JT)a;
        jo[6 * n + d] = (JT)(-c);
        jo[7 * n + d] = (JT)c;
      }
      break;
    }
    case VXG_KIND_VCCS: {  // voltax/elements/controlled.py:46-60
      const double gm = prm(g, 0, b, d);
      const double i = gm * (u[2] - u[3]);
      if (wf) {
        fo[d] = i;
        fo[n + d] = -i;
        fo[2 * n + d] = 0.0;
        fo[3 * n + d] = 0.0;
      }
      if (wq) {
#pragma unroll
        for (int e = 0; e < 4; ++e) qo[e * n + d] = 0.0;
      }
      if (wj) {
        const JT a = (JT)(cf * gm);
#pragma unroll
        for (int e = 0; e < 16; ++e) jo[e * n + d] = JT(0);
        jo[2 * n + d] = a;
        jo[3 * n + d] = -a;
        jo[6 * n + d] = -a;
        jo[7 * n + d] = a;
      }
      break;
    }
  }
}

}  // namespace vxg

namespace vxg {
// Local unknowns of device d from the state, node table in global memory.
__device__ __forceinline__ void gather_u(const GroupDev& g, int d, const double* zz,
                                         double* u) {
#pragma unroll
  for (int i = 0; i < kMaxM; ++i) {
    if (i < g.T) {
      const int node = g.nodes[d * g.T + i];
      u[i] = node >= 0 ? zz[node] : 0.0;
    } else if (i < g.m) {
      u[i] = zz[g.int_offset + d * g.K + (i - g.T)];
    } else {
      u[i] = 0.0;
    }
  }
}
}  // namespace vxg
