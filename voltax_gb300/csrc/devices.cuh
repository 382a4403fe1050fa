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
//   waveforms    voltax/signals.py:58-114
// voltax differentiates these by forward-mode AD; the derivatives below are
// the same chain rule written out by hand.
#pragma once

#include "internal.cuh"

namespace vxg {

struct DevEval {
  double I[kMaxM];
  double Q[kMaxM];
  double J[kMaxM * kMaxM];
};

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

struct EkvIn {
  double sign, i_spec, vth, dvth, n, vt, lam, c_ox, cov_w;
};

__device__ __forceinline__ EkvIn ekv_params(const GroupDev& g, int b, int d) {
  EkvIn p;
  p.sign = prm(g, 0, b, d);
  p.i_spec = prm(g, 1, b, d);
  p.vth = prm(g, 2, b, d);
  p.dvth = prm(g, 3, b, d);
  p.n = prm(g, 4, b, d);
  p.vt = prm(g, 5, b, d);
  p.lam = prm(g, 6, b, d);
  p.c_ox = prm(g, 7, b, d);
  p.cov_w = prm(g, 8, b, d);
  return p;
}

// EKV in the n-frame. x = (vd, vg, vs, vb) mirrored voltages. Outputs the
// drain current, the four charges and their derivatives d/dx_k. Because the
// device output is sign * F(sign * v), d output / d v = dF/dx: the
// derivatives need no sign.
__device__ inline void ekv_eval(const EkvIn& p, const double x[4], bool want_i, bool want_q,
                         double* ids, double dids[4], double q[4], double dq[4][4]) {
  const double vd = x[0], vg = x[1], vs = x[2], vb = x[3];
  const double two_vt = 2.0 * p.vt;
  const double vp = (vg - vb - p.vth - p.dvth) / p.n;
  const double af = (vp - (vs - vb)) / two_vt;
  const double ar = (vp - (vd - vb)) / two_vt;
  double spf, sgf, spr, sgr;
  softplus_and_sigmoid(af, &spf, &sgf);
  softplus_and_sigmoid(ar, &spr, &sgr);
  const double i_f = spf * spf, i_r = spr * spr;
  const double dif = 2.0 * spf * sgf, dir = 2.0 * spr * sgr;  // d i / d a
  // d a / d (vd, vg, vs, vb)
  const double dvp_g = 1.0 / p.n;
  const double daf[4] = {0.0, dvp_g / two_vt, -1.0 / two_vt, (1.0 - dvp_g) / two_vt};
  const double dar[4] = {-1.0 / two_vt, dvp_g / two_vt, 0.0, (1.0 - dvp_g) / two_vt};
  if (want_i) {
    const double vds = vd - vs;
    const double root = sqrt(vds * vds + 1e-3 * 1e-3);
    const double sabs = root - 1e-3;
    const double dsabs = vds / root;
    const double mfac = 1.0 + p.lam * sabs;
    *ids = p.i_spec * (i_f - i_r) * mfac;
    const double dmf[4] = {p.lam * dsabs, 0.0, -p.lam * dsabs, 0.0};
    for (int k = 0; k < 4; ++k)
      dids[k] = p.i_spec * ((dif * daf[k] - dir * dar[k]) * mfac + (i_f - i_r) * dmf[k]);
  }
  if (want_q) {
    const double xf = sqrt(0.25 + i_f), xr = sqrt(0.25 + i_r);
    const double scale = p.c_ox * p.n * p.vt;
    const double s = xf + xr;
    const double s2 = s * s;
    const double c415 = 4.0 / 15.0;
    const double nd = 3 * xr * xr * xr + 6 * xr * xr * xf + 4 * xr * xf * xf + 2 * xf * xf * xf;
    const double ns = 3 * xf * xf * xf + 6 * xf * xf * xr + 4 * xf * xr * xr + 2 * xr * xr * xr;
    const double q_d = -scale * (c415 * nd / s2 - 0.5);
    const double q_s = -scale * (c415 * ns / s2 - 0.5);
    const double q_i = q_d + q_s;
    const double kb = -(p.n - 1.0) / p.n;
    const double q_b = kb * (p.c_ox * (vg - vb) + q_i);
    const double q_g = -(q_i + q_b);
    const double q_gs = p.cov_w * (vg - vs), q_gd = p.cov_w * (vg - vd);
    q[0] = q_d + -q_gd;
    q[1] = q_g + (q_gs + q_gd);
    q[2] = q_s + -q_gs;
    q[3] = q_b + 0.0;
    // derivatives of N/s^2 with respect to xf, xr
    const double s3 = s2 * s;
    const double dnd_f = 6 * xr * xr + 8 * xr * xf + 6 * xf * xf;
    const double dnd_r = 9 * xr * xr + 12 * xr * xf + 4 * xf * xf;
    const double dns_f = 9 * xf * xf + 12 * xf * xr + 4 * xr * xr;
    const double dns_r = 6 * xf * xf + 8 * xf * xr + 6 * xr * xr;
    const double gd_f = (dnd_f * s - 2 * nd) / s3, gd_r = (dnd_r * s - 2 * nd) / s3;
    const double gs_f = (dns_f * s - 2 * ns) / s3, gs_r = (dns_r * s - 2 * ns) / s3;
    const double dxf_da = dif / (2.0 * xf), dxr_da = dir / (2.0 * xr);
    for (int k = 0; k < 4; ++k) {
      const double dxf = dxf_da * daf[k], dxr = dxr_da * dar[k];
      const double dqd = -scale * c415 * (gd_f * dxf + gd_r * dxr);
      const double dqs = -scale * c415 * (gs_f * dxf + gs_r * dxr);
      const double dqi = dqd + dqs;
      const double dvgb = (k == 1 ? 1.0 : 0.0) - (k == 3 ? 1.0 : 0.0);
      const double dqb = kb * (p.c_ox * dvgb + dqi);
      const double dqg = -(dqi + dqb);
      const double dgs = p.cov_w * ((k == 1 ? 1.0 : 0.0) - (k == 2 ? 1.0 : 0.0));
      const double dgd = p.cov_w * ((k == 1 ? 1.0 : 0.0) - (k == 0 ? 1.0 : 0.0));
      dq[0][k] = dqd - dgd;
      dq[1][k] = dqg + (dgs + dgd);
      dq[2][k] = dqs - dgs;
      dq[3][k] = dqb;
    }
  }
}

// Evaluate device d of group g for instance b. u holds the m local unknowns.
__device__ inline void eval_device(const GroupDev& g, int b, int d, const double* u, double t,
                            double cf, double cq, bool want_f, bool want_q, bool want_j,
                            DevEval& o) {
  const int m = g.m;
  for (int i = 0; i < m; ++i) {
    o.I[i] = 0.0;
    o.Q[i] = 0.0;
  }
  for (int i = 0; i < m * m; ++i) o.J[i] = 0.0;
  switch (g.kind) {
    case VXG_KIND_CONDUCTANCE: {
      const double gg = prm(g, 0, b, d);
      const double i = (u[0] - u[1]) * gg;
      o.I[0] = i;
      o.I[1] = -i;
      if (want_j && cf != 0.0) {
        const double a = cf * gg;
        o.J[0] = a;
        o.J[1] = -a;
        o.J[2] = -a;
        o.J[3] = a;
      }
      break;
    }
    case VXG_KIND_CAPACITOR: {
      const double c = prm(g, 0, b, d);
      const double q = c * (u[0] - u[1]);
      o.Q[0] = q;
      o.Q[1] = -q;
      if (want_j && cq != 0.0) {
        const double a = cq * c;
        o.J[0] = a;
        o.J[1] = -a;
        o.J[2] = -a;
        o.J[3] = a;
      }
      break;
    }
    case VXG_KIND_VSOURCE: {
      const double i = u[2];
      o.I[0] = i;
      o.I[1] = -i;
      o.I[2] = (u[0] - u[1]) - wave_value(g, b, d, t);
      if (want_j && cf != 0.0) {  // rows (p, n, eq), cols (vp, vn, i)
        o.J[0 * 3 + 2] = cf;
        o.J[1 * 3 + 2] = -cf;
        o.J[2 * 3 + 0] = cf;
        o.J[2 * 3 + 1] = -cf;
      }
      break;
    }
    case VXG_KIND_ISOURCE: {
      const double i = wave_value(g, b, d, t);
      o.I[0] = i;
      o.I[1] = -i;
      break;
    }
    case VXG_KIND_EKV: {
      const EkvIn p = ekv_params(g, b, d);
      double x[4];
      for (int k = 0; k < 4; ++k) x[k] = p.sign * u[k];
      const bool need_i = want_f || (want_j && cf != 0.0);
      const bool need_q = want_q || (want_j && cq != 0.0);
      double ids = 0.0, dids[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0}, dq[4][4];
      ekv_eval(p, x, need_i, need_q, &ids, dids, q, dq);
      if (need_i) {
        o.I[0] = p.sign * ids;
        o.I[2] = p.sign * -ids;
        o.I[1] = p.sign * 0.0;
        o.I[3] = p.sign * 0.0;
      }
      if (need_q)
        for (int k = 0; k < 4; ++k) o.Q[k] = p.sign * q[k];
      if (want_j) {
        for (int j = 0; j < 4; ++j) {
          double jd = 0.0, js = 0.0;
          if (cf != 0.0) {
            jd = cf * dids[j];
            js = cf * -dids[j];
          }
          double r0 = jd, r1 = 0.0, r2 = js, r3 = 0.0;
          if (cq != 0.0) {
            r0 = r0 + cq * dq[0][j];
            r1 = r1 + cq * dq[1][j];
            r2 = r2 + cq * dq[2][j];
            r3 = r3 + cq * dq[3][j];
          }
          o.J[0 * 4 + j] = r0;
          o.J[1 * 4 + j] = r1;
          o.J[2 * 4 + j] = r2;
          o.J[3 * 4 + j] = r3;
        }
      }
      break;
    }
  }
}

}  // namespace vxg
