/*
 * cvx.c -- compiled CPU restatement of the voltax Newton loop, used as the
 * timed CPU baseline (TEST INFRASTRUCTURE: only tests/, the smoke check and
 * bench.py's CPU legs call it; the product never does).
 *
 * One circuit instance, FP64 throughout, single-threaded:
 *   device physics + local Jacobians   voltax/elements/{passive,sources,mosfet}.py,
 *                                      voltax/signals.py:58-114 (derivatives by
 *                                      hand; voltax uses forward-mode AD)
 *   stamping (sequential, canonical    voltax/sparse.py:220-249, circuit.py:209-226
 *   group/device/row/column order)
 *   block-LDU refactorization per      voltax/sparse.py:543-572 (per supernode in
 *   supernode, partial pivoting in     postorder rather than padded per-level
 *   the pivot block; solves            batches, i.e. without the padding work)
 *                                      voltax/sparse.py:575-595
 *   damped Newton, gmin stepping,      voltax/analysis.py:208-266, 333-378,
 *   DC, BE / trapezoidal transient     410-480
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { K_COND = 0, K_CAP = 1, K_VSRC = 2, K_ISRC = 3, K_EKV = 4, K_L1 = 5,
       K_DIODE = 6, K_IND = 7, K_VCCS = 8, K_BJT = 9, K_VCVS = 10, K_CCCS = 11,
       K_CCVS = 12, K_XFMR = 13, K_IOPAMP = 14, K_OPAMP = 15, K_SWITCH = 16 };
enum { W_CONST = 0, W_STEP = 1, W_PULSE = 2 };
enum { M_DC = 0, M_BE = 1, M_TRAP = 2 };

typedef struct {
  int kind, n, T, K, wave, n_params, int_offset;
  const int* nodes;     /* n*T, -1 = ground */
  const double* params; /* n_params rows of n values */
  const int* jpos;      /* n*m*m pattern positions, nnz = dropped */
} cvx_group;

typedef struct {
  int S, nv, nnz, n_groups;
  const cvx_group* groups;
  const long long* indptr;
  const int* indices;
  const int* rows;
  int n_sn;
  const int* k;
  const int* r;
  const long long* panel;
  const long long* piv_ptr;
  const int* piv;
  const long long* bord_ptr;
  const int* bord;
  const long long* a_pos;
  long long work;
  const long long* schur_ptr; /* n_sn+1 */
  const long long* schur_tgt; /* per supernode r*r panel positions */
} cvx_sys;

typedef struct {
  int max_steps;
  double rtol, atol, max_dv, gmin;
  int gmin_steps, direct_steps;
  const double* gmins; /* gmin_steps + 1 */
} cvx_opts;

/* ------------------------------------------------------------- waveforms */
static double clamp01(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }

static double py_mod(double x, double y) {
  double r = fmod(x, y);
  if (r != 0.0 && ((r < 0.0) != (y < 0.0))) r += y;
  return r;
}

static double wave(const cvx_group* g, int d, double t) {
  const double* p = g->params;
  const int n = g->n;
  if (g->wave == W_CONST) return p[d];
  if (g->wave == W_STEP) {
    double v0 = p[d], v1 = p[n + d], delay = p[2 * n + d], rise = p[3 * n + d];
    return v0 + (v1 - v0) * clamp01((t - delay) / rise);
  }
  {
    double v1 = p[d], v2 = p[n + d], delay = p[2 * n + d], rise = p[3 * n + d];
    double fall = p[4 * n + d], width = p[5 * n + d], period = p[6 * n + d];
    double tc = py_mod(t - delay, period);
    double up = clamp01(tc / (rise + 1e-30));
    double tfe = rise + width + fall;
    double down = clamp01((tfe - tc) / (fall + 1e-30));
    double value = v1 + (v2 - v1) * (up < down ? up : down);
    return t < delay ? v1 : value;
  }
}

/* ----------------------------------------------------------------- EKV */
static void softplus2(double x, double* sp, double* sg) {
  double e = exp(-fabs(x));
  *sp = (x > 0.0 ? x : 0.0) + log1p(e);
  *sg = x >= 0.0 ? 1.0 / (1.0 + e) : e / (1.0 + e);
}

/* outputs I, Q (4) and J = cf dI/dv + cq dQ/dv (4x4) of one EKV device */
static void ekv(const cvx_group* g, int d, const double* v, double cf, double cq, int wj,
                double* I, double* Q, double* J) {
  const double* p = g->params;
  const int n = g->n;
  const double sign = p[d], i_spec = p[n + d], vth = p[2 * n + d], dvth = p[3 * n + d];
  const double nn = p[4 * n + d], vt = p[5 * n + d], lam = p[6 * n + d];
  const double c_ox = p[7 * n + d], cov_w = p[8 * n + d];
  const double vd = sign * v[0], vg = sign * v[1], vs = sign * v[2], vb = sign * v[3];
  const double two_vt = 2.0 * vt;
  const double vp = (vg - vb - vth - dvth) / nn;
  double spf, sgf, spr, sgr;
  softplus2((vp - (vs - vb)) / two_vt, &spf, &sgf);
  softplus2((vp - (vd - vb)) / two_vt, &spr, &sgr);
  const double i_f = spf * spf, i_r = spr * spr;
  const double dif = 2.0 * spf * sgf, dir = 2.0 * spr * sgr;
  const double g1 = 1.0 / nn;
  const double daf[4] = {0.0, g1 / two_vt, -1.0 / two_vt, (1.0 - g1) / two_vt};
  const double dar[4] = {-1.0 / two_vt, g1 / two_vt, 0.0, (1.0 - g1) / two_vt};
  const double vds = vd - vs;
  const double root = sqrt(vds * vds + 1e-3 * 1e-3);
  const double mfac = 1.0 + lam * (root - 1e-3);
  const double ids = i_spec * (i_f - i_r) * mfac;
  const double dsa = vds / root;
  const double dmf[4] = {lam * dsa, 0.0, -lam * dsa, 0.0};
  I[0] = sign * ids;
  I[1] = 0.0;
  I[2] = sign * -ids;
  I[3] = 0.0;
  const double xf = sqrt(0.25 + i_f), xr = sqrt(0.25 + i_r);
  const double scale = c_ox * nn * vt;
  const double s = xf + xr, s2 = s * s, s3 = s2 * s;
  const double c415 = 4.0 / 15.0;
  const double nd = 3 * xr * xr * xr + 6 * xr * xr * xf + 4 * xr * xf * xf + 2 * xf * xf * xf;
  const double ns = 3 * xf * xf * xf + 6 * xf * xf * xr + 4 * xf * xr * xr + 2 * xr * xr * xr;
  const double q_d = -scale * (c415 * nd / s2 - 0.5);
  const double q_s = -scale * (c415 * ns / s2 - 0.5);
  const double q_i = q_d + q_s;
  const double kb = -(nn - 1.0) / nn;
  const double q_b = kb * (c_ox * (vg - vb) + q_i);
  const double q_g = -(q_i + q_b);
  const double q_gs = cov_w * (vg - vs), q_gd = cov_w * (vg - vd);
  Q[0] = sign * (q_d - q_gd);
  Q[1] = sign * (q_g + (q_gs + q_gd));
  Q[2] = sign * (q_s - q_gs);
  Q[3] = sign * q_b;
  if (!wj) return;
  const double gd_f = ((6 * xr * xr + 8 * xr * xf + 6 * xf * xf) * s - 2 * nd) / s3;
  const double gd_r = ((9 * xr * xr + 12 * xr * xf + 4 * xf * xf) * s - 2 * nd) / s3;
  const double gs_f = ((9 * xf * xf + 12 * xf * xr + 4 * xr * xr) * s - 2 * ns) / s3;
  const double gs_r = ((6 * xf * xf + 8 * xf * xr + 6 * xr * xr) * s - 2 * ns) / s3;
  const double dxf_da = dif / (2.0 * xf), dxr_da = dir / (2.0 * xr);
  for (int kk = 0; kk < 4; ++kk) {
    const double dids = i_spec * ((dif * daf[kk] - dir * dar[kk]) * mfac + (i_f - i_r) * dmf[kk]);
    const double dxf = dxf_da * daf[kk], dxr = dxr_da * dar[kk];
    const double dqd = -scale * c415 * (gd_f * dxf + gd_r * dxr);
    const double dqs = -scale * c415 * (gs_f * dxf + gs_r * dxr);
    const double dqi = dqd + dqs;
    const double dvgb = (kk == 1 ? 1.0 : 0.0) - (kk == 3 ? 1.0 : 0.0);
    const double dqb = kb * (c_ox * dvgb + dqi);
    const double dqg = -(dqi + dqb);
    const double dgs = cov_w * ((kk == 1 ? 1.0 : 0.0) - (kk == 2 ? 1.0 : 0.0));
    const double dgd = cov_w * ((kk == 1 ? 1.0 : 0.0) - (kk == 0 ? 1.0 : 0.0));
    J[0 * 4 + kk] = cf * dids + cq * (dqd - dgd);
    J[1 * 4 + kk] = cq * (dqg + (dgs + dgd));
    J[2 * 4 + kk] = cf * -dids + cq * (dqs - dgs);
    J[3 * 4 + kk] = cq * dqb;
  }
}

/* Level 1 MOSFET (voltax/elements/mosfet.py:208-257); max/min split the
 * derivative 1/2 : 1/2 at a tie, as jnp.maximum / jnp.minimum do. Rows: sign,
 * kp W/L, vth, dvth, lam, gamma, phi, smooth, cov W (then derived rows). */
static double tie_gt(double a, double b) { return a > b ? 1.0 : (a == b ? 0.5 : 0.0); }

static void l1_vt(double vsb, double vt0, double gamma, double phi, double* vt, double* dvt) {
  if (gamma == 0.0) { *vt = vt0; *dvt = 0.0; return; }
  const double sphi = sqrt(phi);
  double root, droot;
  if (vsb >= 0.0) {
    root = sqrt(phi + fmax(vsb, 0.0));
    droot = tie_gt(vsb, 0.0) * 0.5 / root;
  } else {
    const double lin = sphi + vsb / (2.0 * sphi);
    root = fmax(lin, 0.0);
    droot = tie_gt(lin, 0.0) / (2.0 * sphi);
  }
  *vt = vt0 + gamma * (root - sphi);
  *dvt = gamma * droot;
}

static void l1_side(double vgs, double vds, double vt, double k, double lam, double s,
                    double* f, double* fgs, double* fds) {
  const double x = vgs - vt;
  double vov, dvov;
  if (s > 0.0) {
    double sp, sg;
    softplus2(x / s, &sp, &sg);
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

static void level1(const cvx_group* g, int d, const double* v, double cf, double cq,
                   double* I, double* Q, double* J) {
  const double* p = g->params;
  const int n = g->n;
  const double sign = p[d], k = p[n + d], vt0 = p[2 * n + d] + p[3 * n + d];
  const double lam = p[4 * n + d], gamma = p[5 * n + d], phi = p[6 * n + d];
  const double sm = p[7 * n + d], cov_w = p[8 * n + d];
  const double vd = sign * v[0], vg = sign * v[1], vs = sign * v[2], vb = sign * v[3];
  const double vds = vd - vs;
  const double dp = tie_gt(vds, 0.0), dn = tie_gt(-vds, 0.0);
  double vtf, dvtf, vtr, dvtr, F, Fgs, Fds, R, Rgs, Rds;
  l1_vt(vs - vb, vt0, gamma, phi, &vtf, &dvtf);
  l1_vt(vd - vb, vt0, gamma, phi, &vtr, &dvtr);
  l1_side(vg - vs, fmax(vds, 0.0), vtf, k, lam, sm, &F, &Fgs, &Fds);
  l1_side(vg - vd, fmax(-vds, 0.0), vtr, k, lam, sm, &R, &Rgs, &Rds);
  const double ids = F - R;
  const double gi[4] = {Fds * dp + Rgs + Rds * dn + Rgs * dvtr, Fgs - Rgs,
                        -Fgs - Fds * dp - Fgs * dvtf - Rds * dn, Fgs * dvtf - Rgs * dvtr};
  I[0] = sign * ids;
  I[1] = 0.0;
  I[2] = sign * -ids;
  I[3] = 0.0;
  const double q_gs = cov_w * (v[1] - v[2]), q_gd = cov_w * (v[1] - v[0]);
  Q[0] = -q_gd;
  Q[1] = q_gs + q_gd;
  Q[2] = -q_gs;
  Q[3] = 0.0;
  const double dq0[4] = {cov_w, -cov_w, 0.0, 0.0};
  const double dq1[4] = {-cov_w, 2.0 * cov_w, -cov_w, 0.0};
  const double dq2[4] = {0.0, -cov_w, cov_w, 0.0};
  for (int kk = 0; kk < 4; ++kk) {
    J[0 * 4 + kk] = cf * gi[kk] + cq * dq0[kk];
    J[1 * 4 + kk] = cq * dq1[kk];
    J[2 * 4 + kk] = cf * -gi[kk] + cq * dq2[kk];
    J[3 * 4 + kk] = 0.0;
  }
}

/* f (cf_on), q and the CSR Jacobian (cf df + cq dq + gmin on node diagonals) */
static void stamp(const cvx_sys* s, const double* z, double t, double cf, double cq,
                  double gmin, double* f, double* q, double* data) {
  const int S = s->S;
  if (f) memset(f, 0, sizeof(double) * S);
  if (q) memset(q, 0, sizeof(double) * S);
  if (data) memset(data, 0, sizeof(double) * (s->nnz + 1));
  for (int gi = 0; gi < s->n_groups; ++gi) {
    const cvx_group* g = &s->groups[gi];
    const int m = g->T + g->K;
    for (int d = 0; d < g->n; ++d) {
      double u[6], I[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, J[36];
      int row[6];
      for (int i = 0; i < g->T; ++i) {
        const int nd = g->nodes[d * g->T + i];
        u[i] = nd >= 0 ? z[nd] : 0.0;
        row[i] = nd;
      }
      for (int i = 0; i < g->K; ++i) {
        row[g->T + i] = g->int_offset + d * g->K + i;
        u[g->T + i] = z[row[g->T + i]];
      }
      memset(J, 0, sizeof(J));
      switch (g->kind) {
        case K_COND: {
          const double gg = g->params[d], i = (u[0] - u[1]) * gg;
          I[0] = i;
          I[1] = -i;
          J[0] = cf * gg; J[1] = -cf * gg; J[2] = -cf * gg; J[3] = cf * gg;
          break;
        }
        case K_CAP: {
          const double c = g->params[d], qq = c * (u[0] - u[1]);
          Q[0] = qq;
          Q[1] = -qq;
          J[0] = cq * c; J[1] = -cq * c; J[2] = -cq * c; J[3] = cq * c;
          break;
        }
        case K_VSRC:
          I[0] = u[2];
          I[1] = -u[2];
          I[2] = (u[0] - u[1]) - wave(g, d, t);
          J[2] = cf; J[5] = -cf; J[6] = cf; J[7] = -cf;
          break;
        case K_ISRC: {
          const double i = wave(g, d, t);
          I[0] = i;
          I[1] = -i;
          break;
        }
        case K_EKV:
          ekv(g, d, u, cf, cq, data != 0, I, Q, J);
          break;
        case K_L1:
          level1(g, d, u, cf, cq, I, Q, J);
          break;
        case K_DIODE: { /* rows: is, 1/(n vt), tt, cj */
          const double* p = g->params;
          const int n = g->n;
          const double is = p[d], inv = p[n + d], tt = p[2 * n + d], cj = p[3 * n + d];
          const double v = u[0] - u[1], x = v * inv, e = exp(fmin(x, 40.0));
          const double ex = x > 40.0 ? e * (1.0 + x - 40.0) : e;
          const double dex = x == 40.0 ? 0.5 * e : e;
          const double i = is * (ex - 1.0), gi = is * dex * inv;
          I[0] = i; I[1] = -i;
          Q[0] = tt * i + cj * v; Q[1] = -Q[0];
          const double a = cf * gi + cq * (tt * gi + cj);
          J[0] = a; J[1] = -a; J[2] = -a; J[3] = a;
          break;
        }
        case K_IND: { /* rows: l, rs; local unknowns (vp, vn, i) */
          const double l = g->params[d], rs = g->params[g->n + d];
          I[0] = u[2]; I[1] = -u[2]; I[2] = rs * u[2] - (u[0] - u[1]);
          Q[2] = l * u[2];
          J[2] = cf; J[5] = -cf; J[6] = -cf; J[7] = cf; J[8] = cf * rs + cq * l;
          break;
        }
        case K_BJT: { /* rows: sign, is, 1/vt, 1/bf, 1/br, 1/vaf, tf, tr, cje, cjc */
          const double* p = g->params;
          const int n = g->n;
          const double sg = p[d], is = p[n + d], ivt = p[2 * n + d], ibf = p[3 * n + d];
          const double ibr = p[4 * n + d], ivaf = p[5 * n + d], tf = p[6 * n + d];
          const double tr = p[7 * n + d], cje = p[8 * n + d], cjc = p[9 * n + d];
          const double vbe = sg * (u[1] - u[2]), vbc = sg * (u[1] - u[0]);
          const double xf = vbe * ivt, xr = vbc * ivt;
          const double ef = exp(fmin(xf, 40.0)), er = exp(fmin(xr, 40.0));
          const double i_f = is * ((xf > 40.0 ? ef * (1.0 + xf - 40.0) : ef) - 1.0);
          const double i_r = is * ((xr > 40.0 ? er * (1.0 + xr - 40.0) : er) - 1.0);
          const double early = 1.0 + (vbe - vbc) * ivaf;
          const double ic = (i_f - i_r) * early - i_r * ibr, ib = i_f * ibf + i_r * ibr;
          I[0] = sg * ic; I[1] = sg * ib; I[2] = sg * (-ic - ib);
          const double q_be = tf * i_f + cje * vbe, q_bc = tr * i_r + cjc * vbc;
          Q[0] = sg * -q_bc; Q[1] = sg * (q_be + q_bc); Q[2] = sg * -q_be;
          const double gf = is * (xf == 40.0 ? 0.5 * ef : ef) * ivt;
          const double gr = is * (xr == 40.0 ? 0.5 * er : er) * ivt;
          const double dbe[3] = {0.0, 1.0, -1.0}, dbc[3] = {-1.0, 1.0, 0.0};
          for (int kk = 0; kk < 3; ++kk) {
            const double dic = (gf * dbe[kk] - gr * dbc[kk]) * early +
                               (i_f - i_r) * ivaf * (dbe[kk] - dbc[kk]) - gr * ibr * dbc[kk];
            const double dib = gf * ibf * dbe[kk] + gr * ibr * dbc[kk];
            const double dqbe = (tf * gf + cje) * dbe[kk], dqbc = (tr * gr + cjc) * dbc[kk];
            J[0 * 3 + kk] = cf * dic - cq * dqbc;
            J[1 * 3 + kk] = cf * dib + cq * (dqbe + dqbc);
            J[2 * 3 + kk] = cf * (-dic - dib) - cq * dqbe;
          }
          break;
        }
        case K_VCVS: { /* (p, n, cp, cn, i) */
          const double a = g->params[d];
          I[0] = u[4]; I[1] = -u[4]; I[4] = (u[0] - u[1]) - a * (u[2] - u[3]);
          J[4] = cf; J[9] = -cf; J[20] = cf; J[21] = -cf; J[22] = -cf * a; J[23] = cf * a;
          break;
        }
        case K_CCCS: { /* (p, n, cp, cn, i_sense) */
          const double a = g->params[d];
          I[0] = a * u[4]; I[1] = -a * u[4]; I[2] = u[4]; I[3] = -u[4]; I[4] = u[2] - u[3];
          J[4] = cf * a; J[9] = -cf * a; J[14] = cf; J[19] = -cf; J[22] = cf; J[23] = -cf;
          break;
        }
        case K_CCVS: { /* (p, n, cp, cn, i, i_sense) */
          const double r = g->params[d];
          I[0] = u[4]; I[1] = -u[4]; I[2] = u[5]; I[3] = -u[5];
          I[4] = (u[0] - u[1]) - r * u[5]; I[5] = u[2] - u[3];
          J[4] = cf; J[10] = -cf; J[17] = cf; J[23] = -cf;
          J[24] = cf; J[25] = -cf; J[29] = -cf * r; J[32] = cf; J[33] = -cf;
          break;
        }
        case K_XFMR: { /* (p1, n1, p2, n2, i1, i2); rows l1, l2, m */
          const int nn = g->n;
          const double l1 = g->params[d], l2 = g->params[nn + d], mm = g->params[2 * nn + d];
          I[0] = u[4]; I[1] = -u[4]; I[2] = u[5]; I[3] = -u[5];
          I[4] = -(u[0] - u[1]); I[5] = -(u[2] - u[3]);
          Q[4] = l1 * u[4] + mm * u[5]; Q[5] = mm * u[4] + l2 * u[5];
          J[4] = cf; J[10] = -cf; J[17] = cf; J[23] = -cf;
          J[24] = -cf; J[25] = cf; J[32] = -cf; J[33] = cf;
          J[28] = cq * l1; J[29] = cq * mm; J[34] = cq * mm; J[35] = cq * l2;
          break;
        }
        case K_IOPAMP: /* (inp, inn, out, i_out) */
          I[2] = -u[3]; I[3] = u[0] - u[1];
          J[11] = -cf; J[12] = cf; J[13] = -cf;
          break;
        case K_OPAMP: { /* rows a0, 1/rout, tau, mid, half, 1/half; (inp, inn, out, x) */
          const double* p = g->params;
          const int nn = g->n;
          const double a0 = p[d], gr = p[nn + d], tau = p[2 * nn + d], mid = p[3 * nn + d];
          const double half = p[4 * nn + d];
          const double th = tanh((a0 * (u[0] - u[1]) - mid) / half);
          I[2] = (u[2] - u[3]) * gr; I[3] = u[3] - (mid + half * th);
          Q[3] = tau * u[3];
          const double ds = a0 * (1.0 - th * th);
          J[10] = cf * gr; J[11] = -cf * gr; J[12] = -cf * ds; J[13] = cf * ds; J[15] = cf + cq * tau;
          break;
        }
        case K_SWITCH: { /* rows log roff, log(roff/ron), vth, 1/vwidth; (p, n, cp, cn) */
          const double* p = g->params;
          const int nn = g->n;
          const double lroff = p[d], lrat = p[nn + d], vth = p[2 * nn + d], iw = p[3 * nn + d];
          double sp, on;
          softplus2((u[2] - u[3] - vth) * iw, &sp, &on);
          const double gg = exp(-lroff + on * lrat), vpn = u[0] - u[1];
          I[0] = gg * vpn; I[1] = -I[0];
          const double a = cf * gg, c = cf * gg * lrat * on * (1.0 - on) * iw * vpn;
          J[0] = a; J[1] = -a; J[2] = c; J[3] = -c; J[4] = -a; J[5] = a; J[6] = -c; J[7] = c;
          break;
        }
        case K_VCCS: {
          const double gm = g->params[d], i = gm * (u[2] - u[3]);
          I[0] = i; I[1] = -i;
          J[2] = cf * gm; J[3] = -cf * gm; J[6] = -cf * gm; J[7] = cf * gm;
          break;
        }
      }
      for (int i = 0; i < m; ++i) {
        if (row[i] < 0) continue;
        if (f) f[row[i]] += I[i];
        if (q) q[row[i]] += Q[i];
      }
      if (data) {
        const int* jp = g->jpos + (long long)d * m * m;
        for (int e = 0; e < m * m; ++e) data[jp[e]] += J[e];
      }
    }
  }
  if (data)
    for (int e = 0; e < s->nnz; ++e)
      if (s->rows[e] < s->nv && s->indices[e] == s->rows[e]) data[e] += gmin;
}

/* ------------------------------------------------------- factor / solve */
static void factor(const cvx_sys* s, const double* data, double* work, int* perm, double* tmp) {
  memset(work, 0, sizeof(double) * s->work);
  for (int e = 0; e < s->nnz; ++e) work[s->a_pos[e]] = data[e];
  for (int j = 0; j < s->n_sn; ++j) {
    const int k = s->k[j], r = s->r[j];
    double* A = work + s->panel[j];
    double* F12 = A + (long long)k * k;
    double* F21 = F12 + (long long)k * r;
    for (int c = 0; c < k; ++c) { /* Gauss-Jordan, partial pivoting */
      int p = c;
      double best = fabs(A[c * k + c]);
      for (int i = c + 1; i < k; ++i)
        if (fabs(A[i * k + c]) > best) { best = fabs(A[i * k + c]); p = i; }
      perm[c] = p;
      if (p != c)
        for (int jj = 0; jj < k; ++jj) { double t = A[p * k + jj]; A[p * k + jj] = A[c * k + jj]; A[c * k + jj] = t; }
      const double dd = A[c * k + c];
      A[c * k + c] = 1.0;
      for (int jj = 0; jj < k; ++jj) A[c * k + jj] /= dd;
      for (int i = 0; i < k; ++i) {
        if (i == c) continue;
        const double fct = A[i * k + c];
        A[i * k + c] = 0.0;
        for (int jj = 0; jj < k; ++jj) A[i * k + jj] -= fct * A[c * k + jj];
      }
    }
    for (int c = k - 1; c >= 0; --c)
      if (perm[c] != c)
        for (int i = 0; i < k; ++i) { double t = A[i * k + c]; A[i * k + c] = A[i * k + perm[c]]; A[i * k + perm[c]] = t; }
    if (!r) continue;
    /* Ub = W F12 */
    for (int cc = 0; cc < r; ++cc) {
      for (int l = 0; l < k; ++l) tmp[l] = F12[(long long)l * r + cc];
      for (int i = 0; i < k; ++i) {
        double acc = 0.0;
        for (int l = 0; l < k; ++l) acc += A[i * k + l] * tmp[l];
        F12[(long long)i * r + cc] = acc;
      }
    }
    /* Schur: work[target] -= F21 Ub; then Lb = F21 W */
    const long long* tg = s->schur_tgt + s->schur_ptr[j];
    for (int a = 0; a < r; ++a) {
      const double* row = F21 + (long long)a * k;
      for (int b = 0; b < r; ++b) {
        double acc = 0.0;
        for (int l = 0; l < k; ++l) acc += row[l] * F12[(long long)l * r + b];
        work[tg[(long long)a * r + b]] -= acc;
      }
      for (int jj = 0; jj < k; ++jj) {
        double acc = 0.0;
        for (int l = 0; l < k; ++l) acc += row[l] * A[l * k + jj];
        tmp[jj] = acc;
      }
      memcpy(F21 + (long long)a * k, tmp, sizeof(double) * k);
    }
  }
}

static void solve(const cvx_sys* s, const double* work, double* x, double* tmp) {
  for (int j = 0; j < s->n_sn; ++j) {
    const int k = s->k[j], r = s->r[j];
    const double* W = work + s->panel[j];
    const double* Lb = W + (long long)k * k + (long long)k * r;
    const int* piv = s->piv + s->piv_ptr[j];
    const int* brd = s->bord + s->bord_ptr[j];
    for (int l = 0; l < k; ++l) tmp[l] = x[piv[l]];
    for (int a = 0; a < r; ++a) {
      double acc = 0.0;
      for (int l = 0; l < k; ++l) acc += Lb[(long long)a * k + l] * tmp[l];
      x[brd[a]] -= acc;
    }
    for (int i = 0; i < k; ++i) {
      double acc = 0.0;
      for (int l = 0; l < k; ++l) acc += W[i * k + l] * tmp[l];
      x[piv[i]] = acc;
    }
  }
  for (int j = s->n_sn - 1; j >= 0; --j) {
    const int k = s->k[j], r = s->r[j];
    const double* Ub = work + s->panel[j] + (long long)k * k;
    const int* piv = s->piv + s->piv_ptr[j];
    const int* brd = s->bord + s->bord_ptr[j];
    for (int i = 0; i < k; ++i) {
      double acc = 0.0;
      for (int a = 0; a < r; ++a) acc += Ub[(long long)i * r + a] * x[brd[a]];
      x[piv[i]] -= acc;
    }
  }
}

/* ---------------------------------------------------------------- Newton */
typedef struct {
  double *f, *q, *fp, *qp, *data, *work, *dz, *tmp;
  int* perm;
} ws_t;

static int newton(const cvx_sys* s, const cvx_opts* o, ws_t* w, int mode, double t, double tp,
                  double gmin, int max_steps, double* z, int* iters) {
  const int S = s->S;
  const double cf = mode == M_TRAP ? 0.5 : 1.0;
  const double cq = mode == M_DC ? 0.0 : 1.0 / (t - tp);
  const double h = t - tp;
  int done = 0, it = 0;
  while (it < max_steps && !done) {
    stamp(s, z, t, cf, cq, gmin, w->f, mode == M_DC ? 0 : w->q, w->data);
    for (int i = 0; i < S; ++i) {
      const double gm = i < s->nv ? gmin * z[i] : 0.0;
      double r;
      if (mode == M_DC) r = w->f[i] + gm;
      else if (mode == M_BE) r = (w->q[i] - w->qp[i]) / h + w->f[i] + gm;
      else r = (w->q[i] - w->qp[i]) / h + 0.5 * (w->f[i] + w->fp[i]) + gm;
      w->dz[i] = -r;
    }
    factor(s, w->data, w->work, w->perm, w->tmp);
    solve(s, w->work, w->dz, w->tmp);
    double m = 0.0;
    int nan_seen = 0;
    for (int i = 0; i < s->nv; ++i) {
      const double v = fabs(w->dz[i]);
      if (isnan(v)) nan_seen = 1;
      else if (v > m) m = v;
    }
    const double dv = nan_seen ? NAN : m;
    const double qd = o->max_dv / (dv + 1e-300);
    const double scale = isnan(qd) ? qd : (qd < 1.0 ? qd : 1.0);
    int ok = 1;
    for (int i = 0; i < S; ++i) {
      const double zn = z[i] + scale * w->dz[i];
      if (!(fabs(w->dz[i]) <= o->atol + o->rtol * fabs(zn))) ok = 0;
      if (!isfinite(zn)) ok = 0;
      z[i] = zn;
    }
    done = ok && scale == 1.0;
    ++it;
  }
  *iters = it;
  return done;
}

int cvx_run(const cvx_sys* s, const cvx_opts* o, int mode, int n_t, const double* ts,
            const double* z0, int dc_first, double* z_out, int* conv, int* iters) {
  const int S = s->S;
  int maxk = 1;
  for (int j = 0; j < s->n_sn; ++j) {
    if (s->k[j] > maxk) maxk = s->k[j];
    if (s->r[j] > maxk) maxk = s->r[j];
  }
  ws_t w;
  w.f = calloc(S, sizeof(double));
  w.q = calloc(S, sizeof(double));
  w.fp = calloc(S, sizeof(double));
  w.qp = calloc(S, sizeof(double));
  w.dz = calloc(S, sizeof(double));
  w.data = calloc(s->nnz + 1, sizeof(double));
  w.work = calloc(s->work > 0 ? s->work : 1, sizeof(double));
  w.tmp = calloc(maxk + S, sizeof(double));
  w.perm = calloc(maxk, sizeof(int));
  double* z = calloc(S, sizeof(double));
  if (!w.f || !w.q || !w.fp || !w.qp || !w.dz || !w.data || !w.work || !w.tmp || !w.perm || !z)
    return 1;
  memcpy(z, z0, sizeof(double) * S);
  int ok = 1, it = 0;
  if (dc_first) {
    ok = newton(s, o, &w, M_DC, ts[0], 0.0, o->gmin,
                o->gmin_steps > 0 ? o->direct_steps : o->max_steps, z, &it);
    if (!ok && o->gmin_steps > 0) {
      memcpy(z, z0, sizeof(double) * S);
      for (int k = 1; k <= o->gmin_steps; ++k) {
        int its = 0;
        ok = newton(s, o, &w, M_DC, ts[0], 0.0, o->gmins[k], o->max_steps, z, &its);
        it += its;
      }
    }
  }
  memcpy(z_out, z, sizeof(double) * S);
  conv[0] = ok;
  iters[0] = it;
  for (int n = 1; n < n_t; ++n) {
    stamp(s, z, ts[n - 1], 1.0, 0.0, 0.0, mode == M_TRAP ? w.fp : 0, w.qp, 0);
    int its = 0;
    conv[n] = newton(s, o, &w, mode, ts[n], ts[n - 1], o->gmin, o->max_steps, z, &its);
    iters[n] = its;
    memcpy(z_out + (long long)n * S, z, sizeof(double) * S);
  }
  free(w.f); free(w.q); free(w.fp); free(w.qp); free(w.dz); free(w.data); free(w.work);
  free(w.tmp); free(w.perm); free(z);
  return 0;
}

/* ---------------------------------------------------- acceptance check
 * KCL residual and Newton-step test of a trajectory computed elsewhere
 * (the GPU): for each time point n, the residual r of `mode` at z_n
 * (voltax/analysis.py:333-378; point 0 is the DC residual f + gmin v when
 * dc_first, else it is skipped), evaluated with z_{n-1} as the previous
 * state, and one Newton step dz = -J(z_n)^-1 r. Writes
 *   kcl[n]   = max_i |r_i|                       (A for KCL rows)
 *   ratio[n] = max_i |dz_i| / (atol + rtol |z_n,i|)
 * so ratio <= 1 means z_n passes voltax's own convergence test
 * (voltax/analysis.py:224-229) once more, at the oracle's FP64 residual. */
int cvx_check(const cvx_sys* s, const cvx_opts* o, int mode, int n_t, const double* ts,
              const double* z_traj, int dc_first, double* kcl, double* ratio) {
  const int S = s->S;
  int maxk = 1;
  for (int j = 0; j < s->n_sn; ++j) {
    if (s->k[j] > maxk) maxk = s->k[j];
    if (s->r[j] > maxk) maxk = s->r[j];
  }
  ws_t w;
  w.f = calloc(S, sizeof(double));
  w.q = calloc(S, sizeof(double));
  w.fp = calloc(S, sizeof(double));
  w.qp = calloc(S, sizeof(double));
  w.dz = calloc(S, sizeof(double));
  w.data = calloc(s->nnz + 1, sizeof(double));
  w.work = calloc(s->work > 0 ? s->work : 1, sizeof(double));
  w.tmp = calloc(maxk + S, sizeof(double));
  w.perm = calloc(maxk, sizeof(int));
  if (!w.f || !w.q || !w.fp || !w.qp || !w.dz || !w.data || !w.work || !w.tmp || !w.perm)
    return 1;
  for (int n = 0; n < n_t; ++n) {
    const double* z = z_traj + (long long)n * S;
    kcl[n] = 0.0;
    ratio[n] = 0.0;
    int md = mode;
    double t = ts[n], tp = 0.0;
    if (n == 0) {
      if (!dc_first) continue;
      md = M_DC;
    } else {
      tp = ts[n - 1];
      stamp(s, z - S, tp, 1.0, 0.0, 0.0, mode == M_TRAP ? w.fp : 0, w.qp, 0);
    }
    const double cf = md == M_TRAP ? 0.5 : 1.0;
    const double cq = md == M_DC ? 0.0 : 1.0 / (t - tp);
    const double h = t - tp;
    stamp(s, z, t, cf, cq, o->gmin, w.f, md == M_DC ? 0 : w.q, w.data);
    double rmax = 0.0;
    int bad = 0;
    for (int i = 0; i < S; ++i) {
      const double gm = i < s->nv ? o->gmin * z[i] : 0.0;
      double r;
      if (md == M_DC) r = w.f[i] + gm;
      else if (md == M_BE) r = (w.q[i] - w.qp[i]) / h + w.f[i] + gm;
      else r = (w.q[i] - w.qp[i]) / h + 0.5 * (w.f[i] + w.fp[i]) + gm;
      if (isnan(r)) bad = 1;
      else if (fabs(r) > rmax) rmax = fabs(r);
      w.dz[i] = -r;
    }
    factor(s, w.data, w.work, w.perm, w.tmp);
    solve(s, w.work, w.dz, w.tmp);
    double worst = 0.0;
    for (int i = 0; i < S; ++i) {
      const double q = fabs(w.dz[i]) / (o->atol + o->rtol * fabs(z[i]));
      if (isnan(q)) bad = 1;
      else if (q > worst) worst = q;
    }
    kcl[n] = bad ? NAN : rmax;
    ratio[n] = bad ? NAN : worst;
  }
  free(w.f); free(w.q); free(w.fp); free(w.qp); free(w.dz); free(w.data); free(w.work);
  free(w.tmp); free(w.perm);
  return 0;
}
