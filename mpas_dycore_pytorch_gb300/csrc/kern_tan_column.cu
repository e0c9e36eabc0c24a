// Forward mode (tangents) of the column stages: the edge mean of theta_m_save, vertical
// implicit coefficients with their Thomas factorisation, the acoustic substep (edge
// update, right-hand side, tangent of the Thomas solve, post-solve), divergence damping,
// large-step recovery and the cold-start preparation.
//
// Each kernel differentiates one forward kernel of kern_column.cu / kern_diag.cu along the
// tangent state d (the same mpasg_fields layout as the values f), with the branches the
// forward takes (upwind sides, the damping layer) frozen at the values.  The value of every
// product, quotient and power comes from f: a tangent kernel runs before its forward kernel
// where the forward updates its inputs in place (and then reads the inputs it needs), after
// it where it needs the forward's outputs (Thomas factors, solve results).  The step driver
// (driver_tan.cu) orders the calls.
#include <cmath>

#include "adj_common.cuh"
#include "pow_exner.cuh"

namespace {

// ---------------------------------------------------------------- theta_m_save edge mean
// theta_edge_save = 0.5 (th_1 + th_2), theta_edge_rsum = 1 / (th_1 + th_2)
__global__ void k_tan_theta_edge(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const double ds = d.theta_m_save[(size_t)c2 * L + k] + d.theta_m_save[(size_t)c1 * L + k];
  const double rs = f.theta_edge_rsum[i];
  d.theta_edge_save[i] = 0.5 * ds;
  d.theta_edge_rsum[i] = -ds * rs * rs;
}

// ---------------------------------------------------------------- vertical implicit coefficients
// (vert_imp_coefs.py:343-428; values from the forward's outputs in f)
MPASG_D double tan_cofwt(const mpasg_mesh& m, const mpasg_fields& f, const mpasg_fields& d, size_t o, int k,
                         double dtseps, double rcv) {
  const double zz = m.zz[o + k], p = f.exner[o + k], rb = m.rho_base[o + k];
  const double rtb = f.rtheta_base[o + k], pb = f.exner_base[o + k], rt = f.rtheta_p[o + k], q = f.qtot[o + k];
  double x = 0.5 * dtseps * rcv * zz * kGravity * rb;
  if (q != 0.0) x = x / (1.0 + q);
  const double s = rtb + rt;
  return x / (s * pb) * (d.exner[o + k] - p * d.rtheta_p[o + k] / s);
}

MPASG_D double tan_coftz(const mpasg_mesh& m, const mpasg_fields& d, size_t o, int k, int L, double dtseps) {
  if (k <= 0 || k >= L) return 0.0;
  return dtseps * (m.fzm[k] * d.theta_m[o + k] + m.fzp[k] * d.theta_m[o + k - 1]);
}

// tangents of cofwt, coftz, cofwz and of the diagonals a, b, c (b, c into d.b_tri / d.c_tri)
__global__ void k_tan_vimp_coefs(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, double dts, double epssm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double dtseps = 0.5 * dts * (1.0 + epssm);
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  const double dcw_k = tan_cofwt(m, f, d, o, k, dtseps, rcv);
  const double dct_k = tan_coftz(m, d, o, k, L, dtseps);
  d.cofwt[o + k] = dcw_k;
  d.coftz[ow + k] = dct_k;
  if (k == 0) {
    d.coftz[ow + L] = 0.0;
    d.cofwz[o] = 0.0;
    d.a_tri[o] = 0.0;
    d.b_tri[o] = 0.0;
    d.c_tri[o] = 0.0;
    return;
  }
  const double zz = m.zz[o + k], zzm = m.zz[o + k - 1];
  const double fzm = m.fzm[k], fzp = m.fzp[k];
  const double z_i = fzm * zz + fzp * zzm;
  const double dcofwz = dtseps * c2 * z_i * m.rdzu[k] * f.cqw[ow + k] * (fzm * d.exner[o + k] + fzp * d.exner[o + k - 1]);
  d.cofwz[o + k] = dcofwz;
  const double cofwz = f.cofwz[o + k];
  const double ct_k = f.coftz[ow + k], ct_km1 = f.coftz[ow + k - 1], ct_kp1 = f.coftz[ow + k + 1];
  const double cw_k = f.cofwt[o + k], cw_km1 = f.cofwt[o + k - 1];
  const double dct_km1 = tan_coftz(m, d, o, k - 1, L, dtseps), dct_kp1 = tan_coftz(m, d, o, k + 1, L, dtseps);
  const double dcw_km1 = tan_cofwt(m, f, d, o, k - 1, dtseps, rcv);
  const double rdzw_k = m.rdzw[k], rdzw_km1 = m.rdzw[k - 1];
  d.a_tri[o + k] = -dcofwz * ct_km1 * rdzw_km1 * zzm - cofwz * dct_km1 * rdzw_km1 * zzm -
                   (dcw_km1 * ct_km1 + cw_km1 * dct_km1) * rdzw_km1;
  d.b_tri[o + k] = dcofwz * (ct_k * rdzw_k * zz + ct_k * rdzw_km1 * zzm) +
                   cofwz * (dct_k * rdzw_k * zz + dct_k * rdzw_km1 * zzm) - dct_k * (cw_k * rdzw_k - cw_km1 * rdzw_km1) -
                   ct_k * (dcw_k * rdzw_k - dcw_km1 * rdzw_km1);
  d.c_tri[o + k] = -dcofwz * ct_kp1 * rdzw_k * zz - cofwz * dct_kp1 * rdzw_k * zz + (dcw_k * ct_kp1 + cw_k * dct_kp1) * rdzw_k;
}

// Thomas factorisation alpha_k = 1 / (b_k - a_k gamma_(k-1)), gamma_k = c_k alpha_k, one
// thread per column
__global__ void k_tan_vimp_factor(mpasg_mesh m, mpasg_fields f, mpasg_fields d) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nCells) return;
  const int L = m.nVertLevels;
  const size_t o = (size_t)c * L;
  double gam = 0.0, dgam = 0.0;
  d.alpha_tri[o] = 0.0;
  d.gamma_tri[o] = 0.0;
  for (int k = 1; k < L; ++k) {
    const double al = f.alpha_tri[o + k];
    const double dal = -al * al * (d.b_tri[o + k] - d.a_tri[o + k] * gam - f.a_tri[o + k] * dgam);
    const double dg = d.c_tri[o + k] * al + f.c_tri[o + k] * dal;
    d.alpha_tri[o + k] = dal;
    d.gamma_tri[o + k] = dg;
    gam = f.gamma_tri[o + k];
    dgam = dg;
  }
}

// ---------------------------------------------------------------- acoustic substep
// edges (acoustic_step.py:576), before the forward edge update
__global__ void k_tan_ac_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, int small_step, double dts,
                               double c2) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  if (small_step == 1) {
    const double r = dts * d.tend_u[i];
    d.ru_p[i] = r;
    d.ruAvg[i] = r;
    return;
  }
  const int c1 = m.cellsOnEdge[2 * e], c2i = m.cellsOnEdge[2 * e + 1];
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2i * L + k;
  const double zzm = 0.5 * (m.zz[i2] + m.zz[i1]);
  double g = (f.rtheta_pp[i2] - f.rtheta_pp[i1]) * m.invDcEdge[e];
  double dg = (d.rtheta_pp[i2] - d.rtheta_pp[i1]) * m.invDcEdge[e];
  if (zzm != 1.0) {
    g = g / zzm;
    dg = dg / zzm;
  }
  const double a = f.cqu_e[i] * 0.5 * c2;
  const double dpgrad = a * ((d.exner[i1] + d.exner[i2]) * g + (f.exner[i1] + f.exner[i2]) * dg) +
                        0.5 * m.zxu[i] * kGravity * (d.rho_pp[i1] + d.rho_pp[i2]);
  const double r = d.ru_p[i] + dts * (d.tend_u[i] - dpgrad);
  d.ru_p[i] = r;
  d.ruAvg[i] = d.ruAvg[i] + r;
}

// tangents of rs / ts of one level (ac_level), with the forward's new ru_p in f and d
struct TanLevel {
  double rs, ts, rho_in, rt_in;
};
MPASG_D TanLevel tan_ac_level(const mpasg_mesh& m, const mpasg_fields& f, const mpasg_fields& d, int c, int k,
                              bool first, double dts, double resm) {
  const int L = m.nVertLevels;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double* geo = m.cell_edge_geo + (size_t)c * me;
  double rs = 0.0, ts = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const size_t ie = (size_t)e * L + k;
    const double w = dts * geo[j];
    rs -= w * d.ru_p[ie];
    ts -= w * (d.ru_p[ie] * f.theta_edge_save[ie] + f.ru_p[ie] * d.theta_edge_save[ie]);
  }
  const size_t o = (size_t)c * L + k;
  const size_t ow = (size_t)c * (L + 1) + k;
  TanLevel t;
  t.rho_in = first ? 0.0 : d.rho_pp[o];
  t.rt_in = first ? 0.0 : d.rtheta_pp[o];
  const double rwp_k = first ? 0.0 : f.rw_p[ow], rwp_k1 = first ? 0.0 : f.rw_p[ow + 1];
  const double drwp_k = first ? 0.0 : d.rw_p[ow], drwp_k1 = first ? 0.0 : d.rw_p[ow + 1];
  t.rs = t.rho_in + dts * d.tend_rho[o] + rs - f.cofrz[k] * resm * (drwp_k1 - drwp_k);
  t.ts = t.rt_in + dts * d.tend_theta[o] + ts -
         resm * m.rdzw[k] * (d.coftz[ow + 1] * rwp_k1 + f.coftz[ow + 1] * drwp_k1 - d.coftz[ow] * rwp_k -
                             f.coftz[ow] * drwp_k);
  return t;
}

// right-hand side (acoustic_step.py:456, :675), after the forward's part 0 (f.ac_rs /
// f.ac_ts hold rs / ts; rho_pp, rtheta_pp, rw_p are still the substep's inputs)
__global__ void k_tan_ac_prep(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl1, int small_step, double dts,
                              double epssm, double resm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const bool first = small_step == 1;
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  TanLevel lv{0.0, 0.0, 0.0, 0.0};
  if (k < L) {
    lv = tan_ac_level(m, f, d, c, k, first, dts, resm);
    d.ac_rs[o + k] = lv.rs;
    d.ac_ts[o + k] = lv.ts;
    d.rtheta_pp_old[o + k] = lv.rt_in;
  }
  const double drwp_k = first ? 0.0 : d.rw_p[ow + k];
  if (k == 0 || k == L) {
    d.ac_x[ow + k] = drwp_k;
    if (first) d.wwAvg[ow + k] = 0.0;
    return;
  }
  const TanLevel lo = tan_ac_level(m, f, d, c, k - 1, first, dts, resm);
  const double dww_in = first ? 0.0 : d.wwAvg[ow + k];
  d.wwAvg[ow + k] = dww_in + 0.5 * (1.0 - epssm) * drwp_k;
  const double zz_k = m.zz[o + k], zz_km1 = m.zz[o + k - 1];
  const double ts_k = f.ac_ts[o + k], ts_km1 = f.ac_ts[o + k - 1];
  const double rt_k = first ? 0.0 : f.rtheta_pp[o + k], rt_km1 = first ? 0.0 : f.rtheta_pp[o + k - 1];
  const double A = (zz_k * ts_k - zz_km1 * ts_km1) + resm * (zz_k * rt_k - zz_km1 * rt_km1);
  const double dA = (zz_k * lv.ts - zz_km1 * lo.ts) + resm * (zz_k * lv.rt_in - zz_km1 * lo.rt_in);
  const double dB = (lv.rs + lo.rs) + resm * (lv.rho_in + lo.rho_in);
  const double C = ts_k + resm * rt_k, D = ts_km1 + resm * rt_km1;
  const double dC = lv.ts + resm * lv.rt_in, dD = lo.ts + resm * lo.rt_in;
  d.ac_x[ow + k] = drwp_k + dts * d.tend_rw[ow + k] - d.cofwz[o + k] * A - f.cofwz[o + k] * dA - f.cofwr[o + k] * dB +
                   d.cofwt[o + k] * C + f.cofwt[o + k] * dC + d.cofwt[o + k - 1] * D + f.cofwt[o + k - 1] * dD;
}

// the Thomas solve's tangent, one thread per column, before the forward solve (f.ac_x
// holds the right-hand side): forward elimination of values and tangents (the eliminated
// values u_k kept in ubuf), then back substitution of both
__global__ void k_tan_ac_solve(mpasg_mesh m, mpasg_fields f, mpasg_fields d, double* __restrict__ ubuf) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nCells) return;
  const int L = m.nVertLevels;
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double* x = f.ac_x + ow;
  double* dx = d.ac_x + ow;
  double* u = ubuf + ow;
  double up = x[0], dup = dx[0];
  u[0] = up;
  for (int k = 1; k < L; ++k) {
    const double a = f.a_tri[o + k], al = f.alpha_tri[o + k];
    const double t = x[k] - a * up;
    const double dt = dx[k] - d.a_tri[o + k] * up - a * dup;
    up = t * al;
    dup = dt * al + t * d.alpha_tri[o + k];
    u[k] = up;
    dx[k] = dup;
  }
  double xn = x[L], dxn = dx[L];
  for (int k = L - 1; k >= 0; --k) {
    const double g = f.gamma_tri[o + k];
    const double xk = u[k] - g * xn;
    const double dxk = dx[k] - d.gamma_tri[o + k] * xn - g * dxn;
    xn = xk;
    dxn = dxk;
    dx[k] = dxk;
  }
}

// damping, ww accumulation and rho_pp / rtheta_pp (k_ac_post), after the forward's part 1
// (f.rw_p holds the damped solution, f.ac_x the undamped one)
MPASG_D double tan_ac_damped(const mpasg_mesh& m, const mpasg_fields& f, const mpasg_fields& d, size_t o, size_t ow,
                             int k, int L, double dts) {
  const double dx = d.ac_x[ow + k];
  if (k == 0 || k == L) return dx;
  const double fzm = m.fzm[k], fzp = m.fzp[k];
  const double zz_i = fzm * m.zz[o + k] + fzp * m.zz[o + k - 1];
  const double rho_i = fzm * f.rho_zz[o + k] + fzp * f.rho_zz[o + k - 1];
  const double drho_i = fzm * d.rho_zz[o + k] + fzp * d.rho_zz[o + k - 1];
  const double dss = m.dss[o + k];
  const double drw_delta = d.rw_save[ow + k] - d.rw[ow + k];
  const double dnum = dx + drw_delta - dts * dss * zz_i * (drho_i * f.w[ow + k] + rho_i * d.w[ow + k]);
  const double den = 1.0 + dts * dss;
  return (den == 1.0 ? dnum : dnum / den) - drw_delta;
}

__global__ void k_tan_ac_post(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl1, double dts, double epssm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double dxr = tan_ac_damped(m, f, d, o, ow, k, L, dts);
  if (k >= 1 && k < L) d.wwAvg[ow + k] = d.wwAvg[ow + k] + 0.5 * (1.0 + epssm) * dxr;
  d.rw_p[ow + k] = dxr;  // read by no other thread of this kernel (they read d.ac_x)
  if (k < L) {
    const double dxr1 = tan_ac_damped(m, f, d, o, ow, k + 1, L, dts);
    const double xr = f.rw_p[ow + k], xr1 = f.rw_p[ow + k + 1];
    d.rho_pp[o + k] = d.ac_rs[o + k] - f.cofrz[k] * (dxr1 - dxr);
    d.rtheta_pp[o + k] = d.ac_ts[o + k] - m.rdzw[k] * (d.coftz[ow + k + 1] * xr1 + f.coftz[ow + k + 1] * dxr1 -
                                                       d.coftz[ow + k] * xr - f.coftz[ow + k] * dxr);
  }
}

// ---------------------------------------------------------------- divergence damping
// ru_p += coef (d2 - d1) / (th_1 + th_2), d = -(rtheta_pp - rtheta_pp_old)
__global__ void k_tan_divdamp(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, double coef) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  const double d1 = -(f.rtheta_pp[i1] - f.rtheta_pp_old[i1]), d2 = -(f.rtheta_pp[i2] - f.rtheta_pp_old[i2]);
  const double t1 = -(d.rtheta_pp[i1] - d.rtheta_pp_old[i1]), t2 = -(d.rtheta_pp[i2] - d.rtheta_pp_old[i2]);
  d.ru_p[i] = d.ru_p[i] + coef * ((t2 - t1) * f.theta_edge_rsum[i] + (d2 - d1) * d.theta_edge_rsum[i]);
}

// ---------------------------------------------------------------- small-step perturbation
// (smlstep_pert.py:197-373) on the tangents: the same linear map, with the slope
// coefficients' selection (tend_u >= 0) taken from the forward's tend_u
__global__ void k_tan_smlstep(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  if (k == 0 || k == L) {
    d.tend_rw[i] = d.tend_w[i];
    return;
  }
  const int me = m.maxEdges;
  const double fzm = m.fzm[k], fzp = m.fzp[k];
  double acc = d.tend_w[i];
  const int n = m.flatTerrain ? 0 : m.nEdgesOnCell[c];
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const size_t o = (size_t)e * L;
    const double du = fzm * d.tend_u[o + k] + fzp * d.tend_u[o + k - 1];
    const size_t zi = ((size_t)c * me + j) * (L + 1) + k;
    const double coef = m.zb_cell[zi] + (f.tend_u[o + k] >= 0.0 ? 1.0 : -1.0) * m.zb3_cell[zi];
    acc = acc - coef * (m.edgesOnCell_sign[c * me + j] * du);
  }
  const size_t o = (size_t)c * L;
  d.tend_rw[i] = (fzm * m.zz[o + k] + fzp * m.zz[o + k - 1]) * acc;
}

// ---------------------------------------------------------------- large-step recovery
// (recover_large_step.py:329-513), before the forward recovery.  Over terrain, w adds the
// slope fluxes of the new ru = ru_save + ru_p with their selection sgn(flux) held fixed:
// sum_j s_j (zb + sgn(fi) zb3) fi_j at interior interfaces (fi_j = fzm ru[k] + fzp ru[k-1]),
// and at the surface w_0 = sum_j s_j (zb + sgn(fs) zb3) fs_j / (cf1 rho_0 + cf2 rho_1 +
// cf3 rho_2), fs_j = cf1 ru[0] + cf2 ru[1] + cf3 ru[2]; w_0 = 0 over flat terrain.
struct SlopeSum {
  double v, d;  // value and tangent
};
// kw >= 1: interface kw's flux fzm ru[kw] + fzp ru[kw-1]; kw == 0: the surface flux
MPASG_D SlopeSum recover_slope_sum(const mpasg_mesh& m, const mpasg_fields& f, const mpasg_fields& d, uint32_t c,
                                   int kw) {
  const int L = m.nVertLevels, me = m.maxEdges, n = m.nEdgesOnCell[c];
  SlopeSum r{0.0, 0.0};
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const size_t o = (size_t)e * L;
    auto ru = [&](int q) { return f.ru_save[o + q] + f.ru_p[o + q]; };
    auto dru = [&](int q) { return d.ru_save[o + q] + d.ru_p[o + q]; };
    double fl, dfl;
    if (kw == 0) {
      fl = m.cf1 * ru(0) + m.cf2 * ru(1) + m.cf3 * ru(2);
      dfl = m.cf1 * dru(0) + m.cf2 * dru(1) + m.cf3 * dru(2);
    } else {
      fl = m.fzm[kw] * ru(kw) + m.fzp[kw] * ru(kw - 1);
      dfl = m.fzm[kw] * dru(kw) + m.fzp[kw] * dru(kw - 1);
    }
    const size_t zi = ((size_t)c * me + j) * (L + 1) + kw;
    const double cs = m.edgesOnCell_sign[c * me + j] * (m.zb_cell[zi] + sgn(fl) * m.zb3_cell[zi]);
    r.v += cs * fl;
    r.d += cs * dfl;
  }
  return r;
}

__global__ void k_tan_recover_cells(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl1, int rk_step,
                                    double inv_ns, double rk_dt) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t oc = (size_t)c * L;
  if (k < L) {
    const size_t o = oc + k;
    const double rho_p = f.rho_p_save[o] + f.rho_pp[o];
    const double rho_zz = rho_p + m.rho_base[o];
    const double drho = d.rho_p_save[o] + d.rho_pp[o];
    double rtp, drtp;
    if (rk_step == 3) {
      rtp = f.rtheta_p_save[o] + f.rtheta_pp[o] - rk_dt * rho_zz * f.rt_diabatic_tend[o];
      drtp = d.rtheta_p_save[o] + d.rtheta_pp[o] - rk_dt * drho * f.rt_diabatic_tend[o];
    } else {
      rtp = f.rtheta_p_save[o] + f.rtheta_pp[o];
      drtp = d.rtheta_p_save[o] + d.rtheta_pp[o];
    }
    const double rtb = f.rtheta_base[o];
    d.rho_p[o] = drho;
    d.rho_zz[o] = drho;
    d.rtheta_p[o] = drtp;
    d.theta_m[o] = drtp / rho_zz - (rtp + rtb) * drho / (rho_zz * rho_zz);
    if (rk_step == 3) {
      const double rcv = kRgas / (kCp - kRgas);
      const double zz = m.zz[o];
      const double ex = mpasg_pow::pow_exner(zz * (kRgas / kP0) * (rtp + rtb), rcv);
      const double dex = rcv * ex * drtp / (rtp + rtb);
      d.exner[o] = dex;
      d.pressure_p[o] = zz * kRgas * (dex * rtp + ex * drtp + rtb * dex);
    }
  }
  const size_t ow = (size_t)c * (L + 1) + k;
  if (k >= 1 && k < L) {
    d.wwAvg[ow] = d.rw_save[ow] + d.wwAvg[ow] * inv_ns;
    const double rw = f.rw_save[ow] + f.rw_p[ow];
    const double drw = d.rw_save[ow] + d.rw_p[ow];
    d.rw[ow] = drw;
    const double den = m.fzm[k] * m.zz[oc + k] + m.fzp[k] * m.zz[oc + k - 1];
    const double wo = den == 1.0 ? rw : rw / den;
    const double dwo = den == 1.0 ? drw : drw / den;
    const double rho_k = f.rho_p_save[oc + k] + f.rho_pp[oc + k] + m.rho_base[oc + k];
    const double rho_km1 = f.rho_p_save[oc + k - 1] + f.rho_pp[oc + k - 1] + m.rho_base[oc + k - 1];
    const double drho_k = d.rho_p_save[oc + k] + d.rho_pp[oc + k];
    const double drho_km1 = d.rho_p_save[oc + k - 1] + d.rho_pp[oc + k - 1];
    const double R = m.fzm[k] * rho_k + m.fzp[k] * rho_km1;
    const double dR = m.fzm[k] * drho_k + m.fzp[k] * drho_km1;
    double num = wo, dnum = dwo;
    if (!m.flatTerrain) {
      const SlopeSum sl = recover_slope_sum(m, f, d, c, k);
      num = num + sl.v;
      dnum = dnum + sl.d;
    }
    d.w[ow] = dnum / R - num * dR / (R * R);
  } else if (k == 0 && !m.flatTerrain) {
    const SlopeSum sl = recover_slope_sum(m, f, d, c, 0);
    auto rho = [&](int q) { return f.rho_p_save[oc + q] + f.rho_pp[oc + q] + m.rho_base[oc + q]; };
    auto drho = [&](int q) { return d.rho_p_save[oc + q] + d.rho_pp[oc + q]; };
    const double D = m.cf1 * rho(0) + m.cf2 * rho(1) + m.cf3 * rho(2);
    const double dD = m.cf1 * drho(0) + m.cf2 * drho(1) + m.cf3 * drho(2);
    d.w[ow] = sl.d / D - sl.v * dD / (D * D);
  } else {
    d.w[ow] = 0.0;
  }
}

__global__ void k_tan_recover_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, double inv_ns) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  d.ruAvg[i] = d.ru_save[i] + d.ruAvg[i] * inv_ns;
  const double ru = f.ru_save[i] + f.ru_p[i];
  const double dru = d.ru_save[i] + d.ru_p[i];
  d.ru[i] = dru;
  const double rho2 = (f.rho_p_save[i1] + f.rho_pp[i1] + m.rho_base[i1]) + (f.rho_p_save[i2] + f.rho_pp[i2] + m.rho_base[i2]);
  const double drho2 = (d.rho_p_save[i1] + d.rho_pp[i1]) + (d.rho_p_save[i2] + d.rho_pp[i2]);
  d.u[i] = 2.0 * dru / rho2 - 2.0 * ru * drho2 / (rho2 * rho2);
}

// ---------------------------------------------------------------- cold-start preparation
// (init_coupled_diagnostics.py:147, dry), after the forward preparation: the tangents of
// theta (= theta_m) and rho arrive in dth / drho, those of u and w in d
__global__ void k_tan_prepare_cells(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl,
                                    const double* __restrict__ dth, const double* __restrict__ drho) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const double zz = m.zz[i];
  const double th = f.theta_m[i], rho_p = f.rho_p[i], rb = m.rho_base[i];
  const double rtp = f.rtheta_p[i], rtb = f.rtheta_base[i], ex = f.exner[i];
  const double dt = dth ? dth[i] : 0.0;
  const double drz = drho ? drho[i] / zz : 0.0;
  const double drtp = dt * rho_p + th * drz + rb * dt;
  const double rcv = kRgas / (kCp - kRgas);
  const double dex = rcv * ex * drtp / (rtp + rtb);
  d.theta_m[i] = dt;
  d.rho_zz[i] = drz;
  d.rho_p[i] = drz;
  d.rtheta_p[i] = drtp;
  d.exner[i] = dex;
  d.pressure_p[i] = zz * kRgas * (dex * rtp + ex * drtp + rtb * dex);
}

__global__ void k_tan_prepare_ru(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const size_t i1 = (size_t)m.cellsOnEdge[2 * e] * L + k, i2 = (size_t)m.cellsOnEdge[2 * e + 1] * L + k;
  d.ru[i] = 0.5 * (d.u[i] * (f.rho_zz[i1] + f.rho_zz[i2]) + f.u[i] * (d.rho_zz[i1] + d.rho_zz[i2]));
}

// rw = (w rho_i - sum_j s_j coef_j flux_j) zz_i at interior interfaces, flux_j = fzm
// ru[k] + fzp ru[k-1], coef_j = zb + sgn(flux_j) zb3 held fixed (no slope terms over flat
// terrain); after k_tan_prepare_ru
__global__ void k_tan_prepare_rw(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  if (k == 0 || k == L) {
    d.rw[i] = 0.0;
    return;
  }
  const size_t oc = (size_t)c * L;
  const double fzm = m.fzm[k], fzp = m.fzp[k];
  const double rho_i = fzp * f.rho_zz[oc + k - 1] + fzm * f.rho_zz[oc + k];
  const double drho_i = fzp * d.rho_zz[oc + k - 1] + fzm * d.rho_zz[oc + k];
  const double zz_i = fzp * m.zz[oc + k - 1] + fzm * m.zz[oc + k];
  double drw = (d.w[i] * rho_i + f.w[i] * drho_i) * zz_i;
  const int me = m.maxEdges;
  const int n = m.flatTerrain ? 0 : m.nEdgesOnCell[c];
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const size_t o = (size_t)e * L;
    const double flux = fzm * f.ru[o + k] + fzp * f.ru[o + k - 1];
    const double dflux = fzm * d.ru[o + k] + fzp * d.ru[o + k - 1];
    const size_t zi = ((size_t)c * me + j) * (L + 1) + k;
    const double coef = m.zb_cell[zi] + sgn(flux) * m.zb3_cell[zi];
    drw -= m.edgesOnCell_sign[c * me + j] * coef * dflux * zz_i;
  }
  d.rw[i] = drw;
}

}  // namespace

// ================================================================= internal cores
int mpasgi_theta_edge_jvp(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, cudaStream_t s) {
  const int L = m->nVertLevels;
  k_tan_theta_edge<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// after the forward mpasg_vert_imp_coefs on f
int mpasgi_vimp_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                         double dts, cudaStream_t s) {
  const int L = m->nVertLevels;
  k_tan_vimp_coefs<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L), dts, c->epssm);
  MPASG_LAUNCH_CHECK();
  k_tan_vimp_factor<<<nblocks(m->nCells, 64), 64, 0, s>>>(*m, *f, *d);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// one acoustic substep of f and d (the forward's two parts with the tangent kernels around
// them); ubuf: (C+1) x (L+1) doubles
int mpasgi_acoustic_jvp_core(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                             int small_step, double dts, double* ubuf, cudaStream_t s) {
  const int L = m->nVertLevels;
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  const double resm = (1.0 - c->epssm) / (1.0 + c->epssm);
  const long long ncw = (long long)m->nCells * (L + 1);
  k_tan_ac_edges<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L), small_step, dts, c2);
  MPASG_LAUNCH_CHECK();
  int rc = mpasgi_acoustic_parts(m, c, f, small_step, dts, s, 0);
  if (rc != MPASG_OK) return rc;
  k_tan_ac_prep<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L + 1), small_step, dts, c->epssm, resm);
  MPASG_LAUNCH_CHECK();
  k_tan_ac_solve<<<nblocks(m->nCells, 64), 64, 0, s>>>(*m, *f, *d, ubuf);
  MPASG_LAUNCH_CHECK();
  rc = mpasgi_acoustic_parts(m, c, f, small_step, dts, s, 1);
  if (rc != MPASG_OK) return rc;
  k_tan_ac_post<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L + 1), dts, c->epssm);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// before the forward divergence damping
int mpasgi_divdamp_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                            double dts, cudaStream_t s) {
  const int L = m->nVertLevels;
  const double coef = 2.0 * c->smdiv * c->len_disp / dts;
  k_tan_divdamp<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L), coef);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// before the forward recovery
int mpasgi_smlstep_jvp_core(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, cudaStream_t s) {
  const int L = m->nVertLevels;
  k_tan_smlstep<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L + 1));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

int mpasgi_recover_jvp_core(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, int rk_step, int ns,
                            double rk_dt, cudaStream_t s) {
  const int L = m->nVertLevels;
  const double inv_ns = 1.0 / (double)ns;
  k_tan_recover_cells<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L + 1), rk_step,
                                                                                inv_ns, rk_dt);
  MPASG_LAUNCH_CHECK();
  k_tan_recover_edges<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L), inv_ns);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// after the forward preparation
int mpasgi_prepare_jvp_core(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, const double* dth,
                            const double* drho, cudaStream_t s) {
  const int L = m->nVertLevels;
  k_tan_prepare_cells<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L), dth, drho);
  MPASG_LAUNCH_CHECK();
  k_tan_prepare_ru<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L));
  MPASG_LAUNCH_CHECK();
  k_tan_prepare_rw<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, s>>>(*m, *f, *d, FastDiv(L + 1));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
