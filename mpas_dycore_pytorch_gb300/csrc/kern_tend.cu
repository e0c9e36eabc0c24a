// Large-step tendencies (the reference's atm_compute_dyn_tend_work,
// mpas_pytorch/dynamics/dyn_tend.py:10836, canonical composition :9390).
//
//   k_tend_cells_a   h_divergence (+ rk 1: Smagorinsky kdiff, tend_rho, dpdz)   sections :9925-9992
//   k_tend_u         u tendency: vertical transport, PV flux, KE gradient, divergence
//                    coupling (+ rk 1: pressure gradient and del2 mixing)        :9993-10315
//   k_del4_vertex / k_del4_cell / k_tend_u_del4   del4 filter of u (rk 1)        :10075-10315
//   k_mix_cells_a / k_mix_cells_b   w and theta del2 / del4 mixing (rk 1)       :10355, :10544
//   k_tend_w_theta   w and theta advection, vertical fluxes, buoyancy, diabatic  :10316-10835
//
// Slot sums follow the reference's order (first slot assigned, then left-to-right).
#include "common.cuh"

namespace {

struct TendScalars {
  double inv_dt, c_s_len2, kdiff_cap, h_mom_visc4, h_theta_visc4, del4u_div, coef3, visc2;
  int rk_step, smag, del4;
};

__global__ void k_tend_cells_a(mpasg_mesh m, mpasg_fields f, FastDiv fl, TendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double hdiv = 0.0;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double wgt = m.edgesOnCell_sign[c * me + j] * m.dvEdge[e];
    double t = wgt * f.ru[(size_t)e * L + k];
    hdiv = (j == 0) ? t : hdiv + t;
  }
  hdiv = hdiv * m.invAreaCell[c];
  f.h_divergence[i] = hdiv;
  if (p.rk_step != 1) return;
  const size_t ow = (size_t)c * (L + 1) + k;
  f.tend_rho[i] = -hdiv - m.rdzw[k] * (f.rw[ow + 1] - f.rw[ow]);
  double q = f.qtot[i];
  f.dpdz[i] = -kGravity * (m.rho_base[i] * q + f.rr_save[i] * (1.0 + q));
  if (p.smag) {
    double dd = 0.0, dof = 0.0;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      double ca = m.defc_a[c * me + j], cb = m.defc_b[c * me + j];
      double ue = f.u[(size_t)e * L + k], ve = f.v[(size_t)e * L + k];
      double ndd = (dd + ca * ue) - cb * ve;
      double ndo = (dof + cb * ue) + ca * ve;
      dd = ndd;
      dof = ndo;
    }
    f.kdiff[i] = fmin(p.c_s_len2 * sqrt(dd * dd + dof * dof), p.kdiff_cap);
  } else {
    f.kdiff[i] = p.visc2;
  }
}

MPASG_D double wduz_at(const double* __restrict__ u, double rwe, int kk, int L, const double* fzm,
                       const double* fzp) {
  if (kk <= 0 || kk >= L) return 0.0;
  if (kk == 1 || kk == L - 1) return rwe * (fzm[kk] * u[kk] + fzp[kk] * u[kk - 1]);
  return flux3(u[kk - 2], u[kk - 1], u[kk], u[kk + 1], rwe, 1.0);
}

__global__ void __launch_bounds__(kBlock) k_tend_u(mpasg_mesh m, mpasg_fields f, FastDiv fl, TendScalars p) {
  __shared__ double s_wd[kBlock];
  const int L = m.nVertLevels;
  const uint32_t n_all = (uint32_t)m.nEdges * L;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n_all;
  uint32_t e = 0, k = 0;
  int c1 = 0, c2 = 0;
  const double* ue = f.u;
  double wd_k = 0.0;
  if (active) {
    e = fl.div(i);
    k = i - e * L;
    c1 = m.cellsOnEdge[2 * e];
    c2 = m.cellsOnEdge[2 * e + 1];
    ue = f.u + (size_t)e * L;
    double rwe_k = 0.5 * (f.rw[(size_t)c1 * (L + 1) + k] + f.rw[(size_t)c2 * (L + 1) + k]);
    wd_k = wduz_at(ue, rwe_k, k, L, m.fzm, m.fzp);
  }
  s_wd[threadIdx.x] = wd_k;  // vertical flux at the interface below level k
  __syncthreads();
  if (!active) return;
  double wd_k1;
  if (k + 1 >= (uint32_t)L) {
    wd_k1 = 0.0;
  } else if (threadIdx.x + 1 < blockDim.x) {
    wd_k1 = s_wd[threadIdx.x + 1];  // same edge, next level
  } else {
    double rwe_k1 = 0.5 * (f.rw[(size_t)c1 * (L + 1) + k + 1] + f.rw[(size_t)c2 * (L + 1) + k + 1]);
    wd_k1 = wduz_at(ue, rwe_k1, k + 1, L, m.fzm, m.fzp);
  }
  double tu = -m.rdzw[k] * (wd_k1 - wd_k);
  // nonlinear Coriolis / PV flux over the TRiSK stencil
  const int n2 = m.nEdgesOnEdge[e];
  const int me2 = m.maxEdges2;
  const double pv_self = f.pv_edge[i];
  // sum_j (w_j u_j) * 0.5 (pv_self + pv_j): the exact power-of-two factor 0.5 is applied
  // once to the sum (scaling by 0.5 commutes with every rounding of the sum)
  double q = 0.0;
  for (int j = 0; j < n2; ++j) {
    int eo = m.edgesOnEdge[e * me2 + j];
    double t = (m.weightsOnEdge[e * me2 + j] * f.u[(size_t)eo * L + k]) * (pv_self + f.pv_edge[(size_t)eo * L + k]);
    q = (j == 0) ? t : q + t;
  }
  q = 0.5 * q;
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  const double inv_dc = m.invDcEdge[e];
  const double rho_e = f.h_edge[i];
  tu = tu + rho_e * (q - (f.ke[i2] - f.ke[i1]) * inv_dc) - ue[k] * 0.5 * (f.h_divergence[i1] + f.h_divergence[i2]);
  if (p.rk_step == 1) {
    double teu = -f.cqu_e[i] * (div_or_one((f.pressure_p[i2] - f.pressure_p[i1]) * inv_dc, 0.5 * (m.zz[i2] + m.zz[i1])) -
                               0.5 * m.zxu[i] * (f.dpdz[i1] + f.dpdz[i2]));
    int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
    double r_dv = fmin(m.invDvEdge[e], 4.0 * inv_dc);
    double u_diff = (f.divergence[i2] - f.divergence[i1]) * inv_dc -
                    (f.vorticity[(size_t)v2 * L + k] - f.vorticity[(size_t)v1 * L + k]) * r_dv;
    f.delsq_u[i] = u_diff;
    double kdiffu = 0.5 * (f.kdiff[i1] + f.kdiff[i2]);
    teu = teu + rho_e * kdiffu * u_diff * m.meshScalingDel2[e];
    f.tend_u_euler[i] = teu;
    f.tend_u[i] = p.del4 ? tu : tu + teu;
  } else {
    f.tend_u[i] = tu + f.tend_u_euler[i];
  }
}

__global__ void k_del4_vertex(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  uint32_t v = fl.div(i), k = i - v * L;
  const int vd = m.vertexDegree;
  double acc = 0.0;
  for (int j = 0; j < vd; ++j) {
    int e = m.edgesOnVertex[v * vd + j];
    double es = m.invAreaTriangle[v] * m.dcEdge[e] * m.edgesOnVertex_sign[v * vd + j];
    double t = es * f.delsq_u[(size_t)e * L + k];
    acc = (j == 0) ? t : acc + t;
  }
  f.delsq_vort[i] = acc;
}

__global__ void k_del4_cell(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double es = m.invAreaCell[c] * m.dvEdge[e] * m.edgesOnCell_sign[c * me + j];
    double t = es * f.delsq_u[(size_t)e * L + k];
    acc = (j == 0) ? t : acc + t;
  }
  f.delsq_div[i] = acc;
}

__global__ void k_tend_u_del4(mpasg_mesh m, mpasg_fields f, FastDiv fl, TendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
  const double inv_dc = m.invDcEdge[e];
  double u_mix = m.meshScalingDel4[e] * p.h_mom_visc4;
  double r_dc4 = u_mix * p.del4u_div * inv_dc;
  double r_dv4 = u_mix * fmin(m.invDvEdge[e], 4.0 * inv_dc);
  double u_diff4 = (f.delsq_div[(size_t)c2 * L + k] - f.delsq_div[(size_t)c1 * L + k]) * r_dc4 -
                   (f.delsq_vort[(size_t)v2 * L + k] - f.delsq_vort[(size_t)v1 * L + k]) * r_dv4;
  double teu = f.tend_u_euler[i] - f.h_edge[i] * u_diff4;
  f.tend_u_euler[i] = teu;
  f.tend_u[i] = f.tend_u[i] + teu;
}

// w / theta del2 mixing and the del2 fields for del4 (rk 1); index space (C, L+1)
__global__ void k_mix_cells_a(mpasg_mesh m, mpasg_fields f, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  if (k >= 1 && k < (uint32_t)L) {  // w
    double dw = 0.0, tw = 0.0;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      double es = 0.5 * ia * m.edgesOnCell_sign[c * me + j] * m.dvEdge[e] * m.invDcEdge[e];
      double flux = es * (f.h_edge[(size_t)e * L + k] + f.h_edge[(size_t)e * L + k - 1]) *
                    (f.w[(size_t)ec2 * (L + 1) + k] - f.w[(size_t)ec1 * (L + 1) + k]);
      dw = dw + flux;
      flux = flux * m.meshScalingDel2[e] * 0.25 *
             (f.kdiff[(size_t)ec1 * L + k] + f.kdiff[(size_t)ec2 * L + k] + f.kdiff[(size_t)ec1 * L + k - 1] +
              f.kdiff[(size_t)ec2 * L + k - 1]);
      tw = tw + flux;
    }
    f.delsq_w[i] = dw;
    f.tend_w_euler[i] = tw;
  } else {
    f.delsq_w[i] = 0.0;
    f.tend_w_euler[i] = 0.0;
  }
  if (k < (uint32_t)L) {  // theta
    const size_t o = (size_t)c * L + k;
    double dt_ = 0.0, tt = 0.0;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      double es = ia * m.edgesOnCell_sign[c * me + j] * m.dvEdge[e] * m.invDcEdge[e];
      double pr = 1.0 * m.meshScalingDel2[e];
      double flux = es * (f.theta_m[(size_t)ec2 * L + k] - f.theta_m[(size_t)ec1 * L + k]) * f.h_edge[(size_t)e * L + k];
      dt_ = dt_ + flux;
      flux = flux * 0.5 * (f.kdiff[(size_t)ec1 * L + k] + f.kdiff[(size_t)ec2 * L + k]) * pr;
      tt = tt + flux;
    }
    f.delsq_theta[o] = dt_;
    f.tend_theta_euler[o] = tt;
  }
}

// del4 parts of w / theta mixing (rk 1)
__global__ void k_mix_cells_b(mpasg_mesh m, mpasg_fields f, FastDiv fl1, TendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  if (k >= 1 && k < (uint32_t)L) {
    double tw = f.tend_w_euler[i];
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      double es = m.meshScalingDel4[e] * (p.h_mom_visc4 * ia) * m.dvEdge[e] * m.edgesOnCell_sign[c * me + j] *
                  m.invDcEdge[e];
      tw = tw - es * (f.delsq_w[(size_t)ec2 * (L + 1) + k] - f.delsq_w[(size_t)ec1 * (L + 1) + k]);
    }
    f.tend_w_euler[i] = tw;
  }
  if (k < (uint32_t)L) {
    const size_t o = (size_t)c * L + k;
    double tt = f.tend_theta_euler[o];
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      double es = m.meshScalingDel4[e] * (p.h_theta_visc4 * 1.0 * ia) * m.dvEdge[e] *
                  m.edgesOnCell_sign[c * me + j] * m.invDcEdge[e];
      tt = tt - es * (f.delsq_theta[(size_t)ec2 * L + k] - f.delsq_theta[(size_t)ec1 * L + k]);
    }
    f.tend_theta_euler[o] = tt;
  }
}

MPASG_D double wdwz_at(const double* w, const double* rw, int kk, int L) {
  if (kk <= 0 || kk >= L) return 0.0;
  if (kk == 1 || kk == L - 1) return 0.25 * (rw[kk] + rw[kk - 1]) * (w[kk] + w[kk - 1]);
  return flux3(w[kk - 2], w[kk - 1], w[kk], w[kk + 1], 0.5 * (rw[kk] + rw[kk - 1]), 1.0);
}

MPASG_D double wdtz_at(const double* th, const double* ths, const double* rw, const double* rws, int kk, int L,
                       const double* fzm, const double* fzp, double coef3) {
  if (kk <= 0 || kk >= L) return 0.0;
  if (kk == L - 1 && kk != 1) return rws[kk] * (fzm[kk] * th[kk] + fzp[kk] * th[kk - 1]);
  double v;
  if (kk == 1)
    v = rw[kk] * (fzm[kk] * th[kk] + fzp[kk] * th[kk - 1]);
  else
    v = flux3(th[kk - 2], th[kk - 1], th[kk], th[kk + 1], rw[kk], coef3);
  return v + (rws[kk] - rw[kk]) * (fzm[kk] * ths[kk] + fzp[kk] * ths[kk - 1]);
}

// Edge-side horizontal advective fluxes of w and theta_m, computed once per edge:
// flux_w_e[e,k] = ru_w * sum_a (adv_coefs +/- adv_coefs_3rd)_a w[advCell_a, k] (w levels 1..L-1)
// flux_th_e[e,k] = ru * sum_a (...)_a theta_m[advCell_a, k] (mass levels 0..L-1).
// The cell sums then apply edgesOnCell_sign (an exact +/-1 factor), which reproduces
// the reference's per-slot (sign * ru) * flux products bit for bit.
__global__ void k_adv_edges(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int na = m.nAdvMax;
  const int nadv = m.nAdvCellsForEdge[e];
  const int32_t* cells = m.advCellsForEdge + (size_t)e * na;
  const double rue = f.ru[i];
  {
    const double* cf = (rue >= 0.0 ? m.adv_coefs_p : m.adv_coefs_m) + (size_t)e * na;
    double acc = 0.0;
    for (int a = 0; a < nadv; ++a) {
      double t = cf[a] * f.theta_m[(size_t)cells[a] * L + k];
      acc = (a == 0) ? t : acc + t;
    }
    f.flux_th_e[i] = rue * acc;
  }
  if (k >= 1) {
    double ru_w = m.fzm[k] * rue + m.fzp[k] * f.ru[i - 1];
    const double* cf = (ru_w >= 0.0 ? m.adv_coefs_p : m.adv_coefs_m) + (size_t)e * na;
    double acc = 0.0;
    for (int a = 0; a < nadv; ++a) {
      double t = cf[a] * f.w[(size_t)cells[a] * (L + 1) + k];
      acc = (a == 0) ? t : acc + t;
    }
    f.flux_w_e[i] = ru_w * acc;
  }
}

// w and theta tendencies; index space (C, L+1)
__global__ void __launch_bounds__(kBlock) k_tend_w_theta(mpasg_mesh m, mpasg_fields f, FastDiv fl1, TendScalars p) {
  __shared__ double s_wd[kBlock], s_wt[kBlock];
  const int L = m.nVertLevels;
  const uint32_t n_all = (uint32_t)m.nCells * (L + 1);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n_all;
  uint32_t c = 0, k = 0;
  double wd_k = 0.0, wt_k = 0.0;
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
    const size_t ow0 = (size_t)c * (L + 1), oc0 = (size_t)c * L;
    wd_k = wdwz_at(f.w + ow0, f.rw + ow0, k, L);
    wt_k = wdtz_at(f.theta_m + oc0, f.theta_m_save + oc0, f.rw + ow0, f.rw_save + ow0, k, L, m.fzm, m.fzp,
                   p.coef3);
  }
  s_wd[threadIdx.x] = wd_k;  // interface fluxes owned by this level
  s_wt[threadIdx.x] = wt_k;
  __syncthreads();
  if (!active) return;
  double wd_k1 = 0.0, wt_k1 = 0.0;
  if (k < (uint32_t)L) {
    if (threadIdx.x + 1 < blockDim.x) {
      wd_k1 = s_wd[threadIdx.x + 1];
      wt_k1 = s_wt[threadIdx.x + 1];
    } else {
      const size_t ow0 = (size_t)c * (L + 1), oc0 = (size_t)c * L;
      wd_k1 = wdwz_at(f.w + ow0, f.rw + ow0, k + 1, L);
      wt_k1 = wdtz_at(f.theta_m + oc0, f.theta_m_save + oc0, f.rw + ow0, f.rw_save + ow0, k + 1, L, m.fzm,
                      m.fzp, p.coef3);
    }
  }
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  const size_t oc = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  if (k >= 1 && k < (uint32_t)L) {
    const double fzm = m.fzm[k], fzp = m.fzp[k];
    double tw = 0.0;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      tw = tw - m.edgesOnCell_sign[c * me + j] * f.flux_w_e[(size_t)e * L + k];
    }
    tw = tw * ia - m.rdzu[k] * (wd_k1 - wd_k);
    double teu = f.tend_w_euler[i];
    if (p.rk_step == 1) {
      teu = teu - f.cqw[ow + k] * (m.rdzu[k] * (f.pressure_p[oc + k] - f.pressure_p[oc + k - 1]) -
                                   (fzm * f.dpdz[oc + k] + fzp * f.dpdz[oc + k - 1]));
      f.tend_w_euler[i] = teu;
    }
    f.tend_w[i] = tw + teu;
  } else {
    f.tend_w[i] = 0.0;
  }
  if (k < (uint32_t)L) {
    const size_t o = oc + k;
    double tt = 0.0;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      double x = -(m.edgesOnCell_sign[c * me + j] * f.flux_th_e[(size_t)e * L + k]);
      tt = (j == 0) ? x : tt + x;
    }
    if (p.rk_step > 1) {
      for (int j = 0; j < n; ++j) {
        int e = m.edgesOnCell[c * me + j];
        int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
        double wgt = m.edgesOnCell_sign[c * me + j] * m.dvEdge[e];
        double flux = wgt * (f.ru_save[(size_t)e * L + k] - f.ru[(size_t)e * L + k]) * 0.5 *
                      (f.theta_m_save[(size_t)ec2 * L + k] + f.theta_m_save[(size_t)ec1 * L + k]);
        tt = tt - flux;
      }
    }
    const double* th = f.theta_m + oc;
    tt = tt * ia - m.rdzw[k] * (wt_k1 - wt_k);
    double rz = f.rho_zz[o];
    double rtd = f.rt_diabatic_tend[o];
    // unfused: the difference cancels strongly (as rounded by the reference)
    f.rthdynten[o] = __dsub_rn(tt, __dmul_rn(f.tend_rho[o], th[k])) / rz;
    tt = tt + rz * rtd;
    tt = tt + f.tend_theta_euler[o];
    f.tend_theta[o] = tt;
  }
}

}  // namespace

extern "C" int mpasg_dyn_tend(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                              void* stream) {
  if (!m || !c || !f || rk_step < 1 || rk_step > 3) return MPASG_E_ARG;
  if (m->nVertLevels < 4) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  TendScalars p;
  p.inv_dt = 1.0 / c->dt;
  double cl = c->c_s * c->len_disp;
  p.c_s_len2 = cl * cl;
  p.kdiff_cap = (0.01 * (c->len_disp * c->len_disp)) * p.inv_dt;
  p.smag = c->horiz_mixing_smagorinsky;
  if (p.smag) {
    p.h_mom_visc4 = c->visc4_2dsmag * (c->len_disp * c->len_disp * c->len_disp);
    p.h_theta_visc4 = p.h_mom_visc4;
  } else {
    p.h_mom_visc4 = c->h_mom_eddy_visc4;
    p.h_theta_visc4 = c->h_theta_eddy_visc4;
  }
  p.visc2 = 0.0;
  p.del4u_div = c->del4u_div_factor;
  p.coef3 = c->coef_3rd_order;
  p.rk_step = rk_step;
  p.del4 = (p.h_mom_visc4 > 0.0) ? 1 : 0;
  const long long ncl = (long long)m->nCells * L, nel = (long long)m->nEdges * L;
  const long long ncw = (long long)m->nCells * (L + 1), nvl = (long long)m->nVertices * L;
  FastDiv fl(L), fl1(L + 1);
  k_tend_cells_a<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, p);
  MPASG_LAUNCH_CHECK();
  k_tend_u<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, p);
  MPASG_LAUNCH_CHECK();
  if (rk_step == 1) {
    if (p.del4) {
      k_del4_vertex<<<nblocks(nvl), kBlock, 0, s>>>(*m, *f, fl);
      MPASG_LAUNCH_CHECK();
      k_del4_cell<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl);
      MPASG_LAUNCH_CHECK();
      k_tend_u_del4<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, p);
      MPASG_LAUNCH_CHECK();
    }
    k_mix_cells_a<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, fl1);
    MPASG_LAUNCH_CHECK();
    if (p.h_mom_visc4 > 0.0 || p.h_theta_visc4 > 0.0) {
      TendScalars q = p;
      if (!(p.h_mom_visc4 > 0.0)) q.h_mom_visc4 = 0.0;
      k_mix_cells_b<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, fl1, q);
      MPASG_LAUNCH_CHECK();
    }
  }
  k_adv_edges<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  k_tend_w_theta<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, fl1, p);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
