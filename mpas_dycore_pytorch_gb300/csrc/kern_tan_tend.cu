// Forward mode (tangents) of the large-step tendencies (atm_compute_dyn_tend_work,
// mpas_pytorch/dynamics/dyn_tend.py:10836) and of the diagnostics
// (atm_compute_solve_diagnostics_work, dynamics/solve_diagnostics.py:1052).
//
// Both run after their forward stage on f: the tendencies' inputs are not changed by it,
// and its intermediates (mass-flux divergence, kdiff, the del2 / del4 fields of u, the
// kinetic energy and vorticity at the vertices, the cell PV) are read from f.  Each tangent
// kernel has the index space and the slot order of its forward kernel (kern_tend.cu,
// kern_diag.cu).  The Smagorinsky deformation is formed with separately rounded products
// and sums, as the reverse mode does, so both modes differentiate kdiff at the same point.
#include <cmath>

#include "adj_common.cuh"

namespace {

struct TanTendScalars {
  double cs2, kdiff_cap, h_mom_visc4, h_theta_visc4, del4u_div, coef3;
  int rk_step, smag, del4;
  int mix_pert;   // vertical mixing of the perturbation from the initial profiles
  AdjDamping dm;  // CAM floor of kdiff, Rayleigh damping of u, vertical mixing
};

// ---- h_divergence, and at rk 1 tend_rho, dpdz and kdiff (k_tend_cells_a)
__global__ void k_tan_cells_a(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, TanTendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double dh = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const double t = m.cell_edge_sdv[c * me + j] * d.ru[(size_t)e * L + k];
    dh = (j == 0) ? t : dh + t;
  }
  dh = dh * m.invAreaCell[c];
  d.h_divergence[i] = dh;
  if (p.rk_step != 1) return;
  const size_t ow = (size_t)c * (L + 1) + k;
  d.tend_rho[i] = -dh - m.rdzw[k] * (d.rw[ow + 1] - d.rw[ow]);
  const double q = f.qtot[i];
  d.dpdz[i] = -kGravity * (d.rr_save[i] * (1.0 + q));
  double dkd = 0.0;
  if (p.smag) {
    double dd = 0.0, dof = 0.0, tdd = 0.0, tdo = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      const double ca = m.defc_a[c * me + j], cb = m.defc_b[c * me + j];
      const size_t ie = (size_t)e * L + k;
      const double ue = f.u[ie], ve = f.v[ie];
      const double ndd = __dsub_rn(__dadd_rn(dd, __dmul_rn(ca, ue)), __dmul_rn(cb, ve));
      const double ndo = __dadd_rn(__dadd_rn(dof, __dmul_rn(cb, ue)), __dmul_rn(ca, ve));
      dd = ndd;
      dof = ndo;
      tdd += ca * d.u[ie] - cb * d.v[ie];
      tdo += cb * d.u[ie] + ca * d.v[ie];
    }
    const double sq = sqrt(__dadd_rn(__dmul_rn(dd, dd), __dmul_rn(dof, dof)));
    const double A = __dmul_rn(p.cs2, sq);
    const double dA = sq > 0.0 ? p.cs2 * (dd * tdd + dof * tdo) / sq : 0.0;
    // min(A, cap): the branch taken; a tie splits the derivative evenly (torch's minimum)
    dkd = A < p.kdiff_cap ? dA : (A == p.kdiff_cap ? 0.5 * dA : 0.0);
    // max(kdiff, CAM floor) on the top levels: the branch taken, ties split evenly
    if (p.dm.ncam > 0 && k >= L - p.dm.ncam) dkd *= adj_max_factor(fmin(A, p.kdiff_cap), adj_cam_floor(p.dm, k, L));
  }
  d.kdiff[i] = dkd;
}

// tangent of the vertical u flux at interface kk of edge e (wduz_at)
MPASG_D double tan_wduz(const mpasg_mesh& m, const mpasg_fields& f, const mpasg_fields& d, int c1, int c2, size_t oe,
                        int kk, int L) {
  if (kk <= 0 || kk >= L) return 0.0;
  const double* u = f.u + oe;
  const double* du = d.u + oe;
  const double rwe = 0.5 * (f.rw[(size_t)c1 * (L + 1) + kk] + f.rw[(size_t)c2 * (L + 1) + kk]);
  const double drwe = 0.5 * (d.rw[(size_t)c1 * (L + 1) + kk] + d.rw[(size_t)c2 * (L + 1) + kk]);
  if (kk == 1 || kk == L - 1) {
    const double fm = m.fzm[kk], fp = m.fzp[kk];
    return drwe * (fm * u[kk] + fp * u[kk - 1]) + rwe * (fm * du[kk] + fp * du[kk - 1]);
  }
  const Flux3Grad g = flux3_grad(u[kk - 2], u[kk - 1], u[kk], u[kk + 1], rwe, 1.0);
  return g.qm2 * du[kk - 2] + g.qm1 * du[kk - 1] + g.q0 * du[kk] + g.qp1 * du[kk + 1] + g.ua * drwe;
}

// ---- u tendency (k_tend_u): vertical transport, PV flux, KE gradient, divergence coupling,
// and at rk 1 the pressure gradient and del2 mixing
// pv u and its tangent pv du + u dpv at every edge level (the PV flux sum's neighbour
// factors, formed once per stage), into the ke_edge scratch of f and d (free outside the
// diagnostics)
__global__ void k_tan_pvu(mpasg_fields f, mpasg_fields d, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double pv = f.pv_edge[i], u = f.u[i];
  f.ke_edge[i] = pv * u;
  d.ke_edge[i] = pv * d.u[i] + u * d.pv_edge[i];
}

__global__ void k_tan_u(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, TanTendScalars p, int defer) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const size_t oe = (size_t)e * L;
  double dtu = -m.rdzw[k] * (tan_wduz(m, f, d, c1, c2, oe, k + 1, L) - tan_wduz(m, f, d, c1, c2, oe, k, L));
  const int n2 = m.nEdgesOnEdge[e];
  const int me2 = m.maxEdges2;
  // q = 0.5 sum_j w_j u_j (pv_self + pv_j) = 0.5 (pv_self sum w u + sum w (pv u)) and its
  // tangent 0.5 (dpv_self sum w u + pv_self sum w du + sum w d(pv u)): four multiply-adds
  // per neighbour over the per-edge factors of k_tan_pvu
  const double pv_self = f.pv_edge[i], dpv_self = d.pv_edge[i];
  double su = 0.0, sp = 0.0, sdu = 0.0, sdp = 0.0;
  for (int j = 0; j < n2; ++j) {
    const int eo = m.edgesOnEdge[e * me2 + j];
    const size_t io = (size_t)eo * L + k;
    const double w = m.weightsOnEdge[e * me2 + j];
    su = fma(w, f.u[io], su);
    sp = fma(w, f.ke_edge[io], sp);
    sdu = fma(w, d.u[io], sdu);
    sdp = fma(w, d.ke_edge[io], sdp);
  }
  const double q = 0.5 * (pv_self * su + sp);
  const double dq = 0.5 * ((dpv_self * su + pv_self * sdu) + sdp);
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  const double inv_dc = m.invDcEdge[e];
  const double rho_e = f.h_edge[i], drho_e = d.h_edge[i];
  const double keg = (f.ke[i2] - f.ke[i1]) * inv_dc, dkeg = (d.ke[i2] - d.ke[i1]) * inv_dc;
  dtu += drho_e * (q - keg) + rho_e * (dq - dkeg) - d.u[i] * 0.5 * (f.h_divergence[i1] + f.h_divergence[i2]) -
         f.u[i] * 0.5 * (d.h_divergence[i1] + d.h_divergence[i2]);
  const double ray = adj_ray_damp(p.dm, k, L);  // tu - rho_edge u damp (every RK stage)
  if (ray != 0.0) dtu -= (drho_e * f.u[i] + rho_e * d.u[i]) * ray;
  if (p.rk_step == 1) {
    const double zzm = 0.5 * (m.zz[i2] + m.zz[i1]);
    double dP = (d.pressure_p[i2] - d.pressure_p[i1]) * inv_dc;
    if (zzm != 1.0) dP = dP / zzm;
    double dteu = -f.cqu_e[i] * (dP - 0.5 * m.zxu[i] * (d.dpdz[i1] + d.dpdz[i2]));
    const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
    const double r_dv = fmin(m.invDvEdge[e], 4.0 * inv_dc);
    const double ud = f.delsq_u[i];
    const double dud = (d.divergence[i2] - d.divergence[i1]) * inv_dc -
                       (d.vorticity[(size_t)v2 * L + k] - d.vorticity[(size_t)v1 * L + k]) * r_dv;
    d.delsq_u[i] = dud;
    const double kdu = 0.5 * (f.kdiff[i1] + f.kdiff[i2]), dkdu = 0.5 * (d.kdiff[i1] + d.kdiff[i2]);
    dteu += m.meshScalingDel2[e] * (drho_e * kdu * ud + rho_e * dkdu * ud + rho_e * kdu * dud);
    d.tend_u_euler[i] = dteu;
    d.tend_u[i] = defer ? dtu : dtu + dteu;
  } else {
    d.tend_u[i] = dtu + d.tend_u_euler[i];
  }
}

// ---- rk 1, del4: curl and divergence of delsq_u's tangent (k_del4_vertex / k_del4_cell)
__global__ void k_tan_del4_vertex(mpasg_mesh m, mpasg_fields d, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  const uint32_t v = fl.div(i), k = i - v * L;
  const int vd = m.vertexDegree;
  double acc = 0.0;
  for (int j = 0; j < vd; ++j) {
    const int e = m.edgesOnVertex[v * vd + j];
    const double es = m.invAreaTriangle[v] * m.dcEdge[e] * m.edgesOnVertex_sign[v * vd + j];
    acc += es * d.delsq_u[(size_t)e * L + k];
  }
  d.delsq_vort[i] = acc;
}

__global__ void k_tan_del4_cell(mpasg_mesh m, mpasg_fields d, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const double es = m.invAreaCell[c] * m.dvEdge[e] * m.edgesOnCell_sign[c * me + j];
    acc += es * d.delsq_u[(size_t)e * L + k];
  }
  d.delsq_div[i] = acc;
}

// ---- rk 1: del4 filter and vertical mixing of u (k_tend_u_finish)
__global__ void k_tan_u_finish(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, TanTendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  double dteu = d.tend_u_euler[i];
  if (p.del4) {
    const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
    const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
    const double inv_dc = m.invDcEdge[e];
    const double u_mix = m.meshScalingDel4[e] * p.h_mom_visc4;
    const double r_dc4 = u_mix * p.del4u_div * inv_dc;
    const double r_dv4 = u_mix * fmin(m.invDvEdge[e], 4.0 * inv_dc);
    const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
    const size_t j1 = (size_t)v1 * L + k, j2 = (size_t)v2 * L + k;
    const double ud4 = (f.delsq_div[i2] - f.delsq_div[i1]) * r_dc4 - (f.delsq_vort[j2] - f.delsq_vort[j1]) * r_dv4;
    const double dud4 = (d.delsq_div[i2] - d.delsq_div[i1]) * r_dc4 - (d.delsq_vort[j2] - d.delsq_vort[j1]) * r_dv4;
    dteu -= d.h_edge[i] * ud4 + f.h_edge[i] * dud4;
  }
  if (p.dm.v_mom > 0.0 && k >= 1 && k + 1 < (uint32_t)L) {
    // teu += h v (d_up - d_dn) / den; the initial profiles of the perturbation form are constants
    const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
    const double* z1p = m.zgrid + (size_t)c1 * (L + 1);
    const double* z2p = m.zgrid + (size_t)c2 * (L + 1);
    const double za = 0.5 * (z1p[k - 1] + z2p[k - 1]), zb = 0.5 * (z1p[k] + z2p[k]);
    const double zc = 0.5 * (z1p[k + 1] + z2p[k + 1]), zd = 0.5 * (z1p[k + 2] + z2p[k + 2]);
    const double zm = 0.5 * (za + zb), z0 = 0.5 * (zb + zc), zp = 0.5 * (zc + zd);
    const double* u = f.u + (size_t)e * L;
    const double* du = d.u + (size_t)e * L;
    double um = u[k - 1], u0 = u[k], up = u[k + 1];
    if (p.mix_pert) {
      const double ca = cos(m.angleEdge[e]), sa = sin(m.angleEdge[e]);
      um = um - m.u_init[k - 1] * ca - m.v_init[k - 1] * sa;
      u0 = u0 - m.u_init[k] * ca - m.v_init[k] * sa;
      up = up - m.u_init[k + 1] * ca - m.v_init[k + 1] * sa;
    }
    const double den = 0.5 * (zp - zm), v = p.dm.v_mom;
    const double s = (up - u0) / (zp - z0) - (u0 - um) / (z0 - zm);
    const double ds = (du[k + 1] - du[k]) / (zp - z0) - (du[k] - du[k - 1]) / (z0 - zm);
    dteu += v * (d.h_edge[i] * s + f.h_edge[i] * ds) / den;
  }
  d.tend_u_euler[i] = dteu;
  d.tend_u[i] = d.tend_u[i] + dteu;
}

// ---- rk 1: w / theta del2 mixing with kdiff and the del2 fields (k_mix_cells_a)
__global__ void k_tan_mix_a(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  if (k >= 1 && k < L) {
    double ddw = 0.0, dtw = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      const int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      const double es = m.cell_edge_es_w[c * me + j];
      const size_t ie = (size_t)e * L + k;
      const double he = f.h_edge[ie] + f.h_edge[ie - 1], dhe = d.h_edge[ie] + d.h_edge[ie - 1];
      const size_t w1 = (size_t)ec1 * (L + 1) + k, w2 = (size_t)ec2 * (L + 1) + k;
      const double dw = f.w[w2] - f.w[w1], ddwv = d.w[w2] - d.w[w1];
      const double flux = es * he * dw;
      const double dflux = es * (dhe * dw + he * ddwv);
      ddw += dflux;
      const size_t a1 = (size_t)ec1 * L + k, a2 = (size_t)ec2 * L + k;
      const double K = 0.25 * (f.kdiff[a1] + f.kdiff[a2] + f.kdiff[a1 - 1] + f.kdiff[a2 - 1]);
      const double dK = 0.25 * (d.kdiff[a1] + d.kdiff[a2] + d.kdiff[a1 - 1] + d.kdiff[a2 - 1]);
      dtw += m.meshScalingDel2[e] * (dflux * K + flux * dK);
    }
    d.delsq_w[i] = ddw;
    d.tend_w_euler[i] = dtw;
  } else {
    d.delsq_w[i] = 0.0;
    d.tend_w_euler[i] = 0.0;
  }
  if (k < L) {
    const size_t o = (size_t)c * L + k;
    double ddt = 0.0, dtt = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      const int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      const double es = m.cell_edge_es_t[c * me + j];
      const size_t a1 = (size_t)ec1 * L + k, a2 = (size_t)ec2 * L + k;
      const size_t ie = (size_t)e * L + k;
      const double dth = f.theta_m[a2] - f.theta_m[a1], ddth = d.theta_m[a2] - d.theta_m[a1];
      const double flux = es * dth * f.h_edge[ie];
      const double dflux = es * (ddth * f.h_edge[ie] + dth * d.h_edge[ie]);
      ddt += dflux;
      const double K = 0.5 * (f.kdiff[a1] + f.kdiff[a2]), dK = 0.5 * (d.kdiff[a1] + d.kdiff[a2]);
      dtt += m.meshScalingDel2[e] * (dflux * K + flux * dK);
    }
    d.delsq_theta[o] = ddt;
    d.tend_theta_euler[o] = dtt;
  }
}

// ---- rk 1: del4 parts of w / theta mixing (k_mix_cells_b, linear in the del2 fields)
__global__ void k_tan_mix_b(mpasg_mesh m, mpasg_fields d, FastDiv fl1, double h_mom_visc4, double h_theta_visc4) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  if (k >= 1 && k < L) {
    double tw = d.tend_w_euler[i];
    const double hm = h_mom_visc4 * ia;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      const int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      const double es = m.meshScalingDel4[e] * hm * m.dvEdge[e] * m.edgesOnCell_sign[c * me + j] * m.invDcEdge[e];
      tw -= es * (d.delsq_w[(size_t)ec2 * (L + 1) + k] - d.delsq_w[(size_t)ec1 * (L + 1) + k]);
    }
    d.tend_w_euler[i] = tw;
  }
  if (k < L) {
    const size_t o = (size_t)c * L + k;
    double tt = d.tend_theta_euler[o];
    const double ht = h_theta_visc4 * ia;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      const int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      const double es = m.meshScalingDel4[e] * ht * m.dvEdge[e] * m.edgesOnCell_sign[c * me + j] * m.invDcEdge[e];
      tt -= es * (d.delsq_theta[(size_t)ec2 * L + k] - d.delsq_theta[(size_t)ec1 * L + k]);
    }
    d.tend_theta_euler[o] = tt;
  }
}

// ---- horizontal advective fluxes of theta and w per edge (k_adv_edges); upwind side frozen
__global__ void k_tan_adv_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const int na = m.nAdvMax;
  const int nadv = m.nAdvCellsForEdge[e];
  const int32_t* cells = m.advCellsForEdge + (size_t)e * na;
  const double* cfp = m.adv_coefs_p + (size_t)e * na;
  const double* cfm = m.adv_coefs_m + (size_t)e * na;
  const double rue = f.ru[i], drue = d.ru[i];
  {
    const double* cf = rue >= 0.0 ? cfp : cfm;
    double acc = 0.0, dacc = 0.0;
    for (int a = 0; a < nadv; ++a) {
      const size_t o = (size_t)cells[a] * L + k;
      acc += cf[a] * f.theta_m[o];
      dacc += cf[a] * d.theta_m[o];
    }
    d.flux_th_e[i] = drue * acc + rue * dacc;
  }
  if (k >= 1) {
    const double ru_w = m.fzm[k] * rue + m.fzp[k] * f.ru[i - 1];
    const double dru_w = m.fzm[k] * drue + m.fzp[k] * d.ru[i - 1];
    const double* cf = ru_w >= 0.0 ? cfp : cfm;
    double acc = 0.0, dacc = 0.0;
    for (int a = 0; a < nadv; ++a) {
      const size_t o = (size_t)cells[a] * (L + 1) + k;
      acc += cf[a] * f.w[o];
      dacc += cf[a] * d.w[o];
    }
    d.flux_w_e[i] = dru_w * acc + ru_w * dacc;
  }
}

// tangent of the vertical w flux at interface q of a column (wdwz_at)
MPASG_D double tan_wdwz(const double* w, const double* rw, const double* dw, const double* drw, int q, int L) {
  if (q <= 0 || q >= L) return 0.0;
  if (q == 1 || q == L - 1)
    return 0.25 * ((drw[q] + drw[q - 1]) * (w[q] + w[q - 1]) + (rw[q] + rw[q - 1]) * (dw[q] + dw[q - 1]));
  const Flux3Grad g = flux3_grad(w[q - 2], w[q - 1], w[q], w[q + 1], 0.5 * (rw[q] + rw[q - 1]), 1.0);
  return g.qm2 * dw[q - 2] + g.qm1 * dw[q - 1] + g.q0 * dw[q] + g.qp1 * dw[q + 1] + g.ua * 0.5 * (drw[q] + drw[q - 1]);
}

// tangent of the vertical theta flux at interface q of a column (wdtz_at, float64 form)
MPASG_D double tan_wdtz(const mpasg_mesh& m, const double* th, const double* ths, const double* rw, const double* rws,
                        const double* dth, const double* dths, const double* drw, const double* drws, int q, int L,
                        double coef3) {
  if (q <= 0 || q >= L) return 0.0;
  const double fm = m.fzm[q], fp = m.fzp[q];
  if (q == L - 1 && q != 1) return drws[q] * (fm * th[q] + fp * th[q - 1]) + rws[q] * (fm * dth[q] + fp * dth[q - 1]);
  double v;
  if (q == 1) {
    v = drw[q] * (fm * th[q] + fp * th[q - 1]) + rw[q] * (fm * dth[q] + fp * dth[q - 1]);
  } else {
    const Flux3Grad g = flux3_grad(th[q - 2], th[q - 1], th[q], th[q + 1], rw[q], coef3);
    v = g.qm2 * dth[q - 2] + g.qm1 * dth[q - 1] + g.q0 * dth[q] + g.qp1 * dth[q + 1] + g.ua * drw[q];
  }
  const double tse = fm * ths[q] + fp * ths[q - 1], dtse = fm * dths[q] + fp * dths[q - 1];
  return v + (drws[q] - drw[q]) * tse + (rws[q] - rw[q]) * dtse;
}

// ---- w and theta tendencies (k_tend_w_theta); index space (C, L+1)
__global__ void k_tan_w_theta(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl1, TanTendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  const size_t oc = (size_t)c * L, ow = (size_t)c * (L + 1);
  if (k >= 1 && k < L) {
    double dtw = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      dtw -= m.edgesOnCell_sign[c * me + j] * d.flux_w_e[(size_t)e * L + k];
    }
    const double* w = f.w + ow;
    const double* rw = f.rw + ow;
    const double* dw = d.w + ow;
    const double* drw = d.rw + ow;
    dtw = dtw * ia - m.rdzu[k] * (tan_wdwz(w, rw, dw, drw, k + 1, L) - tan_wdwz(w, rw, dw, drw, k, L));
    double dteu = d.tend_w_euler[i];
    if (p.rk_step == 1) {
      const double dres = m.rdzu[k] * (d.pressure_p[oc + k] - d.pressure_p[oc + k - 1]) -
                          (m.fzm[k] * d.dpdz[oc + k] + m.fzp[k] * d.dpdz[oc + k - 1]);
      dteu -= f.cqw[ow + k] * dres;
      if (p.dm.v_mom > 0.0) {  // vertical mixing of w: v rho_half (w_up - w_down) rdzu
        const double rho_half = 0.5 * (f.rho_zz[oc + k] + f.rho_zz[oc + k - 1]);
        const double drho_half = 0.5 * (d.rho_zz[oc + k] + d.rho_zz[oc + k - 1]);
        const double wud = (w[k + 1] - w[k]) * m.rdzw[k] - (w[k] - w[k - 1]) * m.rdzw[k - 1];
        const double dwud = (dw[k + 1] - dw[k]) * m.rdzw[k] - (dw[k] - dw[k - 1]) * m.rdzw[k - 1];
        dteu += p.dm.v_mom * (drho_half * wud + rho_half * dwud) * m.rdzu[k];
      }
      d.tend_w_euler[i] = dteu;
    }
    d.tend_w[i] = dtw + dteu;
  } else {
    d.tend_w[i] = 0.0;
  }
  if (k < L) {
    const size_t o = oc + k;
    double dtt = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      dtt -= m.edgesOnCell_sign[c * me + j] * d.flux_th_e[(size_t)e * L + k];
    }
    if (p.rk_step > 1) {
      for (int j = 0; j < n; ++j) {
        const int e = m.edgesOnCell[c * me + j];
        const size_t ie = (size_t)e * L + k;
        dtt -= m.cell_edge_sdv[c * me + j] * ((d.ru_save[ie] - d.ru[ie]) * f.theta_edge_save[ie] +
                                              (f.ru_save[ie] - f.ru[ie]) * d.theta_edge_save[ie]);
      }
    }
    dtt = dtt * ia -
          m.rdzw[k] * (tan_wdtz(m, f.theta_m + oc, f.theta_m_save + oc, f.rw + ow, f.rw_save + ow, d.theta_m + oc,
                                d.theta_m_save + oc, d.rw + ow, d.rw_save + ow, k + 1, L, p.coef3) -
                       tan_wdtz(m, f.theta_m + oc, f.theta_m_save + oc, f.rw + ow, f.rw_save + ow, d.theta_m + oc,
                                d.theta_m_save + oc, d.rw + ow, d.rw_save + ow, k, L, p.coef3));
    dtt += d.rho_zz[o] * f.rt_diabatic_tend[o];
    double dtte = d.tend_theta_euler[o];
    if (p.rk_step == 1 && p.dm.v_theta > 0.0 && k >= 1 && k + 1 < L) {
      // vertical mixing of theta: v rho_zz diff / den, the initial profile a constant
      const double* zg = m.zgrid + (size_t)c * (L + 1);
      const double zm = 0.5 * (zg[k - 1] + zg[k]), z0 = 0.5 * (zg[k] + zg[k + 1]), zp = 0.5 * (zg[k + 1] + zg[k + 2]);
      const double* th = f.theta_m + oc;
      const double* dth = d.theta_m + oc;
      double tm = th[k - 1], t0 = th[k], tp = th[k + 1];
      if (p.mix_pert) {
        const double* ti = m.t_init + oc;
        tm = tm - ti[k - 1];
        t0 = t0 - ti[k];
        tp = tp - ti[k + 1];
      }
      const double diff = (tp - t0) / (zp - z0) - (t0 - tm) / (z0 - zm);
      const double ddiff = (dth[k + 1] - dth[k]) / (zp - z0) - (dth[k] - dth[k - 1]) / (z0 - zm);
      dtte += p.dm.v_theta * (d.rho_zz[o] * diff + f.rho_zz[o] * ddiff) / (0.5 * (zp - zm));
      d.tend_theta_euler[o] = dtte;
    }
    d.tend_theta[o] = dtt + dtte;
  }
}

// ================================================================= diagnostics
__global__ void k_tan_diag_edges_a(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  d.h_edge[i] = 0.5 * (d.rho_zz[(size_t)c1 * L + k] + d.rho_zz[(size_t)c2 * L + k]);
  d.ke_edge[i] = m.edge_dcdv[e] * 2.0 * f.u[i] * d.u[i];
}

__global__ void k_tan_diag_vertices(mpasg_mesh m, mpasg_fields d, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  const uint32_t v = fl.div(i), k = i - v * L;
  const int vd = m.vertexDegree;
  double vort = 0.0, kev = 0.0;
  for (int j = 0; j < vd; ++j) {
    const int e = m.edgesOnVertex[v * vd + j];
    vort += m.vertex_edge_sdc[v * vd + j] * d.u[(size_t)e * L + k];
    kev += d.ke_edge[(size_t)e * L + k];
  }
  const double iat = m.invAreaTriangle[v];
  vort *= iat;
  d.vorticity[i] = vort;
  d.ke_vertex[i] = 0.25 * iat * kev;
  d.pv_vertex[i] = vort;
}

__global__ void k_tan_diag_cells(mpasg_mesh m, mpasg_fields d, FastDiv fl, int apvm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double div = 0.0, ke = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    div += m.cell_edge_sdv[c * me + j] * d.u[(size_t)e * L + k];
    ke += d.ke_edge[(size_t)e * L + k];
  }
  const double ia = m.invAreaCell[c];
  const double ke_fact = 1.0 - 0.375;
  ke = ke_fact * ((0.25 * ke) * ia);
  const int vd = m.vertexDegree;
  double pvc = 0.0;
  for (int j = 0; j < n; ++j) {
    const int v = m.verticesOnCell[c * me + j];
    const int kk = m.kiteForCell[c * me + j];
    if (v >= m.nVertices || kk < 0) continue;
    const double kite = m.kiteAreasOnVertex[v * vd + kk];
    ke += (1.0 - ke_fact) * kite * d.ke_vertex[(size_t)v * L + k] * ia;
    if (apvm) pvc += kite * d.pv_vertex[(size_t)v * L + k] * ia;
  }
  d.divergence[i] = div * ia;
  d.ke[i] = ke;
  if (apvm) d.pv_cell[i] = pvc;
}

__global__ void k_tan_diag_edges_b(mpasg_mesh m, mpasg_fields f, mpasg_fields d, FastDiv fl, int recompute_v,
                                   double apvm_dt, int apvm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
  const size_t j1 = (size_t)v1 * L + k, j2 = (size_t)v2 * L + k;
  double dpve = 0.5 * (d.pv_vertex[j1] + d.pv_vertex[j2]);
  double dvv;
  if (recompute_v) {
    const int n2 = m.nEdgesOnEdge[e];
    const int me2 = m.maxEdges2;
    dvv = 0.0;
    for (int j = 0; j < n2; ++j)
      dvv += m.weightsOnEdge[e * me2 + j] * d.u[(size_t)m.edgesOnEdge[e * me2 + j] * L + k];
    d.v[i] = dvv;
  } else {
    dvv = d.v[i];
  }
  if (apvm) {
    const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
    const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
    const double gt = (f.pv_vertex[j2] - f.pv_vertex[j1]) * m.invDvEdge[e];
    const double dgt = (d.pv_vertex[j2] - d.pv_vertex[j1]) * m.invDvEdge[e];
    const double gn = (f.pv_cell[i2] - f.pv_cell[i1]) * m.invDcEdge[e];
    const double dgn = (d.pv_cell[i2] - d.pv_cell[i1]) * m.invDcEdge[e];
    dpve -= apvm_dt * (dvv * gt + f.v[i] * dgt + d.u[i] * gn + f.u[i] * dgn);
  }
  d.pv_edge[i] = dpve;
}

}  // namespace

// after the forward tendencies of rk stage rk_step on f
int mpasgi_dyn_tend_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                             int rk_step, cudaStream_t s) {
  const int L = m->nVertLevels;
  const long long ncl = (long long)m->nCells * L, nel = (long long)m->nEdges * L;
  const long long ncw = (long long)m->nCells * (L + 1), nvl = (long long)m->nVertices * L;
  FastDiv fl(L), fl1(L + 1);
  TanTendScalars p{};
  const double cl = c->c_s * c->len_disp;
  p.cs2 = cl * cl;
  p.kdiff_cap = (0.01 * (c->len_disp * c->len_disp)) * (1.0 / c->dt);
  p.smag = c->horiz_mixing_smagorinsky;
  if (p.smag) {
    p.h_mom_visc4 = c->visc4_2dsmag * std::pow(c->len_disp, 3.0);
    p.h_theta_visc4 = p.h_mom_visc4;
  } else {
    p.h_mom_visc4 = c->h_mom_eddy_visc4;
    p.h_theta_visc4 = c->h_theta_eddy_visc4;
  }
  p.del4u_div = c->del4u_div_factor;
  p.coef3 = c->coef_3rd_order;
  p.rk_step = rk_step;
  p.del4 = p.h_mom_visc4 > 0.0 ? 1 : 0;
  p.mix_pert = c->mix_perturbation ? 1 : 0;
  p.dm = adj_damping(c);
  const int defer = (p.del4 || p.dm.v_mom > 0.0) ? 1 : 0;  // as the forward's TendScalars.defer
  k_tan_cells_a<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, *d, fl, p);
  MPASG_LAUNCH_CHECK();
  k_tan_pvu<<<nblocks(nel), kBlock, 0, s>>>(*f, *d, nel);
  MPASG_LAUNCH_CHECK();
  k_tan_u<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *d, fl, p, defer);
  MPASG_LAUNCH_CHECK();
  if (rk_step == 1) {
    if (p.del4) {
      k_tan_del4_vertex<<<nblocks(nvl), kBlock, 0, s>>>(*m, *d, fl);
      MPASG_LAUNCH_CHECK();
      k_tan_del4_cell<<<nblocks(ncl), kBlock, 0, s>>>(*m, *d, fl);
      MPASG_LAUNCH_CHECK();
    }
    if (defer) {
      k_tan_u_finish<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *d, fl, p);
      MPASG_LAUNCH_CHECK();
    }
    k_tan_mix_a<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *d, fl1);
    MPASG_LAUNCH_CHECK();
    if (p.h_mom_visc4 > 0.0 || p.h_theta_visc4 > 0.0) {
      k_tan_mix_b<<<nblocks(ncw), kBlock, 0, s>>>(*m, *d, fl1, p.h_mom_visc4 > 0.0 ? p.h_mom_visc4 : 0.0,
                                                  p.h_theta_visc4);
      MPASG_LAUNCH_CHECK();
    }
  }
  k_tan_adv_edges<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *d, fl);
  MPASG_LAUNCH_CHECK();
  k_tan_w_theta<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *d, fl1, p);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// after the forward diagnostics of rk stage rk_step (3: and the preparation) on f
int mpasgi_diag_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                         int rk_step, cudaStream_t s) {
  const int L = m->nVertLevels;
  FastDiv fl(L);
  const int apvm = c->apvm_upwinding > 0.0 ? 1 : 0;
  k_tan_diag_edges_a<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *d, fl);
  MPASG_LAUNCH_CHECK();
  k_tan_diag_vertices<<<nblocks((long long)m->nVertices * L), kBlock, 0, s>>>(*m, *d, fl);
  MPASG_LAUNCH_CHECK();
  k_tan_diag_cells<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *d, fl, apvm);
  MPASG_LAUNCH_CHECK();
  k_tan_diag_edges_b<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *d, fl, rk_step == 3 ? 1 : 0,
                                                                          c->apvm_upwinding * c->dt, apvm);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
