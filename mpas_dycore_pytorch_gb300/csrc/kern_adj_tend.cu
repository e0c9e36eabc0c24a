// Reverse mode of the large-step tendencies (the reference's atm_compute_dyn_tend_work,
// mpas_pytorch/dynamics/dyn_tend.py:10836; the reference differentiates it through the
// ordered-transpose custom Functions at :1194, :1413, :1568, :3860).
//
// The forward stage (kern_tend.cu) forms cell sums over edges, edge values from two cells,
// the TRiSK sum over edgesOnEdge, the advection stencils and column fluxes.  Each is read
// backwards as a gather over the outputs that read the thread's input: an edge collects its
// two cells (slot of the edge in each cell from the transposed connectivity), a cell its
// edges, a vertex its edges, an edge its TRiSK neighbours, a cell the advection-stencil
// slots that read it (CSR), a level its neighbour levels.  Per-edge partial products that a
// cell or vertex gather needs are written to the work buffer first.  No atomics: every
// cotangent is a fixed-order sum, so results are bitwise reproducible.
//
// Values the derivatives need and the forward does not keep (the mass-flux divergence, the
// Smagorinsky deformation and kdiff, the del2 field of u and its del4 divergence and curl)
// are recomputed here from the stage's inputs, with the forward's expressions.
#include "adj_common.cuh"

namespace {

struct AdjTendScalars {
  double cs2, kdiff_cap, h_mom_visc4, h_theta_visc4, del4u_div, coef3, visc2;
  int rk_step, smag, del4;
  int mix_pert;  // vertical mixing of the perturbation from the initial profiles
  AdjDamping dm;  // CAM floor of kdiff, Rayleigh damping of u, vertical mixing
};

// ---- values: mass-flux divergence (every rk) and, at rk 1, Smagorinsky deformation and kdiff
__global__ void k_tadj_values(mpasg_mesh m, mpasg_fields f, FastDiv fl, AdjTendScalars p, double* __restrict__ hd,
                              double* __restrict__ kd, double* __restrict__ dd_out, double* __restrict__ do_out) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double h = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const double t = m.cell_edge_sdv[c * me + j] * f.ru[(size_t)e * L + k];
    h = (j == 0) ? t : h + t;
  }
  hd[i] = h * m.invAreaCell[c];
  if (p.rk_step != 1) return;
  if (p.smag) {
    // Separately rounded products and sums in the reference's order: over a nearly rigid
    // flow the deformation is a few roundings of its terms, and the direction of kdiff's
    // derivative (dd, do) / |(dd, do)| follows those roundings exactly.
    double dd = 0.0, dof = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.edgesOnCell[c * me + j];
      const double ca = m.defc_a[c * me + j], cb = m.defc_b[c * me + j];
      const double ue = f.u[(size_t)e * L + k], ve = f.v[(size_t)e * L + k];
      const double ndd = __dsub_rn(__dadd_rn(dd, __dmul_rn(ca, ue)), __dmul_rn(cb, ve));
      const double ndo = __dadd_rn(__dadd_rn(dof, __dmul_rn(cb, ue)), __dmul_rn(ca, ve));
      dd = ndd;
      dof = ndo;
    }
    double kdv = fmin(__dmul_rn(p.cs2, sqrt(__dadd_rn(__dmul_rn(dd, dd), __dmul_rn(dof, dof)))), p.kdiff_cap);
    if (p.dm.ncam > 0 && (int)k >= L - p.dm.ncam) kdv = fmax(kdv, adj_cam_floor(p.dm, (int)k, L));
    kd[i] = kdv;
    dd_out[i] = dd;
    do_out[i] = dof;
  } else {
    kd[i] = (p.dm.ncam > 0 && (int)k >= L - p.dm.ncam) ? fmax(p.visc2, adj_cam_floor(p.dm, (int)k, L)) : p.visc2;
  }
}

// ---- values (rk 1, del4): del2 of u on the edges (the forward's delsq_u = u_diff)
__global__ void k_tadj_udiff(mpasg_mesh m, mpasg_fields f, FastDiv fl, double* __restrict__ ud) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
  const double inv_dc = m.invDcEdge[e];
  const double r_dv = fmin(m.invDvEdge[e], 4.0 * inv_dc);
  ud[i] = (f.divergence[(size_t)c2 * L + k] - f.divergence[(size_t)c1 * L + k]) * inv_dc -
          (f.vorticity[(size_t)v2 * L + k] - f.vorticity[(size_t)v1 * L + k]) * r_dv;
}

// ---- values (rk 1, del4): its divergence (cells) and curl (vertices), as k_del4_cell / k_del4_vertex
__global__ void k_tadj_del4_cells(mpasg_mesh m, FastDiv fl, const double* __restrict__ ud, double* __restrict__ dsd) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const double t = (m.invAreaCell[c] * m.dvEdge[e] * m.edgesOnCell_sign[c * me + j]) * ud[(size_t)e * L + k];
    acc = (j == 0) ? t : acc + t;
  }
  dsd[i] = acc;
}

__global__ void k_tadj_del4_vertices(mpasg_mesh m, FastDiv fl, const double* __restrict__ ud,
                                     double* __restrict__ dsv) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  const uint32_t v = fl.div(i), k = i - v * L;
  const int vd = m.vertexDegree;
  double acc = 0.0;
  for (int j = 0; j < vd; ++j) {
    const int e = m.edgesOnVertex[v * vd + j];
    const double t = (m.invAreaTriangle[v] * m.dcEdge[e] * m.edgesOnVertex_sign[v * vd + j]) * ud[(size_t)e * L + k];
    acc = (j == 0) ? t : acc + t;
  }
  dsv[i] = acc;
}

// vertical theta flux at interface q (k_tend_w_theta's wdtz_at, float64 form) and its
// partial derivatives with respect to theta_m[q-2..q+1], theta_m_save[q-1..q], rw[q], rw_save[q]
struct WdtzGrad {
  double th[4];  // q-2, q-1, q, q+1
  double ths[2];  // q-1, q
  double rw, rws;
};
MPASG_D WdtzGrad wdtz_grad(const mpasg_mesh& m, const double* th, const double* ths, const double* rw,
                           const double* rws, int q, int L, double coef3) {
  WdtzGrad d = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0}, 0.0, 0.0};
  const double fm = m.fzm[q], fp = m.fzp[q];
  if (q == L - 1 && q != 1) {
    d.th[2] = rws[q] * fm;
    d.th[1] = rws[q] * fp;
    d.rws = fm * th[q] + fp * th[q - 1];
    return d;
  }
  if (q == 1) {
    d.th[2] = rw[q] * fm;
    d.th[1] = rw[q] * fp;
    d.rw = fm * th[q] + fp * th[q - 1];
  } else {
    const Flux3Grad g = flux3_grad(th[q - 2], th[q - 1], th[q], th[q + 1], rw[q], coef3);
    d.th[0] = g.qm2;
    d.th[1] = g.qm1;
    d.th[2] = g.q0;
    d.th[3] = g.qp1;
    d.rw = g.ua;
  }
  const double tse = fm * ths[q] + fp * ths[q - 1];
  d.rw -= tse;
  d.rws = tse;
  d.ths[1] = (rws[q] - rw[q]) * fm;
  d.ths[0] = (rws[q] - rw[q]) * fp;
  return d;
}

// vertical w flux at interface q (wdwz_at) and its partials: w[q-2..q+1], rw[q-1], rw[q]
struct WdwzGrad {
  double w[4];
  double rwm, rw;
};
MPASG_D WdwzGrad wdwz_grad(const double* w, const double* rw, int q, int L) {
  WdwzGrad d = {{0.0, 0.0, 0.0, 0.0}, 0.0, 0.0};
  if (q == 1 || q == L - 1) {
    const double a = 0.25 * (w[q] + w[q - 1]), b = 0.25 * (rw[q] + rw[q - 1]);
    d.rw = a;
    d.rwm = a;
    d.w[2] = b;
    d.w[1] = b;
    return d;
  }
  const Flux3Grad g = flux3_grad(w[q - 2], w[q - 1], w[q], w[q + 1], 0.5 * (rw[q] + rw[q - 1]), 1.0);
  d.w[0] = g.qm2;
  d.w[1] = g.qm1;
  d.w[2] = g.q0;
  d.w[3] = g.qp1;
  d.rw = 0.5 * g.ua;
  d.rwm = 0.5 * g.ua;
  return d;
}

// ---- columns of the theta and w tendencies read backwards (index space C x (L+1)):
// vertical fluxes of theta and w, the flux divergences' area factor, the buoyancy /
// pressure-gradient residual (rk 1), the diabatic term, and the Euler tendencies
// (collected for the mixing at rk 1, passed through at rk 2 and 3)
__global__ void k_tadj_columns(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1, AdjTendScalars p,
                               double* __restrict__ tt1b, double* __restrict__ tw1b, double* __restrict__ tweb,
                               double* __restrict__ tteb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t oc = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double ia = m.invAreaCell[c];
  const double* th = f.theta_m + oc;
  const double* ths = f.theta_m_save + oc;
  const double* rw = f.rw + ow;
  const double* rws = f.rw_save + ow;
  const double* w = f.w + ow;
  auto Gtt = [&](int q) { return (q >= 0 && q < L) ? g.tend_theta[oc + q] : 0.0; };
  auto Gtw = [&](int q) { return (q >= 1 && q <= L - 1) ? g.tend_w[ow + q] : 0.0; };
  auto wdtzb = [&](int q) { return Gtt(q) * (q < L ? m.rdzw[q] : 0.0) - Gtt(q - 1) * (q >= 1 ? m.rdzw[q - 1] : 0.0); };
  auto wdwzb = [&](int q) { return Gtw(q) * m.rdzu[q < L ? q : 0] * (q <= L - 1 ? 1.0 : 0.0) -
                                   Gtw(q - 1) * (q - 1 >= 1 ? m.rdzu[q - 1] : 0.0); };
  // ---- mass level k: theta
  if (k < L) {
    const size_t o = oc + k;
    const double G = g.tend_theta[o];
    g.rho_zz[o] += G * f.rt_diabatic_tend[o];
    tt1b[o] = G * ia;
    double gth = 0.0, gths = 0.0;
    for (int q = k - 1; q <= k + 2; ++q) {
      if (q < 1 || q > L - 1) continue;
      const double b = wdtzb(q);
      if (b == 0.0) continue;
      const WdtzGrad d = wdtz_grad(m, th, ths, rw, rws, q, L, p.coef3);
      const int s = k - (q - 2);  // position of level k in q-2..q+1
      gth += b * d.th[s];
      if (k == q - 1) gths += b * d.ths[0];
      if (k == q) gths += b * d.ths[1];
    }
    g.theta_m[o] += gth;
    g.theta_m_save[o] += gths;
    if (p.rk_step == 1) {
      tteb[o] = G + g.tend_theta_euler[o];
    } else {
      g.tend_theta_euler[o] += G;
    }
  }
  // ---- w level k: rw / rw_save from the theta flux, w / rw from the w flux
  double grw = 0.0, grws = 0.0, gw = 0.0;
  if (k >= 1 && k <= L - 1) {
    const double b = wdtzb(k);
    const WdtzGrad d = wdtz_grad(m, th, ths, rw, rws, k, L, p.coef3);
    grw += b * d.rw;
    grws += b * d.rws;
  }
  for (int q = k - 1; q <= k + 2; ++q) {
    if (q < 1 || q > L - 1) continue;
    const double b = wdwzb(q);
    if (b == 0.0) continue;
    const WdwzGrad d = wdwz_grad(w, rw, q, L);
    gw += b * d.w[k - (q - 2)];
    if (k == q) grw += b * d.rw;
    if (k == q - 1) grw += b * d.rwm;
  }
  g.rw[ow + k] += grw;
  g.rw_save[ow + k] += grws;
  g.w[ow + k] += gw;
  if (k >= 1 && k <= L - 1) {
    const double G = g.tend_w[ow + k];
    tw1b[ow + k] = G * ia;
    if (p.rk_step == 1) {
      tweb[ow + k] = G + g.tend_w_euler[ow + k];
    } else {
      g.tend_w_euler[ow + k] += G;
    }
  } else {
    tw1b[ow + k] = 0.0;
    tweb[ow + k] = 0.0;
  }
}

// ---- rk 1: pressure gradient / buoyancy residual of tend_w_euler read backwards, per
// mass level: -> pressure_p, rr_save (through dpdz)
__global__ void k_tadj_wres(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, const double* __restrict__ tweb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const size_t ow = (size_t)c * (L + 1);
  double gpp = 0.0, gdp = 0.0;
  if (k >= 1) {
    const double t = tweb[ow + k] * f.cqw[ow + k];
    gpp += -t * m.rdzu[k];
    gdp += t * m.fzm[k];
  }
  if (k + 1 <= L - 1) {
    const double t = tweb[ow + k + 1] * f.cqw[ow + k + 1];
    gpp += t * m.rdzu[k + 1];
    gdp += t * m.fzp[k + 1];
  }
  g.pressure_p[i] += gpp;
  g.rr_save[i] += gdp * (-kGravity) * (1.0 + f.qtot[i]);
}

// ---- edges: horizontal advective fluxes of theta and w read backwards (and, at rk > 1,
// the theta flux of the change of ru within the dynamics substep).  Writes the cotangents
// of the stencil sums (fltb, flwb) for the cell gather, adds to ru, ru_save and the
// edge-sum cotangent of theta_m_save.
// sgn_x >= 0 by the bits (no float64 comparison): true for +0 and -0
MPASG_D bool nonneg(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 || b == (long long)0x8000000000000000ull;
}

// Each thread forms the w stencil sum of its own level k once and shares the product with
// its flux cotangent; level k also needs level k+1's (shared memory, recomputed at the
// block's edge).  The upwind sides of the theta and w stencils are stored as bits in sel
// for the cell gather.
__global__ void __launch_bounds__(kBlock) k_tadj_adv_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields g,
                                                           mpasg_transpose t, FastDiv fl, AdjTendScalars p,
                                                           const double* __restrict__ tt1b,
                                                           const double* __restrict__ tw1b, double* __restrict__ fltb,
                                                           double* __restrict__ flwb, uint8_t* __restrict__ sel) {
  __shared__ double s_pw[kBlock];
  const int L = m.nVertLevels;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nEdges * L;
  const int me = m.maxEdges, na = m.nAdvMax;
  uint32_t e = 0;
  int k = 0, nadv = 0;
  const int32_t* cells = m.advCellsForEdge;
  // cotangents of the edge fluxes from the two cells' sums (x = -sign * flux)
  auto edge_b = [&](const double* src, int kk, size_t pitch) {
    double s = 0.0;
    for (int q = 0; q < 2; ++q) {
      const int j = t.edgeCellSlot[2 * e + q];
      if (j < 0) continue;
      const int c = m.cellsOnEdge[2 * e + q];
      s -= src[(size_t)c * pitch + kk] * m.edgesOnCell_sign[c * me + j];
    }
    return s;
  };
  auto adv_sum = [&](const double* fld, int kk, size_t pitch, bool up) {
    const double* cf = (up ? m.adv_coefs_p : m.adv_coefs_m) + (size_t)e * na;
    double acc = 0.0;
    for (int a = 0; a < nadv; ++a) {
      const double tt = cf[a] * fld[(size_t)cells[a] * pitch + kk];
      acc = (a == 0) ? tt : acc + tt;
    }
    return acc;
  };
  auto ru_w = [&](int kk) { return m.fzm[kk] * f.ru[(size_t)e * L + kk] + m.fzp[kk] * f.ru[(size_t)e * L + kk - 1]; };
  auto w_part = [&](int kk, bool* up) {  // fweb_kk * sum_a cf_a w_a, and the flux cotangent's product
    const double rwk = ru_w(kk);
    *up = nonneg(rwk);
    return edge_b(tw1b, kk, L + 1) * adv_sum(f.w, kk, L + 1, *up);
  };
  double pw = 0.0;
  bool up_w = true;
  if (active) {
    e = fl.div(i);
    k = (int)(i - e * L);
    nadv = m.nAdvCellsForEdge[e];
    cells = m.advCellsForEdge + (size_t)e * na;
    if (k >= 1) pw = w_part(k, &up_w);
  }
  s_pw[threadIdx.x] = pw;
  __syncthreads();
  if (!active) return;
  const double rue = f.ru[i];
  const bool up_t = nonneg(rue);
  // theta
  const double fteb = edge_b(tt1b, k, L);
  double gru = fteb * adv_sum(f.theta_m, k, L, up_t);
  fltb[i] = fteb * rue;
  // w at level k (k >= 1) and k + 1: ru_w = fzm ru_k + fzp ru_(k-1)
  if (k >= 1) {
    gru += pw * m.fzm[k];
    flwb[i] = edge_b(tw1b, k, L + 1) * ru_w(k);
  } else {
    flwb[i] = 0.0;
  }
  if (k + 1 <= L - 1) {
    bool dummy;
    const double pw1 = threadIdx.x + 1 < blockDim.x ? s_pw[threadIdx.x + 1] : w_part(k + 1, &dummy);
    gru += pw1 * m.fzp[k + 1];
  }
  sel[i] = (uint8_t)((up_t ? 1 : 0) | (k >= 1 && up_w ? 2 : 0));
  if (p.rk_step > 1) {  // - sum_j (sign dvEdge)_j (ru_save - ru) theta_edge_save
    double s_sdv = 0.0;
    for (int q = 0; q < 2; ++q) {
      const int j = t.edgeCellSlot[2 * e + q];
      if (j < 0) continue;
      const int c = m.cellsOnEdge[2 * e + q];
      s_sdv -= tt1b[(size_t)c * L + k] * m.cell_edge_sdv[c * me + j];
    }
    const double the = f.theta_edge_save[i];
    g.ru_save[i] += s_sdv * the;
    gru -= s_sdv * the;
    g.theta_edge_save[i] += 0.5 * s_sdv * (f.ru_save[i] - rue);
  }
  g.ru[i] += gru;
}

// ---- cells: the advection stencils transposed (CSR of (edge, slot) readers): theta, w;
// the upwind sides come from sel (bit 0 theta, bit 1 w)
__global__ void k_tadj_adv_cells(mpasg_mesh m, mpasg_fields g, mpasg_transpose t, FastDiv fl1, FastDiv fna,
                                 const double* __restrict__ fltb, const double* __restrict__ flwb,
                                 const uint8_t* __restrict__ sel) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  double gth = 0.0, gw = 0.0;
  const int p0 = t.advPtr[c], p1 = t.advPtr[c + 1];
  const bool th = k < L, wl = k >= 1 && k <= L - 1;
  for (int q = p0; q < p1; ++q) {
    const int es = t.advIdx[q];
    const uint32_t e = fna.div((uint32_t)es);
    const size_t ie = (size_t)e * L + k;
    const double cp = m.adv_coefs_p[es], cm = m.adv_coefs_m[es];
    if (th) {
      const uint8_t b = sel[ie];
      gth += ((b & 1) ? cp : cm) * fltb[ie];
      if (wl) gw += ((b & 2) ? cp : cm) * flwb[ie];
    }
  }
  if (th) g.theta_m[(size_t)c * L + k] += gth;
  g.w[i] += gw;
}

// ---- edges: the u tendency read backwards (vertical transport, PV flux, kinetic-energy
// gradient, divergence coupling; at rk 1 the pressure gradient and del2 / del4 mixing)
// qa = G rho_edge per edge level: the cotangent of the PV flux q of that edge, which every
// TRiSK neighbour of the edge reads
// per edge level, the factors the PV-flux transpose reads at every neighbour: qa = G
// rho_edge (the cotangent of that edge's PV flux sum), qa pv_edge, and pv_edge u (the
// forward sum's neighbour factor), so each neighbour costs four multiply-adds
__global__ void k_tadj_qa(int n, const double* __restrict__ gtu, const double* __restrict__ h,
                          const double* __restrict__ pv, const double* __restrict__ u, double* __restrict__ qa,
                          double* __restrict__ qapv, double* __restrict__ pvu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double q = gtu[i] * h[i];
  qa[i] = q;
  qapv[i] = q * pv[i];
  pvu[i] = pv[i] * u[i];
}

// The vertical-transport part per interface q of the edge: its flux's cotangent
// b_q = rdzw_q G_q - rdzw_(q-1) G_(q-1) times the flux's partials with respect to u at
// levels q-2 .. q+1 (c[0..3]; the second-order interfaces q = 1, L-1 read q-1, q only),
// and with respect to the interface's rw mean (pr)
struct WduzPart {
  double c[4];
  double pr;
};
MPASG_D WduzPart wduz_part(const mpasg_mesh& m, const mpasg_fields& f, const double* ue, const double* Gtu, int c1,
                           int c2, int q, int L) {
  WduzPart w = {{0.0, 0.0, 0.0, 0.0}, 0.0};
  if (q < 1 || q > L - 1) return w;
  double b = 0.0;
  if (q <= L - 1) b += Gtu[q] * m.rdzw[q];
  b -= Gtu[q - 1] * m.rdzw[q - 1];
  const double rwe = 0.5 * (f.rw[(size_t)c1 * (L + 1) + q] + f.rw[(size_t)c2 * (L + 1) + q]);
  if (q == 1 || q == L - 1) {
    const double br = b * rwe;
    w.c[2] = br * m.fzm[q];
    w.c[1] = br * m.fzp[q];
    w.pr = b * (m.fzm[q] * ue[q] + m.fzp[q] * ue[q - 1]);
    return w;
  }
  const Flux3Grad d = flux3_grad(ue[q - 2], ue[q - 1], ue[q], ue[q + 1], rwe, 1.0);
  w.c[0] = b * d.qm2;
  w.c[1] = b * d.qm1;
  w.c[2] = b * d.q0;
  w.c[3] = b * d.qp1;
  w.pr = b * d.ua;
  return w;
}

// Each thread forms the parts of its own interface k once; level k collects c[3], c[2],
// c[1], c[0] of interfaces k-1, k, k+1, k+2 from its neighbours in the block (shared
// memory), recomputing the few that fall outside it.
__global__ void __launch_bounds__(kBlock) k_tadj_u(mpasg_mesh m, mpasg_fields f, mpasg_fields g, mpasg_transpose t,
                                                   FastDiv fl, AdjTendScalars p, const double* __restrict__ hd,
                                                   const double* __restrict__ kd, const double* __restrict__ ud,
                                                   const double* __restrict__ dsd, const double* __restrict__ dsv,
                                                   double* __restrict__ pke, double* __restrict__ phd,
                                                   double* __restrict__ prwe, double* __restrict__ ppp,
                                                   double* __restrict__ pkd, double* __restrict__ udb,
                                                   double* __restrict__ pd4, const double* __restrict__ qa,
                                                   double* __restrict__ pdz, const double* __restrict__ qapv,
                                                   const double* __restrict__ pvu) {
  __shared__ double s_c[4][kBlock];
  const int L = m.nVertLevels;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nEdges * L;
  uint32_t e = 0;
  int k = 0, c1 = 0, c2 = 0;
  const double* ue = f.u;
  const double* Gtu = g.tend_u;
  WduzPart own = {{0.0, 0.0, 0.0, 0.0}, 0.0};
  if (active) {
    e = fl.div(i);
    k = (int)(i - e * L);
    c1 = m.cellsOnEdge[2 * e];
    c2 = m.cellsOnEdge[2 * e + 1];
    ue = f.u + (size_t)e * L;
    Gtu = g.tend_u + (size_t)e * L;
    own = wduz_part(m, f, ue, Gtu, c1, c2, k, L);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) s_c[j][threadIdx.x] = own.c[j];
  __syncthreads();
  if (!active) return;
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  const double G = Gtu[k];
  const double rho_e = f.h_edge[i];
  const double inv_dc = m.invDcEdge[e];
  // PV flux q_e = 0.5 sum_j w_j u_j (pv_e + pv_j), with its transpose over edgesOnEdge: the
  // neighbour eo's sum reads u_e and pv_e at its slot jt (cotangent of q_eo: G_eo rho_edge_eo)
  // four sums over the stencil, combined after the loop (four multiply-adds per slot, the
  // per-edge products from k_tadj_qa): s1 = sum w u, s2 = sum w (pv u), s3 = sum wt A,
  // s4 = sum wt (A pv), A = G_eo rho_edge_eo
  const int n2 = m.nEdgesOnEdge[e], me2 = m.maxEdges2;
  const double pv_self = f.pv_edge[i], u_self = ue[k];
  double s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
  for (int j = 0; j < n2; ++j) {
    const int eo = m.edgesOnEdge[e * me2 + j];
    const size_t io = (size_t)eo * L + k;
    const double w = m.weightsOnEdge[e * me2 + j];
    s1 = fma(w, f.u[io], s1);
    s2 = fma(w, pvu[io], s2);
    const int jt = t.eoeTransSlot[e * me2 + j];
    if (jt < 0) continue;
    const double wt = m.weightsOnEdge[(size_t)eo * me2 + jt];
    s3 = fma(wt, qa[io], s3);
    s4 = fma(wt, qapv[io], s4);
  }
  const double q = 0.5 * (pv_self * s1 + s2);
  double gh = G * (q - (f.ke[i2] - f.ke[i1]) * inv_dc);
  pke[i] = G * rho_e * inv_dc;
  double gu = -G * 0.5 * (hd[i1] + hd[i2]) + 0.5 * (pv_self * s3 + s4);
  const double ray = adj_ray_damp(p.dm, k, L);  // tu - rho_edge u damp (every RK stage)
  if (ray != 0.0) {
    gu -= G * rho_e * ray;
    gh -= G * u_self * ray;
  }
  g.pv_edge[i] += 0.5 * (G * rho_e * s1 + u_self * s3);
  phd[i] = -G * u_self * 0.5;
  // vertical transport: interfaces k-1 .. k+2 of this edge
  for (int qq = k - 1; qq <= k + 2; ++qq) {
    if (qq < 1 || qq > L - 1) continue;
    const int lane = (int)threadIdx.x + (qq - k);
    const int slot = k - (qq - 2);
    if (lane >= 0 && lane < (int)blockDim.x)
      gu += s_c[slot][lane];
    else
      gu += wduz_part(m, f, ue, Gtu, c1, c2, qq, L).c[slot];
  }
  prwe[i] = (k >= 1 && k <= L - 1) ? own.pr : 0.0;
  if (p.rk_step == 1) {
    const double teub = G + g.tend_u_euler[i];
    const double zzm = 0.5 * (m.zz[i2] + m.zz[i1]);
    const double pg = -teub * f.cqu_e[i] * inv_dc;
    ppp[i] = zzm == 1.0 ? pg : pg / zzm;
    // terrain: + cqu 0.5 zxu (dpdz_1 + dpdz_2), the same partial for both cells
    if (pdz) pdz[i] = teub * f.cqu_e[i] * 0.5 * m.zxu[i];
    const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
    const double r_dv = fmin(m.invDvEdge[e], 4.0 * inv_dc);
    const double u_diff = (f.divergence[i2] - f.divergence[i1]) * inv_dc -
                          (f.vorticity[(size_t)v2 * L + k] - f.vorticity[(size_t)v1 * L + k]) * r_dv;
    const double kdiffu = 0.5 * (kd[i1] + kd[i2]);
    const double msd2 = m.meshScalingDel2[e];
    const double tm = teub * msd2;
    gh += tm * kdiffu * u_diff;
    pkd[i] = 0.5 * tm * rho_e * u_diff;
    udb[i] = tm * rho_e * kdiffu;
    if (p.del4) {
      const double u_mix = m.meshScalingDel4[e] * p.h_mom_visc4;
      const double r_dc4 = u_mix * p.del4u_div * inv_dc;
      const double r_dv4 = u_mix * r_dv;
      const double u_diff4 = (dsd[i2] - dsd[i1]) * r_dc4 - (dsv[(size_t)v2 * L + k] - dsv[(size_t)v1 * L + k]) * r_dv4;
      gh += -teub * u_diff4;
      pd4[i] = -teub * rho_e;
    }
  } else {
    g.tend_u_euler[i] += G;
  }
  (void)ud;
  g.h_edge[i] += gh;
  g.u[i] += gu;
}

// ---- cells: the u tendency's per-edge partials gathered (index space C x (L+1)):
// ke, the mass-flux divergence, pressure_p, kdiff, the del4 divergence, over terrain dpdz
// (-> rr_save, dpdz = -g (rho_base qtot + rr_save (1 + qtot))) (mass levels); rw through the
// edge-interface mean (w levels)
__global__ void k_tadj_u_cells(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1, AdjTendScalars p,
                               const double* __restrict__ pke, const double* __restrict__ phd,
                               const double* __restrict__ prwe, const double* __restrict__ ppp,
                               const double* __restrict__ pkd, const double* __restrict__ pd4,
                               const double* __restrict__ pdz, double* __restrict__ hdb, double* __restrict__ kdb,
                               double* __restrict__ dsdb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double gke = 0.0, ghd = 0.0, gpp = 0.0, gkd = 0.0, gds = 0.0, grw = 0.0, gdz = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const int side = cell_side(m, e, (int)c);
    if (k < L) {
      const size_t ie = (size_t)e * L + k;
      gke += side ? -pke[ie] : pke[ie];
      ghd += phd[ie];
      if (p.rk_step == 1) {
        gpp += side ? ppp[ie] : -ppp[ie];
        gkd += pkd[ie];
        if (pdz) gdz += pdz[ie];
        if (p.del4) {
          const double inv_dc = m.invDcEdge[e];
          const double r_dc4 = m.meshScalingDel4[e] * p.h_mom_visc4 * p.del4u_div * inv_dc;
          gds += side ? pd4[ie] * r_dc4 : -pd4[ie] * r_dc4;
        }
      }
    }
    if (k >= 1 && k <= L - 1) grw += 0.5 * prwe[(size_t)e * L + k];
  }
  g.rw[i] += grw;
  if (k == L) return;
  const size_t o = (size_t)c * L + k;
  g.ke[o] += gke;
  hdb[o] = ghd;
  if (p.rk_step == 1) {
    g.pressure_p[o] += gpp;
    kdb[o] = gkd;
    dsdb[o] = gds;
    if (pdz) g.rr_save[o] += gdz * (-kGravity) * (1.0 + f.qtot[o]);
  }
}

// ---- vertices (rk 1, del4): the del4 curl's cotangent
__global__ void k_tadj_dsv(mpasg_mesh m, FastDiv fl, AdjTendScalars p, const double* __restrict__ pd4,
                           double* __restrict__ dsvb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  const uint32_t v = fl.div(i);
  const int k = (int)(i - v * L);
  const int vd = m.vertexDegree;
  double a = 0.0;
  for (int j = 0; j < vd; ++j) {
    const int e = m.edgesOnVertex[v * vd + j];
    if (e >= m.nEdges) continue;
    const double inv_dc = m.invDcEdge[e];
    const double r_dv4 = m.meshScalingDel4[e] * p.h_mom_visc4 * fmin(m.invDvEdge[e], 4.0 * inv_dc);
    const double pp = pd4[(size_t)e * L + k] * r_dv4;
    a += vertex_side(m, e, (int)v) ? -pp : pp;
  }
  dsvb[i] = a;
}

// ---- edges (rk 1): total cotangent of u_diff (del2 + del4 through delsq_u)
__global__ void k_tadj_udiff_b(mpasg_mesh m, mpasg_transpose t, FastDiv fl, AdjTendScalars p,
                               const double* __restrict__ dsdb, const double* __restrict__ dsvb,
                               double* __restrict__ udb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  if (!p.del4) return;
  const int me = m.maxEdges, vd = m.vertexDegree;
  double a = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int jv = t.edgeVertexSlot[2 * e + s];
    if (jv >= 0) {
      const int v = m.verticesOnEdge[2 * e + s];
      a += dsvb[(size_t)v * L + k] * (m.invAreaTriangle[v] * m.dcEdge[e] * m.edgesOnVertex_sign[v * vd + jv]);
    }
    const int jc = t.edgeCellSlot[2 * e + s];
    if (jc >= 0) {
      const int c = m.cellsOnEdge[2 * e + s];
      a += dsdb[(size_t)c * L + k] * (m.invAreaCell[c] * m.dvEdge[e] * m.edgesOnCell_sign[c * me + jc]);
    }
  }
  udb[i] += a;
}

// ---- cells / vertices (rk 1): u_diff's cotangent -> divergence, vorticity
__global__ void k_tadj_div(mpasg_mesh m, mpasg_fields g, FastDiv fl, const double* __restrict__ udb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double a = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const double b = udb[(size_t)e * L + k] * m.invDcEdge[e];
    a += cell_side(m, e, (int)c) ? b : -b;
  }
  g.divergence[i] += a;
}

__global__ void k_tadj_vort(mpasg_mesh m, mpasg_fields g, FastDiv fl, const double* __restrict__ udb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  const uint32_t v = fl.div(i);
  const int k = (int)(i - v * L);
  const int vd = m.vertexDegree;
  double a = 0.0;
  for (int j = 0; j < vd; ++j) {
    const int e = m.edgesOnVertex[v * vd + j];
    if (e >= m.nEdges) continue;
    const double r_dv = fmin(m.invDvEdge[e], 4.0 * m.invDcEdge[e]);
    const double b = udb[(size_t)e * L + k] * r_dv;
    a += vertex_side(m, e, (int)v) ? -b : b;
  }
  g.vorticity[i] += a;
}

// ---- rk 1 mixing: edges, the del4 parts' cotangents of delsq_theta / delsq_w per edge
__global__ void k_tadj_mix_a(mpasg_mesh m, mpasg_transpose t, FastDiv fl, AdjTendScalars p,
                             const double* __restrict__ tteb, const double* __restrict__ tweb, double* __restrict__ a4t,
                             double* __restrict__ a4w) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int me = m.maxEdges;
  double at = 0.0, aw = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int j = t.edgeCellSlot[2 * e + s];
    if (j < 0) continue;
    const int c = m.cellsOnEdge[2 * e + s];
    const double ia = m.invAreaCell[c];
    const double base = m.meshScalingDel4[e];
    const double sg = m.edgesOnCell_sign[c * me + j];
    // es = msd4 * (visc4 * ia) * dv * sign * invDc, as k_mix_cells_b forms it
    const double es_t = base * (p.h_theta_visc4 * 1.0 * ia) * m.dvEdge[e] * sg * m.invDcEdge[e];
    const double es_w = base * (p.h_mom_visc4 * ia) * m.dvEdge[e] * sg * m.invDcEdge[e];
    at += tteb[(size_t)c * L + k] * es_t;
    if (k >= 1) aw += tweb[(size_t)c * (L + 1) + k] * es_w;
  }
  a4t[i] = p.h_theta_visc4 > 0.0 ? at : 0.0;
  a4w[i] = p.h_mom_visc4 > 0.0 ? aw : 0.0;
}

// ---- rk 1 mixing: cells, delsq_theta / delsq_w cotangents (index space C x (L+1))
__global__ void k_tadj_mix_b(mpasg_mesh m, FastDiv fl1, const double* __restrict__ a4t,
                             const double* __restrict__ a4w, double* __restrict__ dstb, double* __restrict__ dswb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double st = 0.0, sw = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const int side = cell_side(m, e, (int)c);
    if (k < L) st += side ? -a4t[(size_t)e * L + k] : a4t[(size_t)e * L + k];
    if (k >= 1 && k <= L - 1) sw += side ? -a4w[(size_t)e * L + k] : a4w[(size_t)e * L + k];
  }
  if (k < L) dstb[(size_t)c * L + k] = st;
  dswb[i] = sw;
}

// ---- rk 1 mixing: edges, the del2 fluxes read backwards: per-edge partials for the cell
// gathers (theta, w, kdiff) and the cotangent of h_edge (rho_edge) from theta's flux; w's
// flux reads rho_edge at two levels, its partial per w level goes to gre
__global__ void k_tadj_mix_c(mpasg_mesh m, mpasg_fields f, mpasg_fields g, mpasg_transpose t, FastDiv fl,
                             const double* __restrict__ kd, const double* __restrict__ tteb,
                             const double* __restrict__ tweb, const double* __restrict__ dstb,
                             const double* __restrict__ dswb, double* __restrict__ bt, double* __restrict__ kdt,
                             double* __restrict__ bw, double* __restrict__ kdw, double* __restrict__ gre) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int me = m.maxEdges;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  const double msd2 = m.meshScalingDel2[e];
  const double rho_e = f.h_edge[i];
  // theta: flux_c = es_t(c) (theta_2 - theta_1) rho_e; tte_c += flux_c 0.5 (kd_1 + kd_2) msd2
  const double dth = f.theta_m[i2] - f.theta_m[i1];
  const double kdm = 0.5 * (kd[i1] + kd[i2]);
  double b = 0.0, kt = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int j = t.edgeCellSlot[2 * e + s];
    if (j < 0) continue;
    const int c = m.cellsOnEdge[2 * e + s];
    const double es = m.cell_edge_es_t[c * me + j];
    const size_t oc = (size_t)c * L + k;
    const double flux = es * dth * rho_e;
    b += (tteb[oc] * kdm * msd2 + dstb[oc]) * es;
    kt += tteb[oc] * flux * 0.5 * msd2;
  }
  g.h_edge[i] += b * dth;
  bt[i] = b * rho_e;
  kdt[i] = kt;
  // w (level k >= 1): flux_c = es_w(c) (rho_e_k + rho_e_(k-1)) (w_2 - w_1)
  double bwk = 0.0, kw = 0.0, gr = 0.0;
  if (k >= 1) {
    const size_t w1 = (size_t)c1 * (L + 1) + k, w2 = (size_t)c2 * (L + 1) + k;
    const double dw = f.w[w2] - f.w[w1];
    const double rsum = rho_e + f.h_edge[i - 1];
    const double kd4 = 0.25 * (kd[i1] + kd[i2] + kd[i1 - 1] + kd[i2 - 1]);
    double bb = 0.0;
    for (int s = 0; s < 2; ++s) {
      const int j = t.edgeCellSlot[2 * e + s];
      if (j < 0) continue;
      const int c = m.cellsOnEdge[2 * e + s];
      const double es = m.cell_edge_es_w[c * me + j];
      const size_t ow = (size_t)c * (L + 1) + k;
      const double flux = es * rsum * dw;
      bb += (tweb[ow] * msd2 * kd4 + dswb[ow]) * es;
      kw += tweb[ow] * flux * msd2 * 0.25;
    }
    gr = bb * dw;
    bwk = bb * rsum;
  }
  bw[i] = bwk;
  kdw[i] = kw;
  gre[i] = gr;
}

// ---- rk 1 mixing: cells, theta / w / kdiff gathers (index space C x (L+1))
__global__ void k_tadj_mix_d(mpasg_mesh m, mpasg_fields g, FastDiv fl1, const double* __restrict__ bt,
                             const double* __restrict__ kdt, const double* __restrict__ bw,
                             const double* __restrict__ kdw, double* __restrict__ kdb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double gth = 0.0, gw = 0.0, gk = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const int side = cell_side(m, e, (int)c);
    const size_t ie = (size_t)e * L;
    if (k < L) {
      gth += side ? bt[ie + k] : -bt[ie + k];
      gk += kdt[ie + k];
      if (k >= 1) gk += kdw[ie + k];
      if (k + 1 <= L - 1) gk += kdw[ie + k + 1];
    }
    if (k >= 1 && k <= L - 1) gw += side ? bw[ie + k] : -bw[ie + k];
  }
  if (k < L) {
    const size_t o = (size_t)c * L + k;
    g.theta_m[o] += gth;
    kdb[o] += gk;
  }
  g.w[i] += gw;
}

// ---- rk 1 mixing: edges, rho_edge's cotangent from w's flux at its two w levels
__global__ void k_tadj_mix_e(mpasg_mesh m, mpasg_fields g, FastDiv fl, const double* __restrict__ gre) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  double a = 0.0;
  if (k >= 1) a += gre[i];
  if (k + 1 <= L - 1) a += gre[i + 1];
  g.h_edge[i] += a;
}

// ---- rk 1 Smagorinsky: kdiff = min(cs2 sqrt(dd^2 + do^2), cap) read backwards (min and
// sqrt with the derivative of the branch taken; ties split as torch's minimum does)
__global__ void k_tadj_kdiff(mpasg_mesh m, FastDiv fl, AdjTendScalars p, const double* __restrict__ kdb,
                             double* __restrict__ ddb_io, double* __restrict__ dob_io) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const double dd = ddb_io[i], dof = dob_io[i];
  const double sq = sqrt(__dadd_rn(__dmul_rn(dd, dd), __dmul_rn(dof, dof)));
  const double A = __dmul_rn(p.cs2, sq);
  double gk = kdb[i];
  const int k = (int)(i - fl.div(i) * (uint32_t)L);
  if (p.dm.ncam > 0 && k >= L - p.dm.ncam)  // max(kdiff, CAM floor): the branch taken
    gk *= adj_max_factor(fmin(A, p.kdiff_cap), adj_cam_floor(p.dm, k, L));
  const double gA = A < p.kdiff_cap ? gk : (A == p.kdiff_cap ? 0.5 * gk : 0.0);
  const double gs = sq > 0.0 ? gA * p.cs2 * 0.5 / sq : 0.0;
  ddb_io[i] = gs * 2.0 * dd;
  dob_io[i] = gs * 2.0 * dof;
}

__global__ void k_tadj_deform(mpasg_mesh m, mpasg_fields g, mpasg_transpose t, FastDiv fl,
                              const double* __restrict__ ddb, const double* __restrict__ dob) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int me = m.maxEdges;
  double gu = 0.0, gv = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int j = t.edgeCellSlot[2 * e + s];
    if (j < 0) continue;
    const int c = m.cellsOnEdge[2 * e + s];
    const double ca = m.defc_a[c * me + j], cb = m.defc_b[c * me + j];
    const double a = ddb[(size_t)c * L + k], b = dob[(size_t)c * L + k];
    gu += a * ca + b * cb;
    gv += -a * cb + b * ca;
  }
  g.u[i] += gu;
  g.v[i] += gv;
}

// ---- rk 1 density tendency: tend_rho = -h_div - rdzw (rw_(k+1) - rw_k), per w level
__global__ void k_tadj_rho(mpasg_mesh m, mpasg_fields g, FastDiv fl1, AdjTendScalars p, double* __restrict__ hdb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t oc = (size_t)c * L;
  if (p.rk_step != 1) return;
  double a = 0.0;
  if (k < L) {
    const double G = g.tend_rho[oc + k];
    a += G * m.rdzw[k];
    hdb[oc + k] += -G;
  }
  if (k >= 1) a -= g.tend_rho[oc + k - 1] * m.rdzw[k - 1];
  g.rw[i] += a;
}

// ---- edges: the mass-flux divergence transposed -> ru
__global__ void k_tadj_hdiv(mpasg_mesh m, mpasg_fields g, mpasg_transpose t, FastDiv fl, const double* __restrict__ hdb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int me = m.maxEdges;
  double a = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int j = t.edgeCellSlot[2 * e + s];
    if (j < 0) continue;
    const int c = m.cellsOnEdge[2 * e + s];
    a += hdb[(size_t)c * L + k] * m.invAreaCell[c] * m.cell_edge_sdv[c * me + j];
  }
  g.ru[i] += a;
}

// ---- rk 1: vertical mixing of u (k_tend_u_finish) read backwards.  At level q (1 <= q <=
// L-2) of an edge: teu += h v (d_up - d_dn) / den, d_up = (u_(q+1) - u_q) / (zp - z0),
// d_dn = (u_q - u_(q-1)) / (z0 - zm), heights the edge means of the two cells' interfaces;
// level k gathers the terms of levels k-1, k, k+1.  The perturbation form's initial profiles
// are constants: they enter only the value d_up - d_dn that rho_edge's cotangent reads.
__global__ void k_tadj_vmix_u(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, AdjTendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const double* z1p = m.zgrid + (size_t)c1 * (L + 1);
  const double* z2p = m.zgrid + (size_t)c2 * (L + 1);
  const size_t oe = (size_t)e * L;
  const double v = p.dm.v_mom;
  double gu = 0.0, gh = 0.0;
  for (int q = k - 1; q <= k + 1; ++q) {
    if (q < 1 || q > L - 2) continue;
    const double za = 0.5 * (z1p[q - 1] + z2p[q - 1]), zb = 0.5 * (z1p[q] + z2p[q]);
    const double zc = 0.5 * (z1p[q + 1] + z2p[q + 1]), zd = 0.5 * (z1p[q + 2] + z2p[q + 2]);
    const double zm = 0.5 * (za + zb), z0 = 0.5 * (zb + zc), zp = 0.5 * (zc + zd);
    const double den = 0.5 * (zp - zm);
    const double G = g.tend_u[oe + q] + g.tend_u_euler[oe + q];  // cotangent of the final teu
    const double a = G * (f.h_edge[oe + q] * v) / den;
    if (q == k) {
      gu -= a / (zp - z0) + a / (z0 - zm);
      double um = f.u[oe + q - 1], u0 = f.u[oe + q], up = f.u[oe + q + 1];
      if (p.mix_pert) {
        const double ca = cos(m.angleEdge[e]), sa = sin(m.angleEdge[e]);
        um = um - m.u_init[q - 1] * ca - m.v_init[q - 1] * sa;
        u0 = u0 - m.u_init[q] * ca - m.v_init[q] * sa;
        up = up - m.u_init[q + 1] * ca - m.v_init[q + 1] * sa;
      }
      gh += G * v * ((up - u0) / (zp - z0) - (u0 - um) / (z0 - zm)) / den;
    } else if (q == k - 1) {
      gu += a / (zp - z0);
    } else {
      gu += a / (z0 - zm);
    }
  }
  g.u[i] += gu;
  g.h_edge[i] += gh;
}

// ---- rk 1: vertical mixing of w and theta (k_tend_w_theta) read backwards (index space
// C x (L+1)).  w at interface q (1 <= q <= L-1): v rho_half (w_up - w_down) rdzu_q with
// rho_half the mean of rho_zz at q-1, q, w_up = (w_(q+1) - w_q) rdzw_q, w_down = (w_q -
// w_(q-1)) rdzw_(q-1), cotangent tweb_q; theta at level q (1 <= q <= L-2): v rho_zz_q diff /
// den, diff = (t_(q+1) - t_q) / (zp - z0) - (t_q - t_(q-1)) / (z0 - zm) from the cell's own
// heights, cotangent tteb_q.  Interface / level j gathers the terms that read it.
__global__ void k_tadj_vmix_cells(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1, AdjTendScalars p,
                                  const double* __restrict__ tweb, const double* __restrict__ tteb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int j = (int)(i - c * (L + 1));
  const size_t oc = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double* rz = f.rho_zz + oc;
  if (p.dm.v_mom > 0.0) {
    const double v = p.dm.v_mom;
    const double* w = f.w + ow;
    double gw = 0.0, gr = 0.0;
    for (int q = j - 1; q <= j + 1; ++q) {
      if (q < 1 || q > L - 1) continue;
      const double b = tweb[ow + q] * v * m.rdzu[q];
      const double rho_half = 0.5 * (rz[q] + rz[q - 1]);
      if (q == j + 1) gw += b * rho_half * m.rdzw[q - 1];                    // w_(q-1) in w_down
      if (q == j) gw -= b * rho_half * (m.rdzw[q] + m.rdzw[q - 1]);          // w_q in both
      if (q == j - 1) gw += b * rho_half * m.rdzw[q];                        // w_(q+1) in w_up
      if (j < L && (q == j || q == j + 1)) {                                   // rho_zz_j in rho_half
        const double wu = (w[q + 1] - w[q]) * m.rdzw[q], wd = (w[q] - w[q - 1]) * m.rdzw[q - 1];
        gr += 0.5 * b * (wu - wd);
      }
    }
    g.w[ow + j] += gw;
    if (j < L) g.rho_zz[oc + j] += gr;
  }
  if (p.dm.v_theta > 0.0 && j < L) {
    const double v = p.dm.v_theta;
    const double* zg = m.zgrid + (size_t)c * (L + 1);
    const double* th = f.theta_m + oc;
    const double* ti = p.mix_pert ? m.t_init + oc : nullptr;
    double gt = 0.0, gr = 0.0;
    for (int q = j - 1; q <= j + 1; ++q) {
      if (q < 1 || q > L - 2) continue;
      const double zm = 0.5 * (zg[q - 1] + zg[q]), z0 = 0.5 * (zg[q] + zg[q + 1]), zp = 0.5 * (zg[q + 1] + zg[q + 2]);
      const double den = 0.5 * (zp - zm);
      const double a = tteb[oc + q] * (v * 1.0 * rz[q]) / den;
      if (q == j) {
        gt -= a / (zp - z0) + a / (z0 - zm);
        double tm = th[q - 1], t0 = th[q], tp = th[q + 1];
        if (p.mix_pert) {
          tm = tm - ti[q - 1];
          t0 = t0 - ti[q];
          tp = tp - ti[q + 1];
        }
        gr += tteb[oc + q] * v * 1.0 * ((tp - t0) / (zp - z0) - (t0 - tm) / (z0 - zm)) / den;
      } else if (q == j - 1) {
        gt += a / (zp - z0);
      } else {
        gt += a / (z0 - zm);
      }
    }
    g.theta_m[oc + j] += gt;
    g.rho_zz[oc + j] += gr;
  }
}

#define CHECK_RC(x)                  \
  do {                               \
    int _rc = (x);                   \
    if (_rc != MPASG_OK) return _rc; \
  } while (0)

}  // namespace

int mpasgi_dyn_tend_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                             const mpasg_transpose* t, int rk_step, const AdjWork& w, cudaStream_t s) {
  const int L = m->nVertLevels;
  const long long ncl = (long long)m->nCells * L, nel = (long long)m->nEdges * L;
  const long long ncw = (long long)m->nCells * (L + 1), nvl = (long long)m->nVertices * L;
  AdjTendScalars p{};
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
  p.visc2 = p.smag ? 0.0 : c->h_theta_eddy_visc2;
  p.del4u_div = c->del4u_div_factor;
  p.coef3 = c->coef_3rd_order;
  p.rk_step = rk_step;
  p.del4 = p.h_mom_visc4 > 0.0 ? 1 : 0;
  p.mix_pert = c->mix_perturbation ? 1 : 0;
  p.dm = adj_damping(c);
  FastDiv fl(L), fl1(L + 1);
  // work: cells
  double* hd = w.c[0];
  double* kd = w.c[1];
  double* ddb = w.c[2];
  double* dob = w.c[3];
  double* tt1b = w.c[4];
  double* tw1b = w.c[5];
  double* tweb = w.c[6];
  double* tteb = w.c[7];
  double* dsd = w.c[8];
  double* hdb = w.c[9];
  double* kdb = w.c[10];
  double* dsdb = w.c[11];
  double* dstb = w.c[12];
  double* dswb = w.c[13];
  // edges
  double* fltb = w.e[0];
  double* flwb = w.e[1];
  double* pke = w.e[3];
  double* phd = w.e[4];
  double* prwe = w.e[5];
  double* ppp = w.e[6];
  double* pkd = w.e[7];
  double* udb = w.e[8];
  double* ud = w.e[9];
  double* pd4 = w.e[10];
  double* a4t = w.e[11];
  double* a4w = w.e[12];
  double* bt = w.e[13];
  double* kdt = w.e[14];
  double* bw = w.e[15];
  double* kdw = w.e[16];
  double* gre = w.e[17];
  double* pdz = m->flatTerrain ? nullptr : w.e[18];  // terrain: dpdz partials of the u tendency
  // vertices
  double* dsv = w.v[0];
  double* dsvb = w.v[1];

  k_tadj_values<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, p, hd, kd, ddb, dob);
  MPASG_LAUNCH_CHECK();
  if (rk_step == 1 && p.del4) {
    k_tadj_udiff<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, ud);
    MPASG_LAUNCH_CHECK();
    k_tadj_del4_cells<<<nblocks(ncl), kBlock, 0, s>>>(*m, fl, ud, dsd);
    MPASG_LAUNCH_CHECK();
    k_tadj_del4_vertices<<<nblocks(nvl), kBlock, 0, s>>>(*m, fl, ud, dsv);
    MPASG_LAUNCH_CHECK();
  }
  k_tadj_columns<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *g, fl1, p, tt1b, tw1b, tweb, tteb);
  MPASG_LAUNCH_CHECK();
  if (rk_step == 1) {
    k_tadj_wres<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, *g, fl, tweb);
    MPASG_LAUNCH_CHECK();
    if (p.dm.v_mom > 0.0 || p.dm.v_theta > 0.0) {
      k_tadj_vmix_cells<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *g, fl1, p, tweb, tteb);
      MPASG_LAUNCH_CHECK();
    }
  }
  uint8_t* sel = reinterpret_cast<uint8_t*>(w.e[2]);  // (E+1) x L bytes within one edge array
  k_tadj_adv_edges<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *g, *t, fl, p, tt1b, tw1b, fltb, flwb, sel);
  MPASG_LAUNCH_CHECK();
  k_tadj_adv_cells<<<nblocks(ncw), kBlock, 0, s>>>(*m, *g, *t, fl1, FastDiv(m->nAdvMax), fltb, flwb, sel);
  MPASG_LAUNCH_CHECK();
  double* qa = w.e[2];  // sel's bytes (read by the advection gather above) are no longer needed
  double* qapv = w.e[19];
  double* pvu = w.e[20];
  k_tadj_qa<<<nblocks(nel), kBlock, 0, s>>>((int)nel, g->tend_u, f->h_edge, f->pv_edge, f->u, qa, qapv, pvu);
  MPASG_LAUNCH_CHECK();
  k_tadj_u<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *g, *t, fl, p, hd, kd, ud, dsd, dsv, pke, phd, prwe, ppp, pkd,
                                          udb, pd4, qa, pdz, qapv, pvu);
  MPASG_LAUNCH_CHECK();
  k_tadj_u_cells<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *g, fl1, p, pke, phd, prwe, ppp, pkd, pd4, pdz, hdb, kdb,
                                                 dsdb);
  MPASG_LAUNCH_CHECK();
  if (rk_step == 1 && p.dm.v_mom > 0.0) {
    k_tadj_vmix_u<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *g, fl, p);
    MPASG_LAUNCH_CHECK();
  }
  if (rk_step == 1) {
    if (p.del4) {
      k_tadj_dsv<<<nblocks(nvl), kBlock, 0, s>>>(*m, fl, p, pd4, dsvb);
      MPASG_LAUNCH_CHECK();
      k_tadj_udiff_b<<<nblocks(nel), kBlock, 0, s>>>(*m, *t, fl, p, dsdb, dsvb, udb);
      MPASG_LAUNCH_CHECK();
    }
    k_tadj_div<<<nblocks(ncl), kBlock, 0, s>>>(*m, *g, fl, udb);
    MPASG_LAUNCH_CHECK();
    k_tadj_vort<<<nblocks(nvl), kBlock, 0, s>>>(*m, *g, fl, udb);
    MPASG_LAUNCH_CHECK();
    // horizontal mixing of theta and w (del2 with kdiff, del4)
    k_tadj_mix_a<<<nblocks(nel), kBlock, 0, s>>>(*m, *t, fl, p, tteb, tweb, a4t, a4w);
    MPASG_LAUNCH_CHECK();
    k_tadj_mix_b<<<nblocks(ncw), kBlock, 0, s>>>(*m, fl1, a4t, a4w, dstb, dswb);
    MPASG_LAUNCH_CHECK();
    k_tadj_mix_c<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *g, *t, fl, kd, tteb, tweb, dstb, dswb, bt, kdt, bw, kdw, gre);
    MPASG_LAUNCH_CHECK();
    k_tadj_mix_d<<<nblocks(ncw), kBlock, 0, s>>>(*m, *g, fl1, bt, kdt, bw, kdw, kdb);
    MPASG_LAUNCH_CHECK();
    k_tadj_mix_e<<<nblocks(nel), kBlock, 0, s>>>(*m, *g, fl, gre);
    MPASG_LAUNCH_CHECK();
    if (p.smag) {
      k_tadj_kdiff<<<nblocks(ncl), kBlock, 0, s>>>(*m, fl, p, kdb, ddb, dob);
      MPASG_LAUNCH_CHECK();
      k_tadj_deform<<<nblocks(nel), kBlock, 0, s>>>(*m, *g, *t, fl, ddb, dob);
      MPASG_LAUNCH_CHECK();
    }
  }
  k_tadj_rho<<<nblocks(ncw), kBlock, 0, s>>>(*m, *g, fl1, p, hdb);
  MPASG_LAUNCH_CHECK();
  k_tadj_hdiv<<<nblocks(nel), kBlock, 0, s>>>(*m, *g, *t, fl, hdb);
  MPASG_LAUNCH_CHECK();
  // the stage's outputs are consumed; at rk 1 so are the Euler tendencies and tend_rho it
  // creates (later stages passed their cotangents through)
  const ZeroSpan zs[] = {{g->tend_u, (m->nEdges + 1LL) * L}, {g->tend_w, (m->nCells + 1LL) * (L + 1)},
                         {g->tend_theta, (m->nCells + 1LL) * L}, {g->tend_u_euler, (m->nEdges + 1LL) * L},
                         {g->tend_w_euler, (m->nCells + 1LL) * (L + 1)}, {g->tend_theta_euler, (m->nCells + 1LL) * L},
                         {g->tend_rho, (m->nCells + 1LL) * L}};
  CHECK_RC(mpasgi_zero_many(zs, rk_step == 1 ? 7 : 3, s));
  return MPASG_OK;
}

extern "C" int mpasg_dyn_tend_vjp(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                                  const mpasg_transpose* t, int rk_step, double* work, void* stream) {
  if (!m || !c || !f || !g || !t || !work || rk_step < 1 || rk_step > 3 || !adj_supported(m, c)) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (rk_step > 1) {  // the edge mean of theta_m_save the rk 2 / 3 flux reads
    mpasg_fields fm = *f;
    CHECK_RC(mpasgi_theta_edge(m, &fm, false, s));
  }
  return mpasgi_dyn_tend_vjp_core(m, c, f, g, t, rk_step, adj_work(m, work), s);
}
