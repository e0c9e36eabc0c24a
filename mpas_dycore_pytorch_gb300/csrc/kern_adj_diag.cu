// Reverse mode of the diagnostics (mpas_pytorch/dynamics/solve_diagnostics.py:1052) and of
// the cold-start preparation (dynamics/init_coupled_diagnostics.py:147 followed by the
// first diagnostics), as deterministic gathers over the transposed connectivity.
#include "adj_common.cuh"

namespace {

// pv at a vertex as the diagnostics form it: fVertex + vorticity
MPASG_D double pv_vertex(const mpasg_mesh& m, const mpasg_fields& f, int v, int k) {
  return m.fVertex[v] + f.vorticity[(size_t)v * m.nVertLevels + k];
}

// cell PV of the APVM upwinding: sum_j kite_j pv_vertex_j / area
__global__ void k_dadj_pvc(mpasg_mesh m, mpasg_fields f, FastDiv fl, double* __restrict__ pvc) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const int me = m.maxEdges, vd = m.vertexDegree;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    const int v = m.verticesOnCell[c * me + j];
    const int kk = m.kiteForCell[c * me + j];
    if (v >= m.nVertices || kk < 0) continue;
    double pt = m.kiteAreasOnVertex[v * vd + kk] * pv_vertex(m, f, v, k);
    pt = pt * ia;
    acc = (j == 0) ? pt : acc + pt;
  }
  pvc[i] = acc;
}

// pv_edge (with APVM) read backwards, per edge level: -> u (APVM normal term), v, and the
// per-edge partials for the vertex (pv1 / pv2) and cell (pc) gathers; at rk 3 the
// cotangent of the recomputed tangential wind goes to vb (v is consumed)
__global__ void k_dadj_edges_b(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, int rk_step, int apvm,
                               double apvm_dt, const double* __restrict__ pvc, double* __restrict__ pv1,
                               double* __restrict__ pv2, double* __restrict__ pc, double* __restrict__ vb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const double G = g.pv_edge[i];
  double at = 0.0, an = 0.0, vbar = g.v[i];
  if (apvm) {
    const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
    const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
    const double gd = -G * apvm_dt;
    const double gpt = (pv_vertex(m, f, v2, k) - pv_vertex(m, f, v1, k)) * m.invDvEdge[e];
    const double gpn = (pvc[(size_t)c2 * L + k] - pvc[(size_t)c1 * L + k]) * m.invDcEdge[e];
    vbar += gd * gpt;
    g.u[i] += gd * gpn;
    at = gd * f.v[i] * m.invDvEdge[e];
    an = gd * f.u[i] * m.invDcEdge[e];
  }
  pv1[i] = 0.5 * G - at;
  pv2[i] = 0.5 * G + at;
  pc[i] = an;
  if (rk_step == 3) {
    vb[i] = vbar;
    g.v[i] = 0.0;
  } else {
    g.v[i] = vbar;
  }
}

// APVM cell PV cotangent (cells)
__global__ void k_dadj_pvc_b(mpasg_mesh m, FastDiv fl, const double* __restrict__ pc, double* __restrict__ pvcb) {
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
    const double p = pc[(size_t)e * L + k];
    a += cell_side(m, e, (int)c) ? p : -p;
  }
  pvcb[i] = a;
}

// vertices: vorticity's total cotangent (through pv_vertex) and the vertex kinetic energy's
__global__ void k_dadj_vertices(mpasg_mesh m, mpasg_fields g, mpasg_transpose t, FastDiv fl, int apvm,
                                const double* __restrict__ pv1, const double* __restrict__ pv2,
                                const double* __restrict__ pvcb, double* __restrict__ vortb, double* __restrict__ kevb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  const uint32_t v = fl.div(i);
  const int k = (int)(i - v * L);
  const int vd = m.vertexDegree;
  double pvb = 0.0, keb = 0.0;
  for (int j = 0; j < vd; ++j) {
    const int e = m.edgesOnVertex[v * vd + j];
    if (e >= m.nEdges) continue;
    const size_t ie = (size_t)e * L + k;
    pvb += vertex_side(m, e, (int)v) ? pv2[ie] : pv1[ie];
  }
  const double kf = 1.0 - 0.375;
  for (int s = 0; s < vd; ++s) {
    const int c = t.cellsOnVertex[v * vd + s];
    const int kk = t.vertexKite[v * vd + s];
    if (c >= m.nCells || kk < 0) continue;
    const double kite = m.kiteAreasOnVertex[v * vd + kk];
    const double ia = m.invAreaCell[c];
    if (apvm) pvb += kite * ia * pvcb[(size_t)c * L + k];
    keb += (1.0 - kf) * kite * ia * g.ke[(size_t)c * L + k];
  }
  vortb[i] = g.vorticity[i] + pvb;
  kevb[i] = keb;
}

// edges: u's cotangent from the circulation, divergence, kinetic energies and (rk 3) the
// TRiSK tangential wind
__global__ void k_dadj_edges_a(mpasg_mesh m, mpasg_fields f, mpasg_fields g, mpasg_transpose t, FastDiv fl,
                               int rk_step, const double* __restrict__ vortb, const double* __restrict__ kevb,
                               const double* __restrict__ vb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int me = m.maxEdges, vd = m.vertexDegree;
  const double kf = 1.0 - 0.375;
  double gu = 0.0, gke = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int jv = t.edgeVertexSlot[2 * e + s];
    if (jv >= 0) {
      const int v = m.verticesOnEdge[2 * e + s];
      const double iat = m.invAreaTriangle[v];
      gu += vortb[(size_t)v * L + k] * iat * m.vertex_edge_sdc[v * vd + jv];
      gke += kevb[(size_t)v * L + k] * 0.25 * iat;
    }
    const int jc = t.edgeCellSlot[2 * e + s];
    if (jc >= 0) {
      const int c = m.cellsOnEdge[2 * e + s];
      const double ia = m.invAreaCell[c];
      const size_t oc = (size_t)c * L + k;
      gu += g.divergence[oc] * ia * m.cell_edge_sdv[c * me + jc];
      gke += g.ke[oc] * kf * 0.25 * ia;
    }
  }
  if (rk_step == 3) {
    const int n2 = m.nEdgesOnEdge[e], me2 = m.maxEdges2;
    for (int j = 0; j < n2; ++j) {
      const int eo = m.edgesOnEdge[e * me2 + j];
      const int jt = t.eoeTransSlot[e * me2 + j];
      if (jt < 0) continue;
      gu += m.weightsOnEdge[(size_t)eo * me2 + jt] * vb[(size_t)eo * L + k];
    }
  }
  gu += gke * m.edge_dcdv[e] * 2.0 * f.u[i];
  g.u[i] += gu;
}

// cells: rho_zz's cotangent from h_edge = 0.5 (rho_1 + rho_2)
__global__ void k_dadj_hedge(mpasg_mesh m, mpasg_fields g, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double a = 0.0;
  for (int j = 0; j < n; ++j) a += 0.5 * g.h_edge[(size_t)m.edgesOnCell[c * me + j] * L + k];
  g.rho_zz[i] += a;
}

// ---------------------------------------------------------------- preparation
// Over terrain, rw at interior interface k of cell c also has the slope terms
// - sum_j s_j coef_j flux_j zz_i, flux_j = fzm ru[e_j][k] + fzp ru[e_j][k-1], coef_j = zb +
// sgn(flux_j) zb3 (a constant selection; init_coupled_diagnostics.py:147): ru's cotangent
// from the interfaces k (fzm) and k+1 (fzp) of both cells
MPASG_D double prepare_slope_cotangent(const mpasg_mesh& m, const mpasg_fields& f, const mpasg_fields& g, uint32_t e,
                                       int k) {
  const int L = m.nVertLevels, me = m.maxEdges;
  const double* ru = f.ru + (size_t)e * L;
  double acc = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int c = m.cellsOnEdge[2 * e + s];
    if (c < 0 || c >= m.nCells) continue;
    const int j = cell_slot(m, c, (int)e);
    if (j < 0) continue;
    const double sign = m.edgesOnCell_sign[c * me + j];
    const size_t oc = (size_t)c * L, ow = (size_t)c * (L + 1);
    for (int kw = k; kw <= k + 1; ++kw) {
      if (kw < 1 || kw > L - 1) continue;
      const double fzm = m.fzm[kw], fzp = m.fzp[kw];
      const double flux = fzm * ru[kw] + fzp * ru[kw - 1];
      const size_t zi = ((size_t)c * me + j) * (L + 1) + kw;
      const double coef = m.zb_cell[zi] + sgn(flux) * m.zb3_cell[zi];
      const double zz_i = fzp * m.zz[oc + kw - 1] + fzm * m.zz[oc + kw];
      acc -= g.rw[ow + kw] * sign * coef * zz_i * (kw == k ? fzm : fzp);
    }
  }
  return acc;
}

// edges: ru = 0.5 u (rho_1 + rho_2) -> u; the rho partial for the cell gather
__global__ void k_padj_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, double* __restrict__ g_u,
                             double* __restrict__ pru) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)(m.nEdges + 1) * L) return;
  if (i >= (uint32_t)m.nEdges * L) {
    g_u[i] = 0.0;
    return;
  }
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  double gru = g.ru[i];
  if (!m.flatTerrain) gru += prepare_slope_cotangent(m, f, g, e, k);
  g_u[i] = g.u[i] + gru * 0.5 * (f.rho_zz[(size_t)c1 * L + k] + f.rho_zz[(size_t)c2 * L + k]);
  pru[i] = gru * 0.5 * f.u[i];
}

// w levels: rw = w rho_i zz_i (+ the slope terms, k_padj_edges) -> w; rho_i's cotangent
__global__ void k_padj_wlev(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1, const double* __restrict__ w_in,
                            double* __restrict__ g_w, double* __restrict__ rho_ib) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)(m.nCells + 1) * (L + 1)) return;
  if (i >= (uint32_t)m.nCells * (L + 1)) {
    g_w[i] = 0.0;
    return;
  }
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  double gw = g.w[i], rib = 0.0;
  if (k >= 1 && k <= L - 1) {
    const size_t o = (size_t)c * L + k;
    const double rho_i = m.fzp[k] * f.rho_zz[o - 1] + m.fzm[k] * f.rho_zz[o];
    const double zz_i = m.fzp[k] * m.zz[o - 1] + m.fzm[k] * m.zz[o];
    const double grw = g.rw[i];
    gw += grw * rho_i * zz_i;
    rib = grw * w_in[i] * zz_i;
  }
  g_w[i] = gw;
  rho_ib[i] = rib;
}

// cells: the coupled diagnostics (theta_m, rho_zz, rho_p, rtheta_p, exner, pressure_p)
// read backwards -> theta, rho (dry: theta_m = theta)
__global__ void k_padj_cells(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, const double* __restrict__ pru,
                             const double* __restrict__ rho_ib, double* __restrict__ g_theta,
                             double* __restrict__ g_rho) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)(m.nCells + 1) * L) return;
  if (i >= (uint32_t)m.nCells * L) {
    g_theta[i] = 0.0;
    g_rho[i] = 0.0;
    return;
  }
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const double rcv = kRgas / (kCp - kRgas);
  const double zz = m.zz[i], rb = m.rho_base[i];
  const double thm = f.theta_m[i], rho_p = f.rho_p[i], rtp = f.rtheta_p[i], rtb = f.rtheta_base[i];
  const double ex = f.exner[i];
  const double gpp = g.pressure_p[i];
  const double gex = g.exner[i] + gpp * zz * kRgas * (rtp + rtb);
  const double E = zz * (kRgas / kP0) * (rtp + rtb);
  const double grtp = g.rtheta_p[i] + gpp * zz * kRgas * ex + gex * rcv * ex / E * zz * (kRgas / kP0);
  const double gthm = g.theta_m[i] + grtp * (rho_p + rb);
  const double grho_p = g.rho_p[i] + grtp * thm;
  double grz = g.rho_zz[i] + grho_p;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  for (int j = 0; j < n; ++j) grz += pru[(size_t)m.edgesOnCell[c * me + j] * L + k];
  const size_t ow = (size_t)c * (L + 1) + k;
  if (k >= 1) grz += m.fzm[k] * rho_ib[ow];
  if (k + 1 <= L - 1) grz += m.fzp[k + 1] * rho_ib[ow + 1];
  g_theta[i] = gthm;
  g_rho[i] = grz / zz;
}

#define CHECK_RC(x)                  \
  do {                               \
    int _rc = (x);                   \
    if (_rc != MPASG_OK) return _rc; \
  } while (0)

}  // namespace

int mpasgi_diag_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                         const mpasg_transpose* t, int rk_step, const AdjWork& w, cudaStream_t s) {
  const int L = m->nVertLevels;
  const long long ncl = (long long)m->nCells * L, nel = (long long)m->nEdges * L;
  const long long nvl = (long long)m->nVertices * L;
  const int apvm = c->apvm_upwinding > 0.0 ? 1 : 0;
  FastDiv fl(L);
  double* pvc = w.c[0];
  double* pvcb = w.c[1];
  double* pv1 = w.e[0];
  double* pv2 = w.e[1];
  double* pc = w.e[2];
  double* vb = w.e[3];
  double* vortb = w.v[0];
  double* kevb = w.v[1];
  if (apvm) {
    k_dadj_pvc<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, pvc);
    MPASG_LAUNCH_CHECK();
  }
  k_dadj_edges_b<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *g, fl, rk_step, apvm, c->apvm_upwinding * c->dt, pvc, pv1,
                                                 pv2, pc, vb);
  MPASG_LAUNCH_CHECK();
  if (apvm) {
    k_dadj_pvc_b<<<nblocks(ncl), kBlock, 0, s>>>(*m, fl, pc, pvcb);
    MPASG_LAUNCH_CHECK();
  }
  k_dadj_vertices<<<nblocks(nvl), kBlock, 0, s>>>(*m, *g, *t, fl, apvm, pv1, pv2, pvcb, vortb, kevb);
  MPASG_LAUNCH_CHECK();
  k_dadj_edges_a<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *g, *t, fl, rk_step, vortb, kevb, vb);
  MPASG_LAUNCH_CHECK();
  k_dadj_hedge<<<nblocks(ncl), kBlock, 0, s>>>(*m, *g, fl);
  MPASG_LAUNCH_CHECK();
  // the stage's outputs are consumed
  const ZeroSpan zs[] = {{g->h_edge, (m->nEdges + 1LL) * L}, {g->pv_edge, (m->nEdges + 1LL) * L},
                         {g->divergence, (m->nCells + 1LL) * L}, {g->ke, (m->nCells + 1LL) * L},
                         {g->vorticity, (m->nVertices + 1LL) * L}};
  CHECK_RC(mpasgi_zero_many(zs, 5, s));
  return MPASG_OK;
}

extern "C" int mpasg_diag_vjp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                              const mpasg_transpose* t, int rk_step, double* work, void* stream) {
  if (!m || !c || !f || !g || !t || !work || !adj_supported(m, c) || c->precision != MPASG_PRECISION_FLOAT64)
    return MPASG_E_ARG;
  CHECK_RC(mpasg_solve_diagnostics(m, c, f, rk_step, stream));
  return mpasgi_diag_vjp_core(m, c, f, g, t, rk_step, adj_work(m, work), (cudaStream_t)stream);
}

extern "C" int mpasg_prepare_vjp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                                 const mpasg_transpose* t, const double* w_in, double* g_u, double* g_w,
                                 double* g_theta, double* g_rho, double* work, void* stream) {
  if (!m || !c || !f || !g || !t || !w_in || !g_u || !g_w || !g_theta || !g_rho || !work || !adj_supported(m, c))
    return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const AdjWork w = adj_work(m, work);
  mpasg_config c64 = *c;  // the preparation's diagnostics are float64 with the full tangential wind
  c64.precision = MPASG_PRECISION_FLOAT64;
  CHECK_RC(mpasgi_diag_vjp_core(m, &c64, f, g, t, 3, w, s));
  const int L = m->nVertLevels;
  FastDiv fl(L), fl1(L + 1);
  double* pru = w.e[4];
  double* rho_ib = w.c[2];
  k_padj_edges<<<nblocks((m->nEdges + 1LL) * L), kBlock, 0, s>>>(*m, *f, *g, fl, g_u, pru);
  MPASG_LAUNCH_CHECK();
  k_padj_wlev<<<nblocks((m->nCells + 1LL) * (L + 1)), kBlock, 0, s>>>(*m, *f, *g, fl1, w_in, g_w, rho_ib);
  MPASG_LAUNCH_CHECK();
  k_padj_cells<<<nblocks((m->nCells + 1LL) * L), kBlock, 0, s>>>(*m, *f, *g, fl, pru, rho_ib, g_theta, g_rho);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
