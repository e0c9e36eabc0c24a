// Diagnostics (mpas_pytorch/dynamics/solve_diagnostics.py:1052, composition :531),
// cell-centre wind reconstruction (dynamics/vector_reconstruction.py:311) and the
// cold-start coupled diagnostics (dynamics/init_coupled_diagnostics.py:147).
#include "common.cuh"

namespace {

// h_edge and the edge kinetic-energy weights
__global__ void k_diag_edges_a(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  f.h_edge[i] = 0.5 * (f.rho_zz[(size_t)c1 * L + k] + f.rho_zz[(size_t)c2 * L + k]);
  double u = f.u[i];
  f.ke_edge[i] = (m.dcEdge[e] * m.dvEdge[e]) * (u * u);
}

// vorticity, vertex kinetic energy and potential vorticity
__global__ void k_diag_vertices(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  uint32_t v = fl.div(i), k = i - v * L;
  const int vd = m.vertexDegree;
  double vort = 0.0, kev = 0.0;
  for (int j = 0; j < vd; ++j) {
    int e = m.edgesOnVertex[v * vd + j];
    double wgt = m.edgesOnVertex_sign[v * vd + j] * m.dcEdge[e];
    double t = wgt * f.u[(size_t)e * L + k];
    double ke = f.ke_edge[(size_t)e * L + k];
    vort = (j == 0) ? t : vort + t;
    kev = (j == 0) ? ke : kev + ke;
  }
  double iat = m.invAreaTriangle[v];
  vort = vort * iat;
  f.vorticity[i] = vort;
  f.ke_vertex[i] = 0.25 * iat * kev;
  f.pv_vertex[i] = m.fVertex[v] + vort;
}

// divergence, cell kinetic energy (with the vertex-kite blend) and cell PV for APVM
__global__ void k_diag_cells(mpasg_mesh m, mpasg_fields f, FastDiv fl, int apvm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double div = 0.0, ke = 0.0;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double wgt = m.edgesOnCell_sign[c * me + j] * m.dvEdge[e];
    double t = wgt * f.u[(size_t)e * L + k];
    double kt = 0.25 * f.ke_edge[(size_t)e * L + k];
    div = (j == 0) ? t : div + t;
    ke = (j == 0) ? kt : ke + kt;
  }
  const double ia = m.invAreaCell[c];
  div = div * ia;
  ke = ke * ia;
  const double ke_fact = 1.0 - 0.375;
  ke = ke_fact * ke;
  const int vd = m.vertexDegree;
  double pvc = 0.0;
  for (int j = 0; j < n; ++j) {
    int v = m.verticesOnCell[c * me + j];
    int kk = m.kiteForCell[c * me + j];
    if (v >= m.nVertices || kk < 0) continue;
    double kite = m.kiteAreasOnVertex[v * vd + kk];
    double t = (1.0 - ke_fact) * kite;
    t = t * f.ke_vertex[(size_t)v * L + k];
    t = t * ia;
    ke = ke + t;
    if (apvm) {
      double pt = kite * f.pv_vertex[(size_t)v * L + k];
      pt = pt * ia;
      pvc = (j == 0) ? pt : pvc + pt;
    }
  }
  f.divergence[i] = div;
  f.ke[i] = ke;
  if (apvm) f.pv_cell[i] = pvc;
}

// pv_edge (with APVM upwinding) and, at rk 3 / preparation, the TRiSK tangential wind
__global__ void k_diag_edges_b(mpasg_mesh m, mpasg_fields f, FastDiv fl, int recompute_v, double apvm_dt,
                               int apvm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
  double pv1 = f.pv_vertex[(size_t)v1 * L + k], pv2 = f.pv_vertex[(size_t)v2 * L + k];
  double pve = 0.5 * (pv1 + pv2);
  double vv;
  if (recompute_v) {
    const int n2 = m.nEdgesOnEdge[e];
    const int me2 = m.maxEdges2;
    vv = 0.0;
    for (int j = 0; j < n2; ++j) {
      int eo = m.edgesOnEdge[e * me2 + j];
      double t = m.weightsOnEdge[e * me2 + j] * f.u[(size_t)eo * L + k];
      vv = (j == 0) ? t : vv + t;
    }
    f.v[i] = vv;
  } else {
    vv = f.v[i];
  }
  if (apvm) {
    int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
    double grad_pvt = (pv2 - pv1) * m.invDvEdge[e];
    double grad_pvn = (f.pv_cell[(size_t)c2 * L + k] - f.pv_cell[(size_t)c1 * L + k]) * m.invDcEdge[e];
    double delta = apvm_dt * (vv * grad_pvt + f.u[i] * grad_pvn);
    pve = pve - delta;
  }
  f.pv_edge[i] = pve;
}

// mpas_reconstruct_2d: RBF reconstruction of the cell-centre wind
__global__ void k_reconstruct(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double x = 0.0, y = 0.0, z = 0.0;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double u = f.u[(size_t)e * L + k];
    const double* cr = m.coeffs_reconstruct + ((size_t)c * me + j) * 3;
    double tx = cr[0] * u, ty = cr[1] * u, tz = cr[2] * u;
    if (j == 0) {
      x = tx; y = ty; z = tz;
    } else {
      x = x + tx; y = y + ty; z = z + tz;
    }
  }
  double lat = m.latCell[c], lon = m.lonCell[c];
  double clat = cos(lat), slat = sin(lat), clon = cos(lon), slon = sin(lon);
  f.uReconstructX[i] = x;
  f.uReconstructY[i] = y;
  f.uReconstructZ[i] = z;
  f.uReconstructZonal[i] = -x * slon + y * clon;
  f.uReconstructMeridional[i] = -(x * clon + y * slon) * slat + z * clat;
}

// ---------------------------------------------------------------- cold-start preparation
__global__ void k_fill(double* p, int n, double v) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = v;
}

__global__ void k_prepare_cells(mpasg_mesh m, mpasg_fields f, FastDiv fl, const double* __restrict__ theta,
                                const double* __restrict__ rho, const double* __restrict__ qv, double rcv) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  double q = qv ? qv[i] : 0.0;
  double zz = m.zz[i];
  double theta_m = theta[i] * (1.0 + kRvord * q);
  double rho_zz = rho[i] / zz;
  double rb = m.rho_base[i], tb = m.theta_base[i];
  double rho_p = rho_zz - rb;
  double rtb = tb * rb;
  // unfused products: rtheta_p cancels to roundoff when the state is near the base state
  double rtp = __dadd_rn(__dmul_rn(theta_m, rho_p), __dmul_rn(rb, theta_m - tb));
  double ex = pow(zz * (kRgas / kP0) * (rtp + rtb), rcv);
  double exb = pow(zz * (kRgas / kP0) * rtb, rcv);
  f.theta_m[i] = theta_m;
  f.rho_zz[i] = rho_zz;
  f.rho_p[i] = rho_p;
  f.rtheta_base[i] = rtb;
  f.rtheta_p[i] = rtp;
  f.exner[i] = ex;
  f.exner_base[i] = exb;
  f.pressure_p[i] = zz * kRgas * __dadd_rn(__dmul_rn(ex, rtp), __dmul_rn(rtb, ex - exb));
  f.pressure_base[i] = zz * kRgas * exb * rtb;
}

__global__ void k_prepare_ru(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  f.ru[i] = 0.5 * f.u[i] * (f.rho_zz[(size_t)c1 * L + k] + f.rho_zz[(size_t)c2 * L + k]);
}

__global__ void k_prepare_rw(mpasg_mesh m, mpasg_fields f, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  if (k == 0 || k == (uint32_t)L) {
    f.rw[i] = 0.0;
    return;
  }
  const size_t oc = (size_t)c * L;
  double fzm = m.fzm[k], fzp = m.fzp[k];
  double rho_i = fzp * f.rho_zz[oc + k - 1] + fzm * f.rho_zz[oc + k];
  double zz_i = fzp * m.zz[oc + k - 1] + fzm * m.zz[oc + k];
  double rw = f.w[i] * rho_i * zz_i;
  const int me = m.maxEdges;
  const int n = m.flatTerrain ? 0 : m.nEdgesOnCell[c];  // zero-slope terms add exact zeros
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double flux = fzm * f.ru[(size_t)e * L + k] + fzp * f.ru[(size_t)e * L + k - 1];
    size_t zi = ((size_t)c * me + j) * (L + 1) + k;
    double coef = m.zb_cell[zi] + sgn(flux) * m.zb3_cell[zi];
    rw = rw - m.edgesOnCell_sign[c * me + j] * coef * flux * zz_i;
  }
  f.rw[i] = rw;
}

}  // namespace

extern "C" int mpasg_solve_diagnostics(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                                       void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  FastDiv fl(L);
  const int apvm = c->apvm_upwinding > 0.0 ? 1 : 0;
  k_diag_edges_a<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  k_diag_vertices<<<nblocks((long long)m->nVertices * L), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  k_diag_cells<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, fl, apvm);
  MPASG_LAUNCH_CHECK();
  k_diag_edges_b<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(
      *m, *f, fl, rk_step == 3 ? 1 : 0, c->apvm_upwinding * c->dt, apvm);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_reconstruct_2d(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  const int L = m->nVertLevels;
  k_reconstruct<<<nblocks((long long)m->nCells * L), kBlock, 0, (cudaStream_t)stream>>>(*m, *f, FastDiv(L));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_prepare(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, const double* theta,
                             const double* rho, const double* qv, void* stream) {
  if (!m || !c || !f || !theta || !rho) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  const double rcv = kRgas / (kCp - kRgas);
  FastDiv fl(L), fl1(L + 1);
  k_prepare_cells<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, fl, theta, rho, qv, rcv);
  MPASG_LAUNCH_CHECK();
  // rho_zz padding row stamped to 1.0 (atmosphere_model.py:529-545)
  k_fill<<<1, 128, 0, s>>>(f->rho_zz + (size_t)m->nCells * L, L, 1.0);
  MPASG_LAUNCH_CHECK();
  k_prepare_ru<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  k_prepare_rw<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, s>>>(*m, *f, fl1);
  MPASG_LAUNCH_CHECK();
  int rc = mpasg_solve_diagnostics(m, c, f, 3, stream);
  if (rc) return rc;
  return mpasg_reconstruct_2d(m, c, f, stream);
}
