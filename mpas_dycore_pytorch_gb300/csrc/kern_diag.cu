// Diagnostics (mpas_pytorch/dynamics/solve_diagnostics.py:1052, composition :531),
// cell-centre wind reconstruction (dynamics/vector_reconstruction.py:311) and the
// cold-start coupled diagnostics (dynamics/init_coupled_diagnostics.py:147).
#include "common.cuh"
#include "pow_exner.cuh"

namespace {

// Every diagnostic kernel is a template on the stencil arithmetic type T (common.cuh):
// double for the float64 form, float for the mixed form.

// h_edge and the edge kinetic-energy weights
template <typename T>
__global__ void k_diag_edges_a(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  f.h_edge[i] = f64(T(0.5) * (cv<T>(f.rho_zz[(size_t)c1 * L + k]) + cv<T>(f.rho_zz[(size_t)c2 * L + k])));
  const T u = fp<T>(f.u, f.u_f32)[i];
  const T dcdv = sizeof(T) == sizeof(double) ? cv<T>(m.edge_dcdv[e]) : G(dcEdge)[e] * G(dvEdge)[e];
  fpw<T>(f.ke_edge, f.ke_edge_f32)[i] = dcdv * (u * u);
}

// vorticity, vertex kinetic energy and potential vorticity
template <typename T>
__global__ void k_diag_vertices(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  uint32_t v = fl.div(i), k = i - v * L;
  const int vd = m.vertexDegree;
  // the circulation sum cancels strongly: float64 in both forms
  double vort = 0.0;
  T kev = T(0);
  for (int j = 0; j < vd; ++j) {
    int e = m.edgesOnVertex[v * vd + j];
    double t = m.vertex_edge_sdc[v * vd + j] * f.u[(size_t)e * L + k];  // (sign * dcEdge) * u
    T ke = fp<T>(f.ke_edge, f.ke_edge_f32)[(size_t)e * L + k];
    vort = (j == 0) ? t : vort + t;
    kev = (j == 0) ? ke : kev + ke;
  }
  const double iat = m.invAreaTriangle[v];
  vort = vort * iat;
  f.vorticity[i] = vort;
  f.ke_vertex[i] = f64(T(0.25) * G(invAreaTriangle)[v] * kev);
  const double pvv = m.fVertex[v] + vort;
  f.pv_vertex[i] = pvv;
  if (sizeof(T) != sizeof(double)) f.pv_vertex_f32[i] = d2f_bits(pvv);
}

// divergence, cell kinetic energy (with the vertex-kite blend) and cell PV for APVM
template <typename T>
__global__ void k_diag_cells(mpasg_mesh m, mpasg_fields f, FastDiv fl, int apvm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  // the divergence sum cancels strongly: float64 in both forms
  double div = 0.0;
  T ke = T(0);
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double t = m.cell_edge_sdv[c * me + j] * f.u[(size_t)e * L + k];  // (sign * dvEdge) * u
    T kt = fp<T>(f.ke_edge, f.ke_edge_f32)[(size_t)e * L + k];
    div = (j == 0) ? t : div + t;
    ke = (j == 0) ? kt : ke + kt;
  }
  div = div * m.invAreaCell[c];
  const T ia = G(invAreaCell)[c];
  // sum_j 0.25 ke_edge_j: the power-of-two factor applied once to the sum (scaling by
  // 0.25 commutes with every rounding of the sum)
  ke = (T(0.25) * ke) * ia;
  const T ke_fact = T(1.0 - 0.375);
  ke = ke_fact * ke;
  const int vd = m.vertexDegree;
  T pvc = T(0);
  for (int j = 0; j < n; ++j) {
    int v = m.verticesOnCell[c * me + j];
    int kk = m.kiteForCell[c * me + j];
    if (v >= m.nVertices || kk < 0) continue;
    T kite = G(kiteAreasOnVertex)[v * vd + kk];
    T t = (T(1) - ke_fact) * kite;
    t = t * cv<T>(f.ke_vertex[(size_t)v * L + k]);
    t = t * ia;
    ke = ke + t;
    if (apvm) {
      T pt = kite * fp<T>(f.pv_vertex, f.pv_vertex_f32)[(size_t)v * L + k];
      pt = pt * ia;
      pvc = (j == 0) ? pt : pvc + pt;
    }
  }
  f.divergence[i] = div;
  f.ke[i] = f64(ke);
  if (apvm) f.pv_cell[i] = f64(pvc);
}

// pv_edge (with APVM upwinding) and, at rk 3 / preparation, the TRiSK tangential wind
template <typename T>
__global__ void k_diag_edges_b(mpasg_mesh m, mpasg_fields f, FastDiv fl, int recompute_v, double apvm_dt,
                               int apvm) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
  const T* pvv = fp<T>(f.pv_vertex, f.pv_vertex_f32);
  const T* u = fp<T>(f.u, f.u_f32);
  const T pv1 = pvv[(size_t)v1 * L + k], pv2 = pvv[(size_t)v2 * L + k];
  T pve = T(0.5) * (pv1 + pv2);
  T vv;
  if (recompute_v) {
    const int n2 = m.nEdgesOnEdge[e];
    const int me2 = m.maxEdges2;
    vv = T(0);
    for (int j = 0; j < n2; ++j) {
      int eo = m.edgesOnEdge[e * me2 + j];
      T t = G(weightsOnEdge)[e * me2 + j] * u[(size_t)eo * L + k];
      vv = (j == 0) ? t : vv + t;
    }
    f.v[i] = f64(vv);
  } else {
    vv = cv<T>(f.v[i]);
  }
  if (apvm) {
    int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
    T grad_pvt = (pv2 - pv1) * G(invDvEdge)[e];
    T grad_pvn = (cv<T>(f.pv_cell[(size_t)c2 * L + k]) - cv<T>(f.pv_cell[(size_t)c1 * L + k])) * G(invDcEdge)[e];
    T delta = cv<T>(apvm_dt) * (vv * grad_pvt + u[i] * grad_pvn);
    pve = pve - delta;
  }
  f.pv_edge[i] = f64(pve);
  if (sizeof(T) != sizeof(double)) f.pv_edge_f32[i] = pve;
}

// mpas_reconstruct_2d: RBF reconstruction of the cell-centre wind
template <typename T>
__global__ void k_reconstruct(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  T x = T(0), y = T(0), z = T(0);
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    T u = fp<T>(f.u, f.u_f32)[(size_t)e * L + k];
    const T* cr = G(coeffs_reconstruct) + ((size_t)c * me + j) * 3;
    T tx = cr[0] * u, ty = cr[1] * u, tz = cr[2] * u;
    if (j == 0) {
      x = tx; y = ty; z = tz;
    } else {
      x = x + tx; y = y + ty; z = z + tz;
    }
  }
  const double* tr = m.cell_trig + (size_t)c * 4;  // cos / sin of the cell's latitude and longitude
  const T clat = cv<T>(tr[0]), slat = cv<T>(tr[1]), clon = cv<T>(tr[2]), slon = cv<T>(tr[3]);
  f.uReconstructX[i] = f64(x);
  f.uReconstructY[i] = f64(y);
  f.uReconstructZ[i] = f64(z);
  f.uReconstructZonal[i] = f64(-x * slon + y * clon);
  f.uReconstructMeridional[i] = f64(-(x * clon + y * slon) * slat + z * clat);
}

// ---------------------------------------------------------------- surface pressure
// physics_interface_surface_pressure (mpas_pytorch/diagnostics.py:10, formula :77-82):
// hydrostatic extrapolation of the lowest two layers plus the lowest-level pressure.
// Separately rounded operations in the reference's order, so the result is bit-exact.
__global__ void k_surface_pressure(int nc, int rows, int L, const double* __restrict__ rho_zz,
                                   const double* __restrict__ zz, const double* __restrict__ qv,
                                   const double* __restrict__ pp, const double* __restrict__ pb,
                                   const double* __restrict__ zgrid, double half_g, double* __restrict__ out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= rows) return;
  if (c >= nc) {
    out[c] = 0.0;  // padding row
    return;
  }
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double tem1 = __dsub_rn(zgrid[ow + 1], zgrid[ow]);
  const double tem2 = __dsub_rn(zgrid[ow + 2], zgrid[ow + 1]);
  const double q0 = qv ? qv[o] : 0.0, q1 = qv ? qv[o + 1] : 0.0;
  const double rho1 = __dmul_rn(__dmul_rn(rho_zz[o], zz[o]), __dadd_rn(1.0, q0));
  const double rho2 = __dmul_rn(__dmul_rn(rho_zz[o + 1], zz[o + 1]), __dadd_rn(1.0, q1));
  const double corr = __ddiv_rn(__dmul_rn(__dmul_rn(0.5, __dsub_rn(rho2, rho1)), tem1), __dadd_rn(tem1, tem2));
  const double hyd = __dmul_rn(__dmul_rn(half_g, tem1), __dsub_rn(rho1, corr));
  out[c] = __dadd_rn(__dadd_rn(hyd, pp[o]), pb[o]);
}

// area-weighted sum of squared anomalies, sum_c w_c (x_c - r_c)^2, in a fixed order
// (one block: strided partial sums, then a shared-memory tree), so it is deterministic
__global__ void __launch_bounds__(1024) k_weighted_sq_sum(long long n, const double* __restrict__ x,
                                                          const double* __restrict__ r,
                                                          const double* __restrict__ w, double* out) {
  __shared__ double part[1024];
  double acc = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = x[i] - (r ? r[i] : 0.0);
    acc = acc + (w ? w[i] : 1.0) * (d * d);
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) part[threadIdx.x] = part[threadIdx.x] + part[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

// Derivatives of the surface pressure (diagnostics.py:77-82) with respect to rho_zz, qv,
// pressure_p and pressure_base.  hyd = A * B with A = (g/2) tem1 and
// B = rho1 - ((0.5 (rho2 - rho1)) tem1) / s, s = tem1 + tem2; read backwards in the order
// torch's reverse mode evaluates that expression, so the result is bit-identical to it.
// One thread per cell-level of the (rows, L) cotangent arrays: levels 0 and 1 of the
// active cells carry the derivative, every other entry is written 0.  Null outputs skip.
__global__ void k_surface_pressure_vjp(int nc, int rows, int L, const double* __restrict__ rho_zz,
                                       const double* __restrict__ zz, const double* __restrict__ qv,
                                       const double* __restrict__ zgrid, double half_g,
                                       const double* __restrict__ g_sp, double* __restrict__ g_rho,
                                       double* __restrict__ g_qv, double* __restrict__ g_pp,
                                       double* __restrict__ g_pb) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)rows * L) return;
  const int c = (int)(i / L), k = (int)(i - (long long)c * L);
  double gr = 0.0, gq = 0.0, gp = 0.0;
  if (c < nc && k < 2) {
    const size_t ow = (size_t)c * (L + 1);
    const double tem1 = __dsub_rn(zgrid[ow + 1], zgrid[ow]);
    const double s = __dadd_rn(tem1, __dsub_rn(zgrid[ow + 2], zgrid[ow + 1]));
    const double g = g_sp[c];
    const double gB = __dmul_rn(g, __dmul_rn(half_g, tem1));
    const double gD = __dmul_rn(0.5, __dmul_rn(__ddiv_rn(-gB, s), tem1));
    const double grho = k == 0 ? __dsub_rn(gB, gD) : gD;  // cotangent of rho1 / rho2
    const double q = qv ? qv[i] : 0.0;
    gr = __dmul_rn(__dmul_rn(grho, __dadd_rn(1.0, q)), zz[i]);
    gq = __dmul_rn(grho, __dmul_rn(rho_zz[i], zz[i]));
    gp = k == 0 ? g : 0.0;
  }
  if (g_rho) g_rho[i] = gr;
  if (g_qv) g_qv[i] = gq;
  if (g_pp) g_pp[i] = gp;
  if (g_pb) g_pb[i] = gp;
}

// Tangent of the surface pressure for tangents of rho_zz, qv, pressure_p, pressure_base
// (null tangent = zero), in the order torch's forward mode evaluates the expression.
__global__ void k_surface_pressure_jvp(int nc, int rows, int L, const double* __restrict__ rho_zz,
                                       const double* __restrict__ zz, const double* __restrict__ qv,
                                       const double* __restrict__ zgrid, double half_g,
                                       const double* __restrict__ t_rho, const double* __restrict__ t_qv,
                                       const double* __restrict__ t_pp, const double* __restrict__ t_pb,
                                       double* __restrict__ t_sp) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= rows) return;
  if (c >= nc) {
    t_sp[c] = 0.0;
    return;
  }
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double tem1 = __dsub_rn(zgrid[ow + 1], zgrid[ow]);
  const double s = __dadd_rn(tem1, __dsub_rn(zgrid[ow + 2], zgrid[ow + 1]));
  double d[2];
  for (int k = 0; k < 2; ++k) {
    const double q = qv ? qv[o + k] : 0.0;
    const double a = t_rho ? __dmul_rn(__dmul_rn(t_rho[o + k], zz[o + k]), __dadd_rn(1.0, q)) : 0.0;
    const double b = t_qv ? __dmul_rn(__dmul_rn(rho_zz[o + k], zz[o + k]), t_qv[o + k]) : 0.0;
    d[k] = __dadd_rn(a, b);
  }
  const double dC = __ddiv_rn(__dmul_rn(__dmul_rn(0.5, __dsub_rn(d[1], d[0])), tem1), s);
  const double hyd = __dmul_rn(__dmul_rn(half_g, tem1), __dsub_rn(d[0], dC));
  t_sp[c] = __dadd_rn(__dadd_rn(hyd, t_pp ? t_pp[o] : 0.0), t_pb ? t_pb[o] : 0.0);
}

// gradient of sum_i w_i (x_i - r_i)^2 scaled by the device scalar *g_out:
// g_x = 2 ((g_out w) (x - r)); g_r (optional) = -g_x
__global__ void k_weighted_sq_sum_vjp(long long n, const double* __restrict__ x, const double* __restrict__ r,
                                      const double* __restrict__ w, const double* __restrict__ g_out,
                                      double* __restrict__ g_x, double* __restrict__ g_r) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = __dsub_rn(x[i], r ? r[i] : 0.0);
  const double g = __dmul_rn(2.0, __dmul_rn(__dmul_rn(*g_out, w ? w[i] : 1.0), d));
  if (g_x) g_x[i] = g;
  if (g_r) g_r[i] = -g;
}

// ---------------------------------------------------------------- cold-start preparation
__global__ void k_fill(double* p, int n, double v) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = v;
}

// DERIVED: theta and rho hold theta_m and rho_zz themselves (the rederivation of a step
// boundary whose prognostics were edited, init_coupled_diagnostics.py:259-261); they may
// alias f.theta_m and f.rho_zz (each thread reads its element before writing it)
template <bool DERIVED>
__global__ void k_prepare_cells(mpasg_mesh m, mpasg_fields f, FastDiv fl, const double* theta,
                                const double* rho, const double* __restrict__ qv, double rcv) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  double zz = m.zz[i];
  double theta_m, rho_zz;
  if (DERIVED) {
    theta_m = theta[i];
    rho_zz = rho[i];
  } else {
    double q = qv ? qv[i] : 0.0;
    theta_m = theta[i] * (1.0 + kRvord * q);
    rho_zz = rho[i] / zz;
  }
  double rb = m.rho_base[i], tb = m.theta_base[i];
  double rho_p = rho_zz - rb;
  double rtb = tb * rb;
  // unfused products: rtheta_p cancels to roundoff when the state is near the base state
  double rtp = __dadd_rn(__dmul_rn(theta_m, rho_p), __dmul_rn(rb, theta_m - tb));
  double ex = mpasg_pow::pow_exner(zz * (kRgas / kP0) * (rtp + rtb), rcv);
  double exb = mpasg_pow::pow_exner(zz * (kRgas / kP0) * rtb, rcv);
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

template <typename T>
int launch_diagnostics(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step, cudaStream_t s) {
  const int L = m->nVertLevels;
  FastDiv fl(L);
  const int apvm = c->apvm_upwinding > 0.0 ? 1 : 0;
  k_diag_edges_a<T><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  k_diag_vertices<T><<<nblocks((long long)m->nVertices * L), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  k_diag_cells<T><<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, fl, apvm);
  MPASG_LAUNCH_CHECK();
  k_diag_edges_b<T><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(
      *m, *f, fl, rk_step == 3 ? 1 : 0, c->apvm_upwinding * c->dt, apvm);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

}  // namespace

extern "C" int mpasg_solve_diagnostics(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                                       void* stream) {
  return mpasgi_solve_diagnostics(m, c, f, rk_step, (cudaStream_t)stream, false);
}

int mpasgi_solve_diagnostics(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                             cudaStream_t s, bool copies_current) {
  if (!m || !c || !f) return MPASG_E_ARG;
  if (c->precision == MPASG_PRECISION_MIXED) {
    if (!copies_current) {
      const int rc = mpasgi_pack_f32(m, f, s);
      if (rc != MPASG_OK) return rc;
    }
    return launch_diagnostics<float>(m, c, f, rk_step, s);
  }
  return launch_diagnostics<double>(m, c, f, rk_step, s);
}

extern "C" int mpasg_reconstruct_2d(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, void* stream) {
  return mpasgi_reconstruct(m, c, f, (cudaStream_t)stream, false);
}

int mpasgi_reconstruct(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, cudaStream_t s,
                       bool copies_current) {
  if (!m || !c || !f) return MPASG_E_ARG;
  const int L = m->nVertLevels;
  if (c->precision == MPASG_PRECISION_MIXED) {
    if (!copies_current) {
      const int rc = mpasgi_pack_f32(m, f, s);
      if (rc != MPASG_OK) return rc;
    }
    k_reconstruct<float><<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, FastDiv(L));
  } else {
    k_reconstruct<double><<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, FastDiv(L));
  }
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

namespace {
template <bool DERIVED>
int prepare(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, const double* theta, const double* rho,
            const double* qv, void* stream) {
  if (!m || !c || !f || !theta || !rho) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  const double rcv = kRgas / (kCp - kRgas);
  FastDiv fl(L), fl1(L + 1);
  k_prepare_cells<DERIVED><<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, fl, theta, rho, qv, rcv);
  MPASG_LAUNCH_CHECK();
  // rho_zz padding row stamped to 1.0 (atmosphere_model.py:529-545)
  k_fill<<<1, 128, 0, s>>>(f->rho_zz + (size_t)m->nCells * L, L, 1.0);
  MPASG_LAUNCH_CHECK();
  k_prepare_ru<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  k_prepare_rw<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, s>>>(*m, *f, fl1);
  MPASG_LAUNCH_CHECK();
  mpasg_config c64 = *c;  // the cold start is float64 in both precisions
  c64.precision = MPASG_PRECISION_FLOAT64;
  int rc = mpasg_solve_diagnostics(m, &c64, f, 3, stream);
  if (rc) return rc;
  return mpasg_reconstruct_2d(m, &c64, f, stream);
}
}  // namespace

extern "C" int mpasg_prepare(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, const double* theta,
                             const double* rho, const double* qv, void* stream) {
  return prepare<false>(m, c, f, theta, rho, qv, stream);
}

extern "C" int mpasg_prepare_derived(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                     const double* theta_m, const double* rho_zz, void* stream) {
  return prepare<true>(m, c, f, theta_m, rho_zz, nullptr, stream);
}

extern "C" int mpasg_surface_pressure(int nCells, int rows, int nVertLevels, const double* rho_zz, const double* zz,
                                      const double* qv, const double* pressure_p, const double* pressure_base,
                                      const double* zgrid, double gravity, double* out, void* stream) {
  if (!rho_zz || !zz || !pressure_p || !pressure_base || !zgrid || !out) return MPASG_E_ARG;
  if (nCells < 0 || (rows != nCells && rows != nCells + 1) || nVertLevels < 2) return MPASG_E_ARG;
  if (rows == 0) return MPASG_OK;
  k_surface_pressure<<<nblocks(rows), kBlock, 0, (cudaStream_t)stream>>>(
      nCells, rows, nVertLevels, rho_zz, zz, qv, pressure_p, pressure_base, zgrid, 0.5 * gravity, out);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_weighted_sq_sum(long long n, const double* x, const double* ref, const double* weight,
                                     double* out, void* stream) {
  if (!x || !out || n < 0) return MPASG_E_ARG;
  k_weighted_sq_sum<<<1, 1024, 0, (cudaStream_t)stream>>>(n, x, ref, weight, out);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_surface_pressure_vjp(int nCells, int rows, int nVertLevels, const double* rho_zz,
                                          const double* zz, const double* qv, const double* zgrid,
                                          double gravity, const double* g_sp, double* g_rho_zz, double* g_qv,
                                          double* g_pressure_p, double* g_pressure_base, void* stream) {
  if (!rho_zz || !zz || !zgrid || !g_sp || nVertLevels < 2 || nCells < 0 ||
      (rows != nCells && rows != nCells + 1))
    return MPASG_E_ARG;
  const long long n = (long long)rows * nVertLevels;
  if (n == 0) return MPASG_OK;
  k_surface_pressure_vjp<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      nCells, rows, nVertLevels, rho_zz, zz, qv, zgrid, 0.5 * gravity, g_sp, g_rho_zz, g_qv, g_pressure_p,
      g_pressure_base);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_surface_pressure_jvp(int nCells, int rows, int nVertLevels, const double* rho_zz,
                                          const double* zz, const double* qv, const double* zgrid,
                                          double gravity, const double* t_rho_zz, const double* t_qv,
                                          const double* t_pressure_p, const double* t_pressure_base,
                                          double* t_sp, void* stream) {
  if (!rho_zz || !zz || !zgrid || !t_sp || nVertLevels < 2 || nCells < 0 ||
      (rows != nCells && rows != nCells + 1))
    return MPASG_E_ARG;
  if (rows == 0) return MPASG_OK;
  k_surface_pressure_jvp<<<nblocks(rows), kBlock, 0, (cudaStream_t)stream>>>(
      nCells, rows, nVertLevels, rho_zz, zz, qv, zgrid, 0.5 * gravity, t_rho_zz, t_qv, t_pressure_p,
      t_pressure_base, t_sp);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_weighted_sq_sum_vjp(long long n, const double* x, const double* ref, const double* weight,
                                         const double* g_out, double* g_x, double* g_ref, void* stream) {
  if (!x || !g_out || n < 0) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_weighted_sq_sum_vjp<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      n, x, ref, weight, g_out, g_x, g_ref);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
