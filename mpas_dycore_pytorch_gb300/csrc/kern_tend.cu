// Large-step tendencies (the reference's atm_compute_dyn_tend_work,
// mpas_pytorch/dynamics/dyn_tend.py:10836, canonical composition :9390).
//
//   k_tend_cells_a   h_divergence (+ rk 1: Smagorinsky kdiff, tend_rho, dpdz)   sections :9925-9992
//   k_tend_u         u tendency: vertical transport, PV flux, KE gradient, divergence
//                    coupling (+ rk 1: pressure gradient and del2 mixing)        :9993-10315
//   k_del4_vertex / k_del4_cell / k_tend_u_finish   del4 filter and vertical mixing of u
//                    (rk 1)                                                      :10075-10315
//   k_mix_cells_a / k_mix_cells_b   w and theta del2 / del4 mixing (rk 1)       :10355, :10544
//   k_adv_edges      horizontal advective fluxes of w and theta, once per edge    :10316, :10442
//   k_tend_w_theta   w and theta flux divergence, vertical fluxes, buoyancy,
//                    diabatic term                                                :10386, :10679
//
// Every kernel is a template on the stencil arithmetic type T (common.cuh): double for
// the float64 form, whose slot sums follow the reference's order (first slot assigned,
// then left to right); float for the mixed form, which reads the float32 copies of the
// geometry and of u, w, rw, pv_edge (fp<T> / G) and float64 fields through cv<T>.
#include <cmath>

#include "common.cuh"

namespace {

struct TendScalars {
  double inv_dt, c_s_len2, kdiff_cap, h_mom_visc4, h_theta_visc4, del4u_div, coef3, visc2;
  double cam_base, v_mom, v_theta;  // CAM damping base, vertical mixing coefficients (0: off)
  double ray_coef;                  // 1 / (levels * timescale): Rayleigh damping of u
  int rk_step, smag, del4;
  int ncam;   // CAM damping levels (0: off)
  int ray_n;  // Rayleigh-damped top levels of u (0: off)
  int mix_pert;  // vertical mixing of the perturbation from the initial profiles
  int defer;  // k_tend_u leaves tend_u_euler to k_tend_u_finish (del4 and / or vertical mixing)
};

// CAM-style damping of the top ncam levels (dyn_tend.py:3434-3456): kdiff raised to
// base * (1 - (L - (k + 1)) / ncam), base = 4 * 2.0833 * len_disp * mpas_cam_coef
MPASG_D double cam_kdiff(double kd, const TendScalars& p, uint32_t k, int L) {
  const double factor = 1.0 - (double)(L - (int)(k + 1)) / (double)p.ncam;
  return fmax(kd, p.cam_base * factor);
}

template <typename T, bool CAM = false>
__global__ void k_tend_cells_a(mpasg_mesh m, mpasg_fields f, FastDiv fl, TendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  // the mass-flux divergence cancels strongly: float64 in both forms
  double hdiv = 0.0;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double t = m.cell_edge_sdv[c * me + j] * f.ru[(size_t)e * L + k];  // (sign * dvEdge) * ru
    hdiv = (j == 0) ? t : hdiv + t;
  }
  hdiv = hdiv * m.invAreaCell[c];
  f.h_divergence[i] = hdiv;
  if (p.rk_step != 1) return;
  const size_t ow = (size_t)c * (L + 1) + k;
  f.tend_rho[i] = -hdiv - m.rdzw[k] * (f.rw[ow + 1] - f.rw[ow]);
  // dpdz nearly balances the vertical pressure gradient (k_tend_w_theta): float64
  double q = f.qtot[i];
  f.dpdz[i] = -kGravity * (m.rho_base[i] * q + f.rr_save[i] * (1.0 + q));
  if (p.smag) {
    const T* defc_a = G(defc_a);
    const T* defc_b = G(defc_b);
    const T* u = fp<T>(f.u, f.u_f32);
    T dd = T(0), dof = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      T ca = defc_a[c * me + j], cb = defc_b[c * me + j];
      T ue = u[(size_t)e * L + k], ve = cv<T>(f.v[(size_t)e * L + k]);
      T ndd = (dd + ca * ue) - cb * ve;
      T ndo = (dof + cb * ue) + ca * ve;
      dd = ndd;
      dof = ndo;
    }
    double kd = f64(vmin(cv<T>(p.c_s_len2) * vsqrt(dd * dd + dof * dof), cv<T>(p.kdiff_cap)));
    if (CAM && (int)k >= L - p.ncam) kd = cam_kdiff(kd, p, k, L);
    f.kdiff[i] = kd;
  } else {  // 2d_fixed: the theta del2 coefficient everywhere
    f.kdiff[i] = (CAM && (int)k >= L - p.ncam) ? cam_kdiff(p.visc2, p, k, L) : p.visc2;
  }
}

// Rayleigh damping of u on the top ray_n levels (dyn_tend.py:2956-2990), every RK stage:
// tend_u - rho_edge u ((k + 1) - k0) / (ray_n timescale), k0 = L - ray_n
template <typename T>
MPASG_D T rayleigh_u(T tu, T rho_e, T u_k, int k, int L, const TendScalars& p) {
  const int k0 = L - p.ray_n;
  if (p.ray_n <= 0 || k < k0) return tu;
  const double damp = (((double)k + 1.0) - (double)k0) * p.ray_coef;
  return tu - rho_e * u_k * cv<T>(damp);
}

template <typename T>
MPASG_D T wduz_at(const T* __restrict__ u, T rwe, int kk, int L, const T* fzm, const T* fzp) {
  if (kk <= 0 || kk >= L) return T(0);
  if (kk == 1 || kk == L - 1) return rwe * (fzm[kk] * u[kk] + fzp[kk] * u[kk - 1]);
  return flux3<T>(u[kk - 2], u[kk - 1], u[kk], u[kk + 1], rwe, T(1));
}

// pv_edge * u at every edge level, the neighbour factor of the float64 PV flux sum (below),
// formed once per tendency stage instead of once per reading edge; stored in ke_edge (the
// diagnostics' edge kinetic-energy scratch, free between two diagnostics stages)
template <typename T>
__global__ void k_pvu(mpasg_mesh m, mpasg_fields f, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fpw<T>(f.ke_edge, f.ke_edge_f32)[i] = fp<T>(f.pv_edge, f.pv_edge_f32)[i] * fp<T>(f.u, f.u_f32)[i];
}

// RAY: Rayleigh damping of u compiled in (a run-time test would cost float64 work in
// every thread of the hot kernel once the compiler predicates it)
template <typename T, bool RAY = false>
__global__ void __launch_bounds__(kBlock) k_tend_u(mpasg_mesh m, mpasg_fields f, FastDiv fl, TendScalars p) {
  __shared__ T s_wd[kBlock];
  const int L = m.nVertLevels;
  const uint32_t n_all = (uint32_t)m.nEdges * L;
  const T* u = fp<T>(f.u, f.u_f32);
  const T* rw = fp<T>(f.rw, f.rw_f32);
  const T* fzm = G(fzm);
  const T* fzp = G(fzp);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n_all;
  uint32_t e = 0, k = 0;
  int c1 = 0, c2 = 0;
  const T* ue = u;
  T wd_k = T(0);
  if (active) {
    e = fl.div(i);
    k = i - e * L;
    c1 = m.cellsOnEdge[2 * e];
    c2 = m.cellsOnEdge[2 * e + 1];
    ue = u + (size_t)e * L;
    T rwe_k = T(0.5) * (rw[(size_t)c1 * (L + 1) + k] + rw[(size_t)c2 * (L + 1) + k]);
    wd_k = wduz_at<T>(ue, rwe_k, k, L, fzm, fzp);
  }
  s_wd[threadIdx.x] = wd_k;  // vertical flux at the interface below level k
  __syncthreads();
  if (!active) return;
  T wd_k1;
  if (k + 1 >= (uint32_t)L) {
    wd_k1 = T(0);
  } else if (threadIdx.x + 1 < blockDim.x) {
    wd_k1 = s_wd[threadIdx.x + 1];  // same edge, next level
  } else {
    T rwe_k1 = T(0.5) * (rw[(size_t)c1 * (L + 1) + k + 1] + rw[(size_t)c2 * (L + 1) + k + 1]);
    wd_k1 = wduz_at<T>(ue, rwe_k1, k + 1, L, fzm, fzp);
  }
  T tu = -G(rdzw)[k] * (wd_k1 - wd_k);
  // nonlinear Coriolis / PV flux over the TRiSK stencil, sum_j w_j u_j 0.5 (pv_self + pv_j)
  // over the slots in order.  float64: as 0.5 (pv_self sum_j w_j u_j + sum_j w_j (pv u)_j),
  // two multiply-adds per neighbour on the float64 pipe that bounds the kernel, (pv u)
  // formed once per edge level by k_pvu; float32: as written, the exact power-of-two
  // factor 0.5 applied once to the sum (the extra pass would cost more than it saves)
  const int n2 = m.nEdgesOnEdge[e];
  const int me2 = m.maxEdges2;
  const T* pv = fp<T>(f.pv_edge, f.pv_edge_f32);
  const T* woe = G(weightsOnEdge);
  const T pv_self = pv[i];
  T q;
  if constexpr (sizeof(T) == sizeof(double)) {
    const double* pvu = f.ke_edge;
    T sa = T(0), sb = T(0);
    for (int j = 0; j < n2; ++j) {
      const size_t io = (size_t)m.edgesOnEdge[e * me2 + j] * L + k;
      const T w = woe[e * me2 + j];
      sa = (j == 0) ? w * u[io] : sa + w * u[io];
      sb = (j == 0) ? w * pvu[io] : sb + w * pvu[io];
    }
    q = T(0.5) * (pv_self * sa + sb);
  } else {
    q = T(0);
    for (int j = 0; j < n2; ++j) {
      int eo = m.edgesOnEdge[e * me2 + j];
      T t = (woe[e * me2 + j] * u[(size_t)eo * L + k]) * (pv_self + pv[(size_t)eo * L + k]);
      q = (j == 0) ? t : q + t;
    }
    q = T(0.5) * q;
  }
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  const T inv_dc = G(invDcEdge)[e];
  const T rho_e = cv<T>(f.h_edge[i]);
  tu = tu + rho_e * (q - dif<T>(f.ke[i2], f.ke[i1]) * inv_dc) -
       ue[k] * T(0.5) * (cv<T>(f.h_divergence[i1]) + cv<T>(f.h_divergence[i2]));
  if (RAY) tu = rayleigh_u<T>(tu, rho_e, ue[k], (int)k, L, p);
  if (p.rk_step == 1) {
    const T* zz = G(zz);
    T teu = -cv<T>(f.cqu_e[i]) * (div_or_one<T>(dif<T>(f.pressure_p[i2], f.pressure_p[i1]) * inv_dc,
                                                T(0.5) * (zz[i2] + zz[i1])) -
                                  T(0.5) * G(zxu)[i] * (cv<T>(f.dpdz[i1]) + cv<T>(f.dpdz[i2])));
    int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
    T r_dv = vmin(G(invDvEdge)[e], T(4) * inv_dc);
    T u_diff = (cv<T>(f.divergence[i2]) - cv<T>(f.divergence[i1])) * inv_dc -
               (cv<T>(f.vorticity[(size_t)v2 * L + k]) - cv<T>(f.vorticity[(size_t)v1 * L + k])) * r_dv;
    f.delsq_u[i] = f64(u_diff);
    T kdiffu = T(0.5) * (cv<T>(f.kdiff[i1]) + cv<T>(f.kdiff[i2]));
    teu = teu + rho_e * kdiffu * u_diff * G(meshScalingDel2)[e];
    f.tend_u_euler[i] = f64(teu);
    f.tend_u[i] = f64(p.defer ? tu : tu + teu);
  } else {
    f.tend_u[i] = f64(tu + cv<T>(f.tend_u_euler[i]));
  }
}

// k_tend_u with V consecutive levels per thread (a tile of the autotuner): the edge's
// connectivity and TRiSK weights are loaded once for V levels, the V neighbour gathers
// are independent, and the interface fluxes at k0 .. k0+V are computed in-thread (the
// top one again by the next chunk).  Per level, the same expressions in the same order as
// k_tend_u; the compiler may fuse multiply-adds differently in the two kernels, so the
// tiles agree to the rounding of one FMA (last bit).
template <typename T, int V, bool RAY = false>
__global__ void __launch_bounds__(kBlock) k_tend_u_chunk(mpasg_mesh m, mpasg_fields f, FastDiv flc, int nchunk,
                                                         TendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * (uint32_t)nchunk) return;
  const uint32_t e = flc.div(i);
  const int k0 = (int)(i - e * (uint32_t)nchunk) * V;
  const T* u = fp<T>(f.u, f.u_f32);
  const T* rw = fp<T>(f.rw, f.rw_f32);
  const T* fzm = G(fzm);
  const T* fzp = G(fzp);
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const T* ue = u + (size_t)e * L;
  T wd[V + 1];
#pragma unroll
  for (int v = 0; v <= V; ++v) {
    const int kk = k0 + v;
    wd[v] = T(0);
    if (kk < L) {
      T rwe = T(0.5) * (rw[(size_t)c1 * (L + 1) + kk] + rw[(size_t)c2 * (L + 1) + kk]);
      wd[v] = wduz_at<T>(ue, rwe, kk, L, fzm, fzp);
    }
  }
  const int n2 = m.nEdgesOnEdge[e];
  const int me2 = m.maxEdges2;
  const T* pv = fp<T>(f.pv_edge, f.pv_edge_f32);
  const T* pvu = fp<T>(f.ke_edge, f.ke_edge_f32);  // float64 only (k_tend_u)
  const T* woe = G(weightsOnEdge);
  constexpr bool kSplit = sizeof(T) == sizeof(double);
  T pv_self[V], sa[V], sb[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    pv_self[v] = (k0 + v < L) ? pv[(size_t)e * L + k0 + v] : T(0);
    sa[v] = T(0);
    sb[v] = T(0);
  }
  for (int j = 0; j < n2; ++j) {
    const int eo = m.edgesOnEdge[e * me2 + j];
    const T w = woe[e * me2 + j];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      if (k0 + v < L) {
        const size_t oo = (size_t)eo * L + k0 + v;
        if (kSplit) {
          sa[v] = (j == 0) ? w * u[oo] : sa[v] + w * u[oo];
          sb[v] = (j == 0) ? w * pvu[oo] : sb[v] + w * pvu[oo];
        } else {
          const T t = (w * u[oo]) * (pv_self[v] + pv[oo]);
          sa[v] = (j == 0) ? t : sa[v] + t;
        }
      }
    }
  }
  const T inv_dc = G(invDcEdge)[e];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int k = k0 + v;
    if (k >= L) break;
    const size_t ie = (size_t)e * L + k;
    T tu = -G(rdzw)[k] * ((k + 1 >= L ? T(0) : wd[v + 1]) - wd[v]);
    const T qv = kSplit ? T(0.5) * (pv_self[v] * sa[v] + sb[v]) : T(0.5) * sa[v];
    const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
    const T rho_e = cv<T>(f.h_edge[ie]);
    tu = tu + rho_e * (qv - dif<T>(f.ke[i2], f.ke[i1]) * inv_dc) -
         ue[k] * T(0.5) * (cv<T>(f.h_divergence[i1]) + cv<T>(f.h_divergence[i2]));
    if (RAY) tu = rayleigh_u<T>(tu, rho_e, ue[k], k, L, p);
    if (p.rk_step == 1) {
      const T* zz = G(zz);
      T teu = -cv<T>(f.cqu_e[ie]) * (div_or_one<T>(dif<T>(f.pressure_p[i2], f.pressure_p[i1]) * inv_dc,
                                                   T(0.5) * (zz[i2] + zz[i1])) -
                                     T(0.5) * G(zxu)[ie] * (cv<T>(f.dpdz[i1]) + cv<T>(f.dpdz[i2])));
      int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
      T r_dv = vmin(G(invDvEdge)[e], T(4) * inv_dc);
      T u_diff = (cv<T>(f.divergence[i2]) - cv<T>(f.divergence[i1])) * inv_dc -
                 (cv<T>(f.vorticity[(size_t)v2 * L + k]) - cv<T>(f.vorticity[(size_t)v1 * L + k])) * r_dv;
      f.delsq_u[ie] = f64(u_diff);
      T kdiffu = T(0.5) * (cv<T>(f.kdiff[i1]) + cv<T>(f.kdiff[i2]));
      teu = teu + rho_e * kdiffu * u_diff * G(meshScalingDel2)[e];
      f.tend_u_euler[ie] = f64(teu);
      f.tend_u[ie] = f64(p.defer ? tu : tu + teu);
    } else {
      f.tend_u[ie] = f64(tu + cv<T>(f.tend_u_euler[ie]));
    }
  }
}

template <typename T>
__global__ void k_del4_vertex(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nVertices * L) return;
  uint32_t v = fl.div(i), k = i - v * L;
  const int vd = m.vertexDegree;
  const T* iat = G(invAreaTriangle);
  const T* dc = G(dcEdge);
  const T* sg = G(edgesOnVertex_sign);
  T acc = T(0);
  for (int j = 0; j < vd; ++j) {
    int e = m.edgesOnVertex[v * vd + j];
    T es = iat[v] * dc[e] * sg[v * vd + j];
    T t = es * cv<T>(f.delsq_u[(size_t)e * L + k]);
    acc = (j == 0) ? t : acc + t;
  }
  f.delsq_vort[i] = f64(acc);
}

template <typename T>
__global__ void k_del4_cell(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T* ia = G(invAreaCell);
  const T* dv = G(dvEdge);
  const T* sg = G(edgesOnCell_sign);
  T acc = T(0);
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    T es = ia[c] * dv[e] * sg[c * me + j];
    T t = es * cv<T>(f.delsq_u[(size_t)e * L + k]);
    acc = (j == 0) ? t : acc + t;
  }
  f.delsq_div[i] = f64(acc);
}

// rk 1 completion of the u tendency when k_tend_u deferred it: del4 filter (if enabled),
// then vertical mixing of u (dyn_tend.py:2730-2780; full state, interior levels, heights
// of the edge's interfaces as the mean of its two cells), then tend_u += tend_u_euler
template <typename T>
__global__ void k_tend_u_finish(mpasg_mesh m, mpasg_fields f, FastDiv fl, TendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  T teu = cv<T>(f.tend_u_euler[i]);
  if (p.del4) {
    const int v1 = m.verticesOnEdge[2 * e], v2 = m.verticesOnEdge[2 * e + 1];
    const T inv_dc = G(invDcEdge)[e];
    T u_mix = G(meshScalingDel4)[e] * cv<T>(p.h_mom_visc4);
    T r_dc4 = u_mix * cv<T>(p.del4u_div) * inv_dc;
    T r_dv4 = u_mix * vmin(G(invDvEdge)[e], T(4) * inv_dc);
    T u_diff4 = (cv<T>(f.delsq_div[(size_t)c2 * L + k]) - cv<T>(f.delsq_div[(size_t)c1 * L + k])) * r_dc4 -
                (cv<T>(f.delsq_vort[(size_t)v2 * L + k]) - cv<T>(f.delsq_vort[(size_t)v1 * L + k])) * r_dv4;
    teu = teu - cv<T>(f.h_edge[i]) * u_diff4;
  }
  if (p.v_mom > 0.0 && k >= 1 && k + 1 < (uint32_t)L) {
    const double* z1p = m.zgrid + (size_t)c1 * (L + 1);
    const double* z2p = m.zgrid + (size_t)c2 * (L + 1);
    const double za = 0.5 * (z1p[k - 1] + z2p[k - 1]), zb = 0.5 * (z1p[k] + z2p[k]);
    const double zc = 0.5 * (z1p[k + 1] + z2p[k + 1]), zd = 0.5 * (z1p[k + 2] + z2p[k + 2]);
    const double zm = 0.5 * (za + zb), z0 = 0.5 * (zb + zc), zp = 0.5 * (zc + zd);
    const double* u = f.u + (size_t)e * L;
    double um = u[k - 1], u0 = u[k], up = u[k + 1];
    if (p.mix_pert) {  // perturbation from the initial profile along the edge normal
      const double ca = cos(m.angleEdge[e]), sa = sin(m.angleEdge[e]);
      um = um - m.u_init[k - 1] * ca - m.v_init[k - 1] * sa;
      u0 = u0 - m.u_init[k] * ca - m.v_init[k] * sa;
      up = up - m.u_init[k + 1] * ca - m.v_init[k + 1] * sa;
    }
    const T d_up = dif<T>(up, u0) / cv<T>(zp - z0);
    const T d_dn = dif<T>(u0, um) / cv<T>(z0 - zm);
    teu = teu + cv<T>(f.h_edge[i]) * cv<T>(p.v_mom) * (d_up - d_dn) / cv<T>(0.5 * (zp - zm));
  }
  f.tend_u_euler[i] = f64(teu);
  f.tend_u[i] = f64(cv<T>(f.tend_u[i]) + teu);
}

// vertical mixing of w at interface k, 1 <= k <= L-1 (dyn_tend.py:4636-4648, rk 1)
MPASG_D double w_vmix(const mpasg_mesh& m, const mpasg_fields& f, size_t oc, size_t ow, uint32_t k, double v) {
  const double rho_half = 0.5 * (f.rho_zz[oc + k] + f.rho_zz[oc + k - 1]);
  const double w_up = (f.w[ow + k + 1] - f.w[ow + k]) * m.rdzw[k];
  const double w_down = (f.w[ow + k] - f.w[ow + k - 1]) * m.rdzw[k - 1];
  return v * rho_half * (w_up - w_down) * m.rdzu[k];
}

// vertical mixing of theta at level k, 1 <= k <= L-2 (dyn_tend.py:5064-5100, rk 1;
// Prandtl factor 1)
MPASG_D double theta_vmix(const mpasg_mesh& m, const mpasg_fields& f, uint32_t c, uint32_t k, int L, double v,
                          int mix_pert) {
  const double* zg = m.zgrid + (size_t)c * (L + 1);
  const double zm = 0.5 * (zg[k - 1] + zg[k]), z0 = 0.5 * (zg[k] + zg[k + 1]), zp = 0.5 * (zg[k + 1] + zg[k + 2]);
  const double* th = f.theta_m + (size_t)c * L;
  double tm = th[k - 1], t0 = th[k], tp = th[k + 1];
  if (mix_pert) {  // perturbation from the initial profile
    const double* ti = m.t_init + (size_t)c * L;
    tm = tm - ti[k - 1];
    t0 = t0 - ti[k];
    tp = tp - ti[k + 1];
  }
  const double diff = (tp - t0) / (zp - z0) - (t0 - tm) / (z0 - zm);
  return v * 1.0 * f.rho_zz[(size_t)c * L + k] * diff / (0.5 * (zp - zm));
}

// w / theta del2 mixing and the del2 fields for del4 (rk 1); index space (C, L+1)
template <typename T>
__global__ void k_mix_cells_a(mpasg_mesh m, mpasg_fields f, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T ia = G(invAreaCell)[c];
  const T* sg = G(edgesOnCell_sign);
  const T* dv = G(dvEdge);
  const T* idc = G(invDcEdge);
  const T* msd2 = G(meshScalingDel2);
  if (k >= 1 && k < (uint32_t)L) {  // w
    const T* w = fp<T>(f.w, f.w_f32);
    T dw = T(0), tw = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      T es = sizeof(T) == sizeof(double) ? cv<T>(m.cell_edge_es_w[c * me + j])  // same product, formed once
                                         : T(0.5) * ia * sg[c * me + j] * dv[e] * idc[e];
      T flux = es * (cv<T>(f.h_edge[(size_t)e * L + k]) + cv<T>(f.h_edge[(size_t)e * L + k - 1])) *
               (w[(size_t)ec2 * (L + 1) + k] - w[(size_t)ec1 * (L + 1) + k]);
      dw = dw + flux;
      flux = flux * msd2[e] * T(0.25) *
             (cv<T>(f.kdiff[(size_t)ec1 * L + k]) + cv<T>(f.kdiff[(size_t)ec2 * L + k]) +
              cv<T>(f.kdiff[(size_t)ec1 * L + k - 1]) + cv<T>(f.kdiff[(size_t)ec2 * L + k - 1]));
      tw = tw + flux;
    }
    f.delsq_w[i] = f64(dw);
    f.tend_w_euler[i] = f64(tw);
  } else {
    f.delsq_w[i] = 0.0;
    f.tend_w_euler[i] = 0.0;
  }
  if (k < (uint32_t)L) {  // theta
    const size_t o = (size_t)c * L + k;
    T dt_ = T(0), tt = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      T es = sizeof(T) == sizeof(double) ? cv<T>(m.cell_edge_es_t[c * me + j]) : ia * sg[c * me + j] * dv[e] * idc[e];
      T pr = T(1) * msd2[e];
      T flux = es * dif<T>(f.theta_m[(size_t)ec2 * L + k], f.theta_m[(size_t)ec1 * L + k]) *
               cv<T>(f.h_edge[(size_t)e * L + k]);
      dt_ = dt_ + flux;
      flux = flux * T(0.5) * (cv<T>(f.kdiff[(size_t)ec1 * L + k]) + cv<T>(f.kdiff[(size_t)ec2 * L + k])) * pr;
      tt = tt + flux;
    }
    f.delsq_theta[o] = f64(dt_);
    f.tend_theta_euler[o] = f64(tt);
  }
}

// del4 parts of w / theta mixing (rk 1)
template <typename T>
__global__ void k_mix_cells_b(mpasg_mesh m, mpasg_fields f, FastDiv fl1, TendScalars p) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T ia = G(invAreaCell)[c];
  const T* sg = G(edgesOnCell_sign);
  const T* dv = G(dvEdge);
  const T* idc = G(invDcEdge);
  const T* msd4 = G(meshScalingDel4);
  if (k >= 1 && k < (uint32_t)L) {
    T tw = cv<T>(f.tend_w_euler[i]);
    const T hm = cv<T>(p.h_mom_visc4) * ia;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      T es = msd4[e] * hm * dv[e] * sg[c * me + j] * idc[e];
      tw = tw - es * (cv<T>(f.delsq_w[(size_t)ec2 * (L + 1) + k]) - cv<T>(f.delsq_w[(size_t)ec1 * (L + 1) + k]));
    }
    f.tend_w_euler[i] = f64(tw);
  }
  if (k < (uint32_t)L) {
    const size_t o = (size_t)c * L + k;
    T tt = cv<T>(f.tend_theta_euler[o]);
    const T ht = cv<T>(p.h_theta_visc4) * T(1) * ia;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
      T es = msd4[e] * ht * dv[e] * sg[c * me + j] * idc[e];
      tt = tt - es * (cv<T>(f.delsq_theta[(size_t)ec2 * L + k]) - cv<T>(f.delsq_theta[(size_t)ec1 * L + k]));
    }
    f.tend_theta_euler[o] = f64(tt);
  }
}

template <typename T>
MPASG_D T wdwz_at(const T* w, const T* rw, int kk, int L) {
  if (kk <= 0 || kk >= L) return T(0);
  if (kk == 1 || kk == L - 1) return T(0.25) * (rw[kk] + rw[kk - 1]) * (w[kk] + w[kk - 1]);
  return flux3<T>(w[kk - 2], w[kk - 1], w[kk], w[kk + 1], T(0.5) * (rw[kk] + rw[kk - 1]), T(1));
}

// vertical theta flux at interface kk: th / ths are theta_m / theta_m_save (float64 form)
// or their deviations from the reference profile (mixed form); rw_t is rw as the stencil
// type, rw / rws the float64 rw and rw_save
template <typename T>
MPASG_D T wdtz_at(const T* th, const T* ths, const T* rw_t, const double* rw, const double* rws, int kk, int L,
                  const T* fzm, const T* fzp, T coef3) {
  if (kk <= 0 || kk >= L) return T(0);
  const T fm = fzm[kk], fp = fzp[kk];
  if (kk == L - 1 && kk != 1) return cv<T>(rws[kk]) * (fm * th[kk] + fp * th[kk - 1]);
  T v;
  if (kk == 1)
    v = rw_t[kk] * (fm * th[kk] + fp * th[kk - 1]);
  else
    v = flux3<T>(th[kk - 2], th[kk - 1], th[kk], th[kk + 1], rw_t[kk], coef3);
  return v + dif<T>(rws[kk], rw[kk]) * (fm * ths[kk] + fp * ths[kk - 1]);
}

// Edge-side horizontal advective fluxes of w and theta_m, computed once per edge:
// flux_w_e[e,k] = ru_w * sum_a (adv_coefs +/- adv_coefs_3rd)_a w[advCell_a, k] (w levels 1..L-1)
// flux_th_e[e,k] = ru * sum_a (...)_a theta_m[advCell_a, k] (mass levels 0..L-1).
// The cell sums then apply edgesOnCell_sign (an exact +/-1 factor), which reproduces
// the reference's per-slot (sign * ru) * flux products bit for bit.  The mixed form
// advects the deviation theta_m - ref_theta (its reference part is added in float64 by
// k_tend_w_theta_mixed) and stores float32 fluxes.
template <typename T>
__global__ void k_adv_edges(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int na = m.nAdvMax;
  const int nadv = m.nAdvCellsForEdge[e];
  const int32_t* cells = m.advCellsForEdge + (size_t)e * na;
  const T* cfp = G(adv_coefs_p) + (size_t)e * na;
  const T* cfm = G(adv_coefs_m) + (size_t)e * na;
  const T rue = cv<T>(f.ru[i]);
  {
    const T* th = fp<T>(f.theta_m, f.theta_dev);
    const T* cf = rue >= T(0) ? cfp : cfm;
    T acc = T(0);
    for (int a = 0; a < nadv; ++a) {
      T t = cf[a] * th[(size_t)cells[a] * L + k];
      acc = (a == 0) ? t : acc + t;
    }
    fpw<T>(f.flux_th_e, f.flux_th_e_f32)[i] = rue * acc;
  }
  if (k >= 1) {
    const T* w = fp<T>(f.w, f.w_f32);
    T ru_w = G(fzm)[k] * rue + G(fzp)[k] * cv<T>(f.ru[i - 1]);
    const T* cf = ru_w >= T(0) ? cfp : cfm;
    T acc = T(0);
    for (int a = 0; a < nadv; ++a) {
      T t = cf[a] * w[(size_t)cells[a] * (L + 1) + k];
      acc = (a == 0) ? t : acc + t;
    }
    fpw<T>(f.flux_w_e, f.flux_w_e_f32)[i] = ru_w * acc;
  }
}

// w and theta tendencies (float64 form); index space (C, L+1)
__global__ void __launch_bounds__(kBlock) k_tend_w_theta(mpasg_mesh m, mpasg_fields f, FastDiv fl1, TendScalars p) {
  using T = double;
  __shared__ T s_wd[kBlock], s_wt[kBlock];
  const int L = m.nVertLevels;
  const uint32_t n_all = (uint32_t)m.nCells * (L + 1);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n_all;
  uint32_t c = 0, k = 0;
  T wd_k = T(0), wt_k = T(0);
  const T coef3 = p.coef3;
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
    const size_t ow0 = (size_t)c * (L + 1), oc0 = (size_t)c * L;
    wd_k = wdwz_at<T>(f.w + ow0, f.rw + ow0, k, L);
    wt_k = wdtz_at<T>(f.theta_m + oc0, f.theta_m_save + oc0, f.rw + ow0, f.rw + ow0, f.rw_save + ow0, k, L, m.fzm,
                      m.fzp, coef3);
  }
  s_wd[threadIdx.x] = wd_k;  // interface fluxes owned by this level
  s_wt[threadIdx.x] = wt_k;
  __syncthreads();
  if (!active) return;
  T wd_k1 = T(0), wt_k1 = T(0);
  if (k < (uint32_t)L) {
    if (threadIdx.x + 1 < blockDim.x) {
      wd_k1 = s_wd[threadIdx.x + 1];
      wt_k1 = s_wt[threadIdx.x + 1];
    } else {
      const size_t ow0 = (size_t)c * (L + 1), oc0 = (size_t)c * L;
      wd_k1 = wdwz_at<T>(f.w + ow0, f.rw + ow0, k + 1, L);
      wt_k1 = wdtz_at<T>(f.theta_m + oc0, f.theta_m_save + oc0, f.rw + ow0, f.rw + ow0, f.rw_save + ow0, k + 1, L,
                         m.fzm, m.fzp, coef3);
    }
  }
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T ia = m.invAreaCell[c];
  const size_t oc = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  if (k >= 1 && k < (uint32_t)L) {
    T tw = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      tw = tw - m.edgesOnCell_sign[c * me + j] * f.flux_w_e[(size_t)e * L + k];
    }
    tw = tw * ia - m.rdzu[k] * (wd_k1 - wd_k);
    T teu = f.tend_w_euler[i];
    if (p.rk_step == 1) {
      // vertical pressure gradient minus buoyancy: a near-hydrostatic residual
      const double res = m.rdzu[k] * (f.pressure_p[oc + k] - f.pressure_p[oc + k - 1]) -
                         (m.fzm[k] * f.dpdz[oc + k] + m.fzp[k] * f.dpdz[oc + k - 1]);
      teu = teu - f.cqw[ow + k] * res;
      if (p.v_mom > 0.0) teu = teu + w_vmix(m, f, oc, ow, k, p.v_mom);
      f.tend_w_euler[i] = teu;
    }
    f.tend_w[i] = tw + teu;
  } else {
    f.tend_w[i] = 0.0;
  }
  if (k < (uint32_t)L) {
    const size_t o = oc + k;
    T tt = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      T x = -(m.edgesOnCell_sign[c * me + j] * f.flux_th_e[(size_t)e * L + k]);
      tt = (j == 0) ? x : tt + x;
    }
    if (p.rk_step > 1) {
      for (int j = 0; j < n; ++j) {
        int e = m.edgesOnCell[c * me + j];
        // (sign dvEdge) (ru_save - ru) 0.5 (theta_2 + theta_1), with the slot product and the
        // edge mean formed once (scaling by 0.5 is exact, so the rounding is unchanged)
        T flux = m.cell_edge_sdv[c * me + j] * (f.ru_save[(size_t)e * L + k] - f.ru[(size_t)e * L + k]) *
                 f.theta_edge_save[(size_t)e * L + k];
        tt = tt - flux;
      }
    }
    tt = tt * ia - m.rdzw[k] * (wt_k1 - wt_k);
    const T rz = f.rho_zz[o];
    const T rtd = f.rt_diabatic_tend[o];
    // unfused: the difference cancels strongly (as rounded by the reference)
    f.rthdynten[o] = sub_rn(tt, mul_rn(f.tend_rho[o], f.theta_m[o])) / rz;
    tt = tt + rz * rtd;
    double tte = f.tend_theta_euler[o];
    if (p.rk_step == 1 && p.v_theta > 0.0 && k >= 1 && k + 1 < (uint32_t)L) {
      tte = tte + theta_vmix(m, f, c, k, L, p.v_theta, p.mix_pert);
      f.tend_theta_euler[o] = tte;
    }
    tt = tt + tte;
    f.tend_theta[o] = tt;
  }
}

// ---------------------------------------------------------------- mixed form, theta split
// theta = ref_theta(k) + theta'.  The flux divergences of theta cancel to a few parts in
// 10^3 of their terms (theta ~ 300 K), too few digits are left in float32; the deviation
// theta' (a few K) is advected in float32 and the reference part, which reduces to
// per-level profile weights times float64 mass fluxes, is added in float64.
__global__ void k_theta_dev(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  (void)c;
  const double r = m.ref_theta[k];
  f.theta_dev[i] = d2f_bits(f.theta_m[i] - r);
  f.theta_save_dev[i] = d2f_bits(f.theta_m_save[i] - r);
}

// float64 vertical flux of the reference profile at interface kk (the reference part of
// wdtz_at: flux3 and second-order interpolations are linear in theta)
MPASG_D double ref_wflux(const mpasg_mesh& m, double rw, double rws, int kk, int L, double coef3) {
  if (kk <= 0 || kk >= L) return 0.0;
  const double w2 = m.ref_theta_w2[kk];
  if (kk == L - 1 && kk != 1) return rws * w2;
  if (kk == 1) return rw * w2 + (rws - rw) * w2;
  return rw * m.ref_theta_w4[kk] + coef3 * fabs(rw) * m.ref_theta_w3[kk] + (rws - rw) * w2;
}

__global__ void __launch_bounds__(kBlock) k_tend_w_theta_mixed(mpasg_mesh m, mpasg_fields f, FastDiv fl1,
                                                               TendScalars p) {
  using T = float;
  __shared__ T s_wd[kBlock], s_wt[kBlock];
  __shared__ double s_wr[kBlock];
  const int L = m.nVertLevels;
  const uint32_t n_all = (uint32_t)m.nCells * (L + 1);
  const T* w = f.w_f32;
  const T* rw = f.rw_f32;
  const T* fzm = m.fzm_f32;
  const T* fzp = m.fzp_f32;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n_all;
  uint32_t c = 0, k = 0;
  T wd_k = T(0), wt_k = T(0);
  double wr_k = 0.0;
  const T coef3 = cv<T>(p.coef3);
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
    const size_t ow0 = (size_t)c * (L + 1), oc0 = (size_t)c * L;
    wd_k = wdwz_at<T>(w + ow0, rw + ow0, k, L);
    wt_k = wdtz_at<T>(f.theta_dev + oc0, f.theta_save_dev + oc0, rw + ow0, f.rw + ow0, f.rw_save + ow0, k, L, fzm,
                      fzp, coef3);
    if (k < (uint32_t)L) wr_k = ref_wflux(m, f.rw[ow0 + k], f.rw_save[ow0 + k], k, L, p.coef3);
  }
  s_wd[threadIdx.x] = wd_k;
  s_wt[threadIdx.x] = wt_k;
  s_wr[threadIdx.x] = wr_k;
  __syncthreads();
  if (!active) return;
  T wd_k1 = T(0), wt_k1 = T(0);
  double wr_k1 = 0.0;
  if (k < (uint32_t)L) {
    if (threadIdx.x + 1 < blockDim.x) {
      wd_k1 = s_wd[threadIdx.x + 1];
      wt_k1 = s_wt[threadIdx.x + 1];
      wr_k1 = s_wr[threadIdx.x + 1];
    } else {
      const size_t ow0 = (size_t)c * (L + 1), oc0 = (size_t)c * L;
      wd_k1 = wdwz_at<T>(w + ow0, rw + ow0, k + 1, L);
      wt_k1 = wdtz_at<T>(f.theta_dev + oc0, f.theta_save_dev + oc0, rw + ow0, f.rw + ow0, f.rw_save + ow0, k + 1,
                         L, fzm, fzp, coef3);
      wr_k1 = ref_wflux(m, f.rw[ow0 + k + 1], f.rw_save[ow0 + k + 1], k + 1, L, p.coef3);
    }
  }
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T ia = m.invAreaCell_f32[c];
  const T* sg = m.edgesOnCell_sign_f32;
  const size_t oc = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  if (k >= 1 && k < (uint32_t)L) {
    T tw = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      tw = tw - sg[c * me + j] * f.flux_w_e_f32[(size_t)e * L + k];
    }
    tw = tw * ia - m.rdzu_f32[k] * (wd_k1 - wd_k);
    T teu = cv<T>(f.tend_w_euler[i]);
    if (p.rk_step == 1) {
      const double res = m.rdzu[k] * (f.pressure_p[oc + k] - f.pressure_p[oc + k - 1]) -
                         (m.fzm[k] * f.dpdz[oc + k] + m.fzp[k] * f.dpdz[oc + k - 1]);
      teu = teu - cv<T>(f.cqw[ow + k]) * cv<T>(res);
      if (p.v_mom > 0.0) teu = teu + cv<T>(w_vmix(m, f, oc, ow, k, p.v_mom));
      f.tend_w_euler[i] = f64(teu);
    }
    f.tend_w[i] = f64(tw + teu);
  } else {
    f.tend_w[i] = 0.0;
  }
  if (k < (uint32_t)L) {
    const size_t o = oc + k;
    const double rt = m.ref_theta[k];
    T tt = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      T x = -(sg[c * me + j] * f.flux_th_e_f32[(size_t)e * L + k]);
      tt = (j == 0) ? x : tt + x;
    }
    // reference part of the horizontal flux divergence: the adv_coefs of an edge sum to
    // its dvEdge (to 1e-11), so it is ref_theta times the float64 mass-flux divergence
    double tmean = -rt * f.h_divergence[o];
    if (p.rk_step > 1) {
      double dsum = 0.0;
      for (int j = 0; j < n; ++j) {
        int e = m.edgesOnCell[c * me + j];
        int ec1 = m.cellsOnEdge[2 * e], ec2 = m.cellsOnEdge[2 * e + 1];
        const double wgt = m.cell_edge_sdv[c * me + j];  // sign * dvEdge (mesh table)
        const double dru = f.ru_save[(size_t)e * L + k] - f.ru[(size_t)e * L + k];
        dsum = dsum + wgt * dru;
        T flux = cv<T>(wgt) * cv<T>(dru) * T(0.5) *
                 (f.theta_save_dev[(size_t)ec2 * L + k] + f.theta_save_dev[(size_t)ec1 * L + k]);
        tt = tt - flux;
      }
      tmean = tmean - rt * dsum * m.invAreaCell[c];
    }
    tt = tt * ia - m.rdzw_f32[k] * (wt_k1 - wt_k);
    tmean = tmean - m.rdzw[k] * (wr_k1 - wr_k);
    const double ttot = f64(tt) + tmean;
    const double rz = f.rho_zz[o];
    // (a diagnostic for physics coupling: the cancelling difference in float64, the
    // quotient in float32)
    f.rthdynten[o] = f64(cv<T>(ttot - f.tend_rho[o] * f.theta_m[o]) / cv<T>(rz));
    double tte = f.tend_theta_euler[o];
    if (p.rk_step == 1 && p.v_theta > 0.0 && k >= 1 && k + 1 < (uint32_t)L) {
      tte = tte + theta_vmix(m, f, c, k, L, p.v_theta, p.mix_pert);
      f.tend_theta_euler[o] = tte;
    }
    f.tend_theta[o] = ttot + rz * f.rt_diabatic_tend[o] + tte;
  }
}

MPASG_HD int tile_levels(int code) { return code == 2 ? 2 : code == 4 ? 4 : 1; }

template <typename T>
int launch_dyn_tend(const mpasg_mesh* m, mpasg_fields* f, const TendScalars& p, int rk_step, cudaStream_t s,
                    int c_tile) {
  const int L = m->nVertLevels;
  const long long ncl = (long long)m->nCells * L, nel = (long long)m->nEdges * L;
  const long long ncw = (long long)m->nCells * (L + 1), nvl = (long long)m->nVertices * L;
  FastDiv fl(L), fl1(L + 1);
  if (sizeof(T) != sizeof(double)) {
    k_theta_dev<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl);
    MPASG_LAUNCH_CHECK();
  }
  if (p.ncam > 0 && rk_step == 1)
    k_tend_cells_a<T, true><<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, p);
  else
    k_tend_cells_a<T><<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, p);
  MPASG_LAUNCH_CHECK();
  if (sizeof(T) == sizeof(double)) {  // the float64 PV flux reads pv_edge * u (k_tend_u)
    k_pvu<T><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, nel);
    MPASG_LAUNCH_CHECK();
  }
  const int vt = tile_levels(c_tile);  // levels per thread of k_tend_u (autotuner choice)
  const bool ray = p.ray_n > 0;
  if (vt == 1) {
    if (ray) k_tend_u<T, true><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, p);
    else k_tend_u<T><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, p);
  } else {
    const int nchunk = (L + vt - 1) / vt;
    const long long nth = (long long)m->nEdges * nchunk;
    if (vt == 2) {
      if (ray) k_tend_u_chunk<T, 2, true><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
      else k_tend_u_chunk<T, 2><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
    } else {
      if (ray) k_tend_u_chunk<T, 4, true><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
      else k_tend_u_chunk<T, 4><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
    }
  }
  MPASG_LAUNCH_CHECK();
  if (rk_step == 1) {
    if (p.del4) {
      k_del4_vertex<T><<<nblocks(nvl), kBlock, 0, s>>>(*m, *f, fl);
      MPASG_LAUNCH_CHECK();
      k_del4_cell<T><<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl);
      MPASG_LAUNCH_CHECK();
    }
    if (p.defer) {
      k_tend_u_finish<T><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, p);
      MPASG_LAUNCH_CHECK();
    }
    k_mix_cells_a<T><<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, fl1);
    MPASG_LAUNCH_CHECK();
    if (p.h_mom_visc4 > 0.0 || p.h_theta_visc4 > 0.0) {
      TendScalars q = p;
      if (!(p.h_mom_visc4 > 0.0)) q.h_mom_visc4 = 0.0;
      k_mix_cells_b<T><<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, fl1, q);
      MPASG_LAUNCH_CHECK();
    }
  }
  k_adv_edges<T><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl);
  MPASG_LAUNCH_CHECK();
  if (sizeof(T) == sizeof(double))
    k_tend_w_theta<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, fl1, p);
  else
    k_tend_w_theta_mixed<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, fl1, p);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

}  // namespace

int mpasgi_theta_dev(const mpasg_mesh* m, mpasg_fields* f, cudaStream_t s) {
  const int L = m->nVertLevels;
  k_theta_dev<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, FastDiv(L));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_dyn_tend(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                              void* stream) {
  return mpasgi_dyn_tend(m, c, f, rk_step, (cudaStream_t)stream, false);
}

int mpasgi_dyn_tend(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step, cudaStream_t s,
                    bool copies_current) {
  if (!m || !c || !f || rk_step < 1 || rk_step > 3) return MPASG_E_ARG;
  if (!copies_current && rk_step > 1 && c->precision != MPASG_PRECISION_MIXED) {
    const int rc = mpasgi_theta_edge(m, f, false, s);  // the edge mean of theta_m_save read below
    if (rc != MPASG_OK) return rc;
  }
  if (m->nVertLevels < 4) return MPASG_E_ARG;
  if (c->precision != MPASG_PRECISION_FLOAT64 && c->precision != MPASG_PRECISION_MIXED) return MPASG_E_ARG;
  TendScalars p;
  p.inv_dt = 1.0 / c->dt;
  double cl = c->c_s * c->len_disp;
  p.c_s_len2 = cl * cl;
  p.kdiff_cap = (0.01 * (c->len_disp * c->len_disp)) * p.inv_dt;
  p.smag = c->horiz_mixing_smagorinsky;
  if (p.smag) {
    p.h_mom_visc4 = c->visc4_2dsmag * std::pow(c->len_disp, 3.0);  // correctly rounded, as len**3
    p.h_theta_visc4 = p.h_mom_visc4;
  } else {
    p.h_mom_visc4 = c->h_mom_eddy_visc4;
    p.h_theta_visc4 = c->h_theta_eddy_visc4;
  }
  p.visc2 = p.smag ? 0.0 : c->h_theta_eddy_visc2;
  p.del4u_div = c->del4u_div_factor;
  p.coef3 = c->coef_3rd_order;
  p.rk_step = rk_step;
  p.del4 = (p.h_mom_visc4 > 0.0) ? 1 : 0;
  if (c->number_cam_damping_levels > m->nVertLevels) return MPASG_E_ARG;
  p.ncam = (c->mpas_cam_coef > 0.0 && c->number_cam_damping_levels > 0) ? c->number_cam_damping_levels : 0;
  p.cam_base = 4.0 * 2.0833 * c->len_disp * c->mpas_cam_coef;
  p.v_mom = c->v_mom_eddy_visc2 > 0.0 ? c->v_mom_eddy_visc2 : 0.0;
  p.v_theta = c->v_theta_eddy_visc2 > 0.0 ? c->v_theta_eddy_visc2 : 0.0;
  p.defer = (p.del4 || p.v_mom > 0.0) ? 1 : 0;
  if (p.v_mom > 0.0 || p.v_theta > 0.0) {
    if (!m->zgrid) return MPASG_E_ARG;
  }
  p.mix_pert = c->mix_perturbation ? 1 : 0;
  if (p.mix_pert && (p.v_mom > 0.0 || p.v_theta > 0.0) && (!m->u_init || !m->v_init || !m->angleEdge || !m->t_init))
    return MPASG_E_ARG;
  p.ray_n = c->rayleigh_damp_u_levels;
  if (p.ray_n > m->nVertLevels || p.ray_n < 0) return MPASG_E_ARG;
  p.ray_coef = p.ray_n > 0 ? 1.0 / ((double)p.ray_n * (c->rayleigh_damp_u_timescale_days * 86400.0)) : 0.0;
  if (c->precision == MPASG_PRECISION_MIXED) {
    if (!copies_current) {
      const int rc = mpasgi_pack_f32(m, f, s);
      if (rc != MPASG_OK) return rc;
    }
    return launch_dyn_tend<float>(m, f, p, rk_step, s, c->tile_tend_u);
  }
  return launch_dyn_tend<double>(m, f, p, rk_step, s, c->tile_tend_u);
}

// Autotuner: times the u-tendency kernel with 1, 2 and 4 levels per thread on the current
// state (rk-2 form, 3 launches each after one warm-up) and keeps the fastest in
// c->tile_tend_u.  Host-synchronising: call it outside stream capture.  The kernels only
// write their outputs (tend_u, ...) and the ke_edge scratch, so the state is unchanged.
extern "C" int mpasg_autotune(const mpasg_mesh* m, mpasg_config* c, mpasg_fields* f, float* times_ms,
                              void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const bool mixed = c->precision == MPASG_PRECISION_MIXED;
  if (mixed) {
    const int rc = mpasgi_pack_f32(m, f, s);
    if (rc != MPASG_OK) return rc;
  }
  TendScalars p{};
  p.rk_step = 2;
  p.coef3 = c->coef_3rd_order;
  const int L = m->nVertLevels;
  const long long nel = (long long)m->nEdges * L;
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return MPASG_E_CUDA;
  if (!mixed) {
    k_pvu<double><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, nel);
    mpasg_count_launch();
    if (cudaGetLastError() != cudaSuccess) return MPASG_E_LAUNCH;
  }
  const int tiles[3] = {1, 2, 4};
  float best = 1e30f;
  int best_tile = 1;
  int rc = MPASG_OK;
  for (int t = 0; t < 3 && rc == MPASG_OK; ++t) {
    const int vt = tiles[t];
    const int nchunk = (L + vt - 1) / vt;
    const long long nth = (long long)m->nEdges * nchunk;
    float ms = 0.0f;
    for (int rep = 0; rep < 4; ++rep) {
      if (rep == 1) cudaEventRecord(a, s);
      if (vt == 1) {
        if (mixed) k_tend_u<float><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, FastDiv(L), p);
        else k_tend_u<double><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, FastDiv(L), p);
      } else if (vt == 2) {
        if (mixed) k_tend_u_chunk<float, 2><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
        else k_tend_u_chunk<double, 2><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
      } else {
        if (mixed) k_tend_u_chunk<float, 4><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
        else k_tend_u_chunk<double, 4><<<nblocks(nth), kBlock, 0, s>>>(*m, *f, FastDiv(nchunk), nchunk, p);
      }
      mpasg_count_launch();
      if (cudaGetLastError() != cudaSuccess) rc = MPASG_E_LAUNCH;
    }
    cudaEventRecord(b, s);
    if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) rc = MPASG_E_CUDA;
    ms /= 3.0f;
    if (times_ms) times_ms[t] = ms;
    if (rc == MPASG_OK && ms < best) {
      best = ms;
      best_tile = vt;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc == MPASG_OK) c->tile_tend_u = best_tile;
  return rc;
}
