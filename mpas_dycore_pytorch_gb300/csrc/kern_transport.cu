// Flux-form scalar transport: explicit RK stages (mpas_pytorch/dynamics/advance_scalars.py:1272,
// composition :861, Pattern-C edge values dynamics/pattern_c.py:234-305) and the monotone
// flux-corrected final stage (dynamics/advance_scalars_mono.py:3332, tile :1476, neighbour
// bounds autodiff/soft_limiter.py:72).  Scalar fields are (C+1, L, S), edge fluxes (E+1, L, S).
#include <mutex>

#include "common.cuh"

namespace {

// Every transport kernel is a template on the stencil arithmetic type T (common.cuh).
// In the mixed form the edge values, flux divergences, bounds and limiter factors are
// float32; the density weighting and the stage update of each scalar are float64.

// sum_m (adv_coefs + sign(uh) adv_coefs_3rd) q[advCell_m]  for every scalar
template <typename T>
__global__ void k_pattern_c(mpasg_mesh m, FastDiv fl, int S, const double* __restrict__ uh,
                            const double* __restrict__ q, double* __restrict__ out, int times_uh) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int na = m.nAdvMax;
  const int nadv = m.nAdvCellsForEdge[e];
  const T u = cv<T>(uh[i]);
  const double* cf = (u >= T(0) ? m.adv_coefs_p : m.adv_coefs_m) + (size_t)e * na;
  T acc[8];
  for (int s = 0; s < S; ++s) acc[s] = T(0);
  for (int a = 0; a < nadv; ++a) {
    int cell = m.advCellsForEdge[e * na + a];
    T w = cv<T>(cf[a]);
    const double* qc = q + ((size_t)cell * L + k) * S;
    for (int s = 0; s < S; ++s) {
      T t = w * cv<T>(qc[s]);
      acc[s] = (a == 0) ? t : acc[s] + t;
    }
  }
  for (int s = 0; s < S; ++s) out[(size_t)i * S + s] = f64(times_uh ? u * acc[s] : acc[s]);
}

template <typename T>
MPASG_D T wdtn_at(const double* sn, const double* ww, int kk, int L, int S, int s, const double* fnm,
                  const double* fnp, T coef3) {
  if (kk <= 0 || kk >= L) return T(0);
  if (kk == 1 || kk == L - 1)
    return cv<T>(ww[kk]) * (cv<T>(fnm[kk]) * cv<T>(sn[kk * S + s]) + cv<T>(fnp[kk]) * cv<T>(sn[(kk - 1) * S + s]));
  return flux3<T>(cv<T>(sn[(kk - 2) * S + s]), cv<T>(sn[(kk - 1) * S + s]), cv<T>(sn[kk * S + s]),
                  cv<T>(sn[(kk + 1) * S + s]), cv<T>(ww[kk]), coef3);
}

// explicit stage update for all scalars at (cell, level)
template <typename T>
__global__ void __launch_bounds__(kBlock) k_scalars_update(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S,
                                                           double dt, double w_old, double w_new, double coef3,
                                                           const double* __restrict__ s_old,
                                                           const double* __restrict__ s_new,
                                                           double* __restrict__ s_out) {
  extern __shared__ __align__(8) unsigned char s_raw[];
  T* s_wdtn = reinterpret_cast<T*>(s_raw);  // [blockDim.x][S]: vertical flux at the interface below
  const int L = m.nVertLevels;
  const T c3 = cv<T>(coef3);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * L;
  uint32_t c = 0, k = 0;
  if (active) {
    c = fl.div(i);
    k = i - c * L;
    const double* sn0 = s_new + (size_t)c * L * S;
    const double* ww0 = f.wwAvg + (size_t)c * (L + 1);
    for (int s = 0; s < S; ++s) s_wdtn[threadIdx.x * S + s] = wdtn_at<T>(sn0, ww0, k, L, S, s, m.fnm, m.fnp, c3);
  }
  __syncthreads();
  if (!active) return;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  T div[8];
  for (int s = 0; s < S; ++s) div[s] = T(0);
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    T w = -cv<T>(m.edgesOnCell_sign[c * me + j]) * cv<T>(f.ruAvg[(size_t)e * L + k]);
    const double* hf = f.hflux + ((size_t)e * L + k) * S;
    for (int s = 0; s < S; ++s) {
      T t = w * cv<T>(hf[s]);
      div[s] = (j == 0) ? t : div[s] + t;
    }
  }
  const T ia = cv<T>(m.invAreaCell[c]);
  const double* sn = s_new + (size_t)c * L * S;
  const double* ww = f.wwAvg + (size_t)c * (L + 1);
  double rho_old = f.rho_zz_old_split[i];
  double rho_i = w_old * rho_old + w_new * f.rho_zz[i];
  double inv = fdiv<T>(1.0, rho_i);
  const bool next_in_block = threadIdx.x + 1 < blockDim.x;
  const T rd = cv<T>(m.rdnw[k]);
  const T dt_t = cv<T>(dt);
  for (int s = 0; s < S; ++s) {
    T tend_col = div[s] * ia + T(0);
    T lo = s_wdtn[threadIdx.x * S + s];
    T hi = (k + 1 >= (uint32_t)L) ? T(0)
           : next_in_block ? s_wdtn[(threadIdx.x + 1) * S + s]
                           : wdtn_at<T>(sn, ww, k + 1, L, S, s, m.fnm, m.fnp, c3);
    T vdiv = rd * (hi - lo);
    s_out[(size_t)i * S + s] = (s_old[(size_t)i * S + s] * rho_old + f64(dt_t * (tend_col - vdiv))) * inv;
  }
}

// ---------------------------------------------------------------- monotone stage
template <typename T>
MPASG_D T mz(T x) { return x > T(0) ? x : T(0); }

// per (cell, level): rho_int, local+neighbour bounds, vertical upwind update,
// vertical parts of the limiter scale sums; stores the high-minus-upwind vertical flux
// at the interface below the level (wflux[c, k, s], k >= 1)
template <typename T>
__global__ void __launch_bounds__(kBlock) k_mono_cells_a(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S,
                                                         double dt, double coef3,
                                                         const double* __restrict__ so_all,
                                                         const double* __restrict__ sn_all) {
  extern __shared__ __align__(8) unsigned char s_raw[];
  T* s_wm = reinterpret_cast<T*>(s_raw);  // [blockDim.x][2 S]: high-minus-upwind and upwind flux below
  const int L = m.nVertLevels;
  const T c3 = cv<T>(coef3);
  const T dt_t = cv<T>(dt);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * L;
  uint32_t c = 0, k = 0;
  if (active) {
    c = fl.div(i);
    k = i - c * L;
    const double* so0 = so_all + (size_t)c * L * S;
    const double* sn0 = sn_all + (size_t)c * L * S;
    const double* ww0 = f.wwAvg + (size_t)c * (L + 1);
    for (int s = 0; s < S; ++s) {
      T fup = T(0), wm = T(0);
      if (k >= 1) {
        T wk = cv<T>(ww0[k]);
        fup = dt_t * (wk * cv<T>(wk >= T(0) ? so0[(k - 1) * S + s] : so0[k * S + s]));
        wm = dt_t * wdtn_at<T>(sn0, ww0, k, L, S, s, m.fnm, m.fnp, c3) - fup;
      }
      s_wm[threadIdx.x * 2 * S + s] = wm;
      s_wm[threadIdx.x * 2 * S + S + s] = fup;
    }
  }
  __syncthreads();
  if (!active) return;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T ia = cv<T>(m.invAreaCell[c]);
  // density at the end of the stage
  T hdiv = T(0);
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    T t = (cv<T>(f.ruAvg[(size_t)e * L + k]) * (-cv<T>(m.edgesOnCell_sign[c * me + j]) * cv<T>(m.dvEdge[e]))) * ia;
    hdiv = (j == 0) ? t : hdiv + t;
  }
  const double* ww = f.wwAvg + (size_t)c * (L + 1);
  double rho_old = f.rho_zz_old_split[i];
  const T rd = cv<T>(m.rdnw[k]);
  double rho_int = rho_old + f64(dt_t * (hdiv - rd * (cv<T>(ww[k + 1]) - cv<T>(ww[k]))));
  f.rho_int[i] = rho_int;
  const double* so = so_all + (size_t)c * L * S;
  const double* sn = sn_all + (size_t)c * L * S;
  for (int s = 0; s < S; ++s) {
    T smax, smin;
    if (k == 0) {
      smax = vmax(cv<T>(so[0 * S + s]), cv<T>(so[1 * S + s]));
      smin = vmin(cv<T>(so[0 * S + s]), cv<T>(so[1 * S + s]));
    } else if (k == (uint32_t)L - 1) {
      smax = vmax(cv<T>(so[k * S + s]), cv<T>(so[(k - 1) * S + s]));
      smin = vmin(cv<T>(so[k * S + s]), cv<T>(so[(k - 1) * S + s]));
    } else {
      smax = vmax(vmax(cv<T>(so[(k - 1) * S + s]), cv<T>(so[k * S + s])), cv<T>(so[(k + 1) * S + s]));
      smin = vmin(vmin(cv<T>(so[(k - 1) * S + s]), cv<T>(so[k * S + s])), cv<T>(so[(k + 1) * S + s]));
    }
    // neighbour extrema (first valid neighbour seeds the running bound)
    T nmax = T(0), nmin = T(0);
    bool seen = false;
    for (int j = 0; j < n; ++j) {
      int nb = m.cellsOnCell[c * me + j];
      if (nb >= m.nCells) continue;
      T val = cv<T>(so_all[((size_t)nb * L + k) * S + s]);
      if (!seen) {
        nmax = val;
        nmin = val;
        seen = true;
      } else {
        nmax = vmax(nmax, val);
        nmin = vmin(nmin, val);
      }
    }
    if (seen) {
      smax = vmax(smax, nmax);
      smin = vmin(smin, nmin);
    }
    // vertical high-order and upwind fluxes at the interfaces below (k) and above (k+1)
    T fup_lo = T(0), fup_hi = T(0), wm_lo = T(0), wm_hi = T(0);
    if (k >= 1) {
      wm_lo = s_wm[threadIdx.x * 2 * S + s];
      fup_lo = s_wm[threadIdx.x * 2 * S + S + s];
      f.wflux[((size_t)c * (L + 1) + k) * S + s] = f64(wm_lo);
    }
    if (k + 1 < (uint32_t)L) {
      if (threadIdx.x + 1 < blockDim.x) {
        wm_hi = s_wm[(threadIdx.x + 1) * 2 * S + s];
        fup_hi = s_wm[(threadIdx.x + 1) * 2 * S + S + s];
      } else {
        T wk = cv<T>(ww[k + 1]);
        fup_hi = dt_t * (wk * cv<T>(wk >= T(0) ? so[k * S + s] : so[(k + 1) * S + s]));
        wm_hi = dt_t * wdtn_at<T>(sn, ww, k + 1, L, S, s, m.fnm, m.fnp, c3) - fup_hi;
      }
    }
    double rows = so[k * S + s] * rho_old;
    if (k + 1 < (uint32_t)L) rows = rows - f64(fup_hi * rd);
    if (k >= 1) rows = rows + f64(fup_lo * rd);
    // prev = interface below (0 at the surface), next = interface above (0 at the top)
    T prev = wm_lo, nxt = wm_hi;
    T sin_ = -rd * ((-mz(-nxt)) - mz(prev));
    T sout = -rd * (mz(nxt) - (-mz(-prev)));
    size_t o = (size_t)i * S + s;
    f.rows[o] = rows;
    f.scale_in[o] = f64(sin_);
    f.scale_out[o] = f64(sout);
    f.s_max[o] = f64(smax);
    f.s_min[o] = f64(smin);
  }
}

// per (edge, level): horizontal upwind flux and high-minus-upwind correction flux
template <typename T>
__global__ void k_mono_edges_a(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S, double dt,
                               const double* __restrict__ so_all) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const T u = cv<T>(f.ruAvg[i]);
  int up = u >= T(0) ? c1 : c2;
  const T dt_t = cv<T>(dt);
  const T dvdt = cv<T>(m.dvEdge[e]) * dt_t;
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    T fup = dvdt * (u * cv<T>(so_all[((size_t)up * L + k) * S + s]));
    f.flux_up[o] = f64(fup);
    f.flux_tmp[o] = f64(dt_t * cv<T>(f.hflux[o]) - fup);
  }
}

// per (cell, level): horizontal upwind update and scale sums, then the limiter factors
template <typename T>
__global__ void k_mono_cells_b(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T ia = cv<T>(m.invAreaCell[c]);
  const T eps = T(1.0e-20);
  const double rint = f.rho_int[i];
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    double rows = f.rows[o];
    T sin_ = cv<T>(f.scale_in[o]), sout = cv<T>(f.scale_out[o]);
    T hsum = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      T sgn_ = cv<T>(m.edgesOnCell_sign[c * me + j]);
      T sw = sgn_ * ia;
      size_t oe = ((size_t)e * L + k) * S + s;
      if (sizeof(T) == sizeof(double))
        rows = rows - f64(cv<T>(f.flux_up[oe]) * sw);  // float64: the reference's running sum
      else
        hsum = hsum - cv<T>(f.flux_up[oe]) * sw;
      T sf = sgn_ * cv<T>(f.flux_tmp[oe]);
      sout = sout - mz(sf) * ia;
      sin_ = sin_ - (-mz(-sf)) * ia;
    }
    if (sizeof(T) != sizeof(double)) rows = rows + f64(hsum);
    const T rows_t = cv<T>(rows), rint_t = cv<T>(rint);
    T a = (cv<T>(f.s_max[o]) * rint_t - rows_t) / (sin_ + eps);
    T b = (cv<T>(f.s_min[o]) * rint_t - rows_t) / (sout - eps);
    f.rows[o] = rows;
    f.scale_in[o] = f64(vmin(vmax(a, T(0)), T(1)));
    f.scale_out[o] = f64(vmin(vmax(b, T(0)), T(1)));
  }
}

// per (edge, level): limited horizontal flux (stored in hflux)
template <typename T>
__global__ void k_mono_edges_b(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    size_t o1 = ((size_t)c1 * L + k) * S + s, o2 = ((size_t)c2 * L + k) * S + s;
    T ft = cv<T>(f.flux_tmp[o]);
    T lim = ft >= T(0) ? vmin(cv<T>(f.scale_out[o1]), cv<T>(f.scale_in[o2]))
                       : vmin(cv<T>(f.scale_in[o1]), cv<T>(f.scale_out[o2]));
    f.hflux[o] = f64(ft * lim);
  }
}

// per (cell, level): apply limited horizontal and vertical fluxes, positivity
template <typename T>
__global__ void k_mono_cells_c(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S, double* __restrict__ s_out) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T ia = cv<T>(m.invAreaCell[c]);
  const double rint = f.rho_int[i];
  const double inv_rint = fdiv<T>(1.0, rint);  // one reciprocal for every scalar of the cell-level
  const size_t oc = (size_t)c * L;
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    // limited vertical fluxes at the interfaces below (k) and above (k+1)
    T wl_lo = T(0), wl_hi = T(0);
    if (k >= 1) {
      T wm = cv<T>(f.wflux[((size_t)c * (L + 1) + k) * S + s]);
      T lim = wm >= T(0) ? vmin(cv<T>(f.scale_out[(oc + k - 1) * S + s]), cv<T>(f.scale_in[(oc + k) * S + s]))
                         : vmin(cv<T>(f.scale_out[(oc + k) * S + s]), cv<T>(f.scale_in[(oc + k - 1) * S + s]));
      wl_lo = wm * lim;
    }
    if (k + 1 < (uint32_t)L) {
      T wm = cv<T>(f.wflux[((size_t)c * (L + 1) + k + 1) * S + s]);
      T lim = wm >= T(0) ? vmin(cv<T>(f.scale_out[(oc + k) * S + s]), cv<T>(f.scale_in[(oc + k + 1) * S + s]))
                         : vmin(cv<T>(f.scale_out[(oc + k + 1) * S + s]), cv<T>(f.scale_in[(oc + k) * S + s]));
      wl_hi = wm * lim;
    }
    double rows = f.rows[o];
    T hsum = T(0);
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      T sw = cv<T>(m.edgesOnCell_sign[c * me + j]) * ia;
      if (sizeof(T) == sizeof(double))
        rows = rows - f64(cv<T>(f.hflux[((size_t)e * L + k) * S + s]) * sw);
      else
        hsum = hsum - cv<T>(f.hflux[((size_t)e * L + k) * S + s]) * sw;
    }
    if (sizeof(T) != sizeof(double)) rows = rows + f64(hsum);
    double st2 = (rows - f64(cv<T>(m.rdnw[k]) * (wl_hi - wl_lo))) * inv_rint;
    s_out[o] = st2 > 0.0 ? st2 : 0.0;
  }
}

}  // namespace

static void time_weights(int advance_density, int rk_step, int order, double* w_old, double* w_new) {
  double wn;
  if (advance_density == 0) wn = 1.0;
  else if (rk_step == 1 && order == 3) wn = 1.0 / 3.0;
  else if ((rk_step == 1 && order == 2) || rk_step == 2) wn = 1.0 / 2.0;
  else wn = 1.0;
  *w_new = wn;
  *w_old = 1.0 - wn;
}

namespace {

// One explicit RK transport stage with the edge values in `hflux` (f->hflux or the
// library-owned scratch): scalars_init, scalars_a -> scalars_b.
template <typename T>
int launch_scalars(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, double* hflux, int rk_step,
                   double dt_stage, cudaStream_t s) {
  const int L = m->nVertLevels, S = c->num_scalars;
  FastDiv fl(L);
  mpasg_fields g = *f;
  g.hflux = hflux;
  k_pattern_c<T><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, fl, S, g.ruAvg, g.scalars_a, hflux, 0);
  MPASG_LAUNCH_CHECK();
  // density weights: advanced with the stage in the split transport loop; the stage's
  // new density in the coupled mode (one dynamics substep, time_integration.py:7930-8200)
  double w_old, w_new;
  time_weights(c->dynamics_split_steps > 1 ? 1 : 0, rk_step, c->time_integration_order, &w_old, &w_new);
  k_scalars_update<T><<<nblocks((long long)m->nCells * L), kBlock, kBlock * S * sizeof(T), s>>>(
      *m, g, fl, S, dt_stage, w_old, w_new, c->coef_3rd_order, g.scalars_init, g.scalars_a, g.scalars_b);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

template <typename T>
int launch_scalars_mono(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, double dt_stage,
                        cudaStream_t s) {
  const int L = m->nVertLevels, S = c->num_scalars;
  FastDiv fl(L);
  const long long nel = (long long)m->nEdges * L, ncl = (long long)m->nCells * L;
  k_pattern_c<T><<<nblocks(nel), kBlock, 0, s>>>(*m, fl, S, f->ruAvg, f->scalars_a, f->hflux, 1);
  MPASG_LAUNCH_CHECK();
  k_mono_cells_a<T><<<nblocks(ncl), kBlock, kBlock * 2 * S * sizeof(T), s>>>(*m, *f, fl, S, dt_stage,
                                                                          c->coef_3rd_order, f->scalars_init,
                                                                          f->scalars_a);
  MPASG_LAUNCH_CHECK();
  k_mono_edges_a<T><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, S, dt_stage, f->scalars_init);
  MPASG_LAUNCH_CHECK();
  k_mono_cells_b<T><<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, S);
  MPASG_LAUNCH_CHECK();
  k_mono_edges_b<T><<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, S);
  MPASG_LAUNCH_CHECK();
  k_mono_cells_c<T><<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, S, f->scalars_b);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

}  // namespace

extern "C" int mpasg_advance_scalars(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                                     double dt_stage, void* stream) {
  if (!m || !c || !f || c->num_scalars < 1 || c->num_scalars > 8) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (c->precision == MPASG_PRECISION_MIXED) return launch_scalars<float>(m, c, f, f->hflux, rk_step, dt_stage, s);
  return launch_scalars<double>(m, c, f, f->hflux, rk_step, dt_stage, s);
}

extern "C" int mpasg_advance_scalars_mono(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                          double dt_stage, void* stream) {
  if (!m || !c || !f || c->num_scalars < 1 || c->num_scalars > 8) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (c->precision == MPASG_PRECISION_MIXED) return launch_scalars_mono<float>(m, c, f, dt_stage, s);
  return launch_scalars_mono<double>(m, c, f, dt_stage, s);
}

// ---------------------------------------------------------------- library-owned scratch
// Edge values of mpasg_advance_scalars_static live here instead of in f->hflux.
static __device__ __align__(256) double g_static_hflux[MPASG_STATIC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
double* g_static_ptr[kMaxDevices] = {};

// Device address of g_static_hflux on the current device, looked up once per device.
// The cached address belongs to the device's primary context: it stays valid for the life
// of the process unless that context is destroyed (cudaDeviceReset), after which a caller
// must not use this entry point on that device again.  A failed lookup clears CUDA's
// sticky last-error state, so it is not reported again by a later, unrelated launch check.
int static_scratch(double** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return MPASG_E_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_hflux) != cudaSuccess || !p) {
      cudaGetLastError();
      return MPASG_E_CUDA;
    }
    g_static_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_static_ptr[dev];
  return MPASG_OK;
}
}  // namespace

extern "C" int mpasg_advance_scalars_static(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                            int rk_step, double dt_stage, void* stream) {
  if (!m || !c || !f || c->num_scalars < 1 || c->num_scalars > 8) return MPASG_E_ARG;
  if (m->nEdges < 0 || m->nCells < 0 || m->nVertLevels < 1) return MPASG_E_ARG;
  const long long need = (long long)m->nEdges * m->nVertLevels * c->num_scalars;
  if (need > MPASG_STATIC_SCRATCH_DOUBLES) return MPASG_E_SCRATCH;
  double* scratch = nullptr;
  const int rc = static_scratch(&scratch);
  if (rc != MPASG_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;  // the caller's struct is left as it is
  if (c->precision == MPASG_PRECISION_MIXED) return launch_scalars<float>(m, c, f, scratch, rk_step, dt_stage, s);
  return launch_scalars<double>(m, c, f, scratch, rk_step, dt_stage, s);
}
