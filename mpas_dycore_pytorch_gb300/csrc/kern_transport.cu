// Flux-form scalar transport: explicit RK stages (mpas_pytorch/dynamics/advance_scalars.py:1272,
// composition :861, Pattern-C edge values dynamics/pattern_c.py:234-305) and the monotone
// flux-corrected final stage (dynamics/advance_scalars_mono.py:3332, tile :1476, neighbour
// bounds autodiff/soft_limiter.py:72).  Scalar fields are (C+1, L, S), edge fluxes (E+1, L, S).
#include <mutex>

#include "common.cuh"

namespace {

// sum_m (adv_coefs + sign(uh) adv_coefs_3rd) q[advCell_m]  for every scalar
__global__ void k_pattern_c(mpasg_mesh m, FastDiv fl, int S, const double* __restrict__ uh,
                            const double* __restrict__ q, double* __restrict__ out, int times_uh) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int na = m.nAdvMax;
  const int nadv = m.nAdvCellsForEdge[e];
  const double u = uh[i];
  const double* cf = (u >= 0.0 ? m.adv_coefs_p : m.adv_coefs_m) + (size_t)e * na;
  double acc[8];
  for (int s = 0; s < S; ++s) acc[s] = 0.0;
  for (int a = 0; a < nadv; ++a) {
    int cell = m.advCellsForEdge[e * na + a];
    double w = cf[a];
    const double* qc = q + ((size_t)cell * L + k) * S;
    for (int s = 0; s < S; ++s) {
      double t = w * qc[s];
      acc[s] = (a == 0) ? t : acc[s] + t;
    }
  }
  for (int s = 0; s < S; ++s) out[(size_t)i * S + s] = times_uh ? u * acc[s] : acc[s];
}

MPASG_D double wdtn_at(const double* sn, const double* ww, int kk, int L, int S, int s, const double* fnm,
                       const double* fnp, double coef3) {
  if (kk <= 0 || kk >= L) return 0.0;
  if (kk == 1 || kk == L - 1) return ww[kk] * (fnm[kk] * sn[kk * S + s] + fnp[kk] * sn[(kk - 1) * S + s]);
  return flux3(sn[(kk - 2) * S + s], sn[(kk - 1) * S + s], sn[kk * S + s], sn[(kk + 1) * S + s], ww[kk], coef3);
}

// explicit stage update for all scalars at (cell, level)
__global__ void __launch_bounds__(kBlock) k_scalars_update(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S,
                                                           double dt, double w_old, double w_new, double coef3,
                                                           const double* __restrict__ s_old,
                                                           const double* __restrict__ s_new,
                                                           double* __restrict__ s_out) {
  extern __shared__ double s_wdtn[];  // [blockDim.x][S]: vertical flux at the interface below
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * L;
  uint32_t c = 0, k = 0;
  if (active) {
    c = fl.div(i);
    k = i - c * L;
    const double* sn0 = s_new + (size_t)c * L * S;
    const double* ww0 = f.wwAvg + (size_t)c * (L + 1);
    for (int s = 0; s < S; ++s) s_wdtn[threadIdx.x * S + s] = wdtn_at(sn0, ww0, k, L, S, s, m.fnm, m.fnp, coef3);
  }
  __syncthreads();
  if (!active) return;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double div[8];
  for (int s = 0; s < S; ++s) div[s] = 0.0;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double w = -m.edgesOnCell_sign[c * me + j] * f.ruAvg[(size_t)e * L + k];
    const double* hf = f.hflux + ((size_t)e * L + k) * S;
    for (int s = 0; s < S; ++s) {
      double t = w * hf[s];
      div[s] = (j == 0) ? t : div[s] + t;
    }
  }
  const double ia = m.invAreaCell[c];
  const double* sn = s_new + (size_t)c * L * S;
  const double* ww = f.wwAvg + (size_t)c * (L + 1);
  double rho_old = f.rho_zz_old_split[i];
  double rho_i = w_old * rho_old + w_new * f.rho_zz[i];
  double inv = 1.0 / rho_i;
  const bool next_in_block = threadIdx.x + 1 < blockDim.x;
  for (int s = 0; s < S; ++s) {
    double tend_col = div[s] * ia + 0.0;
    double lo = s_wdtn[threadIdx.x * S + s];
    double hi = (k + 1 >= (uint32_t)L) ? 0.0
                : next_in_block ? s_wdtn[(threadIdx.x + 1) * S + s]
                                : wdtn_at(sn, ww, k + 1, L, S, s, m.fnm, m.fnp, coef3);
    double vdiv = m.rdnw[k] * (hi - lo);
    s_out[(size_t)i * S + s] = (s_old[(size_t)i * S + s] * rho_old + dt * (tend_col - vdiv)) * inv;
  }
}

// ---------------------------------------------------------------- monotone stage
MPASG_D double mz(double x) { return x > 0.0 ? x : 0.0; }

// per (cell, level): rho_int, local+neighbour bounds, vertical upwind update,
// vertical parts of the limiter scale sums; stores the high-minus-upwind vertical flux
// at the interface below the level (wflux[c, k, s], k >= 1)
__global__ void __launch_bounds__(kBlock) k_mono_cells_a(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S,
                                                         double dt, double coef3,
                                                         const double* __restrict__ so_all,
                                                         const double* __restrict__ sn_all) {
  extern __shared__ double s_wm[];  // [blockDim.x][2 S]: high-minus-upwind flux and upwind flux below
  const int L = m.nVertLevels;
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
      double fup = 0.0, wm = 0.0;
      if (k >= 1) {
        double wk = ww0[k];
        fup = dt * (wk * (wk >= 0.0 ? so0[(k - 1) * S + s] : so0[k * S + s]));
        wm = dt * wdtn_at(sn0, ww0, k, L, S, s, m.fnm, m.fnp, coef3) - fup;
      }
      s_wm[threadIdx.x * 2 * S + s] = wm;
      s_wm[threadIdx.x * 2 * S + S + s] = fup;
    }
  }
  __syncthreads();
  if (!active) return;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  // density at the end of the stage
  double hdiv = 0.0;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double t = (f.ruAvg[(size_t)e * L + k] * (-m.edgesOnCell_sign[c * me + j] * m.dvEdge[e])) * ia;
    hdiv = (j == 0) ? t : hdiv + t;
  }
  const double* ww = f.wwAvg + (size_t)c * (L + 1);
  double rho_old = f.rho_zz_old_split[i];
  double rho_int = rho_old + dt * (hdiv - m.rdnw[k] * (ww[k + 1] - ww[k]));
  f.rho_int[i] = rho_int;
  const double* so = so_all + (size_t)c * L * S;
  const double* sn = sn_all + (size_t)c * L * S;
  const double rd = m.rdnw[k];
  for (int s = 0; s < S; ++s) {
    double smax, smin;
    if (k == 0) {
      smax = fmax(so[0 * S + s], so[1 * S + s]);
      smin = fmin(so[0 * S + s], so[1 * S + s]);
    } else if (k == (uint32_t)L - 1) {
      smax = fmax(so[k * S + s], so[(k - 1) * S + s]);
      smin = fmin(so[k * S + s], so[(k - 1) * S + s]);
    } else {
      smax = fmax(fmax(so[(k - 1) * S + s], so[k * S + s]), so[(k + 1) * S + s]);
      smin = fmin(fmin(so[(k - 1) * S + s], so[k * S + s]), so[(k + 1) * S + s]);
    }
    // neighbour extrema (first valid neighbour seeds the running bound)
    double nmax = 0.0, nmin = 0.0;
    bool seen = false;
    for (int j = 0; j < n; ++j) {
      int nb = m.cellsOnCell[c * me + j];
      if (nb >= m.nCells) continue;
      double val = so_all[((size_t)nb * L + k) * S + s];
      if (!seen) {
        nmax = val;
        nmin = val;
        seen = true;
      } else {
        nmax = fmax(nmax, val);
        nmin = fmin(nmin, val);
      }
    }
    if (seen) {
      smax = fmax(smax, nmax);
      smin = fmin(smin, nmin);
    }
    // vertical high-order and upwind fluxes at the interfaces below (k) and above (k+1)
    double fup_lo = 0.0, fup_hi = 0.0, wm_lo = 0.0, wm_hi = 0.0;
    if (k >= 1) {
      wm_lo = s_wm[threadIdx.x * 2 * S + s];
      fup_lo = s_wm[threadIdx.x * 2 * S + S + s];
      f.wflux[((size_t)c * (L + 1) + k) * S + s] = wm_lo;
    }
    if (k + 1 < (uint32_t)L) {
      if (threadIdx.x + 1 < blockDim.x) {
        wm_hi = s_wm[(threadIdx.x + 1) * 2 * S + s];
        fup_hi = s_wm[(threadIdx.x + 1) * 2 * S + S + s];
      } else {
        double wk = ww[k + 1];
        fup_hi = dt * (wk * (wk >= 0.0 ? so[k * S + s] : so[(k + 1) * S + s]));
        wm_hi = dt * wdtn_at(sn, ww, k + 1, L, S, s, m.fnm, m.fnp, coef3) - fup_hi;
      }
    }
    double rows = so[k * S + s] * rho_old;
    if (k + 1 < (uint32_t)L) rows = rows - fup_hi * rd;
    if (k >= 1) rows = rows + fup_lo * rd;
    // prev = interface below (0 at the surface), next = interface above (0 at the top)
    double prev = wm_lo, nxt = wm_hi;
    double sin_ = -rd * ((-mz(-nxt)) - mz(prev));
    double sout = -rd * (mz(nxt) - (-mz(-prev)));
    size_t o = (size_t)i * S + s;
    f.rows[o] = rows;
    f.scale_in[o] = sin_;
    f.scale_out[o] = sout;
    f.s_max[o] = smax;
    f.s_min[o] = smin;
  }
}

// per (edge, level): horizontal upwind flux and high-minus-upwind correction flux
__global__ void k_mono_edges_a(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S, double dt,
                               const double* __restrict__ so_all) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  double u = f.ruAvg[i];
  int up = u >= 0.0 ? c1 : c2;
  double dvdt = m.dvEdge[e] * dt;
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    double fup = dvdt * (u * so_all[((size_t)up * L + k) * S + s]);
    f.flux_up[o] = fup;
    f.flux_tmp[o] = dt * f.hflux[o] - fup;
  }
}

// per (cell, level): horizontal upwind update and scale sums, then the limiter factors
__global__ void k_mono_cells_b(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  const double eps = 1.0e-20;
  const double rint = f.rho_int[i];
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    double rows = f.rows[o], sin_ = f.scale_in[o], sout = f.scale_out[o];
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      double sgn_ = m.edgesOnCell_sign[c * me + j];
      double sw = sgn_ * ia;
      size_t oe = ((size_t)e * L + k) * S + s;
      rows = rows - f.flux_up[oe] * sw;
      double sf = sgn_ * f.flux_tmp[oe];
      sout = sout - mz(sf) * ia;
      sin_ = sin_ - (-mz(-sf)) * ia;
    }
    double a = (f.s_max[o] * rint - rows) / (sin_ + eps);
    double b = (f.s_min[o] * rint - rows) / (sout - eps);
    f.rows[o] = rows;
    f.scale_in[o] = fmin(fmax(a, 0.0), 1.0);
    f.scale_out[o] = fmin(fmax(b, 0.0), 1.0);
  }
}

// per (edge, level): limited horizontal flux (stored in hflux)
__global__ void k_mono_edges_b(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    size_t o1 = ((size_t)c1 * L + k) * S + s, o2 = ((size_t)c2 * L + k) * S + s;
    double ft = f.flux_tmp[o];
    double lim = ft >= 0.0 ? fmin(f.scale_out[o1], f.scale_in[o2]) : fmin(f.scale_in[o1], f.scale_out[o2]);
    f.hflux[o] = ft * lim;
  }
}

// per (cell, level): apply limited horizontal and vertical fluxes, positivity
__global__ void k_mono_cells_c(mpasg_mesh m, mpasg_fields f, FastDiv fl, int S, double* __restrict__ s_out) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const double ia = m.invAreaCell[c];
  const double rint = f.rho_int[i];
  const size_t oc = (size_t)c * L;
  for (int s = 0; s < S; ++s) {
    size_t o = (size_t)i * S + s;
    // limited vertical fluxes at the interfaces below (k) and above (k+1)
    double wl_lo = 0.0, wl_hi = 0.0;
    if (k >= 1) {
      double wm = f.wflux[((size_t)c * (L + 1) + k) * S + s];
      double lim = wm >= 0.0 ? fmin(f.scale_out[(oc + k - 1) * S + s], f.scale_in[(oc + k) * S + s])
                             : fmin(f.scale_out[(oc + k) * S + s], f.scale_in[(oc + k - 1) * S + s]);
      wl_lo = wm * lim;
    }
    if (k + 1 < (uint32_t)L) {
      double wm = f.wflux[((size_t)c * (L + 1) + k + 1) * S + s];
      double lim = wm >= 0.0 ? fmin(f.scale_out[(oc + k) * S + s], f.scale_in[(oc + k + 1) * S + s])
                             : fmin(f.scale_out[(oc + k + 1) * S + s], f.scale_in[(oc + k) * S + s]);
      wl_hi = wm * lim;
    }
    double rows = f.rows[o];
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      double sw = m.edgesOnCell_sign[c * me + j] * ia;
      rows = rows - f.hflux[((size_t)e * L + k) * S + s] * sw;
    }
    double st2 = (rows - m.rdnw[k] * (wl_hi - wl_lo)) / rint;
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

extern "C" int mpasg_advance_scalars(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                                     double dt_stage, void* stream) {
  if (!m || !c || !f || c->num_scalars < 1 || c->num_scalars > 8) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels, S = c->num_scalars;
  FastDiv fl(L);
  k_pattern_c<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, fl, S, f->ruAvg, f->scalars_a, f->hflux, 0);
  MPASG_LAUNCH_CHECK();
  double w_old, w_new;
  time_weights(1, rk_step, c->time_integration_order, &w_old, &w_new);
  k_scalars_update<<<nblocks((long long)m->nCells * L), kBlock, kBlock * S * sizeof(double), s>>>(
      *m, *f, fl, S, dt_stage, w_old, w_new, c->coef_3rd_order, f->scalars_init, f->scalars_a, f->scalars_b);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_advance_scalars_mono(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                          double dt_stage, void* stream) {
  if (!m || !c || !f || c->num_scalars < 1 || c->num_scalars > 8) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels, S = c->num_scalars;
  FastDiv fl(L);
  const long long nel = (long long)m->nEdges * L, ncl = (long long)m->nCells * L;
  k_pattern_c<<<nblocks(nel), kBlock, 0, s>>>(*m, fl, S, f->ruAvg, f->scalars_a, f->hflux, 1);
  MPASG_LAUNCH_CHECK();
  k_mono_cells_a<<<nblocks(ncl), kBlock, kBlock * 2 * S * sizeof(double), s>>>(*m, *f, fl, S, dt_stage, c->coef_3rd_order, f->scalars_init,
                                                  f->scalars_a);
  MPASG_LAUNCH_CHECK();
  k_mono_edges_a<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, S, dt_stage, f->scalars_init);
  MPASG_LAUNCH_CHECK();
  k_mono_cells_b<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, S);
  MPASG_LAUNCH_CHECK();
  k_mono_edges_b<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, fl, S);
  MPASG_LAUNCH_CHECK();
  k_mono_cells_c<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, fl, S, f->scalars_b);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// ---------------------------------------------------------------- library-owned scratch
// Edge values of mpasg_advance_scalars_static live here instead of in f->hflux.
static __device__ __align__(256) double g_static_hflux[MPASG_STATIC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
double* g_static_ptr[kMaxDevices] = {};

// Device address of g_static_hflux on the current device, looked up once per device.
int static_scratch(double** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MPASG_E_CUDA;
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_hflux) != cudaSuccess || !p) return MPASG_E_CUDA;
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
  mpasg_fields g = *f;  // the caller's struct is left as it is
  g.hflux = scratch;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels, S = c->num_scalars;
  FastDiv fl(L);
  k_pattern_c<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, fl, S, g.ruAvg, g.scalars_a, g.hflux, 0);
  MPASG_LAUNCH_CHECK();
  double w_old, w_new;
  time_weights(1, rk_step, c->time_integration_order, &w_old, &w_new);
  k_scalars_update<<<nblocks((long long)m->nCells * L), kBlock, kBlock * S * sizeof(double), s>>>(
      *m, g, fl, S, dt_stage, w_old, w_new, c->coef_3rd_order, g.scalars_init, g.scalars_a, g.scalars_b);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
