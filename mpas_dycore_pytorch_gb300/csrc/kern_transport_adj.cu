// Adjoint (vector-Jacobian product) of one large step's split scalar transport with
// explicit stages (mpas_pytorch/dynamics/advance_scalars.py:1272 composed as in
// time_integration.py:3954-4700): the step maps the scalars at its start linearly to the
// scalars at its end, given the step's averaged mass fluxes and densities, so the
// adjoint is exact.  Each explicit stage is
//
//   s_out = (s_old rho_old + dt_k (H(s_in) - V(s_in))) / rho_k,
//   rho_k = w_old rho_old + w_new rho_new,
//   H(x)_c = invArea_c sum_j (-sign_cj uh_e) sum_m coef(e, m, sign uh_e) x[advCell(e, m)],
//   V(x)_k = rdnw_k (wdtn_{k+1} - wdtn_k), wdtn from flux3 (2 <= k <= L-2) or the
//            second-order interpolation (k = 1, L-1) of x with the fixed wwAvg,
//
// with (s_old, s_in) = (s0, s0), (s0, out1), (s0, out2) for the three stages.  The
// transposed horizontal operator is a gather on both sides: edges collect the cotangents
// of their two cells (k_tadj_edges), then every cell collects its (edge, slot) pairs of
// the advection stencil from a transposed adjacency list built on the host
// (k_tadj_cells_h); no atomics, so the result is deterministic.  The vertical operator is
// column-local (k_tadj_cells_v).
#include "common.cuh"

namespace {

// z = dt g / rho_k: the cotangent of (H - V) at (cell, level, scalar)
MPASG_D double tadj_z(const double* g, const double* rho_old, const double* rho_new, double dt, double w_old,
                      double w_new, size_t cl, int S, int s) {
  const double rk = w_old * rho_old[cl] + w_new * rho_new[cl];
  return dt * g[cl * S + s] / rk;
}

// vertical part of s_in's cotangent and the s_old cotangent (accumulated), per (cell, level)
__global__ void k_tadj_cells_v(mpasg_mesh m, FastDiv fl, int S, double dt, double w_old, double w_new,
                               double coef3, const double* __restrict__ ww, const double* __restrict__ rho_old,
                               const double* __restrict__ rho_new, const double* __restrict__ g,
                               double* __restrict__ gold, double* __restrict__ sbar) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const size_t o = (size_t)c * L;
  const double* w = ww + (size_t)c * (L + 1);
  const double rk = w_old * rho_old[i] + w_new * rho_new[i];
  for (int s = 0; s < S; ++s) {
    gold[(size_t)i * S + s] += g[(size_t)i * S + s] / rk * rho_old[i];
    double acc = 0.0;
    // interfaces kk whose flux reads level k: kk = k - 1 .. k + 2
    for (int kk = (int)k - 1; kk <= (int)k + 2; ++kk) {
      if (kk < 1 || kk > L - 1) continue;
      // cotangent of wdtn_kk (1 <= kk <= L-1): vdiv_{kk-1} = rdnw (wdtn_kk - ...) and
      // vdiv_kk = rdnw (... - wdtn_kk), and s_out carries -vdiv
      const double wb = -m.rdnw[kk - 1] * tadj_z(g, rho_old, rho_new, dt, w_old, w_new, o + kk - 1, S, s) +
                        m.rdnw[kk] * tadj_z(g, rho_old, rho_new, dt, w_old, w_new, o + kk, S, s);
      const double ua = w[kk];
      double cf = 0.0;
      if (kk == 1 || kk == L - 1) {
        if ((int)k == kk) cf = ua * m.fnm[kk];
        else if ((int)k == kk - 1) cf = ua * m.fnp[kk];
      } else {
        const double au = coef3 * fabs(ua);
        const int d = (int)k - kk;  // -2, -1, 0, +1
        if (d == -2) cf = (-ua - au) / 12.0;
        else if (d == -1) cf = (7.0 * ua + 3.0 * au) / 12.0;
        else if (d == 0) cf = (7.0 * ua - 3.0 * au) / 12.0;
        else if (d == 1) cf = (-ua + au) / 12.0;
      }
      acc += wb * cf;
    }
    sbar[(size_t)i * S + s] = acc;
  }
}

// edge cotangent of the horizontal edge values: uh_e sum_{two cells} (-sign invArea) z_c
__global__ void k_tadj_edges(mpasg_mesh m, FastDiv fl, int S, double dt, double w_old, double w_new,
                             const double* __restrict__ uh, const double* __restrict__ edge_cell_w,
                             const double* __restrict__ rho_old, const double* __restrict__ rho_new,
                             const double* __restrict__ g, double* __restrict__ hb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int c0 = m.cellsOnEdge[2 * e], c1 = m.cellsOnEdge[2 * e + 1];
  const double w0 = edge_cell_w[2 * e], w1 = edge_cell_w[2 * e + 1];
  const double u = uh[i];
  for (int s = 0; s < S; ++s) {
    double acc = 0.0;
    if (c0 < m.nCells) acc += w0 * tadj_z(g, rho_old, rho_new, dt, w_old, w_new, (size_t)c0 * L + k, S, s);
    if (c1 < m.nCells) acc += w1 * tadj_z(g, rho_old, rho_new, dt, w_old, w_new, (size_t)c1 * L + k, S, s);
    hb[(size_t)i * S + s] = u * acc;
  }
}

// horizontal part of s_in's cotangent: every (edge, slot) of the advection stencils that
// reads this cell, in the order of the transposed adjacency list
__global__ void k_tadj_cells_h(mpasg_mesh m, FastDiv fl, int S, const double* __restrict__ uh,
                               const int32_t* __restrict__ adj_ptr, const int32_t* __restrict__ adj_es,
                               const double* __restrict__ hb, double* __restrict__ sbar) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  uint32_t c = fl.div(i), k = i - c * L;
  const int na = m.nAdvMax;
  const int p0 = adj_ptr[c], p1 = adj_ptr[c + 1];
  double acc[8];
  for (int s = 0; s < S; ++s) acc[s] = 0.0;
  for (int p = p0; p < p1; ++p) {
    const int es = adj_es[p];
    const int e = es / na;
    const size_t ie = (size_t)e * L + k;
    const double cf = (uh[ie] >= 0.0 ? m.adv_coefs_p : m.adv_coefs_m)[es];
    for (int s = 0; s < S; ++s) acc[s] += cf * hb[ie * S + s];
  }
  for (int s = 0; s < S; ++s) sbar[(size_t)i * S + s] += acc[s];
}

__global__ void k_tadj_finish(long long n, const double* __restrict__ a, const double* __restrict__ b,
                              double* __restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}

}  // namespace

namespace {
// One explicit stage's adjoint: g (cotangent of the stage output) -> sbar (cotangent of
// the stage input, active rows) and gold += (cotangent of s_old); hb: edge scratch.
int tadj_stage(const mpasg_mesh* m, int S, double dt, double w_old, double w_new, double coef3, const double* ruavg,
               const double* wwavg, const double* rho_old, const double* rho_new, const int32_t* adj_ptr,
               const int32_t* adj_es, const double* edge_cell_w, const double* g, double* gold, double* sbar,
               double* hb, cudaStream_t s) {
  const int L = m->nVertLevels;
  FastDiv fl(L);
  const long long ncl = (long long)m->nCells * L, nel = (long long)m->nEdges * L;
  k_tadj_cells_v<<<nblocks(ncl), kBlock, 0, s>>>(*m, fl, S, dt, w_old, w_new, coef3, wwavg, rho_old, rho_new, g,
                                                 gold, sbar);
  MPASG_LAUNCH_CHECK();
  k_tadj_edges<<<nblocks(nel), kBlock, 0, s>>>(*m, fl, S, dt, w_old, w_new, ruavg, edge_cell_w, rho_old, rho_new, g,
                                               hb);
  MPASG_LAUNCH_CHECK();
  k_tadj_cells_h<<<nblocks(ncl), kBlock, 0, s>>>(*m, fl, S, ruavg, adj_ptr, adj_es, hb, sbar);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

bool tadj_supported(const mpasg_config* c) {
  return c->num_scalars >= 1 && c->num_scalars <= 8 && !c->monotonic && !c->scalar_advection_off;
}
}  // namespace

extern "C" int mpasg_transport_vjp(const mpasg_mesh* m, const mpasg_config* c, const double* ruavg,
                                   const double* wwavg, const double* rho_old, const double* rho_new,
                                   const int32_t* adj_ptr, const int32_t* adj_es, const double* edge_cell_w,
                                   const double* g_out, double* g_in, double* work, void* stream) {
  if (!m || !c || !ruavg || !wwavg || !rho_old || !rho_new || !adj_ptr || !adj_es || !edge_cell_w || !g_out ||
      !g_in || !work)
    return MPASG_E_ARG;
  if (!tadj_supported(c) || c->dynamics_split_steps < 2) return MPASG_E_ARG;
  const int S = c->num_scalars;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  // work: three cell cotangent buffers, then the edge cotangents ((E+1) L S)
  const long long ncs = (long long)(m->nCells + 1) * L * S;
  double* ga = work;
  double* gb = ga + ncs;
  double* gacc = gb + ncs;
  double* hb = gacc + ncs;
  if (cudaMemsetAsync(gacc, 0, ncs * sizeof(double), s) != cudaSuccess) return MPASG_E_CUDA;
  if (cudaMemsetAsync(ga, 0, ncs * sizeof(double), s) != cudaSuccess) return MPASG_E_CUDA;
  if (cudaMemsetAsync(gb, 0, ncs * sizeof(double), s) != cudaSuccess) return MPASG_E_CUDA;
  const double dt = c->dt;
  const double dts[3] = {c->time_integration_order == 2 ? dt / 2.0 : dt / 3.0, dt / 2.0, dt};
  const long long ncl = (long long)m->nCells * L;
  const double* g = g_out;
  double* outs[3] = {ga, gb, ga};  // stage 3 -> ga, stage 2 -> gb, stage 1 -> ga
  for (int rk = 3; rk >= 1; --rk) {
    double w_new;
    if (rk == 1 && c->time_integration_order == 3) w_new = 1.0 / 3.0;
    else if ((rk == 1 && c->time_integration_order == 2) || rk == 2) w_new = 1.0 / 2.0;
    else w_new = 1.0;
    double* sbar = outs[3 - rk];
    const int rc = tadj_stage(m, S, dts[rk - 1], 1.0 - w_new, w_new, c->coef_3rd_order, ruavg, wwavg, rho_old,
                              rho_new, adj_ptr, adj_es, edge_cell_w, g, gacc, sbar, hb, s);
    if (rc != MPASG_OK) return rc;
    g = sbar;  // the previous stage's output cotangent
  }
  // s_in of stage 1 is the step's start: its cotangent joins the s_old cotangents; the
  // padding row passes through the step unchanged (copied with the scalars)
  k_tadj_finish<<<nblocks(ncl * S), kBlock, 0, s>>>(ncl * S, gacc, ga, g_in);
  MPASG_LAUNCH_CHECK();
  if (cudaMemcpyAsync(g_in + ncl * S, g_out + ncl * S, (size_t)L * S * sizeof(double), cudaMemcpyDeviceToDevice,
                      s) != cudaSuccess)
    return MPASG_E_CUDA;
  return MPASG_OK;
}

extern "C" int mpasg_transport_vjp_stage(const mpasg_mesh* m, const mpasg_config* c, double dt_stage, double w_old,
                                         double w_new, const double* ruavg, const double* wwavg,
                                         const double* rho_old, const double* rho_new, const int32_t* adj_ptr,
                                         const int32_t* adj_es, const double* edge_cell_w, const double* g_out,
                                         double* g_sin, double* g_sold, double* work_edges, void* stream) {
  if (!m || !c || !ruavg || !wwavg || !rho_old || !rho_new || !adj_ptr || !adj_es || !edge_cell_w || !g_out ||
      !g_sin || !g_sold || !work_edges || g_sin == g_out)
    return MPASG_E_ARG;
  if (!tadj_supported(c)) return MPASG_E_ARG;
  return tadj_stage(m, c->num_scalars, dt_stage, w_old, w_new, c->coef_3rd_order, ruavg, wwavg, rho_old, rho_new,
                    adj_ptr, adj_es, edge_cell_w, g_out, g_sold, g_sin, work_edges, (cudaStream_t)stream);
}
