// Shared pieces of the dynamics derivatives (reverse mode): the work-buffer layout and the
// internal entry points the stage VJPs and the step driver share.
#pragma once

#include "common.cuh"

// Work buffer of the dynamics VJPs: kAdjE edge arrays (E+1) x L, kAdjC cell arrays
// (C+1) x (L+1) and kAdjV vertex arrays (V+1) x L, each 256-byte aligned.
constexpr int kAdjE = 21, kAdjC = 16, kAdjV = 4;

struct AdjWork {
  double* e[kAdjE];
  double* c[kAdjC];
  double* v[kAdjV];
};

inline long long adj_round(long long n) { return (n + 31) / 32 * 32; }

inline long long adj_work_doubles(const mpasg_mesh* m) {
  const long long L = m->nVertLevels;
  return kAdjE * adj_round((m->nEdges + 1LL) * L) + kAdjC * adj_round((m->nCells + 1LL) * (L + 1)) +
         kAdjV * adj_round((m->nVertices + 1LL) * L);
}

inline AdjWork adj_work(const mpasg_mesh* m, double* w) {
  AdjWork a;
  const long long L = m->nVertLevels;
  const long long ne = adj_round((m->nEdges + 1LL) * L), nc = adj_round((m->nCells + 1LL) * (L + 1)),
                  nv = adj_round((m->nVertices + 1LL) * L);
  for (int i = 0; i < kAdjE; ++i, w += ne) a.e[i] = w;
  for (int i = 0; i < kAdjC; ++i, w += nc) a.c[i] = w;
  for (int i = 0; i < kAdjV; ++i, w += nv) a.v[i] = w;
  return a;
}

// Supported configurations of the dynamics derivatives (see mpasg.h): the arrays the
// vertical mixing reads (zgrid; the initial profiles of its perturbation form) must be there
inline bool adj_supported(const mpasg_mesh* m, const mpasg_config* c) {
  const bool vmix = c->v_mom_eddy_visc2 > 0.0 || c->v_theta_eddy_visc2 > 0.0;
  if (vmix && !m->zgrid) return false;
  if (vmix && c->mix_perturbation && (!m->u_init || !m->v_init || !m->angleEdge || !m->t_init)) return false;
  if (c->number_cam_damping_levels > m->nVertLevels || c->rayleigh_damp_u_levels > m->nVertLevels) return false;
  return c->moist_end < c->moist_start && m->nVertLevels >= 4;
}

// Damping options the derivatives differentiate, with the forward's expressions
// (kern_tend.cu TendScalars): CAM-style top-level kdiff floor base * (1 - (L - (k + 1)) /
// ncam) for the top ncam levels (dyn_tend.py:3434-3456), Rayleigh damping of u on the top
// ray_n levels with coefficient ((k + 1) - (L - ray_n)) * ray_coef (dyn_tend.py:2956-2990),
// vertical mixing coefficients of u / w and theta (0: off)
struct AdjDamping {
  double cam_base, ray_coef, v_mom, v_theta;
  int ncam, ray_n;
};
inline AdjDamping adj_damping(const mpasg_config* c) {
  AdjDamping d;
  d.ncam = (c->mpas_cam_coef > 0.0 && c->number_cam_damping_levels > 0) ? c->number_cam_damping_levels : 0;
  d.cam_base = 4.0 * 2.0833 * c->len_disp * c->mpas_cam_coef;
  d.ray_n = c->rayleigh_damp_u_levels > 0 ? c->rayleigh_damp_u_levels : 0;
  d.ray_coef = d.ray_n > 0 ? 1.0 / ((double)d.ray_n * (c->rayleigh_damp_u_timescale_days * 86400.0)) : 0.0;
  d.v_mom = c->v_mom_eddy_visc2 > 0.0 ? c->v_mom_eddy_visc2 : 0.0;
  d.v_theta = c->v_theta_eddy_visc2 > 0.0 ? c->v_theta_eddy_visc2 : 0.0;
  return d;
}
// the CAM floor of kdiff at level k (k >= L - ncam)
MPASG_D double adj_cam_floor(const AdjDamping& d, int k, int L) {
  return d.cam_base * (1.0 - (double)(L - (k + 1)) / (double)d.ncam);
}
// derivative factor of max(x, floor) with respect to x: 1, 0 or, on a tie, 1/2 (torch's
// maximum splits a tie evenly)
MPASG_D double adj_max_factor(double x, double floor) { return x > floor ? 1.0 : (x == floor ? 0.5 : 0.0); }
// Rayleigh damping coefficient of u at level k (0 below the damped layer)
MPASG_D double adj_ray_damp(const AdjDamping& d, int k, int L) {
  const int k0 = L - d.ray_n;
  return (d.ray_n <= 0 || k < k0) ? 0.0 : (((double)k + 1.0) - (double)k0) * d.ray_coef;
}

// 1 when cell c is the second cell (cellsOnEdge[e][1]) of edge e
MPASG_D int cell_side(const mpasg_mesh& m, int e, int c) { return m.cellsOnEdge[2 * e] == c ? 0 : 1; }
// the slot of edge e in edgesOnCell[c] (-1 if absent)
MPASG_D int cell_slot(const mpasg_mesh& m, int c, int e) {
  const int me = m.maxEdges, n = m.nEdgesOnCell[c];
  for (int j = 0; j < n; ++j)
    if (m.edgesOnCell[c * me + j] == e) return j;
  return -1;
}
// 1 when vertex v is the second vertex (verticesOnEdge[e][1]) of edge e
MPASG_D int vertex_side(const mpasg_mesh& m, int e, int v) { return m.verticesOnEdge[2 * e] == v ? 0 : 1; }

// partial derivatives of flux3 (common.cuh; dyn_tend.py:839,853) with respect to its
// arguments qm2, qm1, q0, qp1, ua; |ua| differentiated as sign(ua), 0 at 0 (torch's abs)
struct Flux3Grad {
  double qm2, qm1, q0, qp1, ua;
};
MPASG_D Flux3Grad flux3_grad(double qm2, double qm1, double q0, double qp1, double ua, double c3) {
  const double au = fabs(ua);
  const double s = ua > 0.0 ? 1.0 : (ua < 0.0 ? -1.0 : 0.0);
  Flux3Grad d;
  d.qm2 = (-ua - c3 * au) * kInv12;
  d.qm1 = (7.0 * ua + 3.0 * c3 * au) * kInv12;
  d.q0 = (7.0 * ua - 3.0 * c3 * au) * kInv12;
  d.qp1 = (-ua + c3 * au) * kInv12;
  d.ua = ((7.0 * (q0 + qm1) - (qp1 + qm2)) + c3 * s * ((qp1 - qm2) - 3.0 * (q0 - qm1))) * kInv12;
  return d;
}

// internal entry points shared by the stage VJPs and the step driver
int mpasgi_acoustic_parts(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int small_step, double dts,
                          cudaStream_t s, int part);
int mpasgi_recover_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                            int rk_step, double rk_dt, const AdjWork& w, cudaStream_t s);
int mpasgi_diag_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                         const mpasg_transpose* t, int rk_step, const AdjWork& w, cudaStream_t s);
int mpasgi_acoustic_vjp_core(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                             const mpasg_transpose* t, int small_step, double dts, const AdjWork& w,
                             cudaStream_t s);
int mpasgi_acoustic_vjp_fwd(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int small_step, double dts,
                            const AdjWork& w, cudaStream_t s);
int mpasgi_acoustic_vjp_rev(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                            const mpasg_transpose* t, int small_step, double dts, const double* rt_in,
                            const double* rwp_in, const AdjWork& w, cudaStream_t s);
int mpasgi_vimp_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                         double dts, const AdjWork& w, cudaStream_t s);
// tend_u's sign for the terrain slope terms: up (1 where tend_u >= 0) if given, else tu
int mpasgi_smlstep_vjp_core(const mpasg_mesh* m, const double* tu, const uint8_t* up, mpasg_fields* g,
                            cudaStream_t s);
// b[i] = x[i] >= 0
int mpasgi_nonneg_bytes(const double* x, uint8_t* b, long long n, cudaStream_t s);
int mpasgi_dyn_tend_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                             const mpasg_transpose* t, int rk_step, const AdjWork& w, cudaStream_t s);
int mpasgi_divdamp_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                            double dts, const AdjWork& w, cudaStream_t s);
int mpasgi_zero(double* p, long long n, cudaStream_t s);
// zero several arrays in one launch (up to kZeroSpans per launch; more take more launches)
constexpr int kZeroSpans = 16;
struct ZeroSpan {
  double* p;
  long long n;
};
int mpasgi_zero_many(const ZeroSpan* spans, int count, cudaStream_t s);

// internal entry points of the forward mode (tangents; kern_tan_*.cu, driver_tan.cu): d is the
// tangent state (mpasg_fields layout).  Stages that update their inputs in place run their
// forward on f inside (acoustic) or after the tangent (divergence damping, recovery); the
// others read the forward's outputs and run after it (vimp, tendencies, diagnostics, preparation).
int mpasgi_theta_edge_jvp(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, cudaStream_t s);
int mpasgi_vimp_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                         double dts, cudaStream_t s);
int mpasgi_acoustic_jvp_core(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                             int small_step, double dts, double* ubuf, cudaStream_t s);
int mpasgi_divdamp_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                            double dts, cudaStream_t s);
// the small-step perturbation on d, its selection from f's tend_u (after the forward one)
int mpasgi_smlstep_jvp_core(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, cudaStream_t s);
int mpasgi_recover_jvp_core(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, int rk_step, int ns,
                            double rk_dt, cudaStream_t s);
int mpasgi_prepare_jvp_core(const mpasg_mesh* m, const mpasg_fields* f, mpasg_fields* d, const double* dth,
                            const double* drho, cudaStream_t s);
int mpasgi_dyn_tend_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                             int rk_step, cudaStream_t s);
int mpasgi_diag_jvp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                         int rk_step, cudaStream_t s);
