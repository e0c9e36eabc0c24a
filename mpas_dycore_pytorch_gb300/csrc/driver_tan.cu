// Forward mode of one large step (the tangent-linear model the reference gets from torch's
// forward-mode AD through atm_srk3, atmosphere_model.py:2041 _run_simulation_jvp): the step
// of the values f and, alongside, of the tangents d, stage by stage (kern_tan_*.cu).  The
// dynamics only: the dry dynamics does not read the scalars, so the transport, the split
// averages it reads and the reconstructed winds are left out.  The values advance through
// the same stage calls as the step itself.
#include "adj_common.cuh"

namespace {

#define CHECK_RC(x)                  \
  do {                               \
    int _rc = (x);                   \
    if (_rc != MPASG_OK) return _rc; \
  } while (0)

__global__ void k_fill_row_t(double* __restrict__ p, int n, double v) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = v;
}

int dcopy(double* dst, const double* src, long long n, cudaStream_t s) {
  if (cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return MPASG_E_CUDA;
  return MPASG_OK;
}

// the saves of a dynamics substep (atm_rk_integration_setup and the substep refresh) of one state
int saves(const mpasg_mesh* m, mpasg_fields* f, cudaStream_t s) {
  const long long L = m->nVertLevels, nc = m->nCells;
  const long long nel = (m->nEdges + 1LL) * L, ncw = (nc + 1) * (L + 1), ncl = (nc + 1) * L;
  k_fill_row_t<<<1, 128, 0, s>>>(f->theta_m + nc * L, (int)L, 0.0);
  MPASG_LAUNCH_CHECK();
  CHECK_RC(dcopy(f->ru_save, f->ru, nel, s));
  CHECK_RC(dcopy(f->rw_save, f->rw, ncw, s));
  CHECK_RC(dcopy(f->rtheta_p_save, f->rtheta_p, ncl, s));
  CHECK_RC(dcopy(f->rho_p_save, f->rho_p, ncl, s));
  CHECK_RC(dcopy(f->theta_m_save, f->theta_m, ncl, s));
  CHECK_RC(dcopy(f->rr_save, f->rho_p, ncl, s));
  return MPASG_OK;
}

int saves_both(const mpasg_mesh* m, mpasg_fields* f, mpasg_fields* d, cudaStream_t s) {
  CHECK_RC(saves(m, f, s));
  CHECK_RC(saves(m, d, s));
  CHECK_RC(mpasgi_theta_edge(m, f, false, s));
  return mpasgi_theta_edge_jvp(m, f, d, s);
}

bool jvp_args_ok(const mpasg_mesh* m, const mpasg_config* c) {
  return adj_supported(m, c) && c->precision == MPASG_PRECISION_FLOAT64 &&
         (c->time_integration_order == 2 || c->time_integration_order == 3) && c->number_of_sub_steps >= 1 &&
         c->dynamics_split_steps >= 1;
}

int step_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields f, mpasg_fields* d, double* ubuf,
             cudaStream_t s) {
  void* stream = (void*)s;
  const int split = c->dynamics_split_steps, order = c->time_integration_order, ns = c->number_of_sub_steps;
  const double dt_dyn = c->dt / split;
  double rk_ts[3], rk_sub[3];
  int nsub[3];
  if (order == 3) {
    rk_ts[0] = dt_dyn / 3.0; rk_ts[1] = dt_dyn / 2.0; rk_ts[2] = dt_dyn;
    rk_sub[0] = dt_dyn / 3.0; rk_sub[1] = dt_dyn / ns; rk_sub[2] = dt_dyn / ns;
    nsub[0] = 1; nsub[1] = ns / 2 > 1 ? ns / 2 : 1; nsub[2] = ns;
  } else {
    rk_ts[0] = dt_dyn / 2.0; rk_ts[1] = dt_dyn / 2.0; rk_ts[2] = dt_dyn;
    rk_sub[0] = rk_sub[1] = rk_sub[2] = dt_dyn / ns;
    nsub[0] = nsub[1] = ns / 2 > 1 ? ns / 2 : 1; nsub[2] = ns;
  }
  CHECK_RC(saves_both(m, &f, d, s));
  CHECK_RC(mpasg_moist_coefficients(m, c, &f, stream));  // dry: constants, no tangent
  for (int sub = 1; sub <= split; ++sub) {
    for (int rk = 1; rk <= 3; ++rk) {
      const double dts = rk_sub[rk - 1];
      if (rk == 1 || (rk == 2 && order == 3)) {
        CHECK_RC(mpasg_vert_imp_coefs(m, c, &f, dts, stream));
        CHECK_RC(mpasgi_vimp_jvp_core(m, c, &f, d, dts, s));
      }
      CHECK_RC(mpasgi_dyn_tend(m, c, &f, rk, s, true));
      CHECK_RC(mpasgi_dyn_tend_jvp_core(m, c, &f, d, rk, s));
      CHECK_RC(mpasg_smlstep_pert(m, c, &f, stream));
      CHECK_RC(mpasgi_smlstep_jvp_core(m, &f, d, s));
      for (int small = 1; small <= nsub[rk - 1]; ++small) {
        CHECK_RC(mpasgi_acoustic_jvp_core(m, c, &f, d, small, dts, ubuf, s));
        CHECK_RC(mpasgi_divdamp_jvp_core(m, c, &f, d, dts, s));
        CHECK_RC(mpasgi_divergence_damping(m, c, &f, dts, s, true));
      }
      CHECK_RC(mpasgi_recover_jvp_core(m, &f, d, rk, nsub[rk - 1], rk_ts[rk - 1], s));
      CHECK_RC(mpasg_recover_large_step(m, c, &f, rk, nsub[rk - 1], rk_ts[rk - 1], stream));
      CHECK_RC(mpasgi_solve_diagnostics(m, c, &f, rk, s, true));
      CHECK_RC(mpasgi_diag_jvp_core(m, c, &f, d, rk, s));
    }
    if (sub < split) CHECK_RC(saves_both(m, &f, d, s));
  }
  return MPASG_OK;
}

}  // namespace

// ================================================================= C ABI
extern "C" int mpasg_step_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                              double* work, void* stream) {
  if (!m || !c || !f || !d || !work || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  return step_jvp(m, c, *f, d, work, (cudaStream_t)stream);
}

extern "C" int mpasg_prepare_jvp(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                                 const double* d_theta, const double* d_rho, void* stream) {
  if (!m || !c || !f || !d || !adj_supported(m, c)) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  CHECK_RC(mpasgi_prepare_jvp_core(m, f, d, d_theta, d_rho, s));
  mpasg_config c64 = *c;  // the preparation's diagnostics: float64 with the full tangential wind
  c64.precision = MPASG_PRECISION_FLOAT64;
  return mpasgi_diag_jvp_core(m, &c64, f, d, 3, s);
}

extern "C" int mpasg_vimp_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                              double dts, void* stream) {
  if (!m || !c || !f || !d || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  CHECK_RC(mpasg_vert_imp_coefs(m, c, f, dts, stream));
  return mpasgi_vimp_jvp_core(m, c, f, d, dts, (cudaStream_t)stream);
}

extern "C" int mpasg_dyn_tend_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                                  int rk_step, void* stream) {
  if (!m || !c || !f || !d || rk_step < 1 || rk_step > 3 || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (rk_step > 1) {  // the edge mean of theta_m_save the rk 2 / 3 flux reads, and its tangent
    CHECK_RC(mpasgi_theta_edge(m, f, false, s));
    CHECK_RC(mpasgi_theta_edge_jvp(m, f, d, s));
  }
  CHECK_RC(mpasgi_dyn_tend(m, c, f, rk_step, s, false));
  return mpasgi_dyn_tend_jvp_core(m, c, f, d, rk_step, s);
}

extern "C" int mpasg_smlstep_jvp(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* d,
                                 void* stream) {
  if (!m || !c || !f || !d || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  return mpasgi_smlstep_jvp_core(m, f, d, (cudaStream_t)stream);
}

extern "C" int mpasg_acoustic_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                                  int small_step, double dts, double* work, void* stream) {
  if (!m || !c || !f || !d || !work || small_step < 1 || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  CHECK_RC(mpasgi_theta_edge(m, f, false, s));
  CHECK_RC(mpasgi_theta_edge_jvp(m, f, d, s));
  return mpasgi_acoustic_jvp_core(m, c, f, d, small_step, dts, work, s);
}

extern "C" int mpasg_divdamp_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                                 double dts, void* stream) {
  if (!m || !c || !f || !d || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  CHECK_RC(mpasgi_theta_edge(m, f, false, s));
  CHECK_RC(mpasgi_theta_edge_jvp(m, f, d, s));
  CHECK_RC(mpasgi_divdamp_jvp_core(m, c, f, d, dts, s));
  return mpasgi_divergence_damping(m, c, f, dts, s, true);
}

extern "C" int mpasg_recover_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                                 int rk_step, int ns, double rk_dt, void* stream) {
  if (!m || !c || !f || !d || ns < 1 || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  CHECK_RC(mpasgi_recover_jvp_core(m, f, d, rk_step, ns, rk_dt, (cudaStream_t)stream));
  return mpasg_recover_large_step(m, c, f, rk_step, ns, rk_dt, stream);
}

extern "C" int mpasg_diag_jvp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* d,
                              int rk_step, void* stream) {
  if (!m || !c || !f || !d || !jvp_args_ok(m, c)) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  CHECK_RC(mpasgi_solve_diagnostics(m, c, f, rk_step, s, false));
  return mpasgi_diag_jvp_core(m, c, f, d, rk_step, s);
}
