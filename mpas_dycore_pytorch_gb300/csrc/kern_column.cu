// Column-oriented stages: moist coefficients, vertical implicit coefficients, the
// acoustic substep (edge pressure-gradient update + per-column implicit solve),
// divergence damping, small-step perturbation and large-step recovery.
//
// Each kernel restates the reference stage's float64 arithmetic in the same operation
// order (mpas_pytorch/dynamics/*.py, cited per kernel); slot sums run in connectivity
// slot order, left to right, so results are deterministic and need no atomics.
#include "common.cuh"

namespace {

// ---------------------------------------------------------------- moist coefficients
// dynamics/moist_coefficients.py:124
__global__ void k_moist_cells(int nc, int L, int S, int ms, int me, const double* __restrict__ sc,
                              double* __restrict__ qtot, double* __restrict__ cqw) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double qprev = 0.0;
  for (int k = 0; k < L; ++k) {
    double q = 0.0;
    for (int s = ms - 1; s < me; ++s) q = q + sc[((size_t)c * L + k) * S + s];
    qtot[(size_t)c * L + k] = q;
    double w;
    if (k == 0) w = 0.0;
    else w = (me >= ms) ? 1.0 / (1.0 + 0.5 * (q + qprev)) : 1.0;
    cqw[(size_t)c * (L + 1) + k] = w;
    qprev = q;
  }
  cqw[(size_t)c * (L + 1) + L] = 0.0;
}

__global__ void k_moist_edges(int ne, int L, FastDiv fl, int ms, int me, const int32_t* __restrict__ coe,
                              const double* __restrict__ qtot, double* __restrict__ cqu) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)ne * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  if (me >= ms) {
    int c1 = coe[2 * e], c2 = coe[2 * e + 1];
    cqu[i] = 1.0 / (1.0 + 0.5 * (qtot[(size_t)c1 * L + k] + qtot[(size_t)c2 * L + k]));
  } else {
    cqu[i] = 1.0;
  }
}

// ---------------------------------------------------------------- vertical implicit coefficients
// dynamics/vert_imp_coefs.py:188 (coefficients :343-446, Thomas factor :100-121)
__global__ void k_vert_imp_coefs(mpasg_mesh m, mpasg_fields f, double dts, double epssm) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = m.nVertLevels;
  const double dtseps = 0.5 * dts * (1.0 + epssm);
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  if (c == 0) {
    for (int k = 0; k < L; ++k) f.cofrz[k] = dtseps * m.rdzw[k];
  }
  if (c >= m.nCells) return;
  const size_t o = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  f.coftz[ow] = 0.0;
  f.coftz[ow + L] = 0.0;
  for (int k = 0; k < L; ++k) {
    double zz = m.zz[o + k], p = f.exner[o + k], t = f.theta_m[o + k];
    double rb = m.rho_base[o + k], rtb = f.rtheta_base[o + k], pb = f.exner_base[o + k];
    double rt = f.rtheta_p[o + k], q = f.qtot[o + k];
    f.cofwt[o + k] = 0.5 * dtseps * rcv * zz * kGravity * rb / (1.0 + q) * p / ((rtb + rt) * pb);
    if (k == 0) {
      f.cofwr[o] = 0.0;
      f.cofwz[o] = 0.0;
    } else {
      double zzm = m.zz[o + k - 1];
      double fzm = m.fzm[k], fzp = m.fzp[k];
      f.cofwr[o + k] = 0.5 * dtseps * kGravity * (fzm * zz + fzp * zzm);
      double z_i = fzm * zz + fzp * zzm;
      double p_i = fzm * p + fzp * f.exner[o + k - 1];
      double t_i = fzm * t + fzp * f.theta_m[o + k - 1];
      f.cofwz[o + k] = dtseps * c2 * z_i * m.rdzu[k] * f.cqw[ow + k] * p_i;
      f.coftz[ow + k] = dtseps * t_i;
    }
  }
  double gam = 0.0;
  f.alpha_tri[o] = 0.0;
  f.gamma_tri[o] = 0.0;
  f.a_tri[o] = 0.0;
  for (int k = 1; k < L; ++k) {
    double cofwz = f.cofwz[o + k], cofwr = f.cofwr[o + k];
    double ct_km1 = f.coftz[ow + k - 1], ct_k = f.coftz[ow + k], ct_kp1 = f.coftz[ow + k + 1];
    double zz_k = m.zz[o + k], zz_km1 = m.zz[o + k - 1];
    double rdzw_k = m.rdzw[k], rdzw_km1 = m.rdzw[k - 1];
    double cofrz_k = dtseps * rdzw_k, cofrz_km1 = dtseps * rdzw_km1;
    double cw_k = f.cofwt[o + k], cw_km1 = f.cofwt[o + k - 1];
    double a = -cofwz * ct_km1 * rdzw_km1 * zz_km1 + cofwr * cofrz_km1 - cw_km1 * ct_km1 * rdzw_km1;
    double b = 1.0 + cofwz * (ct_k * rdzw_k * zz_k + ct_k * rdzw_km1 * zz_km1) -
               ct_k * (cw_k * rdzw_k - cw_km1 * rdzw_km1) + cofwr * (cofrz_k - cofrz_km1);
    double cc = -cofwz * ct_kp1 * rdzw_k * zz_k - cofwr * cofrz_k + cw_k * ct_kp1 * rdzw_k;
    double alpha = 1.0 / (b - a * gam);
    gam = cc * alpha;
    f.a_tri[o + k] = a;
    f.alpha_tri[o + k] = alpha;
    f.gamma_tri[o + k] = gam;
  }
}

// ---------------------------------------------------------------- acoustic substep, edges
// dynamics/acoustic_step.py:576 (_acoustic_step_horizontal_momentum_update)
__global__ void k_acoustic_edges(mpasg_mesh m, mpasg_fields f, FastDiv fl, int small_step,
                                 double dts, double c2) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  if (small_step != 1) {
    int c1 = m.cellsOnEdge[2 * e], c2i = m.cellsOnEdge[2 * e + 1];
    size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2i * L + k;
    double pgrad = ((f.rtheta_pp[i2] - f.rtheta_pp[i1]) * m.invDcEdge[e]) / (0.5 * (m.zz[i2] + m.zz[i1]));
    pgrad = f.cqu_e[i] * 0.5 * c2 * (f.exner[i1] + f.exner[i2]) * pgrad;
    pgrad = pgrad + 0.5 * m.zxu[i] * kGravity * (f.rho_pp[i1] + f.rho_pp[i2]);
    double rup = f.ru_p[i] + dts * (f.tend_u[i] - pgrad);
    f.ru_p[i] = rup;
    f.ruAvg[i] = f.ruAvg[i] + rup;
  } else {
    double rup = dts * f.tend_u[i];
    f.ru_p[i] = rup;
    f.ruAvg[i] = rup;
  }
}

// ---------------------------------------------------------------- acoustic substep, columns
// dynamics/acoustic_step.py:456 (cell flux sums), :675 (RHS), :772 (Thomas solve,
// implicit Rayleigh damping, post-solve rho_pp / rtheta_pp); Thomas sweeps from
// autodiff/tridiagonal_solve.py:56-63.  One thread owns one column; pass 1 streams
// upward (fluxes, RHS, forward elimination), pass 2 downward (back substitution,
// Rayleigh damping, post-solve update).
__global__ void k_acoustic_columns(mpasg_mesh m, mpasg_fields f, int small_step, double dts,
                                   double epssm, double resm) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nCells) return;
  const int L = m.nVertLevels;
  const int me = m.maxEdges;
  const size_t o = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  const bool first = (small_step == 1);
  const int nEoC = m.nEdgesOnCell[c];
  const double inv_area = m.invAreaCell[c];
  const double* th1 = f.theta_m_save;  // time-level-1 theta_m

  double rwp_k = first ? 0.0 : f.rw_p[ow];
  double rwp_top = first ? 0.0 : f.rw_p[ow + L];
  if (first) {
    f.rw_p[ow] = 0.0;
    f.rw_p[ow + L] = 0.0;
    f.wwAvg[ow] = 0.0;
    f.wwAvg[ow + L] = 0.0;
  }
  double x_prev = rwp_k;  // forward-eliminated value at k-1 (k = 0: boundary)
  double rs_prev = 0.0, ts_prev = 0.0, rho_prev = 0.0, rt_prev = 0.0;
  for (int k = 0; k < L; ++k) {
    double rs = 0.0, ts = 0.0;
    for (int j = 0; j < nEoC; ++j) {
      int e = m.edgesOnCell[c * me + j];
      double wgt = m.edgesOnCell_sign[c * me + j] * m.dvEdge[e];
      double flux = dts * wgt * f.ru_p[(size_t)e * L + k] * inv_area;
      int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
      double th_e = 0.5 * (th1[(size_t)c2 * L + k] + th1[(size_t)c1 * L + k]);
      if (j == 0) {
        rs = -flux;
        ts = -(flux * th_e);
      } else {
        rs = rs + (-flux);
        ts = ts + (-(flux * th_e));
      }
    }
    double rho_in = first ? 0.0 : f.rho_pp[o + k];
    double rt_in = first ? 0.0 : f.rtheta_pp[o + k];
    double rwp_k1 = (k + 1 < L) ? (first ? 0.0 : f.rw_p[ow + k + 1]) : rwp_top;
    f.rtheta_pp_old[o + k] = rt_in;
    double cofrz = f.cofrz[k];
    double rdzw = m.rdzw[k];
    rs = rho_in + dts * f.tend_rho[o + k] + rs - cofrz * resm * (rwp_k1 - rwp_k);
    ts = rt_in + dts * f.tend_theta[o + k] + ts -
         resm * rdzw * (f.coftz[ow + k + 1] * rwp_k1 - f.coftz[ow + k] * rwp_k);
    f.rho_pp[o + k] = rs;     // holds rs until pass 2
    f.rtheta_pp[o + k] = ts;  // holds ts until pass 2
    if (k >= 1) {
      double ww_in = first ? 0.0 : f.wwAvg[ow + k];
      f.wwAvg[ow + k] = ww_in + 0.5 * (1.0 - epssm) * rwp_k;
      double zz_k = m.zz[o + k], zz_km1 = m.zz[o + k - 1];
      double cofwz = f.cofwz[o + k], cofwr = f.cofwr[o + k];
      double cw_k = f.cofwt[o + k], cw_km1 = f.cofwt[o + k - 1];
      double rhs = rwp_k + dts * f.tend_rw[ow + k] -
                   cofwz * ((zz_k * ts - zz_km1 * ts_prev) + resm * (zz_k * rt_in - zz_km1 * rt_prev)) -
                   cofwr * ((rs + rs_prev) + resm * (rho_in + rho_prev)) + cw_k * (ts + resm * rt_in) +
                   cw_km1 * (ts_prev + resm * rt_prev);
      double x = (rhs - f.a_tri[o + k] * x_prev) * f.alpha_tri[o + k];
      f.rw_p[ow + k] = x;
      x_prev = x;
    }
    rs_prev = rs;
    ts_prev = ts;
    rho_prev = rho_in;
    rt_prev = rt_in;
    rwp_k = rwp_k1;
  }
  // pass 2: back substitution, Rayleigh damping, post-solve
  double xs_next = rwp_top;  // solved (pre-damping) value at k+1
  double xr_next = rwp_top;  // damped value at k+1
  for (int k = L - 1; k >= 0; --k) {
    double xk = (k >= 1) ? f.rw_p[ow + k] : (first ? 0.0 : f.rw_p[ow]);
    double xs = xk - f.gamma_tri[o + k] * xs_next;
    double xr = xs;
    if (k >= 1) {
      double fzm = m.fzm[k], fzp = m.fzp[k];
      double zz_i = fzm * m.zz[o + k] + fzp * m.zz[o + k - 1];
      double rho_i = fzm * f.rho_zz[o + k] + fzp * f.rho_zz[o + k - 1];
      double dss = m.dss[o + k];
      double rw_delta = f.rw_save[ow + k] - f.rw[ow + k];
      xr = (xs + rw_delta - dts * dss * zz_i * rho_i * f.w[ow + k]) / (1.0 + dts * dss) - rw_delta;
      f.wwAvg[ow + k] = f.wwAvg[ow + k] + 0.5 * (1.0 + epssm) * xr;
    }
    f.rw_p[ow + k] = xr;
    double rs = f.rho_pp[o + k], ts = f.rtheta_pp[o + k];
    f.rho_pp[o + k] = rs - f.cofrz[k] * (xr_next - xr);
    f.rtheta_pp[o + k] = ts - m.rdzw[k] * (f.coftz[ow + k + 1] * xr_next - f.coftz[ow + k] * xr);
    xs_next = xs;
    xr_next = xr;
  }
}

// ---------------------------------------------------------------- divergence damping
// dynamics/divergence_damping.py:187-299
__global__ void k_divergence_damping(mpasg_mesh m, mpasg_fields f, FastDiv fl, double coef) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  double d1 = -(f.rtheta_pp[i1] - f.rtheta_pp_old[i1]);
  double d2 = -(f.rtheta_pp[i2] - f.rtheta_pp_old[i2]);
  f.ru_p[i] = f.ru_p[i] + coef * (d2 - d1) / (f.theta_m_save[i1] + f.theta_m_save[i2]);
}

// ---------------------------------------------------------------- small-step perturbation
// dynamics/smlstep_pert.py:197-373
__global__ void k_smlstep_pert(mpasg_mesh m, mpasg_fields f, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  if (k == 0 || k == (uint32_t)L) {
    f.tend_rw[i] = f.tend_w[i];
    return;
  }
  const int me = m.maxEdges;
  double fzm = m.fzm[k], fzp = m.fzp[k];
  double acc = f.tend_w[i];
  const int n = m.nEdgesOnCell[c];
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double ut_k = f.tend_u[(size_t)e * L + k];
    double u_i = fzm * ut_k + fzp * f.tend_u[(size_t)e * L + k - 1];
    double flux = m.edgesOnCell_sign[c * me + j] * u_i;
    size_t zi = ((size_t)c * me + j) * (L + 1) + k;
    double coef = m.zb_cell[zi] + sgn(ut_k) * m.zb3_cell[zi];
    acc = acc - coef * flux;
  }
  size_t o = (size_t)c * L;
  f.tend_rw[i] = (fzm * m.zz[o + k] + fzp * m.zz[o + k - 1]) * acc;
}

// ---------------------------------------------------------------- large-step recovery
// dynamics/recover_large_step.py:414-466 (density / theta / Exner), :485-513 (edges),
// :329-411 (w from omega with zb/zb3 slot fluxes)
__global__ void k_recover_cells(mpasg_mesh m, mpasg_fields f, FastDiv fl1, int rk_step, double inv_ns,
                                double rk_dt) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  const size_t o = (size_t)c * L + k;
  if (k < (uint32_t)L) {
    double rho_p = f.rho_p_save[o] + f.rho_pp[o];
    double rho_zz = rho_p + m.rho_base[o];
    double rtheta_p;
    if (rk_step == 3)
      rtheta_p = f.rtheta_p_save[o] + f.rtheta_pp[o] - rk_dt * rho_zz * f.rt_diabatic_tend[o];
    else
      rtheta_p = f.rtheta_p_save[o] + f.rtheta_pp[o];
    double rtb = f.rtheta_base[o];
    f.rho_p[o] = rho_p;
    f.rho_zz[o] = rho_zz;
    f.rtheta_p[o] = rtheta_p;
    f.theta_m[o] = (rtheta_p + rtb) / rho_zz;
    if (rk_step == 3) {
      const double rcv = kRgas / (kCp - kRgas);
      double zz = m.zz[o];
      double ex = pow(zz * (kRgas / kP0) * (rtheta_p + rtb), rcv);
      f.exner[o] = ex;
      f.pressure_p[o] = zz * kRgas * __dadd_rn(__dmul_rn(ex, rtheta_p), __dmul_rn(rtb, ex - f.exner_base[o]));
    }
  }
  if (k >= 1 && k < (uint32_t)L) {
    size_t ow = (size_t)c * (L + 1) + k;
    double rws = f.rw_save[ow];
    f.wwAvg[ow] = rws + f.wwAvg[ow] * inv_ns;
    double rw = rws + f.rw_p[ow];
    f.rw[ow] = rw;
    size_t oc = (size_t)c * L;
    f.w[ow] = rw / (m.fzm[k] * m.zz[oc + k] + m.fzp[k] * m.zz[oc + k - 1]);
  }
}

__global__ void k_recover_edges(mpasg_mesh m, mpasg_fields f, FastDiv fl, double inv_ns) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  double rus = f.ru_save[i];
  f.ruAvg[i] = rus + f.ruAvg[i] * inv_ns;
  double ru = rus + f.ru_p[i];
  f.ru[i] = ru;
  f.u[i] = 2.0 * ru / (f.rho_zz[(size_t)c1 * L + k] + f.rho_zz[(size_t)c2 * L + k]);
}

__global__ void k_recover_w(mpasg_mesh m, mpasg_fields f, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  if (k == (uint32_t)L) {
    f.w[i] = 0.0;
    return;
  }
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const size_t oc = (size_t)c * L;
  if (k == 0) {
    double surf = 0.0;
    for (int j = 0; j < n; ++j) {
      int e = m.edgesOnCell[c * me + j];
      const double* ru = f.ru + (size_t)e * L;
      double fs = m.cf1 * ru[0] + m.cf2 * ru[1] + m.cf3 * ru[2];
      size_t zi = ((size_t)c * me + j) * (L + 1);
      double cs = m.zb_cell[zi] + sgn(fs) * m.zb3_cell[zi];
      double sc = m.edgesOnCell_sign[c * me + j] * cs * fs;
      surf = (j == 0) ? sc : surf + sc;
    }
    f.w[i] = surf / (m.cf1 * f.rho_zz[oc] + m.cf2 * f.rho_zz[oc + 1] + m.cf3 * f.rho_zz[oc + 2]);
    return;
  }
  double fzm = m.fzm[k], fzp = m.fzp[k];
  double acc = f.w[i];  // omega-derived part from k_recover_cells
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    double fi = fzm * f.ru[(size_t)e * L + k] + fzp * f.ru[(size_t)e * L + k - 1];
    size_t zi = ((size_t)c * me + j) * (L + 1) + k;
    double ci = m.zb_cell[zi] + sgn(fi) * m.zb3_cell[zi];
    acc = acc + m.edgesOnCell_sign[c * me + j] * ci * fi;
  }
  f.w[i] = acc / (fzm * f.rho_zz[oc + k] + fzp * f.rho_zz[oc + k - 1]);
}

}  // namespace

// ================================================================= C ABI
extern "C" int mpasg_moist_coefficients(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                        void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  k_moist_cells<<<nblocks(m->nCells), kBlock, 0, s>>>(m->nCells, L, c->num_scalars, c->moist_start,
                                                      c->moist_end, f->scalars, f->qtot, f->cqw);
  MPASG_LAUNCH_CHECK();
  k_moist_edges<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(
      m->nEdges, L, FastDiv(L), c->moist_start, c->moist_end, m->cellsOnEdge, f->qtot, f->cqu_e);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_vert_imp_coefs(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                    double dts, void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  k_vert_imp_coefs<<<nblocks(m->nCells, 128), 128, 0, (cudaStream_t)stream>>>(*m, *f, dts, c->epssm);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_acoustic_step(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                   int small_step, double dts, void* stream) {
  if (!m || !c || !f || small_step < 1) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  const double resm = (1.0 - c->epssm) / (1.0 + c->epssm);
  k_acoustic_edges<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, FastDiv(L), small_step,
                                                                         dts, c2);
  MPASG_LAUNCH_CHECK();
  k_acoustic_columns<<<nblocks(m->nCells, 128), 128, 0, s>>>(*m, *f, small_step, dts, c->epssm, resm);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_divergence_damping(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                        double dts, void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  const int L = m->nVertLevels;
  double coef = 2.0 * c->smdiv * c->len_disp / dts;
  k_divergence_damping<<<nblocks((long long)m->nEdges * L), kBlock, 0, (cudaStream_t)stream>>>(
      *m, *f, FastDiv(L), coef);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_smlstep_pert(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                  void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  const int L = m->nVertLevels;
  k_smlstep_pert<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, (cudaStream_t)stream>>>(
      *m, *f, FastDiv(L + 1));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_recover_large_step(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                        int rk_step, int ns, double rk_dt, void* stream) {
  if (!m || !c || !f || ns < 1) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  const double inv_ns = 1.0 / (double)ns;
  long long ncw = (long long)m->nCells * (L + 1);
  k_recover_cells<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1), rk_step, inv_ns, rk_dt);
  MPASG_LAUNCH_CHECK();
  k_recover_edges<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, FastDiv(L), inv_ns);
  MPASG_LAUNCH_CHECK();
  k_recover_w<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
