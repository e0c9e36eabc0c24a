// Column-oriented stages: moist coefficients, vertical implicit coefficients, the
// acoustic substep (edge pressure-gradient update + per-column implicit solve),
// divergence damping, small-step perturbation and large-step recovery.
//
// Each kernel restates the reference stage's float64 arithmetic in the same operation
// order (mpas_pytorch/dynamics/*.py, cited per kernel); slot sums run in connectivity
// slot order, left to right, so results are deterministic and need no atomics.
#include "common.cuh"
#include "pow_exner.cuh"

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
// dynamics/vert_imp_coefs.py:188 (coefficients :343-446, Thomas factor :100-121).
// k_vimp_coefs builds every level's coefficients and tridiagonal diagonals in parallel
// (neighbour levels shared through shared memory); k_vimp_factor runs the sequential
// Thomas factorisation, one thread per column.
struct VimpLevel {
  double cofwt, coftz;
};

// (float64 in both forms; T selects the division: exact in the float64 form, Newton
// reciprocal in the mixed form)
template <typename T>
MPASG_D VimpLevel vimp_level(const mpasg_mesh& m, const mpasg_fields& f, size_t o, size_t ow, int k,
                             double dtseps, double rcv) {
  VimpLevel v;
  double zz = m.zz[o + k], p = f.exner[o + k];
  double rb = m.rho_base[o + k], rtb = f.rtheta_base[o + k], pb = f.exner_base[o + k];
  double rt = f.rtheta_p[o + k], q = f.qtot[o + k];
  if (sizeof(T) == sizeof(double)) {
    // x / (1 + q) is x itself when q == 0 (dry columns): the division is skipped, not changed
    const double x = 0.5 * dtseps * rcv * zz * kGravity * rb;
    v.cofwt = fdiv<T>((q == 0.0 ? x : fdiv<T>(x, 1.0 + q)) * p, (rtb + rt) * pb);
  }
  else {  // mixed form: the dry case needs no 1 / (1 + q); constants folded into one factor
    const double x = (dtseps * (0.5 * rcv * kGravity)) * zz * rb;
    v.cofwt = (q == 0.0 ? x : fdiv<T>(x, 1.0 + q)) * p * rcp_nr((rtb + rt) * pb);
  }
  v.coftz = (k == 0) ? 0.0 : dtseps * (m.fzm[k] * f.theta_m[o + k] + m.fzp[k] * f.theta_m[o + k - 1]);
  return v;
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_vimp_coefs(mpasg_mesh m, mpasg_fields f, FastDiv fl, double dts,
                                                       double epssm) {
  __shared__ double s_cw[kBlock], s_ct[kBlock];
  const int L = m.nVertLevels;
  const double dtseps = 0.5 * dts * (1.0 + epssm);
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * L;
  uint32_t c = 0, k = 0;
  size_t o = 0, ow = 0;
  VimpLevel me_{0.0, 0.0};
  if (active) {
    c = fl.div(i);
    k = i - c * L;
    o = (size_t)c * L;
    ow = (size_t)c * (L + 1);
    me_ = vimp_level<T>(m, f, o, ow, k, dtseps, rcv);
    if (c == 0) f.cofrz[k] = dtseps * m.rdzw[k];
  }
  s_cw[threadIdx.x] = me_.cofwt;
  s_ct[threadIdx.x] = me_.coftz;
  __syncthreads();
  if (!active) return;
  f.cofwt[o + k] = me_.cofwt;
  f.coftz[ow + k] = me_.coftz;
  if (k == 0) {
    f.cofwr[o] = 0.0;
    f.cofwz[o] = 0.0;
    f.coftz[ow + L] = 0.0;
    f.a_tri[o] = 0.0;
    f.b_tri[o] = 1.0;
    f.c_tri[o] = 0.0;
    return;
  }
  const double zz = m.zz[o + k], zzm = m.zz[o + k - 1];
  const double fzm = m.fzm[k], fzp = m.fzp[k];
  const double cofwr = 0.5 * dtseps * kGravity * (fzm * zz + fzp * zzm);
  const double z_i = fzm * zz + fzp * zzm;
  const double p_i = fzm * f.exner[o + k] + fzp * f.exner[o + k - 1];
  const double cofwz = dtseps * c2 * z_i * m.rdzu[k] * f.cqw[ow + k] * p_i;
  f.cofwr[o + k] = cofwr;
  f.cofwz[o + k] = cofwz;
  // neighbour levels (k-1 below, k+1 above) from shared memory or recomputed at block edges
  VimpLevel lo = (threadIdx.x >= 1) ? VimpLevel{s_cw[threadIdx.x - 1], s_ct[threadIdx.x - 1]}
                                    : vimp_level<T>(m, f, o, ow, k - 1, dtseps, rcv);
  double ct_kp1 = 0.0;
  if (k + 1 < (uint32_t)L)
    ct_kp1 = (threadIdx.x + 1 < blockDim.x) ? s_ct[threadIdx.x + 1]
                                            : vimp_level<T>(m, f, o, ow, k + 1, dtseps, rcv).coftz;
  const double ct_km1 = lo.coftz, ct_k = me_.coftz;
  const double cw_k = me_.cofwt, cw_km1 = lo.cofwt;
  const double rdzw_k = m.rdzw[k], rdzw_km1 = m.rdzw[k - 1];
  const double cofrz_k = dtseps * rdzw_k, cofrz_km1 = dtseps * rdzw_km1;
  if (sizeof(T) == sizeof(double)) {  // the reference's expressions (vert_imp_coefs.py:388-428)
    f.a_tri[o + k] = -cofwz * ct_km1 * rdzw_km1 * zzm + cofwr * cofrz_km1 - cw_km1 * ct_km1 * rdzw_km1;
    f.b_tri[o + k] = 1.0 + cofwz * (ct_k * rdzw_k * zz + ct_k * rdzw_km1 * zzm) -
                     ct_k * (cw_k * rdzw_k - cw_km1 * rdzw_km1) + cofwr * (cofrz_k - cofrz_km1);
    f.c_tri[o + k] = -cofwz * ct_kp1 * rdzw_k * zz - cofwr * cofrz_k + cw_k * ct_kp1 * rdzw_k;
  } else {  // mixed form: the same float64 coefficients with the common factors taken out
    const double tm = ct_km1 * rdzw_km1, tp = ct_kp1 * rdzw_k;
    f.a_tri[o + k] = cofwr * cofrz_km1 - tm * (cofwz * zzm + cw_km1);
    f.b_tri[o + k] = 1.0 + ct_k * (cofwz * (rdzw_k * zz + rdzw_km1 * zzm) - (cw_k * rdzw_k - cw_km1 * rdzw_km1)) +
                     cofwr * (cofrz_k - cofrz_km1);
    f.c_tri[o + k] = tp * (cw_k - cofwz * zz) - cofwr * cofrz_k;
  }
}

template <typename T>
__global__ void k_vimp_factor(mpasg_mesh m, mpasg_fields f) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nCells) return;
  const int L = m.nVertLevels;
  const size_t o = (size_t)c * L;
  double gam = 0.0;
  f.alpha_tri[o] = 0.0;
  f.gamma_tri[o] = 0.0;
  for (int k = 1; k < L; ++k) {
    double alpha = fdiv<T>(1.0, f.b_tri[o + k] - f.a_tri[o + k] * gam);
    gam = f.c_tri[o + k] * alpha;
    f.alpha_tri[o + k] = alpha;
    f.gamma_tri[o + k] = gam;
    if (sizeof(T) != sizeof(double)) f.tri_m[o + k] = -(alpha * f.a_tri[o + k]);
  }
}

// ---------------------------------------------------------------- acoustic substep, edges
// dynamics/acoustic_step.py:576 (_acoustic_step_horizontal_momentum_update)
// The increment dts (tend_u - pgrad) is formed in the stencil type T; ru_p and ruAvg
// accumulate in float64.
template <typename T>
__global__ void k_acoustic_edges(mpasg_mesh m, mpasg_fields f, FastDiv fl, int small_step,
                                 double dts, double c2) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  if (small_step != 1) {
    int c1 = m.cellsOnEdge[2 * e], c2i = m.cellsOnEdge[2 * e + 1];
    size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2i * L + k;
    T pgrad = div_or_one<T>((cv<T>(f.rtheta_pp[i2]) - cv<T>(f.rtheta_pp[i1])) * cv<T>(m.invDcEdge[e]),
                            T(0.5) * (cv<T>(m.zz[i2]) + cv<T>(m.zz[i1])));
    pgrad = cv<T>(f.cqu_e[i]) * T(0.5) * cv<T>(c2) * (cv<T>(f.exner[i1]) + cv<T>(f.exner[i2])) * pgrad;
    pgrad = pgrad + T(0.5) * cv<T>(m.zxu[i]) * T(kGravity) * (cv<T>(f.rho_pp[i1]) + cv<T>(f.rho_pp[i2]));
    double rup = f.ru_p[i] + f64(cv<T>(dts) * (cv<T>(f.tend_u[i]) - pgrad));
    f.ru_p[i] = rup;
    f.ruAvg[i] = f.ruAvg[i] + rup;
  } else {
    double rup = f64(cv<T>(dts) * cv<T>(f.tend_u[i]));
    f.ru_p[i] = rup;
    f.ruAvg[i] = rup;
  }
}

// ---------------------------------------------------------------- acoustic substep, columns
// dynamics/acoustic_step.py:456 (cell flux sums), :675 (RHS), :772 (Thomas solve,
// implicit Rayleigh damping, post-solve rho_pp / rtheta_pp); Thomas sweeps from
// autodiff/tridiagonal_solve.py:56-63.  Three kernels: k_ac_prep (every level in
// parallel: flux sums, rs / ts, tridiagonal right-hand side), k_ac_thomas (one thread
// per column: forward elimination and back substitution only) and k_ac_post (every
// level in parallel: Rayleigh damping, ww accumulation, rho_pp / rtheta_pp update).

// rs / ts of one level before the implicit solve (acoustic_step.py :456, :675 first half)
struct AcLevel {
  double rs, ts, rho_in, rt_in;
};

// The horizontal flux sums (and dts times the tendencies) are formed in the stencil
// type T; the right-hand side combines them with the implicit coefficients in float64.
template <typename T>
MPASG_D AcLevel ac_level(const mpasg_mesh& m, const mpasg_fields& f, int c, int k, bool first, double dts,
                         double resm) {
  const int L = m.nVertLevels;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const T dts_t = cv<T>(dts);
  // sign * dvEdge * invAreaCell per slot (mesh constant) and the edge mean of the
  // time-level-1 theta_m (formed once per dynamics substep by k_theta_edge): four float64
  // operations per edge instead of eight
  const double* geo = m.cell_edge_geo + (size_t)c * me;
  T rs = T(0), ts = T(0);
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    T flux = (dts_t * cv<T>(geo[j])) * cv<T>(f.ru_p[(size_t)e * L + k]);
    T th_e = cv<T>(f.theta_edge_save[(size_t)e * L + k]);
    if (j == 0) {
      rs = -flux;
      ts = -(flux * th_e);
    } else {
      rs = rs + (-flux);
      ts = ts + (-(flux * th_e));
    }
  }
  const size_t o = (size_t)c * L + k;
  const size_t ow = (size_t)c * (L + 1) + k;
  AcLevel a;
  a.rho_in = first ? 0.0 : f.rho_pp[o];
  a.rt_in = first ? 0.0 : f.rtheta_pp[o];
  double rwp_k = first ? 0.0 : f.rw_p[ow];
  double rwp_k1 = first ? 0.0 : f.rw_p[ow + 1];
  a.rs = a.rho_in + f64(dts_t * cv<T>(f.tend_rho[o])) + f64(rs) - f.cofrz[k] * resm * (rwp_k1 - rwp_k);
  a.ts = a.rt_in + f64(dts_t * cv<T>(f.tend_theta[o])) + f64(ts) -
         resm * m.rdzw[k] * (f.coftz[ow + 1] * rwp_k1 - f.coftz[ow] * rwp_k);
  return a;
}

// edge mean of theta_m_save, 0.5 (theta_2 + theta_1), the value the acoustic right-hand
// side takes per edge, and the reciprocal of the sum that divergence damping divides by
// (theta_m_save only changes at the dynamics substep boundaries)
// MIXED: the mixed form's divergence damping reads the reciprocal as float32, so it is
// the float32 reciprocal of the float32 sum (no float64 division)
template <bool MIXED>
__global__ void k_theta_edge(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const double sum = f.theta_m_save[(size_t)c2 * L + k] + f.theta_m_save[(size_t)c1 * L + k];
  f.theta_edge_save[i] = 0.5 * sum;
  // divergence damping multiplies instead of dividing
  f.theta_edge_rsum[i] = MIXED ? f2d_bits(1.0f / d2f_bits(sum)) : 1.0 / sum;
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_ac_prep(mpasg_mesh m, mpasg_fields f, FastDiv fl1, int small_step,
                                                    double dts, double epssm, double resm) {
  __shared__ AcLevel s_lv[kBlock];
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * (L + 1);
  const bool first = (small_step == 1);
  uint32_t c = 0, k = 0;
  AcLevel lv{0.0, 0.0, 0.0, 0.0};
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
    if (k < (uint32_t)L) lv = ac_level<T>(m, f, c, k, first, dts, resm);
  }
  s_lv[threadIdx.x] = lv;
  __syncthreads();
  if (!active) return;
  const size_t o = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  if (k < (uint32_t)L) {
    f.ac_rs[o + k] = lv.rs;
    f.ac_ts[o + k] = lv.ts;
    f.rtheta_pp_old[o + k] = lv.rt_in;
  }
  const double rwp_k = first ? 0.0 : f.rw_p[ow + k];
  if (k == 0 || k == (uint32_t)L) {  // boundary values pass through the solve unchanged
    f.ac_x[ow + k] = rwp_k;
    if (first) f.wwAvg[ow + k] = 0.0;
    return;
  }
  AcLevel lo = (threadIdx.x >= 1) ? s_lv[threadIdx.x - 1] : ac_level<T>(m, f, c, k - 1, first, dts, resm);
  const double ww_in = first ? 0.0 : f.wwAvg[ow + k];
  f.wwAvg[ow + k] = ww_in + 0.5 * (1.0 - epssm) * rwp_k;
  const double zz_k = m.zz[o + k], zz_km1 = m.zz[o + k - 1];
  const double cw_k = f.cofwt[o + k], cw_km1 = f.cofwt[o + k - 1];
  f.ac_x[ow + k] = rwp_k + dts * f.tend_rw[ow + k] -
                   f.cofwz[o + k] * ((zz_k * lv.ts - zz_km1 * lo.ts) + resm * (zz_k * lv.rt_in - zz_km1 * lo.rt_in)) -
                   f.cofwr[o + k] * ((lv.rs + lo.rs) + resm * (lv.rho_in + lo.rho_in)) +
                   cw_k * (lv.ts + resm * lv.rt_in) + cw_km1 * (lo.ts + resm * lo.rt_in);
}

__global__ void k_ac_thomas(mpasg_mesh m, mpasg_fields f) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nCells) return;
  const int L = m.nVertLevels;
  const size_t o = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  double* x = f.ac_x + ow;
  double xp = x[0];
  for (int k = 1; k < L; ++k) {
    xp = (x[k] - f.a_tri[o + k] * xp) * f.alpha_tri[o + k];
    x[k] = xp;
  }
  double xn = x[L];
  for (int k = L - 1; k >= 0; --k) {
    xn = x[k] - f.gamma_tri[o + k] * xn;
    x[k] = xn;
  }
}

// ---------------------------------------------------------------- acoustic columns, mixed form
// The acoustic perturbations (rho_pp, rtheta_pp, rw_p, ru_p) are within-stage increments
// without a large mean; the mixed form forms their right-hand sides and post-solve
// increments in float32 and accumulates them in float64 (ac_rs, ac_ts, ac_x, rho_pp,
// rtheta_pp, wwAvg); the tridiagonal solve stays float64.  theta at the edges is split
// into the reference profile and the float32 deviation (theta_save_dev).
struct AcLevelF {
  float drs, dts, rho_in, rt_in;  // float32 increments of rs / ts, and the inputs
};

MPASG_D AcLevelF ac_level_mixed(const mpasg_mesh& m, const mpasg_fields& f, int c, int k, bool first, float dts,
                                float resm, double* rs64, double* ts64) {
  const int L = m.nVertLevels;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  const float ia = m.invAreaCell_f32[c];
  float rs = 0.0f, tsd = 0.0f;
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    const float wgt = m.edgesOnCell_sign_f32[c * me + j] * m.dvEdge_f32[e];
    const float flux = dts * wgt * cv<float>(f.ru_p[(size_t)e * L + k]) * ia;
    int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
    const float th_e = 0.5f * (f.theta_save_dev[(size_t)c2 * L + k] + f.theta_save_dev[(size_t)c1 * L + k]);
    rs = rs - flux;
    tsd = tsd - flux * th_e;
  }
  const float ts = cv<float>(m.ref_theta[k]) * rs + tsd;  // sum_j -flux_j (ref + theta'_j)
  const size_t o = (size_t)c * L + k;
  const size_t ow = (size_t)c * (L + 1) + k;
  AcLevelF a;
  const double rho_in = first ? 0.0 : f.rho_pp[o];
  const double rt_in = first ? 0.0 : f.rtheta_pp[o];
  a.rho_in = cv<float>(rho_in);
  a.rt_in = cv<float>(rt_in);
  const float rwp_k = first ? 0.0f : cv<float>(f.rw_p[ow]);
  const float rwp_k1 = first ? 0.0f : cv<float>(f.rw_p[ow + 1]);
  a.drs = dts * cv<float>(f.tend_rho[o]) + rs - cv<float>(f.cofrz[k]) * resm * (rwp_k1 - rwp_k);
  a.dts = dts * cv<float>(f.tend_theta[o]) + ts -
          resm * m.rdzw_f32[k] * (cv<float>(f.coftz[ow + 1]) * rwp_k1 - cv<float>(f.coftz[ow]) * rwp_k);
  if (rs64) *rs64 = rho_in + f64(a.drs);
  if (ts64) *ts64 = rt_in + f64(a.dts);
  return a;
}

__global__ void __launch_bounds__(kBlock) k_ac_prep_mixed(mpasg_mesh m, mpasg_fields f, FastDiv fl1,
                                                          int small_step, float dts, float epssm, float resm) {
  __shared__ AcLevelF s_lv[kBlock];
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * (L + 1);
  const bool first = (small_step == 1);
  uint32_t c = 0, k = 0;
  AcLevelF lv{0.0f, 0.0f, 0.0f, 0.0f};
  double rs64 = 0.0, ts64 = 0.0;
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
    if (k < (uint32_t)L) lv = ac_level_mixed(m, f, c, k, first, dts, resm, &rs64, &ts64);
  }
  s_lv[threadIdx.x] = lv;
  __syncthreads();
  if (!active) return;
  const size_t o = (size_t)c * L;
  const size_t ow = (size_t)c * (L + 1);
  if (k < (uint32_t)L) {
    f.ac_rs[o + k] = rs64;
    f.ac_ts[o + k] = ts64;
    f.rtheta_pp_old[o + k] = first ? 0.0 : f.rtheta_pp[o + k];
  }
  const double rwp_k = first ? 0.0 : f.rw_p[ow + k];
  if (k == 0 || k == (uint32_t)L) {  // boundary values pass through the solve unchanged
    f.ac_x[ow + k] = rwp_k;
    if (first) f.wwAvg[ow + k] = 0.0;
    return;
  }
  const AcLevelF lo = (threadIdx.x >= 1) ? s_lv[threadIdx.x - 1]
                                         : ac_level_mixed(m, f, c, k - 1, first, dts, resm, nullptr, nullptr);
  const double ww_in = first ? 0.0 : f.wwAvg[ow + k];
  const float rwp = cv<float>(rwp_k);
  f.wwAvg[ow + k] = ww_in + f64(0.5f * (1.0f - epssm) * rwp);
  const float zz_k = m.zz_f32[o + k], zz_km1 = m.zz_f32[o + k - 1];
  const float cw_k = cv<float>(f.cofwt[o + k]), cw_km1 = cv<float>(f.cofwt[o + k - 1]);
  const float ts_k = lv.rt_in + lv.dts, ts_km1 = lo.rt_in + lo.dts;
  const float rs_k = lv.rho_in + lv.drs, rs_km1 = lo.rho_in + lo.drs;
  const float inc = dts * cv<float>(f.tend_rw[ow + k]) -
                    cv<float>(f.cofwz[o + k]) *
                        ((zz_k * ts_k - zz_km1 * ts_km1) + resm * (zz_k * lv.rt_in - zz_km1 * lo.rt_in)) -
                    cv<float>(f.cofwr[o + k]) * ((rs_k + rs_km1) + resm * (lv.rho_in + lo.rho_in)) +
                    cw_k * (ts_k + resm * lv.rt_in) + cw_km1 * (ts_km1 + resm * lo.rt_in);
  f.ac_x[ow + k] = rwp_k + f64(inc);
}

// Rayleigh damping of the solution (float64); levels without damping pass through
MPASG_D double ac_damped_mixed(const mpasg_mesh& m, const mpasg_fields& f, size_t o, size_t ow, int k, int L,
                               double x, double dts) {
  if (k == 0 || k == L) return x;
  const double dss = m.dss[o + k];
  if (dss == 0.0) return x;
  double fzm = m.fzm[k], fzp = m.fzp[k];
  double zz_i = fzm * m.zz[o + k] + fzp * m.zz[o + k - 1];
  double rho_i = fzm * f.rho_zz[o + k] + fzp * f.rho_zz[o + k - 1];
  double rw_delta = f.rw_save[ow + k] - f.rw[ow + k];
  double num = x + rw_delta - dts * dss * zz_i * rho_i * f.w[ow + k];
  return fdiv<float>(num, 1.0 + dts * dss) - rw_delta;
}

__global__ void __launch_bounds__(kBlock) k_ac_post_mixed(mpasg_mesh m, mpasg_fields f, FastDiv fl1, double dts,
                                                          float epssm) {
  __shared__ double s_xr[kBlock];
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * (L + 1);
  uint32_t c = 0, k = 0;
  size_t o = 0, ow = 0;
  double xr = 0.0;
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
    o = (size_t)c * L;
    ow = (size_t)c * (L + 1);
    xr = ac_damped_mixed(m, f, o, ow, k, L, f.ac_x[ow + k], dts);
  }
  s_xr[threadIdx.x] = xr;
  __syncthreads();
  if (!active) return;
  f.rw_p[ow + k] = xr;
  if (k >= 1 && k < (uint32_t)L) f.wwAvg[ow + k] = f.wwAvg[ow + k] + f64(0.5f * (1.0f + epssm) * cv<float>(xr));
  if (k == (uint32_t)L) return;
  const double xr1 = (threadIdx.x + 1 < blockDim.x) ? s_xr[threadIdx.x + 1]
                                                    : ac_damped_mixed(m, f, o, ow, k + 1, L, f.ac_x[ow + k + 1], dts);
  const float x0 = cv<float>(xr), x1 = cv<float>(xr1);
  f.rho_pp[o + k] = f.ac_rs[o + k] - f64(cv<float>(f.cofrz[k]) * dif<float>(xr1, xr));
  f.rtheta_pp[o + k] = f.ac_ts[o + k] - f64(m.rdzw_f32[k] * (cv<float>(f.coftz[ow + k + 1]) * x1 -
                                                             cv<float>(f.coftz[ow + k]) * x0));
}

// The same sweeps with the columns staged through shared memory: one warp solves 32
// columns; the block's x, a, alpha and gamma are loaded and stored with coalesced
// accesses (consecutive threads read consecutive levels of a column) into a [level][33]
// layout, so the sequential sweeps read shared memory instead of waiting on one global
// load per level.  The staging runs on all kThomasThreads threads (4 warps, 4x the loads
// in flight: the copy, not the sweep, bounded the one-warp version), the sweeps on the
// first warp.  Same arithmetic as k_ac_thomas.
constexpr int kThomasCols = 32;
constexpr int kThomasPitch = kThomasCols + 1;
constexpr int kThomasThreads = 128;

__global__ void __launch_bounds__(kThomasThreads) k_ac_thomas_staged(mpasg_mesh m, mpasg_fields f, FastDiv fl,
                                                                     FastDiv fl1) {
  extern __shared__ double s_col[];
  const int L = m.nVertLevels;
  double* sx = s_col;                              // (L+1) x pitch
  double* sa = sx + (size_t)(L + 1) * kThomasPitch;  // L x pitch each
  double* sal = sa + (size_t)L * kThomasPitch;
  double* sg = sal + (size_t)L * kThomasPitch;
  const int c0 = blockIdx.x * kThomasCols;
  const int ncol = min(kThomasCols, m.nCells - c0);
  const int t = threadIdx.x;
  const uint32_t nw = (uint32_t)ncol * (L + 1), nl = (uint32_t)ncol * L;
  const double* gx = f.ac_x + (size_t)c0 * (L + 1);
  const size_t o0 = (size_t)c0 * L;
  for (uint32_t idx = t; idx < nw; idx += kThomasThreads) {
    uint32_t col = fl1.div(idx), k = idx - col * (L + 1);
    sx[k * kThomasPitch + col] = gx[idx];
  }
  for (uint32_t idx = t; idx < nl; idx += kThomasThreads) {
    uint32_t col = fl.div(idx), k = idx - col * L;
    sa[k * kThomasPitch + col] = f.a_tri[o0 + idx];
    sal[k * kThomasPitch + col] = f.alpha_tri[o0 + idx];
    sg[k * kThomasPitch + col] = f.gamma_tri[o0 + idx];
  }
  __syncthreads();
  if (t < ncol) {
    double xp = sx[t];
    for (int k = 1; k < L; ++k) {
      xp = (sx[k * kThomasPitch + t] - sa[k * kThomasPitch + t] * xp) * sal[k * kThomasPitch + t];
      sx[k * kThomasPitch + t] = xp;
    }
    double xn = sx[L * kThomasPitch + t];
    for (int k = L - 1; k >= 0; --k) {
      xn = sx[k * kThomasPitch + t] - sg[k * kThomasPitch + t] * xn;
      sx[k * kThomasPitch + t] = xn;
    }
  }
  __syncthreads();
  double* gxo = f.ac_x + (size_t)c0 * (L + 1);
  for (uint32_t idx = t; idx < nw; idx += kThomasThreads) {
    uint32_t col = fl1.div(idx), k = idx - col * (L + 1);
    gxo[idx] = sx[k * kThomasPitch + col];
  }
}

// Mixed form (still float64): u_k = alpha_k x_k + m_k u_(k-1) with m_k = -alpha_k a_k
// precomputed by the factorisation, so the serial dependence is one FMA per level
// (alpha_k x_k does not depend on the chain and issues ahead).
__global__ void __launch_bounds__(kThomasThreads) k_ac_thomas_staged_mixed(mpasg_mesh m, mpasg_fields f,
                                                                           FastDiv fl, FastDiv fl1) {
  extern __shared__ double s_col[];
  const int L = m.nVertLevels;
  double* sx = s_col;
  double* sm = sx + (size_t)(L + 1) * kThomasPitch;
  double* sal = sm + (size_t)L * kThomasPitch;
  double* sg = sal + (size_t)L * kThomasPitch;
  const int c0 = blockIdx.x * kThomasCols;
  const int ncol = min(kThomasCols, m.nCells - c0);
  const int t = threadIdx.x;
  const uint32_t nw = (uint32_t)ncol * (L + 1), nl = (uint32_t)ncol * L;
  const double* gx = f.ac_x + (size_t)c0 * (L + 1);
  const size_t o0 = (size_t)c0 * L;
  for (uint32_t idx = t; idx < nw; idx += kThomasThreads) {
    uint32_t col = fl1.div(idx), k = idx - col * (L + 1);
    sx[k * kThomasPitch + col] = gx[idx];
  }
  for (uint32_t idx = t; idx < nl; idx += kThomasThreads) {
    uint32_t col = fl.div(idx), k = idx - col * L;
    sm[k * kThomasPitch + col] = f.tri_m[o0 + idx];
    sal[k * kThomasPitch + col] = f.alpha_tri[o0 + idx];
    sg[k * kThomasPitch + col] = f.gamma_tri[o0 + idx];
  }
  __syncthreads();
  if (t < ncol) {
    double xp = sx[t];
    for (int k = 1; k < L; ++k) {
      xp = fma(sm[k * kThomasPitch + t], xp, sal[k * kThomasPitch + t] * sx[k * kThomasPitch + t]);
      sx[k * kThomasPitch + t] = xp;
    }
    double xn = sx[L * kThomasPitch + t];
    for (int k = L - 1; k >= 0; --k) {
      xn = fma(-sg[k * kThomasPitch + t], xn, sx[k * kThomasPitch + t]);
      sx[k * kThomasPitch + t] = xn;
    }
  }
  __syncthreads();
  double* gxo = f.ac_x + (size_t)c0 * (L + 1);
  for (uint32_t idx = t; idx < nw; idx += kThomasThreads) {
    uint32_t col = fl1.div(idx), k = idx - col * (L + 1);
    gxo[idx] = sx[k * kThomasPitch + col];
  }
}

// Thomas factorisation (k_vimp_factor) with the columns staged the same way: a, b, c in
// and alpha, gamma (and the mixed form's tri_m) out through a [level][33] layout with
// coalesced copies by 4 warps; the division chain of each column runs on the first warp
// from shared memory.  Same arithmetic as k_vimp_factor.
template <typename T>
__global__ void __launch_bounds__(kThomasThreads) k_vimp_factor_staged(mpasg_mesh m, mpasg_fields f, FastDiv fl) {
  extern __shared__ double s_col[];
  const int L = m.nVertLevels;
  double* sa = s_col;  // L x pitch each
  double* sb = sa + (size_t)L * kThomasPitch;
  double* sc = sb + (size_t)L * kThomasPitch;
  double* sal = sc + (size_t)L * kThomasPitch;
  double* sg = sal + (size_t)L * kThomasPitch;
  const int c0 = blockIdx.x * kThomasCols;
  const int ncol = min(kThomasCols, m.nCells - c0);
  const int t = threadIdx.x;
  const uint32_t nl = (uint32_t)ncol * L;
  const size_t o0 = (size_t)c0 * L;
  for (uint32_t idx = t; idx < nl; idx += kThomasThreads) {
    uint32_t col = fl.div(idx), k = idx - col * L;
    sa[k * kThomasPitch + col] = f.a_tri[o0 + idx];
    sb[k * kThomasPitch + col] = f.b_tri[o0 + idx];
    sc[k * kThomasPitch + col] = f.c_tri[o0 + idx];
  }
  __syncthreads();
  if (t < ncol) {
    double gam = 0.0;
    sal[t] = 0.0;
    sg[t] = 0.0;
    for (int k = 1; k < L; ++k) {
      const double alpha = fdiv<T>(1.0, sb[k * kThomasPitch + t] - sa[k * kThomasPitch + t] * gam);
      gam = sc[k * kThomasPitch + t] * alpha;
      sal[k * kThomasPitch + t] = alpha;
      sg[k * kThomasPitch + t] = gam;
    }
  }
  __syncthreads();
  for (uint32_t idx = t; idx < nl; idx += kThomasThreads) {
    uint32_t col = fl.div(idx), k = idx - col * L;
    const double alpha = sal[k * kThomasPitch + col];
    f.alpha_tri[o0 + idx] = alpha;
    f.gamma_tri[o0 + idx] = sg[k * kThomasPitch + col];
    if (sizeof(T) != sizeof(double) && k > 0) f.tri_m[o0 + idx] = -(alpha * sa[k * kThomasPitch + col]);
  }
}

size_t vimp_factor_smem_bytes(int L) { return (size_t)5 * L * kThomasPitch * sizeof(double); }

// tri_m = -alpha_tri * a_tri (the mixed forward-sweep factor) from the stored factors
__global__ void k_tri_m(long long n, const double* __restrict__ a, const double* __restrict__ al,
                        double* __restrict__ tm) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) tm[i] = -(al[i] * a[i]);
}

size_t thomas_smem_bytes(int L) { return (size_t)(4 * L + 1) * kThomasPitch * sizeof(double); }

MPASG_D double ac_damped(const mpasg_mesh& m, const mpasg_fields& f, size_t o, size_t ow, int k, int L, double x,
                         double dts) {
  if (k == 0 || k == L) return x;
  double fzm = m.fzm[k], fzp = m.fzp[k];
  double zz_i = fzm * m.zz[o + k] + fzp * m.zz[o + k - 1];
  double rho_i = fzm * f.rho_zz[o + k] + fzp * f.rho_zz[o + k - 1];
  double dss = m.dss[o + k];
  double rw_delta = f.rw_save[ow + k] - f.rw[ow + k];
  double num = x + rw_delta - dts * dss * zz_i * rho_i * f.w[ow + k];
  double den = 1.0 + dts * dss;
  return (den == 1.0 ? num : num / den) - rw_delta;  // x / 1.0 == x below the damping layer
}

__global__ void __launch_bounds__(kBlock) k_ac_post(mpasg_mesh m, mpasg_fields f, FastDiv fl1, double dts,
                                                    double epssm) {
  __shared__ double s_xr[kBlock];
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * (L + 1);
  uint32_t c = 0, k = 0;
  size_t o = 0, ow = 0;
  double xr = 0.0;
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
    o = (size_t)c * L;
    ow = (size_t)c * (L + 1);
    xr = ac_damped(m, f, o, ow, k, L, f.ac_x[ow + k], dts);
  }
  s_xr[threadIdx.x] = xr;
  __syncthreads();
  if (!active) return;
  f.rw_p[ow + k] = xr;
  if (k >= 1 && k < (uint32_t)L) f.wwAvg[ow + k] = f.wwAvg[ow + k] + 0.5 * (1.0 + epssm) * xr;
  if (k == (uint32_t)L) return;
  double xr1 = (threadIdx.x + 1 < blockDim.x) ? s_xr[threadIdx.x + 1]
                                              : ac_damped(m, f, o, ow, k + 1, L, f.ac_x[ow + k + 1], dts);
  f.rho_pp[o + k] = f.ac_rs[o + k] - f.cofrz[k] * (xr1 - xr);
  f.rtheta_pp[o + k] = f.ac_ts[o + k] - m.rdzw[k] * (f.coftz[ow + k + 1] * xr1 - f.coftz[ow + k] * xr);
}

// ---------------------------------------------------------------- divergence damping
// dynamics/divergence_damping.py:187-299
// (the increment in the stencil type T, ru_p accumulated in float64)
template <typename T>
__global__ void k_divergence_damping(mpasg_mesh m, mpasg_fields f, FastDiv fl, double coef) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  uint32_t e = fl.div(i), k = i - e * L;
  int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  T d1 = -dif<T>(f.rtheta_pp[i1], f.rtheta_pp_old[i1]);  // substep change: float64 difference
  T d2 = -dif<T>(f.rtheta_pp[i2], f.rtheta_pp_old[i2]);
  // / (theta_m_save_1 + theta_m_save_2) as a product with the reciprocal formed once per
  // dynamics substep (k_theta_edge); within one rounding of the quotient
  f.ru_p[i] = f.ru_p[i] + f64(cv<T>(coef) * (d2 - d1) * cv<T>(f.theta_edge_rsum[i]));
}

// ---------------------------------------------------------------- small-step perturbation
// dynamics/smlstep_pert.py:197-373
template <typename T>
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
  const T fzm = cv<T>(m.fzm[k]), fzp = cv<T>(m.fzp[k]);
  T acc = cv<T>(f.tend_w[i]);
  const int n = m.flatTerrain ? 0 : m.nEdgesOnCell[c];  // zero-slope terms add exact zeros
  for (int j = 0; j < n; ++j) {
    int e = m.edgesOnCell[c * me + j];
    T ut_k = cv<T>(f.tend_u[(size_t)e * L + k]);
    T u_i = fzm * ut_k + fzp * cv<T>(f.tend_u[(size_t)e * L + k - 1]);
    T flux = cv<T>(m.edgesOnCell_sign[c * me + j]) * u_i;
    size_t zi = ((size_t)c * me + j) * (L + 1) + k;
    T coef = cv<T>(m.zb_cell[zi]) + (ut_k >= T(0) ? T(1) : T(-1)) * cv<T>(m.zb3_cell[zi]);
    acc = acc - coef * flux;
  }
  size_t o = (size_t)c * L;
  f.tend_rw[i] = f64((fzm * cv<T>(m.zz[o + k]) + fzp * cv<T>(m.zz[o + k - 1])) * acc);
}

// ---------------------------------------------------------------- large-step recovery
// dynamics/recover_large_step.py:414-466 (density / theta / Exner), :485-513 (edges),
// :329-411 (w from omega with zb/zb3 slot fluxes)
// Binomial coefficients C(a, n) = a (a-1) ... (a-n+1) / n!, n = 0..11 (compile time).
struct BinomTable {
  double c[12];
};
__host__ __device__ constexpr BinomTable binom_table(double a) {
  BinomTable b{};
  double t = 1.0;
  b.c[0] = 1.0;
  for (int n = 1; n < 12; ++n) {
    t = t * (a - (n - 1)) / n;
    b.c[n] = t;
  }
  return b;
}

// (1 + x)^(R/cv) - 1 for |x| < 0.02 by its binomial series, 11 terms in float64 Horner
// form (truncation below 1e-19 relative): no cancellation against 1, unlike pow - 1.
MPASG_D double pow1p_rcv_m1(double x) {
  constexpr BinomTable t = binom_table(kRgas / (kCp - kRgas));
  double p = t.c[11];
#pragma unroll
  for (int n = 10; n >= 1; --n) p = fma(p, x, t.c[n]);
  return p * x;
}

// Float64 in both forms; T selects the division (exact / Newton reciprocal) and, at
// rk 3, the Exner function: pow in the float64 form; in the mixed form the identity
// exner = exner_base (1 + x)^(R/cv), x = rtheta_p / rtheta_base, with the increment
// exner - exner_base = exner_base pow1p_rcv_m1(x) (pow when |x| >= 0.02), so the
// pressure perturbation needs no difference of nearly equal Exner values.
// FLAT (flat terrain, no slope terms): w itself is finished here as well, omega-derived
// part over the interface density, with the level below's density from the neighbouring
// thread (shared memory) -- the same expressions k_recover_w evaluates, one launch fewer.
template <typename T, bool FLAT = false>
__global__ void __launch_bounds__(kBlock) k_recover_cells(mpasg_mesh m, mpasg_fields f, FastDiv fl1, int rk_step,
                                                          double inv_ns, double rk_dt) {
  __shared__ double s_rho[FLAT ? kBlock : 1];
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < (uint32_t)m.nCells * (L + 1);
  if (!FLAT && !active) return;
  uint32_t c = 0, k = 0;
  if (active) {
    c = fl1.div(i);
    k = i - c * (L + 1);
  }
  const size_t o = (size_t)c * L + k;
  if (FLAT) {
    s_rho[threadIdx.x] = (active && k < (uint32_t)L) ? f.rho_p_save[o] + f.rho_pp[o] + m.rho_base[o] : 0.0;
    __syncthreads();
    if (!active) return;
  }
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
    f.theta_m[o] = sizeof(T) == sizeof(double) ? (rtheta_p + rtb) / rho_zz : (rtheta_p + rtb) * rcp_nr1(rho_zz);
    if (rk_step == 3) {
      const double rcv = kRgas / (kCp - kRgas);
      double zz = m.zz[o];
      if (sizeof(T) == sizeof(double)) {
        double ex = mpasg_pow::pow_exner(zz * (kRgas / kP0) * (rtheta_p + rtb), rcv);
        f.exner[o] = ex;
        f.pressure_p[o] = zz * kRgas * __dadd_rn(__dmul_rn(ex, rtheta_p), __dmul_rn(rtb, ex - f.exner_base[o]));
      } else {
        const double exb = f.exner_base[o];
        const double x = fdiv<T>(rtheta_p, rtb);
        double ex, dex;  // exner and exner - exner_base
        if (fabs(x) < 0.02) {
          dex = exb * pow1p_rcv_m1(x);
          ex = exb + dex;
        } else {
          ex = mpasg_pow::pow_exner(zz * (kRgas / kP0) * (rtheta_p + rtb), rcv);
          dex = ex - exb;
        }
        f.exner[o] = ex;
        f.pressure_p[o] = zz * kRgas * (ex * rtheta_p + rtb * dex);
      }
    }
  }
  if (k >= 1 && k < (uint32_t)L) {
    size_t ow = (size_t)c * (L + 1) + k;
    double rws = f.rw_save[ow];
    f.wwAvg[ow] = rws + f.wwAvg[ow] * inv_ns;
    double rw = rws + f.rw_p[ow];
    f.rw[ow] = rw;
    if (sizeof(T) != sizeof(double)) f.rw_f32[ow] = d2f_bits(rw);
    size_t oc = (size_t)c * L;
    const double den = m.fzm[k] * m.zz[oc + k] + m.fzp[k] * m.zz[oc + k - 1];
    const double wo = den == 1.0 ? rw : fdiv<T>(rw, den);
    if (!FLAT) {
      f.w[ow] = wo;
    } else {
      const double rho_k = s_rho[threadIdx.x];
      const double rho_km1 = threadIdx.x >= 1 ? s_rho[threadIdx.x - 1]
                                              : f.rho_p_save[oc + k - 1] + f.rho_pp[oc + k - 1] + m.rho_base[oc + k - 1];
      const double wk = fdiv<T>(wo, m.fzm[k] * rho_k + m.fzp[k] * rho_km1);
      f.w[ow] = wk;
      if (sizeof(T) != sizeof(double)) f.w_f32[ow] = d2f_bits(wk);
    }
  } else if (FLAT) {  // bottom and top interfaces: no slope flux, w = 0
    const size_t ow = (size_t)c * (L + 1) + k;
    f.w[ow] = 0.0;
    if (sizeof(T) != sizeof(double)) f.w_f32[ow] = 0.0f;
  }
}

template <typename T>
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
  const double rho2 = f.rho_zz[(size_t)c1 * L + k] + f.rho_zz[(size_t)c2 * L + k];
  const double u = sizeof(T) == sizeof(double) ? 2.0 * ru / rho2 : 2.0 * ru * rcp_nr1(rho2);
  f.u[i] = u;
  if (sizeof(T) != sizeof(double)) f.u_f32[i] = d2f_bits(u);
}

template <typename T>
__global__ void k_recover_w(mpasg_mesh m, mpasg_fields f, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  uint32_t c = fl1.div(i), k = i - c * (L + 1);
  constexpr bool kMixed = sizeof(T) != sizeof(double);  // also refresh the float32 copy of w
  if (k == (uint32_t)L) {
    f.w[i] = 0.0;
    if (kMixed) f.w_f32[i] = 0.0f;
    return;
  }
  const int me = m.maxEdges;
  const int n = m.flatTerrain ? 0 : m.nEdgesOnCell[c];  // zero-slope terms add exact zeros
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
    const double w0 = fdiv<T>(surf, m.cf1 * f.rho_zz[oc] + m.cf2 * f.rho_zz[oc + 1] + m.cf3 * f.rho_zz[oc + 2]);
    f.w[i] = w0;
    if (kMixed) f.w_f32[i] = d2f_bits(w0);
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
  const double wk = fdiv<T>(acc, fzm * f.rho_zz[oc + k] + fzp * f.rho_zz[oc + k - 1]);
  f.w[i] = wk;
  if (kMixed) f.w_f32[i] = d2f_bits(wk);
}

template <typename T>
int launch_recover(const mpasg_mesh* m, mpasg_fields* f, int rk_step, double inv_ns, double rk_dt, cudaStream_t s) {
  const int L = m->nVertLevels;
  const long long ncw = (long long)m->nCells * (L + 1);
  if (m->flatTerrain)
    k_recover_cells<T, true><<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1), rk_step, inv_ns, rk_dt);
  else
    k_recover_cells<T><<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1), rk_step, inv_ns, rk_dt);
  MPASG_LAUNCH_CHECK();
  k_recover_edges<T><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, FastDiv(L), inv_ns);
  MPASG_LAUNCH_CHECK();
  if (!m->flatTerrain) {  // slope fluxes need the new ru of k_recover_edges
    k_recover_w<T><<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1));
    MPASG_LAUNCH_CHECK();
  }
  return MPASG_OK;
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
  cudaStream_t s = (cudaStream_t)stream;
  const int L = m->nVertLevels;
  // the staged factorisation needs more than 48 KB of dynamic shared memory: opt in once
  // per device (the first call on a device should come before any stream capture)
  const size_t smem = vimp_factor_smem_bytes(L);
  static bool smem_opt_in[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MPASG_E_CUDA;
  if (!smem_opt_in[dev])
    smem_opt_in[dev] = cudaFuncSetAttribute(k_vimp_factor_staged<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            200 * 1024) == cudaSuccess &&
                       cudaFuncSetAttribute(k_vimp_factor_staged<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            200 * 1024) == cudaSuccess;
  const bool staged = smem_opt_in[dev] && smem <= 200 * 1024;
  const int nblk = nblocks(m->nCells, kThomasCols);
  if (c->precision == MPASG_PRECISION_MIXED) {
    k_vimp_coefs<float><<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, FastDiv(L), dts, c->epssm);
    MPASG_LAUNCH_CHECK();
    if (staged) k_vimp_factor_staged<float><<<nblk, kThomasThreads, smem, s>>>(*m, *f, FastDiv(L));
    else k_vimp_factor<float><<<nblocks(m->nCells, 64), 64, 0, s>>>(*m, *f);
  } else {
    k_vimp_coefs<double><<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, FastDiv(L), dts, c->epssm);
    MPASG_LAUNCH_CHECK();
    if (staged) k_vimp_factor_staged<double><<<nblk, kThomasThreads, smem, s>>>(*m, *f, FastDiv(L));
    else k_vimp_factor<double><<<nblocks(m->nCells, 64), 64, 0, s>>>(*m, *f);
  }
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_acoustic_step(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                   int small_step, double dts, void* stream) {
  return mpasgi_acoustic_step(m, c, f, small_step, dts, (cudaStream_t)stream, false);
}

int mpasgi_theta_edge(const mpasg_mesh* m, mpasg_fields* f, bool mixed, cudaStream_t s) {
  const int L = m->nVertLevels;
  if (mixed)
    k_theta_edge<true><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, FastDiv(L));
  else
    k_theta_edge<false><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, FastDiv(L));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

int mpasgi_acoustic_parts(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int small_step, double dts,
                          cudaStream_t s, int part);

int mpasgi_acoustic_step(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int small_step, double dts,
                         cudaStream_t s, bool copies_current) {
  if (!m || !c || !f || small_step < 1) return MPASG_E_ARG;
  if (!copies_current) {
    // the edge theta the right-hand side reads
    const int rc = mpasgi_theta_edge(m, f, c->precision == MPASG_PRECISION_MIXED, s);
    if (rc != MPASG_OK) return rc;
  }
  if (c->precision == MPASG_PRECISION_MIXED && !copies_current) {
    const int rc = mpasgi_theta_dev(m, f, s);  // the float32 theta deviations read below
    if (rc != MPASG_OK) return rc;
    const long long n = (long long)m->nCells * m->nVertLevels;
    k_tri_m<<<nblocks(n), kBlock, 0, s>>>(n, f->a_tri, f->alpha_tri, f->tri_m);  // forward-sweep factor
    MPASG_LAUNCH_CHECK();
  }
  return mpasgi_acoustic_parts(m, c, f, small_step, dts, s, -1);
}

// The acoustic substep in two parts (part -1: both): part 0 updates ru_p / ruAvg on the
// edges and builds the columns' right-hand sides (ac_x holds the tridiagonal right-hand
// side after it); part 1 solves and finishes the columns.
int mpasgi_acoustic_parts(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int small_step, double dts,
                          cudaStream_t s, int part) {
  const int L = m->nVertLevels;
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  const double resm = (1.0 - c->epssm) / (1.0 + c->epssm);
  const long long ncw = (long long)m->nCells * (L + 1);
  const bool mixed = c->precision == MPASG_PRECISION_MIXED;
  if (part != 1) {
    if (mixed) {
      k_acoustic_edges<float><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, FastDiv(L), small_step,
                                                                                  dts, c2);
      MPASG_LAUNCH_CHECK();
      k_ac_prep_mixed<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1), small_step, (float)dts,
                                                      (float)c->epssm, (float)resm);
      MPASG_LAUNCH_CHECK();
    } else {
      k_acoustic_edges<double><<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, FastDiv(L), small_step,
                                                                                   dts, c2);
      MPASG_LAUNCH_CHECK();
      k_ac_prep<double><<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1), small_step, dts, c->epssm, resm);
      MPASG_LAUNCH_CHECK();
    }
    if (part == 0) return MPASG_OK;
  }
  // the staged solve needs more than 48 KB of dynamic shared memory: opt in once per
  // device (the first call on a device should come before any stream capture)
  const size_t smem = thomas_smem_bytes(L);
  static bool smem_opt_in[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MPASG_E_CUDA;
  if (!smem_opt_in[dev])
    smem_opt_in[dev] =
        cudaFuncSetAttribute(k_ac_thomas_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
            cudaSuccess &&
        cudaFuncSetAttribute(k_ac_thomas_staged_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
            cudaSuccess;
  if (smem_opt_in[dev] && smem <= 200 * 1024 && mixed)
    k_ac_thomas_staged_mixed<<<nblocks(m->nCells, kThomasCols), kThomasThreads, smem, s>>>(*m, *f, FastDiv(L),
                                                                                        FastDiv(L + 1));
  else if (smem_opt_in[dev] && smem <= 200 * 1024)
    k_ac_thomas_staged<<<nblocks(m->nCells, kThomasCols), kThomasThreads, smem, s>>>(*m, *f, FastDiv(L),
                                                                                  FastDiv(L + 1));
  else if (mixed)
    return MPASG_E_ARG;  // the mixed sweep needs the staged kernel (L <= 200)
  else
    k_ac_thomas<<<nblocks(m->nCells, 64), 64, 0, s>>>(*m, *f);
  MPASG_LAUNCH_CHECK();
  if (mixed)
    k_ac_post_mixed<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1), dts, (float)c->epssm);
  else
    k_ac_post<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, FastDiv(L + 1), dts, c->epssm);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_divergence_damping(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                        double dts, void* stream) {
  return mpasgi_divergence_damping(m, c, f, dts, (cudaStream_t)stream, false);
}

int mpasgi_divergence_damping(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, double dts,
                              cudaStream_t stream, bool copies_current) {
  if (!m || !c || !f) return MPASG_E_ARG;
  const int L = m->nVertLevels;
  if (!copies_current) {
    // the reciprocal edge sums read below
    const int rc = mpasgi_theta_edge(m, f, c->precision == MPASG_PRECISION_MIXED, stream);
    if (rc != MPASG_OK) return rc;
  }
  double coef = 2.0 * c->smdiv * c->len_disp / dts;
  if (c->precision == MPASG_PRECISION_MIXED)
    k_divergence_damping<float><<<nblocks((long long)m->nEdges * L), kBlock, 0, (cudaStream_t)stream>>>(
        *m, *f, FastDiv(L), coef);
  else
    k_divergence_damping<double><<<nblocks((long long)m->nEdges * L), kBlock, 0, (cudaStream_t)stream>>>(
        *m, *f, FastDiv(L), coef);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_smlstep_pert(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                  void* stream) {
  if (!m || !c || !f) return MPASG_E_ARG;
  const int L = m->nVertLevels;
  if (c->precision == MPASG_PRECISION_MIXED)
    k_smlstep_pert<float><<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, (cudaStream_t)stream>>>(
        *m, *f, FastDiv(L + 1));
  else
    k_smlstep_pert<double><<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, (cudaStream_t)stream>>>(
        *m, *f, FastDiv(L + 1));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_recover_large_step(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f,
                                        int rk_step, int ns, double rk_dt, void* stream) {
  if (!m || !c || !f || ns < 1) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const double inv_ns = 1.0 / (double)ns;
  if (c->precision == MPASG_PRECISION_MIXED)
    return launch_recover<float>(m, f, rk_step, inv_ns, rk_dt, s);
  return launch_recover<double>(m, f, rk_step, inv_ns, rk_dt, s);
}
