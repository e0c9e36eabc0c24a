// Reverse mode of the column stages: vertical implicit coefficients with their Thomas
// factorisation, the small-step perturbation, the acoustic substep (transposed Thomas
// solve inside), divergence damping and large-step recovery.
//
// Each kernel is the transpose of one forward kernel of kern_column.cu, written as a gather
// over the outputs that read the thread's input (vertical neighbours through the level
// index, horizontal ones through the transposed connectivity), so every cotangent is one
// deterministic sum.  Cotangents live in `g` under the forward field names; work holds the
// per-edge partial products a later cell gather reads.
#include "adj_common.cuh"

namespace {

__global__ void k_zero(double* __restrict__ p, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

__global__ void k_copy(double* __restrict__ d, const double* __restrict__ s, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = s[i];
}

// ---------------------------------------------------------------- vert_imp_coefs
// Thomas factorisation (alpha_k = 1 / (b_k - a_k gamma_(k-1)), gamma_k = c_k alpha_k) read
// backwards, one thread per column: alpha / gamma cotangents -> a (accumulated), b, c.
__global__ void k_vimp_factor_vjp(mpasg_mesh m, mpasg_fields f, mpasg_fields g, double* __restrict__ gb,
                                  double* __restrict__ gc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nCells) return;
  const int L = m.nVertLevels;
  const size_t o = (size_t)c * L;
  double carry = 0.0;
  for (int k = L - 1; k >= 1; --k) {
    const double ag = g.gamma_tri[o + k] + carry;
    const double al = f.alpha_tri[o + k];
    gc[o + k] = ag * al;
    const double tot = g.alpha_tri[o + k] + ag * f.c_tri[o + k];
    const double d = -tot * al * al;
    gb[o + k] = d;
    g.a_tri[o + k] += -d * f.gamma_tri[o + k - 1];
    carry = -d * f.a_tri[o + k];
  }
  gb[o] = 0.0;
  gc[o] = 0.0;
}

// The same with 32 columns staged through shared memory ([level][33] layout, coalesced
// copies by 4 warps, the sweeps on the first warp), as the forward factorisation does.
constexpr int kFacCols = 32;
constexpr int kFacPitch = kFacCols + 1;
constexpr int kFacThreads = 128;

__global__ void __launch_bounds__(kFacThreads) k_vimp_factor_vjp_staged(mpasg_mesh m, mpasg_fields f, mpasg_fields g,
                                                                        FastDiv fl, double* __restrict__ gb,
                                                                        double* __restrict__ gc) {
  extern __shared__ double sm[];
  const int L = m.nVertLevels;
  const size_t plane = (size_t)L * kFacPitch;
  double* s_gg = sm;              // gamma's cotangent in, c's out
  double* s_gal = sm + plane;     // alpha's cotangent in, b's out
  double* s_al = sm + 2 * plane;
  double* s_c = sm + 3 * plane;
  double* s_gam = sm + 4 * plane;
  double* s_a = sm + 5 * plane;
  double* s_ga = sm + 6 * plane;
  const int c0 = blockIdx.x * kFacCols;
  const int ncol = min(kFacCols, m.nCells - c0);
  const int t = threadIdx.x;
  const uint32_t nl = (uint32_t)ncol * L;
  const size_t o0 = (size_t)c0 * L;
  for (uint32_t idx = t; idx < nl; idx += kFacThreads) {
    const uint32_t col = fl.div(idx), k = idx - col * L;
    const size_t q = k * kFacPitch + col;
    s_gg[q] = g.gamma_tri[o0 + idx];
    s_gal[q] = g.alpha_tri[o0 + idx];
    s_al[q] = f.alpha_tri[o0 + idx];
    s_c[q] = f.c_tri[o0 + idx];
    s_gam[q] = f.gamma_tri[o0 + idx];
    s_a[q] = f.a_tri[o0 + idx];
    s_ga[q] = 0.0;
  }
  __syncthreads();
  if (t < ncol) {
    double carry = 0.0;
    for (int k = L - 1; k >= 1; --k) {
      const size_t q = k * kFacPitch + t;
      const double ag = s_gg[q] + carry;
      const double al = s_al[q];
      s_gg[q] = ag * al;
      const double d = -(s_gal[q] + ag * s_c[q]) * al * al;
      s_gal[q] = d;
      s_ga[q] = -d * s_gam[q - kFacPitch];
      carry = -d * s_a[q];
    }
    s_gg[t] = 0.0;
    s_gal[t] = 0.0;
  }
  __syncthreads();
  for (uint32_t idx = t; idx < nl; idx += kFacThreads) {
    const uint32_t col = fl.div(idx), k = idx - col * L;
    const size_t q = k * kFacPitch + col;
    gc[o0 + idx] = s_gg[q];
    gb[o0 + idx] = s_gal[q];
    g.a_tri[o0 + idx] += s_ga[q];
  }
}

size_t vimp_factor_vjp_smem_bytes(int L) { return (size_t)7 * L * kFacPitch * sizeof(double); }

// a / b / c diagonals (vert_imp_coefs.py:388-428) read backwards: total cotangents of
// cofwz (levels 1..L-1), coftz (0..L) and cofwt (0..L-1), written to wz / tz / wt.
__global__ void k_vimp_diag_vjp(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1,
                                const double* __restrict__ gb, const double* __restrict__ gc,
                                double* __restrict__ wz, double* __restrict__ tz, double* __restrict__ wt) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  auto in = [&](int q) { return q >= 1 && q <= L - 1; };
  auto ab = [&](int q) { return in(q) ? g.a_tri[o + q] : 0.0; };
  auto bb = [&](int q) { return in(q) ? gb[o + q] : 0.0; };
  auto cb = [&](int q) { return in(q) ? gc[o + q] : 0.0; };
  auto ctz = [&](int q) { return f.coftz[ow + q]; };
  auto cwz = [&](int q) { return f.cofwz[o + q]; };
  auto cwt = [&](int q) { return f.cofwt[o + q]; };
  auto zz = [&](int q) { return m.zz[o + q]; };
  auto rdzw = [&](int q) { return m.rdzw[q]; };
  // coftz at level k (0..L)
  double t = g.coftz[ow + k];
  if (in(k + 1)) t += ab(k + 1) * (-cwz(k + 1) * rdzw(k) * zz(k) - cwt(k) * rdzw(k));
  if (in(k)) t += bb(k) * (cwz(k) * (rdzw(k) * zz(k) + rdzw(k - 1) * zz(k - 1)) - (cwt(k) * rdzw(k) - cwt(k - 1) * rdzw(k - 1)));
  if (in(k - 1)) t += cb(k - 1) * (-cwz(k - 1) * rdzw(k - 1) * zz(k - 1) + cwt(k - 1) * rdzw(k - 1));
  tz[ow + k] = t;
  if (k == L) return;
  // cofwz at level k (1..L-1)
  double z = 0.0;
  if (in(k))
    z = g.cofwz[o + k] + ab(k) * (-ctz(k - 1) * rdzw(k - 1) * zz(k - 1)) +
        bb(k) * ctz(k) * (rdzw(k) * zz(k) + rdzw(k - 1) * zz(k - 1)) + cb(k) * (-ctz(k + 1) * rdzw(k) * zz(k));
  wz[o + k] = z;
  // cofwt at level k (0..L-1)
  double w = g.cofwt[o + k];
  if (in(k + 1)) w += ab(k + 1) * (-ctz(k) * rdzw(k)) + bb(k + 1) * (ctz(k + 1) * rdzw(k));
  if (in(k)) w += bb(k) * (-ctz(k) * rdzw(k)) + cb(k) * (ctz(k + 1) * rdzw(k));
  wt[o + k] = w;
}

// coefficients (vert_imp_coefs.py:343-386) read backwards: -> exner, theta_m, rtheta_p
__global__ void k_vimp_coef_vjp(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, double dts, double epssm,
                                const double* __restrict__ wz, const double* __restrict__ tz,
                                const double* __restrict__ wt) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  const double dtseps = 0.5 * dts * (1.0 + epssm);
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  auto fac = [&](int q) {  // d cofwz_q / d p_i
    const double z_i = m.fzm[q] * m.zz[o + q] + m.fzp[q] * m.zz[o + q - 1];
    return dtseps * c2 * z_i * m.rdzu[q] * f.cqw[ow + q];
  };
  double gp = 0.0, gt = 0.0;
  if (k >= 1) {
    gp += wz[o + k] * fac(k) * m.fzm[k];
    gt += tz[ow + k] * dtseps * m.fzm[k];
  }
  if (k + 1 <= L - 1) {
    gp += wz[o + k + 1] * fac(k + 1) * m.fzp[k + 1];
    gt += tz[ow + k + 1] * dtseps * m.fzp[k + 1];
  }
  const double q = f.qtot[o + k];
  const double x0 = 0.5 * dtseps * rcv * m.zz[o + k] * kGravity * m.rho_base[o + k];
  const double x = q == 0.0 ? x0 : x0 / (1.0 + q);  // dry columns: no division
  const double pb = f.exner_base[o + k];
  const double den = (f.rtheta_base[o + k] + f.rtheta_p[o + k]) * pb;
  const double w = wt[o + k];
  const double rden = 1.0 / den;
  gp += w * x * rden;
  g.exner[o + k] += gp;
  g.theta_m[o + k] += gt;
  g.rtheta_p[o + k] += w * (-x * f.exner[o + k] * pb * rden * rden);
}

// ---------------------------------------------------------------- small-step perturbation
// Over terrain, interior interface k of cell c: tend_rw = Z (tend_w - sum_j coef_j s_j
// (fzm tend_u[e_j][k] + fzp tend_u[e_j][k-1])), Z = fzm zz[k] + fzp zz[k-1], coef_j =
// zb + (tend_u[e_j][k] >= 0 ? 1 : -1) zb3 (smlstep_pert.py:197-373; the selection is
// constant).  Per edge level k: tend_u's cotangent from the interfaces k (fzm) and k+1
// (fzp) of both cells, read before k_smlstep_vjp consumes tend_rw's.  The sign of tend_u
// comes from up (1: >= 0) when given, else from tu.
__global__ void k_smlstep_vjp_slopes(mpasg_mesh m, mpasg_fields g, FastDiv fl, const double* __restrict__ tu,
                                     const uint8_t* __restrict__ up) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int me = m.maxEdges;
  double acc = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int c = m.cellsOnEdge[2 * e + s];
    if (c < 0 || c >= m.nCells) continue;
    const int j = cell_slot(m, c, (int)e);
    if (j < 0) continue;
    const double sign = m.edgesOnCell_sign[c * me + j];
    const size_t oc = (size_t)c * L, ow = (size_t)c * (L + 1);
    for (int kw = k; kw <= k + 1; ++kw) {
      if (kw < 1 || kw > L - 1) continue;
      const size_t ie = (size_t)e * L + kw;
      const bool pos = up ? up[ie] != 0 : tu[ie] >= 0.0;
      const size_t zi = ((size_t)c * me + j) * (L + 1) + kw;
      const double coef = m.zb_cell[zi] + (pos ? 1.0 : -1.0) * m.zb3_cell[zi];
      const double Z = m.fzm[kw] * m.zz[oc + kw] + m.fzp[kw] * m.zz[oc + kw - 1];
      const double wgt = kw == k ? m.fzm[kw] : m.fzp[kw];
      acc -= coef * sign * wgt * Z * g.tend_rw[ow + kw];
    }
  }
  g.tend_u[i] += acc;
}

// 1 where tend_u >= 0 (the slope coefficients' selection, kept for the reverse pass)
__global__ void k_nonneg_bytes(const double* __restrict__ x, uint8_t* __restrict__ b, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = x[i] >= 0.0 ? 1 : 0;
}

// tend_rw = Z tend_w at interior levels (Z = zz_i), tend_w itself at the ends
__global__ void k_smlstep_vjp(mpasg_mesh m, mpasg_fields g, FastDiv fl1) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t o = (size_t)c * L;
  double s = 1.0;
  if (k >= 1 && k <= L - 1) s = m.fzm[k] * m.zz[o + k] + m.fzp[k] * m.zz[o + k - 1];
  g.tend_w[i] += g.tend_rw[i] * s;
  g.tend_rw[i] = 0.0;
}

// ---------------------------------------------------------------- acoustic substep
// rho_pp / rtheta_pp from the solution, the ww accumulation and the implicit Rayleigh
// damping (k_ac_post) read backwards, per w level: -> x (cotangent of the undamped
// solution) in g.ac_x, rho_i's cotangent in rho_ib, and rw / rw_save / w / coftz.
__global__ void k_ac_vjp_post(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1, double dts,
                              double* __restrict__ rho_ib) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t o = (size_t)c * L + k;  // mass level k (valid for k < L)
  const size_t ow = i;
  const double sol2 = f.rw_p[ow];
  double sb = g.rw_p[ow];
  double gct = 0.0;
  if (k < L) {
    sb += g.rho_pp[o] * f.cofrz[k] + g.rtheta_pp[o] * m.rdzw[k] * f.coftz[ow];
    gct += g.rtheta_pp[o] * m.rdzw[k] * sol2;
  }
  if (k > 0) {
    sb -= g.rho_pp[o - 1] * f.cofrz[k - 1] + g.rtheta_pp[o - 1] * m.rdzw[k - 1] * f.coftz[ow];
    gct -= g.rtheta_pp[o - 1] * m.rdzw[k - 1] * sol2;
  }
  g.coftz[ow] += gct;
  double xb = sb, rib = 0.0;
  if (k >= 1 && k <= L - 1) {
    const double dss = m.dss[o];
    const double den = 1.0 + dts * dss;
    const double zz_i = m.fzm[k] * m.zz[o] + m.fzp[k] * m.zz[o - 1];
    const double rho_i = m.fzm[k] * f.rho_zz[o] + m.fzp[k] * f.rho_zz[o - 1];
    xb = den == 1.0 ? sb : sb / den;
    const double rwdb = xb - sb;
    g.rw_save[ow] += rwdb;
    g.rw[ow] -= rwdb;
    g.w[ow] += xb * (-dts * dss * zz_i * rho_i);
    rib = xb * (-dts * dss * zz_i * f.w[ow]);
  }
  g.ac_x[ow] = xb;
  rho_ib[ow] = rib;
}

// Thomas sweeps (autodiff/tridiagonal_solve.py:232-291) transposed for one column: xb
// holds the solution's cotangent on entry and the right-hand side's on return; the a, alpha
// and gamma cotangents accumulate into ga / gal / gg.  The forward-elimination values come
// back from the solution: u_k = x_k + gamma_k x_(k+1) and t_k = rhs_k - a_k u_(k-1) = u_k / alpha_k,
// with 1 / alpha_k by the Newton-refined reciprocal (common.cuh; within 2 ulp, no division).
// Strides: xs / xbs for the (L+1)-level arrays, cs for the L-level ones.
MPASG_D void solve_vjp_column(int L, const double* x, int xs, double* xb, int xbs, const double* a,
                              const double* al, const double* gam, int cs, double* ga, double* gal, double* gg) {
  double prev = 0.0;
  for (int k = 0; k <= L; ++k) {
    const double au = xb[k * xbs] - (k > 0 ? gam[(k - 1) * cs] * prev : 0.0);
    if (k < L) gg[k * cs] += -au * x[(k + 1) * xs];
    xb[k * xbs] = au;
    prev = au;
  }
  double carry = 0.0;
  for (int k = L - 1; k >= 1; --k) {
    const double au = xb[k * xbs] + carry;
    const double u_k = x[k * xs] + gam[k * cs] * x[(k + 1) * xs];
    const double u_km1 = x[(k - 1) * xs] + gam[(k - 1) * cs] * x[k * xs];
    gal[k * cs] += au * (u_k * rcp_nr(al[k * cs]));
    const double at = au * al[k * cs];
    xb[k * xbs] = at;
    ga[k * cs] += -at * u_km1;
    carry = -at * a[k * cs];
  }
  xb[0] += carry;
}

// one thread per column, straight from global memory (fallback when the staged kernel's
// shared memory does not fit)
__global__ void k_ac_vjp_solve(mpasg_mesh m, mpasg_fields f, mpasg_fields g) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nCells) return;
  const int L = m.nVertLevels;
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  solve_vjp_column(L, f.ac_x + ow, 1, g.ac_x + ow, 1, f.a_tri + o, f.alpha_tri + o, f.gamma_tri + o, 1,
                   g.a_tri + o, g.alpha_tri + o, g.gamma_tri + o);
}

// The same with 32 columns staged through shared memory ([level][33] layout, coalesced
// copies by 4 warps, the sweeps on the first warp), as the forward Thomas kernels do.
constexpr int kSolveCols = 32;
constexpr int kSolvePitch = kSolveCols + 1;
constexpr int kSolveThreads = 128;

__global__ void __launch_bounds__(kSolveThreads) k_ac_vjp_solve_staged(mpasg_mesh m, mpasg_fields f, mpasg_fields g,
                                                                       FastDiv fl, FastDiv fl1) {
  extern __shared__ double sm[];
  const int L = m.nVertLevels;
  double* sx = sm;                                   // (L+1) x pitch: the solution x
  double* sb = sx + (size_t)(L + 1) * kSolvePitch;   // (L+1) x pitch: xb in, the rhs cotangent out
  double* s1 = sb + (size_t)(L + 1) * kSolvePitch;   // (L+1) x pitch: first sweep's values
  double* sa = s1 + (size_t)(L + 1) * kSolvePitch;   // L x pitch each below
  double* sal = sa + (size_t)L * kSolvePitch;
  double* sg = sal + (size_t)L * kSolvePitch;
  double* s2 = sg + (size_t)L * kSolvePitch;         // second sweep's values before the alpha scaling
  const int c0 = blockIdx.x * kSolveCols;
  const int ncol = min(kSolveCols, m.nCells - c0);
  const int t = threadIdx.x;
  const uint32_t nw = (uint32_t)ncol * (L + 1), nl = (uint32_t)ncol * L;
  const size_t ow0 = (size_t)c0 * (L + 1), o0 = (size_t)c0 * L;
  for (uint32_t idx = t; idx < nw; idx += kSolveThreads) {
    const uint32_t col = fl1.div(idx), k = idx - col * (L + 1);
    sx[k * kSolvePitch + col] = f.ac_x[ow0 + idx];
    sb[k * kSolvePitch + col] = g.ac_x[ow0 + idx];
  }
  for (uint32_t idx = t; idx < nl; idx += kSolveThreads) {
    const uint32_t col = fl.div(idx), k = idx - col * L;
    sa[k * kSolvePitch + col] = f.a_tri[o0 + idx];
    sal[k * kSolvePitch + col] = f.alpha_tri[o0 + idx];
    sg[k * kSolvePitch + col] = f.gamma_tri[o0 + idx];
  }
  __syncthreads();
  // the two sweeps keep only their recurrences (solve_vjp_column's order of operations):
  // au_k = xb_k - gamma_(k-1) au_(k-1) upwards, then au'_k = au_k + carry, xb_k = au'_k alpha_k,
  // carry = -xb_k a_k downwards; the cotangents of a, alpha, gamma follow in parallel
  if (t < ncol) {
    double prev = 0.0;
    for (int k = 0; k <= L; ++k) {
      const double au = sb[k * kSolvePitch + t] - (k > 0 ? sg[(k - 1) * kSolvePitch + t] * prev : 0.0);
      s1[k * kSolvePitch + t] = au;
      prev = au;
    }
    double carry = 0.0;
    for (int k = L - 1; k >= 1; --k) {
      const double au = s1[k * kSolvePitch + t] + carry;
      s2[k * kSolvePitch + t] = au;
      const double at = au * sal[k * kSolvePitch + t];
      sb[k * kSolvePitch + t] = at;
      carry = -at * sa[k * kSolvePitch + t];
    }
    sb[L * kSolvePitch + t] = s1[L * kSolvePitch + t];
    sb[t] = s1[t] + carry;
  }
  __syncthreads();
  for (uint32_t idx = t; idx < nw; idx += kSolveThreads) {
    const uint32_t col = fl1.div(idx), k = idx - col * (L + 1);
    g.ac_x[ow0 + idx] = sb[k * kSolvePitch + col];
  }
  for (uint32_t idx = t; idx < nl; idx += kSolveThreads) {
    const uint32_t col = fl.div(idx), k = idx - col * L;
    const size_t q = k * kSolvePitch + col;
    const double xk1 = sx[q + kSolvePitch];
    g.gamma_tri[o0 + idx] += -s1[q] * xk1;
    if (k >= 1) {
      const double u_k = sx[q] + sg[q] * xk1;
      const double u_km1 = sx[q - kSolvePitch] + sg[q - kSolvePitch] * sx[q];
      const double au = s2[q];
      g.alpha_tri[o0 + idx] += au * (u_k * rcp_nr(sal[q]));
      g.a_tri[o0 + idx] += -(au * sal[q]) * u_km1;
    }
  }
}

size_t solve_vjp_smem_bytes(int L) { return (size_t)(3 * (L + 1) + 4 * L) * kSolvePitch * sizeof(double); }

// The tridiagonal right-hand side (acoustic_step.py:675) and rs / ts read backwards, per
// mass level: -> tend_theta, tend_rho, cofwz, cofwt, the rs / ts cotangents (rsb, tsb), the
// input perturbations rho_pp / rtheta_pp (consumed and rewritten) and rho_zz through the
// Rayleigh term's interface density.
__global__ void k_ac_vjp_cells(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, int first, double dts,
                               double resm, const double* __restrict__ rt_in, const double* __restrict__ rho_ib,
                               double* __restrict__ rsb_out, double* __restrict__ tsb_out) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const size_t oc = (size_t)c * L, ow = (size_t)c * (L + 1);
  const size_t o = oc + k;
  auto r = [&](int q) { return (q >= 1 && q <= L - 1) ? g.ac_x[ow + q] : 0.0; };
  auto ts = [&](int q) { return f.ac_ts[oc + q]; };
  auto rti = [&](int q) { return first ? 0.0 : rt_in[oc + q]; };
  auto zz = [&](int q) { return m.zz[oc + q]; };
  double tsb = g.rtheta_pp[o], rsb = g.rho_pp[o], rtinb = 0.0, rhoinb = 0.0, gwt = 0.0;
  if (k >= 1) {
    const double rm = r(k);
    const double cwz = f.cofwz[o], cwt = f.cofwt[o], cwr = f.cofwr[o];
    tsb += rm * (cwt - cwz * zz(k));
    rtinb += rm * resm * (cwt - cwz * zz(k));
    rsb += -rm * cwr;
    rhoinb += -rm * cwr * resm;
    g.cofwz[o] += -rm * ((zz(k) * ts(k) - zz(k - 1) * ts(k - 1)) + resm * (zz(k) * rti(k) - zz(k - 1) * rti(k - 1)));
    gwt += rm * (ts(k) + resm * rti(k));
  }
  if (k + 1 <= L - 1) {
    const double r1 = r(k + 1);
    const double cwz1 = f.cofwz[o + 1], cwt = f.cofwt[o], cwr1 = f.cofwr[o + 1];
    tsb += r1 * (cwz1 * zz(k) + cwt);
    rtinb += r1 * resm * (cwz1 * zz(k) + cwt);
    rsb += -r1 * cwr1;
    rhoinb += -r1 * cwr1 * resm;
    gwt += r1 * (ts(k) + resm * rti(k));
  }
  g.cofwt[o] += gwt;
  rtinb += tsb;
  rhoinb += rsb;
  g.tend_theta[o] += dts * tsb;
  g.tend_rho[o] += dts * rsb;
  rsb_out[o] = rsb;
  tsb_out[o] = tsb;
  double grz = 0.0;
  if (k >= 1) grz += m.fzm[k] * rho_ib[ow + k];
  if (k + 1 <= L - 1) grz += m.fzp[k + 1] * rho_ib[ow + k + 1];
  g.rho_zz[o] += grz;
  if (first) {
    g.rho_pp[o] = 0.0;
    g.rtheta_pp[o] = 0.0;
  } else {
    g.rho_pp[o] = rhoinb;
    g.rtheta_pp[o] = rtinb + g.rtheta_pp_old[o];
  }
  g.rtheta_pp_old[o] = 0.0;
}

// the input rw_p's cotangent (right-hand side and rs / ts), tend_rw and coftz, per w level
__global__ void k_ac_vjp_wlev(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1, int first, double dts,
                              double resm, const double* __restrict__ rwp_in, const double* __restrict__ rsb,
                              const double* __restrict__ tsb) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  const size_t oc = (size_t)c * L;
  const double rb = g.ac_x[i];
  const double rwp = first ? 0.0 : rwp_in[i];
  const double ct = f.coftz[i];
  double rwpb = rb, gct = 0.0;
  if (k < L) {
    rwpb += rsb[oc + k] * f.cofrz[k] * resm + tsb[oc + k] * resm * m.rdzw[k] * ct;
    gct += tsb[oc + k] * resm * m.rdzw[k] * rwp;
  }
  if (k > 0) {
    rwpb -= rsb[oc + k - 1] * f.cofrz[k - 1] * resm + tsb[oc + k - 1] * resm * m.rdzw[k - 1] * ct;
    gct -= tsb[oc + k - 1] * resm * m.rdzw[k - 1] * rwp;
  }
  g.coftz[i] += gct;
  if (k >= 1 && k <= L - 1) g.tend_rw[i] += dts * rb;
  g.rw_p[i] = first ? 0.0 : rwpb;
}

// edge update ru_p += dts (tend_u - pgrad) and the cell flux sums' edge terms read
// backwards, per edge level: -> ru_p (input), tend_u, theta_edge_save (edge-sum cotangent),
// and the pressure-gradient partials pex / prt / prho that the cell gather collects.
__global__ void k_ac_vjp_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields g, mpasg_transpose t, FastDiv fl, int first,
                               double dts, double c2, const double* __restrict__ rsb, const double* __restrict__ tsb,
                               const double* __restrict__ rt_in, double* __restrict__ pex, double* __restrict__ prt,
                               double* __restrict__ prho) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int me = m.maxEdges;
  double gnew = g.ru_p[i];
  const double the = f.theta_edge_save[i], rupn = f.ru_p[i];
  double sth = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int j = t.edgeCellSlot[2 * e + s];
    if (j < 0) continue;
    const int c = m.cellsOnEdge[2 * e + s];
    const double wgt = dts * m.cell_edge_geo[(size_t)c * me + j];
    const size_t oc = (size_t)c * L + k;
    gnew += -(rsb[oc] + tsb[oc] * the) * wgt;
    sth += -tsb[oc] * wgt * rupn;
  }
  g.theta_edge_save[i] += 0.5 * sth;
  g.tend_u[i] += dts * gnew;
  if (first) {
    g.ru_p[i] = 0.0;
    return;
  }
  g.ru_p[i] = gnew;
  const double pg = -dts * gnew;
  const int c1 = m.cellsOnEdge[2 * e], c2i = m.cellsOnEdge[2 * e + 1];
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2i * L + k;
  const double den = 0.5 * (m.zz[i2] + m.zz[i1]);
  const double rden = den == 1.0 ? 1.0 : 1.0 / den;  // one division for both terms
  const double d = (rt_in[i2] - rt_in[i1]) * m.invDcEdge[e];
  const double pg1 = den == 1.0 ? d : d * rden;
  const double exs = f.exner[i1] + f.exner[i2];
  const double cqu = f.cqu_e[i];
  pex[i] = pg * cqu * 0.5 * c2 * pg1;
  const double pe = pg * cqu * 0.5 * c2 * exs;
  prt[i] = (den == 1.0 ? pe : pe * rden) * m.invDcEdge[e];
  prho[i] = pg * 0.5 * m.zxu[i] * kGravity;
}

// the pressure-gradient partials gathered on the cells: exner, rtheta_pp, rho_pp
__global__ void k_ac_vjp_pgrad_cells(mpasg_mesh m, mpasg_fields g, FastDiv fl, const double* __restrict__ pex,
                                     const double* __restrict__ prt, const double* __restrict__ prho) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double ge = 0.0, gr = 0.0, gp = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const size_t ie = (size_t)e * L + k;
    ge += pex[ie];
    gr += cell_side(m, e, (int)c) ? prt[ie] : -prt[ie];
    gp += prho[ie];
  }
  g.exner[i] += ge;
  g.rtheta_pp[i] += gr;
  g.rho_pp[i] += gp;
}

// ---------------------------------------------------------------- divergence damping
__global__ void k_divdamp_vjp_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, double coef,
                                    double* __restrict__ pd) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  const size_t i1 = (size_t)c1 * L + k, i2 = (size_t)c2 * L + k;
  const double G = g.ru_p[i];
  const double rs = f.theta_edge_rsum[i];
  const double d1 = -(f.rtheta_pp[i1] - f.rtheta_pp_old[i1]);
  const double d2 = -(f.rtheta_pp[i2] - f.rtheta_pp_old[i2]);
  pd[i] = G * coef * rs;
  g.theta_edge_save[i] += -G * coef * (d2 - d1) * rs * rs;
}

__global__ void k_divdamp_vjp_cells(mpasg_mesh m, mpasg_fields g, FastDiv fl, const double* __restrict__ pd) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  double a = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.edgesOnCell[c * me + j];
    const double p = pd[(size_t)e * L + k];
    a += cell_side(m, e, (int)c) ? -p : p;
  }
  g.rtheta_pp[i] += a;
  g.rtheta_pp_old[i] -= a;
}

// ---------------------------------------------------------------- large-step recovery
// Over terrain, w at interior interface k of cell c is (wo + sum_j s_j c_j fi_j) / R with
// fi_j = fzm ru[e_j][k] + fzp ru[e_j][k-1], c_j = zb + sgn(fi_j) zb3 (a constant selection),
// and at the surface w_0 = sum_j s_j cs_j fs_j / (cf1 rho_0 + cf2 rho_1 + cf3 rho_2), fs_j =
// cf1 ru[e_j][0] + cf2 ru[e_j][1] + cf3 ru[e_j][2] (recover_large_step.py:329-411).  pw
// holds the cotangent of each interface's numerator (k_recover_vjp_wlev); edge level k
// reads interfaces k (fzm), k+1 (fzp) and, for k < 3, the surface (cf_(k+1)) of both cells.
MPASG_D double recover_slope_cotangent(const mpasg_mesh& m, const mpasg_fields& f, const double* __restrict__ pw,
                                       uint32_t e, int k) {
  const int L = m.nVertLevels, me = m.maxEdges;
  const double* ru = f.ru + (size_t)e * L;
  double acc = 0.0;
  for (int s = 0; s < 2; ++s) {
    const int c = m.cellsOnEdge[2 * e + s];
    if (c < 0 || c >= m.nCells) continue;
    const int j = cell_slot(m, c, (int)e);
    if (j < 0) continue;
    const double sign = m.edgesOnCell_sign[c * me + j];
    const size_t ow = (size_t)c * (L + 1), zb0 = ((size_t)c * me + j) * (L + 1);
    for (int kw = k; kw <= k + 1; ++kw) {
      if (kw < 1 || kw > L - 1) continue;
      const double fi = m.fzm[kw] * ru[kw] + m.fzp[kw] * ru[kw - 1];
      const double ci = m.zb_cell[zb0 + kw] + sgn(fi) * m.zb3_cell[zb0 + kw];
      acc += pw[ow + kw] * sign * ci * (kw == k ? m.fzm[kw] : m.fzp[kw]);
    }
    if (k < 3) {
      const double fs = m.cf1 * ru[0] + m.cf2 * ru[1] + m.cf3 * ru[2];
      const double cs = m.zb_cell[zb0] + sgn(fs) * m.zb3_cell[zb0];
      acc += pw[ow] * sign * cs * (k == 0 ? m.cf1 : (k == 1 ? m.cf2 : m.cf3));
    }
  }
  return acc;
}

__global__ void k_recover_vjp_edges(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl,
                                    double* __restrict__ pden, const double* __restrict__ pw) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nEdges * L) return;
  const uint32_t e = fl.div(i);
  const int k = (int)(i - e * L);
  const int c1 = m.cellsOnEdge[2 * e], c2 = m.cellsOnEdge[2 * e + 1];
  // one reciprocal of the edge density sum (float64 division is a long instruction sequence)
  const double rden = 1.0 / (f.rho_zz[(size_t)c1 * L + k] + f.rho_zz[(size_t)c2 * L + k]);
  const double gu = g.u[i];
  double gru = g.ru[i] + gu * 2.0 * rden;
  if (pw) gru += recover_slope_cotangent(m, f, pw, e, k);
  g.ru_save[i] += gru;
  g.ru_p[i] += gru;
  pden[i] = -gu * f.u[i] * rden;
  g.u[i] = 0.0;
  g.ru[i] = 0.0;
}

// pw (terrain only, else null): the cotangent of each interface's numerator for the
// slope terms of k_recover_vjp_edges; rho_ib at the surface slot: the cotangent of the
// surface denominator cf1 rho_0 + cf2 rho_1 + cf3 rho_2
__global__ void k_recover_vjp_wlev(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl1,
                                   double* __restrict__ rho_ib, double* __restrict__ pw) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * (L + 1)) return;
  const uint32_t c = fl1.div(i);
  const int k = (int)(i - c * (L + 1));
  double rib = 0.0, rwpb = 0.0, num = 0.0;
  if (k >= 1 && k <= L - 1) {
    const size_t o = (size_t)c * L + k;
    const double gw = g.w[i];
    const double rho_i = m.fzm[k] * f.rho_zz[o] + m.fzp[k] * f.rho_zz[o - 1];
    const double zz_i = m.fzm[k] * m.zz[o] + m.fzp[k] * m.zz[o - 1];
    const double wmb = gw / rho_i;
    rib = -wmb * f.w[i];
    rwpb = (zz_i == 1.0 ? wmb : wmb / zz_i) + g.rw[i];
    g.rw_save[i] += rwpb;
    num = wmb;
  } else if (k == 0 && pw) {
    const size_t o = (size_t)c * L;
    const double den = m.cf1 * f.rho_zz[o] + m.cf2 * f.rho_zz[o + 1] + m.cf3 * f.rho_zz[o + 2];
    num = g.w[i] / den;
    rib = -num * f.w[i];
  }
  if (pw) pw[i] = num;
  g.rw_p[i] += rwpb;
  rho_ib[i] = rib;
  g.w[i] = 0.0;
  g.rw[i] = 0.0;
}

__global__ void k_recover_vjp_cells(mpasg_mesh m, mpasg_fields f, mpasg_fields g, FastDiv fl, int rk_step,
                                    double rk_dt, const double* __restrict__ pden, const double* __restrict__ rho_ib) {
  const int L = m.nVertLevels;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)m.nCells * L) return;
  const uint32_t c = fl.div(i);
  const int k = (int)(i - c * L);
  const size_t o = i, ow = (size_t)c * (L + 1) + k;
  const double rz = f.rho_zz[o], th = f.theta_m[o], rtp = f.rtheta_p[o], rtb = f.rtheta_base[o];
  const double gth = g.theta_m[o];
  const double gthr = gth / rz;
  double rtpb = g.rtheta_p[o] + gthr;
  if (rk_step == 3) {
    const double rcv = kRgas / (kCp - kRgas);
    const double zz = m.zz[o], ex = f.exner[o];
    const double gp = g.pressure_p[o];
    const double gex = g.exner[o] + gp * zz * kRgas * (rtp + rtb);
    const double E = zz * (kRgas / kP0) * (rtp + rtb);
    rtpb += gp * zz * kRgas * ex + gex * rcv * ex * (zz * (kRgas / kP0) / E);
    g.exner[o] = 0.0;
    g.pressure_p[o] = 0.0;
  }
  double rzb = g.rho_zz[o] - gthr * th;
  const int me = m.maxEdges;
  const int n = m.nEdgesOnCell[c];
  for (int j = 0; j < n; ++j) rzb += pden[(size_t)m.edgesOnCell[c * me + j] * L + k];
  if (k >= 1) rzb += m.fzm[k] * rho_ib[ow];
  if (k + 1 <= L - 1) rzb += m.fzp[k + 1] * rho_ib[ow + 1];
  if (!m.flatTerrain && k < 3) rzb += (k == 0 ? m.cf1 : (k == 1 ? m.cf2 : m.cf3)) * rho_ib[(size_t)c * (L + 1)];
  if (rk_step == 3) rzb += -rtpb * rk_dt * f.rt_diabatic_tend[o];
  g.rtheta_p_save[o] += rtpb;
  g.rtheta_pp[o] += rtpb;
  const double rpb = g.rho_p[o] + rzb;
  g.rho_p_save[o] += rpb;
  g.rho_pp[o] += rpb;
  g.rho_zz[o] = 0.0;
  g.theta_m[o] = 0.0;
  g.rtheta_p[o] = 0.0;
  g.rho_p[o] = 0.0;
}

int zero(double* p, long long n, cudaStream_t s) {
  if (n <= 0) return MPASG_OK;
  k_zero<<<nblocks(n), kBlock, 0, s>>>(p, n);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

int dcopy(double* d, const double* src, long long n, cudaStream_t s) {
  if (n <= 0) return MPASG_OK;
  k_copy<<<nblocks(n), kBlock, 0, s>>>(d, src, n);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

#define CHECK_RC(x)                  \
  do {                               \
    int _rc = (x);                   \
    if (_rc != MPASG_OK) return _rc; \
  } while (0)

}  // namespace

int mpasgi_zero(double* p, long long n, cudaStream_t s) { return zero(p, n, s); }

int mpasgi_nonneg_bytes(const double* x, uint8_t* b, long long n, cudaStream_t s) {
  if (n <= 0) return MPASG_OK;
  k_nonneg_bytes<<<nblocks(n), kBlock, 0, s>>>(x, b, n);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

namespace {
struct ZeroList {
  double* p[kZeroSpans];
  long long n[kZeroSpans];
};
// blockIdx.y picks the array; a grid-stride loop over its length
__global__ void k_zero_many(ZeroList z) {
  double* p = z.p[blockIdx.y];
  const long long n = z.n[blockIdx.y];
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = 0.0;
}
}  // namespace

int mpasgi_zero_many(const ZeroSpan* spans, int count, cudaStream_t s) {
  for (int b = 0; b < count; b += kZeroSpans) {
    ZeroList z{};
    long long nmax = 0;
    const int k = count - b < kZeroSpans ? count - b : kZeroSpans;
    for (int j = 0; j < k; ++j) {
      z.p[j] = spans[b + j].p;
      z.n[j] = spans[b + j].n;
      if (z.n[j] > nmax) nmax = z.n[j];
    }
    if (nmax <= 0) continue;
    long long gx = (nmax + kBlock - 1) / kBlock;
    if (gx > 1216) gx = 1216;  // 8 blocks per SM of 152, grid-stride beyond
    k_zero_many<<<dim3((unsigned)gx, (unsigned)k), kBlock, 0, s>>>(z);
    MPASG_LAUNCH_CHECK();
  }
  return MPASG_OK;
}

// ================================================================= internal cores
// The acoustic substep's forward pass for its reverse mode: keeps the substep's inputs
// (rho_pp, rtheta_pp, rw_p) in the work buffer, then leaves f as the forward substep does (ru_p, rho_pp, rtheta_pp, rtheta_pp_old, rw_p
// updated; ac_rs / ac_ts / ac_x hold rs, ts and the undamped solution).
int mpasgi_acoustic_vjp_fwd(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int small_step, double dts,
                            const AdjWork& w, cudaStream_t s) {
  const int L = m->nVertLevels;
  const long long ncl = (long long)m->nCells * L;
  const long long ncw = (long long)m->nCells * (L + 1);
  CHECK_RC(dcopy(w.c[0], f->rho_pp, ncl, s));
  CHECK_RC(dcopy(w.c[1], f->rtheta_pp, ncl, s));
  CHECK_RC(dcopy(w.c[2], f->rw_p, ncw, s));
  return mpasgi_acoustic_parts(m, c, f, small_step, dts, s, -1);
}

// The reverse pass proper (after mpasgi_acoustic_vjp_fwd on the same f and work).
int mpasgi_acoustic_vjp_rev(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                            const mpasg_transpose* t, int small_step, double dts, const double* rt_in,
                            const double* rwp_in, const AdjWork& w, cudaStream_t s) {
  const int L = m->nVertLevels;
  const long long ncl = (long long)m->nCells * L, nel = (long long)m->nEdges * L;
  const long long ncw = (long long)m->nCells * (L + 1);
  const bool first = small_step == 1;
  double* rho_ib = w.c[4];
  double* rsb = w.c[5];
  double* tsb = w.c[6];
  const double rcv = kRgas / (kCp - kRgas);
  const double c2 = kCp * rcv;
  const double resm = (1.0 - c->epssm) / (1.0 + c->epssm);
  FastDiv fl(L), fl1(L + 1);
  k_ac_vjp_post<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *g, fl1, dts, rho_ib);
  MPASG_LAUNCH_CHECK();
  // the staged solve needs more than 48 KB of dynamic shared memory: opt in once per device
  // (the first call on a device should come before any stream capture)
  const size_t smem = solve_vjp_smem_bytes(L);
  static bool opt_in[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MPASG_E_CUDA;
  if (!opt_in[dev])
    opt_in[dev] = cudaFuncSetAttribute(k_ac_vjp_solve_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       200 * 1024) == cudaSuccess;
  if (opt_in[dev] && smem <= 200 * 1024)
    k_ac_vjp_solve_staged<<<nblocks(m->nCells, kSolveCols), kSolveThreads, smem, s>>>(*m, *f, *g, fl, fl1);
  else
    k_ac_vjp_solve<<<nblocks(m->nCells, 64), 64, 0, s>>>(*m, *f, *g);
  MPASG_LAUNCH_CHECK();
  k_ac_vjp_cells<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, *g, fl, first ? 1 : 0, dts, resm, rt_in, rho_ib, rsb, tsb);
  MPASG_LAUNCH_CHECK();
  k_ac_vjp_wlev<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *g, fl1, first ? 1 : 0, dts, resm, rwp_in, rsb, tsb);
  MPASG_LAUNCH_CHECK();
  k_ac_vjp_edges<<<nblocks(nel), kBlock, 0, s>>>(*m, *f, *g, *t, fl, first ? 1 : 0, dts, c2, rsb, tsb, rt_in,
                                                 w.e[1], w.e[2], w.e[3]);
  MPASG_LAUNCH_CHECK();
  if (!first) {
    k_ac_vjp_pgrad_cells<<<nblocks(ncl), kBlock, 0, s>>>(*m, *g, fl, w.e[1], w.e[2], w.e[3]);
    MPASG_LAUNCH_CHECK();
  }
  return MPASG_OK;
}

int mpasgi_acoustic_vjp_core(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                             const mpasg_transpose* t, int small_step, double dts, const AdjWork& w,
                             cudaStream_t s) {
  CHECK_RC(mpasgi_acoustic_vjp_fwd(m, c, f, small_step, dts, w, s));
  return mpasgi_acoustic_vjp_rev(m, c, f, g, t, small_step, dts, w.c[1], w.c[2], w, s);
}

int mpasgi_divdamp_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                            double dts, const AdjWork& w, cudaStream_t s) {
  const int L = m->nVertLevels;
  const double coef = 2.0 * c->smdiv * c->len_disp / dts;
  FastDiv fl(L);
  k_divdamp_vjp_edges<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *g, fl, coef, w.e[4]);
  MPASG_LAUNCH_CHECK();
  k_divdamp_vjp_cells<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *g, fl, w.e[4]);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

int mpasgi_recover_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                            int rk_step, double rk_dt, const AdjWork& w, cudaStream_t s) {
  (void)c;
  const int L = m->nVertLevels;
  FastDiv fl(L), fl1(L + 1);
  double* pw = m->flatTerrain ? nullptr : w.c[8];  // slope terms: numerator cotangents
  k_recover_vjp_wlev<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, s>>>(*m, *f, *g, fl1, w.c[7], pw);
  MPASG_LAUNCH_CHECK();
  k_recover_vjp_edges<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *f, *g, fl, w.e[5], pw);
  MPASG_LAUNCH_CHECK();
  k_recover_vjp_cells<<<nblocks((long long)m->nCells * L), kBlock, 0, s>>>(*m, *f, *g, fl, rk_step, rk_dt, w.e[5],
                                                                          w.c[7]);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

int mpasgi_vimp_vjp_core(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                         double dts, const AdjWork& w, cudaStream_t s) {
  const int L = m->nVertLevels;
  const long long ncl = (long long)m->nCells * L, ncw = (long long)m->nCells * (L + 1);
  double* gb = w.c[8];
  double* gc = w.c[9];
  // the staged kernel needs more than 48 KB of dynamic shared memory: opt in once per device
  // (the first call on a device should come before any stream capture)
  const size_t smem = vimp_factor_vjp_smem_bytes(L);
  static bool opt_in[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MPASG_E_CUDA;
  if (!opt_in[dev])
    opt_in[dev] = cudaFuncSetAttribute(k_vimp_factor_vjp_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       200 * 1024) == cudaSuccess;
  if (opt_in[dev] && smem <= 200 * 1024)
    k_vimp_factor_vjp_staged<<<nblocks(m->nCells, kFacCols), kFacThreads, smem, s>>>(*m, *f, *g, FastDiv(L), gb, gc);
  else
    k_vimp_factor_vjp<<<nblocks(m->nCells, 64), 64, 0, s>>>(*m, *f, *g, gb, gc);
  MPASG_LAUNCH_CHECK();
  k_vimp_diag_vjp<<<nblocks(ncw), kBlock, 0, s>>>(*m, *f, *g, FastDiv(L + 1), gb, gc, w.c[10], w.c[11], w.c[7]);
  MPASG_LAUNCH_CHECK();
  k_vimp_coef_vjp<<<nblocks(ncl), kBlock, 0, s>>>(*m, *f, *g, FastDiv(L), dts, c->epssm, w.c[10], w.c[11], w.c[7]);
  MPASG_LAUNCH_CHECK();
  // the coefficients' cotangents are consumed
  const ZeroSpan zs[] = {{g->cofwz, ncl}, {g->coftz, ncw}, {g->cofwt, ncl},
                         {g->a_tri, ncl}, {g->alpha_tri, ncl}, {g->gamma_tri, ncl}};
  CHECK_RC(mpasgi_zero_many(zs, 6, s));
  return MPASG_OK;
}

int mpasgi_smlstep_vjp_core(const mpasg_mesh* m, const double* tu, const uint8_t* up, mpasg_fields* g,
                            cudaStream_t s) {
  const int L = m->nVertLevels;
  if (!m->flatTerrain) {
    if (!tu && !up) return MPASG_E_ARG;
    k_smlstep_vjp_slopes<<<nblocks((long long)m->nEdges * L), kBlock, 0, s>>>(*m, *g, FastDiv(L), tu, up);
    MPASG_LAUNCH_CHECK();
  }
  k_smlstep_vjp<<<nblocks((long long)m->nCells * (L + 1)), kBlock, 0, s>>>(*m, *g, FastDiv(L + 1));
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

// ================================================================= C ABI
extern "C" long long mpasg_dyn_vjp_work_doubles(const mpasg_mesh* m) {
  if (!m) return -1;
  return adj_work_doubles(m);
}

extern "C" int mpasg_vimp_vjp(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                              double dts, double* work, void* stream) {
  if (!m || !c || !f || !g || !work || !adj_supported(m, c)) return MPASG_E_ARG;
  return mpasgi_vimp_vjp_core(m, c, f, g, dts, adj_work(m, work), (cudaStream_t)stream);
}

extern "C" int mpasg_smlstep_vjp(const mpasg_mesh* m, const mpasg_config* c, const mpasg_fields* f, mpasg_fields* g,
                                 void* stream) {
  if (!m || !c || !f || !g || !adj_supported(m, c)) return MPASG_E_ARG;
  return mpasgi_smlstep_vjp_core(m, f->tend_u, nullptr, g, (cudaStream_t)stream);
}

extern "C" int mpasg_acoustic_vjp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                                  const mpasg_transpose* t, int small_step, double dts, double* work, void* stream) {
  if (!m || !c || !f || !g || !t || !work || small_step < 1 || !adj_supported(m, c) ||
      c->precision != MPASG_PRECISION_FLOAT64)
    return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  CHECK_RC(mpasgi_theta_edge(m, f, false, s));
  return mpasgi_acoustic_vjp_core(m, c, f, g, t, small_step, dts, adj_work(m, work), s);
}

extern "C" int mpasg_divdamp_vjp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                                 double dts, double* work, void* stream) {
  if (!m || !c || !f || !g || !work || !adj_supported(m, c)) return MPASG_E_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  CHECK_RC(mpasgi_theta_edge(m, f, false, s));
  return mpasgi_divdamp_vjp_core(m, c, f, g, dts, adj_work(m, work), s);
}

extern "C" int mpasg_recover_vjp(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, mpasg_fields* g,
                                 int rk_step, int ns, double rk_dt, double* work, void* stream) {
  if (!m || !c || !f || !g || !work || ns < 1 || !adj_supported(m, c) || c->precision != MPASG_PRECISION_FLOAT64)
    return MPASG_E_ARG;
  CHECK_RC(mpasg_recover_large_step(m, c, f, rk_step, ns, rk_dt, stream));
  return mpasgi_recover_vjp_core(m, c, f, g, rk_step, rk_dt, adj_work(m, work), (cudaStream_t)stream);
}
