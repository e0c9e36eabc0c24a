// Derivatives of the column tridiagonal operators (the reference's custom autograd
// Functions TridiagonalSolve, mpas_pytorch/autodiff/tridiagonal_solve.py:177, and
// TridiagonalFactorize, autodiff/tridiagonal_factor.py:145): forward, reverse (VJP) and
// forward-mode (JVP) sweeps, one thread per column, float64.  Arrays are row-major
// (n_cols, L) for a / b / c / alpha / gamma and (n_cols, L+1) for rhs / out.
//
//   factor:  alpha_k = 1 / (b_k - a_k gamma_(k-1)),  gamma_k = c_k alpha_k   (k >= 1)
//   solve:   u_k = (rhs_k - a_k u_(k-1)) alpha_k  (1 <= k < L),  u_0 = rhs_0, u_L = rhs_L
//            out_k = u_k - gamma_k out_(k+1)  (k = L-1 .. 0),  out_L = u_L
#include "common.cuh"

namespace {

__global__ void k_tri_solve(long long n, int L, const double* __restrict__ a, const double* __restrict__ al,
                            const double* __restrict__ g, const double* __restrict__ rhs,
                            double* __restrict__ out) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  double* x = out + ow;
  double u = rhs[ow];
  x[0] = u;
  for (int k = 1; k < L; ++k) {
    u = (rhs[ow + k] - a[o + k] * u) * al[o + k];
    x[k] = u;
  }
  double xn = rhs[ow + L];
  x[L] = xn;
  for (int k = L - 1; k >= 0; --k) {
    xn = x[k] - g[o + k] * xn;
    x[k] = xn;
  }
}

// Reverse mode of the solve.  adj_u (the adjoint of the eliminated values) is kept in
// grad_rhs and the recomputed u in grad_alpha until they are overwritten by the final
// gradients: level k of each is read before it is written, in the order of the sweeps.
__global__ void k_tri_solve_vjp(long long n, int L, const double* __restrict__ a, const double* __restrict__ al,
                                const double* __restrict__ g, const double* __restrict__ rhs,
                                const double* __restrict__ out, const double* __restrict__ gout,
                                double* __restrict__ ga, double* __restrict__ gal, double* __restrict__ gg,
                                double* __restrict__ grhs) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  // back substitution, reversed: adj_out propagates upward; adj_u_k = adj_out_k
  double adj = gout[ow];
  for (int k = 0; k < L; ++k) {
    grhs[ow + k] = adj;
    gg[o + k] = -adj * out[ow + k + 1];
    adj = gout[ow + k + 1] - g[o + k] * adj;
  }
  grhs[ow + L] = adj;
  // forward elimination, recomputed: u_k into gal[k] (k <= L-2 is all that is read)
  double u = rhs[ow];
  if (L > 1) gal[o] = u;
  for (int k = 1; k < L - 1; ++k) {
    u = (rhs[ow + k] - a[o + k] * u) * al[o + k];
    gal[o + k] = u;
  }
  // elimination, reversed
  for (int k = L - 1; k >= 1; --k) {
    const double um = gal[o + k - 1];
    const double t = rhs[ow + k] - a[o + k] * um;
    const double adj_u = grhs[ow + k];
    const double adj_t = adj_u * al[o + k];
    gal[o + k] = adj_u * t;
    grhs[ow + k] = adj_t;
    ga[o + k] = -adj_t * um;
    grhs[ow + k - 1] = grhs[ow + k - 1] - adj_t * a[o + k];
  }
  if (L > 0) {
    ga[o] = 0.0;
    gal[o] = 0.0;
  }
}

// Forward mode of the solve (null tangents are zero).  d_u is formed in dout, then the
// back substitution runs in place.
__global__ void k_tri_solve_jvp(long long n, int L, const double* __restrict__ a, const double* __restrict__ al,
                                const double* __restrict__ g, const double* __restrict__ rhs,
                                const double* __restrict__ out, const double* __restrict__ da,
                                const double* __restrict__ dal, const double* __restrict__ dg,
                                const double* __restrict__ drhs, double* __restrict__ dout) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t o = (size_t)c * L, ow = (size_t)c * (L + 1);
  double* d = dout + ow;
  double u = rhs[ow];
  double du = drhs ? drhs[ow] : 0.0;
  d[0] = du;
  d[L] = drhs ? drhs[ow + L] : 0.0;
  for (int k = 1; k < L; ++k) {
    const double t = rhs[ow + k] - a[o + k] * u;
    const double dt = (drhs ? drhs[ow + k] : 0.0) - (da ? da[o + k] : 0.0) * u - a[o + k] * du;
    du = dt * al[o + k] + t * (dal ? dal[o + k] : 0.0);
    u = t * al[o + k];
    d[k] = du;
  }
  double dn = d[L];
  for (int k = L - 1; k >= 0; --k) {
    dn = d[k] - (dg ? dg[o + k] : 0.0) * out[ow + k + 1] - g[o + k] * dn;
    d[k] = dn;
  }
}

__global__ void k_tri_factor(long long n, int L, const double* __restrict__ a, const double* __restrict__ b,
                             const double* __restrict__ cc, double* __restrict__ al, double* __restrict__ g) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t o = (size_t)c * L;
  double gam = 0.0;
  if (L > 0) {
    al[o] = 0.0;
    g[o] = 0.0;
  }
  for (int k = 1; k < L; ++k) {
    const double alpha = 1.0 / (b[o + k] - a[o + k] * gam);
    gam = cc[o + k] * alpha;
    al[o + k] = alpha;
    g[o + k] = gam;
  }
}

__global__ void k_tri_factor_vjp(long long n, int L, const double* __restrict__ a, const double* __restrict__ cc,
                                 const double* __restrict__ al, const double* __restrict__ g,
                                 const double* __restrict__ gal, const double* __restrict__ gg,
                                 double* __restrict__ ga, double* __restrict__ gb, double* __restrict__ gc) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t o = (size_t)c * L;
  if (L == 0) return;
  double adj_g = gg[o + L - 1];
  for (int k = L - 1; k >= 1; --k) {
    const double alpha = al[o + k];
    gc[o + k] = adj_g * alpha;
    const double tot = gal[o + k] + adj_g * cc[o + k];
    const double d_adj = -tot * (alpha * alpha);
    gb[o + k] = d_adj;
    ga[o + k] = -d_adj * g[o + k - 1];
    adj_g = gg[o + k - 1] - d_adj * a[o + k];
  }
  ga[o] = 0.0;
  gb[o] = 0.0;
  gc[o] = 0.0;
}

__global__ void k_tri_factor_jvp(long long n, int L, const double* __restrict__ a, const double* __restrict__ cc,
                                 const double* __restrict__ al, const double* __restrict__ g,
                                 const double* __restrict__ da, const double* __restrict__ db,
                                 const double* __restrict__ dc, double* __restrict__ dal, double* __restrict__ dg) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t o = (size_t)c * L;
  if (L == 0) return;
  dal[o] = 0.0;
  dg[o] = 0.0;
  double dgp = 0.0;
  for (int k = 1; k < L; ++k) {
    const double alpha = al[o + k];
    const double term = (db ? db[o + k] : 0.0) - (da ? da[o + k] : 0.0) * g[o + k - 1] - a[o + k] * dgp;
    const double d_alpha = -(alpha * alpha) * term;
    dgp = (dc ? dc[o + k] : 0.0) * alpha + cc[o + k] * d_alpha;
    dal[o + k] = d_alpha;
    dg[o + k] = dgp;
  }
}

inline int cols_ok(long long n, int L) { return n >= 0 && L >= 1 ? MPASG_OK : MPASG_E_ARG; }

}  // namespace

extern "C" int mpasg_tridiag_solve(long long n, int L, const double* a, const double* alpha, const double* gamma,
                                   const double* rhs, double* out, void* stream) {
  if (cols_ok(n, L) || !a || !alpha || !gamma || !rhs || !out) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_tri_solve<<<nblocks(n, 128), 128, 0, (cudaStream_t)stream>>>(n, L, a, alpha, gamma, rhs, out);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_tridiag_solve_vjp(long long n, int L, const double* a, const double* alpha,
                                       const double* gamma, const double* rhs, const double* out,
                                       const double* grad_out, double* grad_a, double* grad_alpha,
                                       double* grad_gamma, double* grad_rhs, void* stream) {
  if (cols_ok(n, L) || !a || !alpha || !gamma || !rhs || !out || !grad_out || !grad_a || !grad_alpha ||
      !grad_gamma || !grad_rhs)
    return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_tri_solve_vjp<<<nblocks(n, 128), 128, 0, (cudaStream_t)stream>>>(n, L, a, alpha, gamma, rhs, out, grad_out,
                                                                    grad_a, grad_alpha, grad_gamma, grad_rhs);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_tridiag_solve_jvp(long long n, int L, const double* a, const double* alpha,
                                       const double* gamma, const double* rhs, const double* out, const double* da,
                                       const double* dalpha, const double* dgamma, const double* drhs,
                                       double* dout, void* stream) {
  if (cols_ok(n, L) || !a || !alpha || !gamma || !rhs || !out || !dout) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_tri_solve_jvp<<<nblocks(n, 128), 128, 0, (cudaStream_t)stream>>>(n, L, a, alpha, gamma, rhs, out, da, dalpha,
                                                                    dgamma, drhs, dout);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_tridiag_factor(long long n, int L, const double* a, const double* b, const double* c,
                                    double* alpha, double* gamma, void* stream) {
  if (cols_ok(n, L) || !a || !b || !c || !alpha || !gamma) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_tri_factor<<<nblocks(n, 128), 128, 0, (cudaStream_t)stream>>>(n, L, a, b, c, alpha, gamma);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_tridiag_factor_vjp(long long n, int L, const double* a, const double* c, const double* alpha,
                                        const double* gamma, const double* grad_alpha, const double* grad_gamma,
                                        double* grad_a, double* grad_b, double* grad_c, void* stream) {
  if (cols_ok(n, L) || !a || !c || !alpha || !gamma || !grad_alpha || !grad_gamma || !grad_a || !grad_b ||
      !grad_c)
    return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_tri_factor_vjp<<<nblocks(n, 128), 128, 0, (cudaStream_t)stream>>>(n, L, a, c, alpha, gamma, grad_alpha,
                                                                     grad_gamma, grad_a, grad_b, grad_c);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}

extern "C" int mpasg_tridiag_factor_jvp(long long n, int L, const double* a, const double* c, const double* alpha,
                                        const double* gamma, const double* da, const double* db, const double* dc,
                                        double* dalpha, double* dgamma, void* stream) {
  if (cols_ok(n, L) || !a || !c || !alpha || !gamma || !dalpha || !dgamma) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  k_tri_factor_jvp<<<nblocks(n, 128), 128, 0, (cudaStream_t)stream>>>(n, L, a, c, alpha, gamma, da, db, dc, dalpha,
                                                                     dgamma);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
