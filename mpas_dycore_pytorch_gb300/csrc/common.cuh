// Shared device helpers for the MPAS step kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mpasg.h"

#define MPASG_HD __host__ __device__ __forceinline__
#define MPASG_D __device__ __forceinline__

// Fast unsigned division by a runtime constant (Granlund-Montgomery, n < 2^31).
struct FastDiv {
  uint32_t d, m, s;
  FastDiv() : d(1), m(0), s(0) {}
  explicit FastDiv(uint32_t div) : d(div) {
    uint32_t l = 0;
    while ((1ull << l) < div) ++l;
    s = l;
    m = (uint32_t)(((1ull << 32) * ((1ull << l) - div)) / div + 1ull);
  }
  MPASG_D uint32_t div(uint32_t n) const { return (__umulhi(n, m) + n) >> s; }
};

// Fortran sign(1.0, x) as the reference's fct_sign_pm: +1 for x >= 0 (and -0.0).
MPASG_D double sgn(double x) { return x >= 0.0 ? 1.0 : -1.0; }

// ---------------------------------------------------------------- stencil arithmetic type
// Stencil kernels are templates on the arithmetic type T: double (plain float64 form) or
// float (mixed form: float64 fields in memory, float32 stencil arithmetic).  On this part
// the hardware float64<->float32 conversions issue on the float64 pipe (about 2 per clock
// per SM, the DFMA rate), so the mixed form converts with integer operations instead:
// binary64 -> binary32 repacks sign, rebiased exponent and the top 23 mantissa bits,
// rounded to nearest (ties away from zero; a mantissa carry rolls into the exponent as
// IEEE ordering allows), magnitudes below 2^-126 become zero; binary32 ->
// binary64 is exact for normal numbers (float32 subnormals become zero; infinities and
// NaNs stay non-finite, so the float64 finite check still sees them).  Field values on
// this path are far inside float32's normal range.
MPASG_D float d2f_bits(double x) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const uint32_t a = hi & 0x7fffffffu;
  uint32_t r = __funnelshift_l(lo, a - 0x38000000u, 3);  // exponent bias 1023 -> 127
  r += (lo >> 28) & 1u;                                   // round half away from zero
  r = a < 0x38100000u ? 0u : r;
  return __uint_as_float(r | (hi & 0x80000000u));
}
MPASG_D double f2d_bits(float x) {
  const uint32_t b = __float_as_uint(x);
  const uint32_t a = b & 0x7fffffffu;
  const bool tiny = a < 0x00800000u;
  uint32_t hi = tiny ? 0u : (a >> 3) + 0x38000000u;
  hi = a >= 0x7f800000u ? (a >> 3) + 0x70000000u : hi;  // exponent 255 -> 2047
  const uint32_t lo = tiny ? 0u : a << 29;
  return __hiloint2double((int)(hi | (b & 0x80000000u)), (int)lo);
}
// cv<T>(x): a float64 value as the stencil type; f64(x): a stencil value stored as float64
template <typename T> MPASG_D T cv(double x);
template <> MPASG_D double cv<double>(double x) { return x; }
template <> MPASG_D float cv<float>(double x) { return d2f_bits(x); }
// fp<T>(d, s): a field or geometry array as the stencil type -- the float64 array in the
// float64 form, its float32 copy in the mixed form (no conversion on load)
template <typename T> MPASG_D const T* fp(const double* d, const float* s);
template <> MPASG_D const double* fp<double>(const double* d, const float*) { return d; }
template <> MPASG_D const float* fp<float>(const double*, const float* s) { return s; }
template <typename T> MPASG_D T* fpw(double* d, float* s);
template <> MPASG_D double* fpw<double>(double* d, float*) { return d; }
template <> MPASG_D float* fpw<float>(double*, float* s) { return s; }
// G(name): mesh geometry array `name` as the stencil type T (kernel-local shorthand)
#define G(name) fp<T>(m.name, m.name##_f32)

// dif<T>(a, b): a - b of two float64 values as the stencil type, the difference taken in
// float64 first (fields with a large mean, e.g. pressure or kinetic energy, whose
// neighbour differences would otherwise lose their leading digits in float32)
template <typename T> MPASG_D T dif(double a, double b) { return cv<T>(a - b); }
template <> MPASG_D double dif<double>(double a, double b) { return a - b; }
MPASG_D double f64(double x) { return x; }
MPASG_D double f64(float x) { return f2d_bits(x); }
MPASG_D double vmin(double a, double b) { return fmin(a, b); }
MPASG_D float vmin(float a, float b) { return fminf(a, b); }
MPASG_D double vmax(double a, double b) { return fmax(a, b); }
MPASG_D float vmax(float a, float b) { return fmaxf(a, b); }
MPASG_D double vabs(double a) { return fabs(a); }
MPASG_D float vabs(float a) { return fabsf(a); }
MPASG_D double vsqrt(double a) { return sqrt(a); }
MPASG_D float vsqrt(float a) { return sqrtf(a); }
// 1 / d in float64 for the mixed form: a float32 reciprocal seed refined by two
// Newton-Raphson steps x <- x + x (1 - d x) (quadratic convergence: 2^-23 -> 2^-46 ->
// float64 rounding), four float64 FMAs instead of a float64 division.  d must be a
// normal float32 magnitude (densities, metric factors).
MPASG_D double rcp_nr(double d) {
  double x = f2d_bits(1.0f / d2f_bits(d));
  double e = fma(-d, x, 1.0);
  x = fma(x, e, x);
  e = fma(-d, x, 1.0);
  return fma(x, e, x);
}
// One Newton-Raphson step from the float32 seed: relative error below 2^-44 (~6e-14),
// for float64 values the mixed form only needs far beyond float32 accuracy.
MPASG_D double rcp_nr1(double d) {
  double x = f2d_bits(1.0f / d2f_bits(d));
  return fma(x, fma(-d, x, 1.0), x);
}
// a / b of float64 operands: the division in the float64 form, a * rcp_nr(b) in the
// mixed form (within 2 ulp)
template <typename T> MPASG_D double fdiv(double a, double b) { return a * rcp_nr(b); }
template <> MPASG_D double fdiv<double>(double a, double b) { return a / b; }

// unfused (separately rounded) products and differences for cancellation-prone terms
MPASG_D double mul_rn(double a, double b) { return __dmul_rn(a, b); }
MPASG_D float mul_rn(float a, float b) { return __fmul_rn(a, b); }
MPASG_D double add_rn(double a, double b) { return __dadd_rn(a, b); }
MPASG_D float add_rn(float a, float b) { return __fadd_rn(a, b); }
MPASG_D double sub_rn(double a, double b) { return __dsub_rn(a, b); }
MPASG_D float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// Third/fourth-order vertical fluxes (dynamics/dyn_tend.py:839,853):
//   flux4 = ua (7 (q0 + qm1) - (qp1 + qm2)) / 12
//   flux3 = flux4 + c3 |ua| ((qp1 - qm2) - 3 (q0 - qm1)) / 12
// evaluated with one multiply by 1/12 instead of two float64 divisions (float64
// division is a long instruction sequence on this part); the sum differs from the
// reference's two-quotient form by at most a couple of units in the last place.
constexpr double kInv12 = 1.0 / 12.0;
template <typename T>
MPASG_D T flux3(T qm2, T qm1, T q0, T qp1, T ua, T c3) {
  return (ua * (T(7) * (q0 + qm1) - (qp1 + qm2)) + c3 * vabs(ua) * ((qp1 - qm2) - T(3) * (q0 - qm1))) * T(kInv12);
}

// x / d with the division skipped when d == 1 (x / 1.0 == x exactly); the height
// coordinate over flat terrain makes most metric denominators exactly one.
template <typename T>
MPASG_D T div_or_one(T x, T d) { return d == T(1) ? x : x / d; }

constexpr double kGravity = 9.80616;
constexpr double kRgas = 287.0;
constexpr double kCp = 1004.5;
constexpr double kP0 = 100000.0;
constexpr double kRvord = 461.6 / 287.0;

// Launch geometry for flat (entity, level[, scalar]) index spaces.
constexpr int kBlock = 256;
inline int nblocks(long long n, int block = kBlock) {
  long long b = (n + block - 1) / block;
  return (int)(b < 1 ? 1 : b);
}

// ---------------------------------------------------------------- internal entry points
// The mixed form's stencils read float32 copies of u, pv_edge, w and rw.  The step driver
// keeps them current (pack once at step start; recover and diagnostics rewrite them), so
// it calls these variants with copies_current = true; the public per-stage entry points
// refresh the copies first.
int mpasgi_pack_f32(const mpasg_mesh* m, mpasg_fields* f, cudaStream_t s);
int mpasgi_dyn_tend(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step, cudaStream_t s,
                    bool copies_current);
int mpasgi_solve_diagnostics(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int rk_step,
                             cudaStream_t s, bool copies_current);
int mpasgi_reconstruct(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, cudaStream_t s,
                       bool copies_current);
// theta_m - ref_theta and theta_m_save - ref_theta (float32) for the mixed form
int mpasgi_theta_dev(const mpasg_mesh* m, mpasg_fields* f, cudaStream_t s);
int mpasgi_theta_edge(const mpasg_mesh* m, mpasg_fields* f, bool mixed, cudaStream_t s);
int mpasgi_divergence_damping(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, double dts,
                              cudaStream_t s, bool copies_current);
int mpasgi_acoustic_step(const mpasg_mesh* m, const mpasg_config* c, mpasg_fields* f, int small_step, double dts,
                         cudaStream_t s, bool copies_current);

// Number of kernels this library has launched (for launch accounting by callers).
extern "C" long long mpasg_launch_count(void);
void mpasg_count_launch();

#define MPASG_LAUNCH_CHECK()                                    \
  do {                                                          \
    mpasg_count_launch();                                       \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return MPASG_E_LAUNCH;               \
  } while (0)
