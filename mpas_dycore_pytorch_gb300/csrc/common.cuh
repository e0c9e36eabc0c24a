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

// Third/fourth-order vertical fluxes (dynamics/dyn_tend.py:839,853):
//   flux4 = ua (7 (q0 + qm1) - (qp1 + qm2)) / 12
//   flux3 = flux4 + c3 |ua| ((qp1 - qm2) - 3 (q0 - qm1)) / 12
// evaluated with one multiply by 1/12 instead of two float64 divisions (float64
// division is a long instruction sequence on this part); the sum differs from the
// reference's two-quotient form by at most a couple of units in the last place.
constexpr double kInv12 = 1.0 / 12.0;
MPASG_D double flux3(double qm2, double qm1, double q0, double qp1, double ua, double c3) {
  return (ua * (7.0 * (q0 + qm1) - (qp1 + qm2)) + c3 * fabs(ua) * ((qp1 - qm2) - 3.0 * (q0 - qm1))) * kInv12;
}

// x / d with the float64 division skipped when d == 1 (x / 1.0 == x exactly); the
// height coordinate over flat terrain makes most metric denominators exactly one.
MPASG_D double div_or_one(double x, double d) { return d == 1.0 ? x : x / d; }

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

// Number of kernels this library has launched (for launch accounting by callers).
extern "C" long long mpasg_launch_count(void);
void mpasg_count_launch();

#define MPASG_LAUNCH_CHECK()                                    \
  do {                                                          \
    mpasg_count_launch();                                       \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return MPASG_E_LAUNCH;               \
  } while (0)
