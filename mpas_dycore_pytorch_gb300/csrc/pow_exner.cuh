// pow_exner(x, y): x**y for the Exner function, rounded to nearest correctly except when
// x**y lies within about 2^-19 units in the last place of a rounding boundary.
//
// The reference evaluates the Exner function (p / p0)**(R / cv) with the host C library's
// pow (glibc rounds correctly in all but ~1 case in 1000 in this range), and the vertically
// implicit acoustic solve amplifies a one-ulp difference in exner into ~1e-12 in w.  CUDA's
// pow is faithful to 2 ulp, which leaves many one-ulp differences; this function agrees
// with a correctly rounded pow, hence with the reference's, nearly everywhere.
//
// Method (Tang's table-driven logarithm and exponential, ACM TOMS 15 (1989) 144 and 16
// (1990) 378, carried in double-double arithmetic):
//   x = 2^e m, m in [1, 2); c = 1 + (j + 1/2)/256 the table point of m's top 8 bits;
//   f = m - c exactly; u = f / c = f (1/c)_hh+lo, |u| <= 2^-9;
//   ln x = e ln2 + ln c + log1p(u),  log1p(u) = u - u^2/2 + u^3 (1/3 - u/4 + ... - u^7/10),
//   with u^2 exact (two_prod) and every term above 2^-80 kept;
//   z = y ln x in double-double; z = (256 k' + j') ln2/256 + t, |t| <= ln2/512;
//   x**y = 2^k' 2^(j'/256) (1 + t + t^2/2 + t^3 (1/6 + ... + t^4/5040)),
//   the leading products exact (two_prod) and summed with error-free additions; one final
//   rounding.  Absolute error before it: below 2^-75 of the result.
// Outside positive normal x, finite y and |y ln x| < 700 the library pow is used.
//
// Compiles for the device (nvcc) and, for its own tests, for the host (a C++ compiler,
// with no contraction of multiply-adds).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define MPASG_POW_HD __device__ __forceinline__
#define MPASG_POW_TABLE static __device__ const
#else
#define MPASG_POW_HD inline
#define MPASG_POW_TABLE static const
#endif

namespace mpasg_pow {

#include "pow_tables.inc"

struct DD {
  double hi, lo;
};

MPASG_POW_HD double fma_rn(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

MPASG_POW_HD int64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  int64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

MPASG_POW_HD double from_bits(int64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

MPASG_POW_HD double tab(const double* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

// error-free transformations: a + b = s + e, a * b = p + e exactly
MPASG_POW_HD DD two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
MPASG_POW_HD DD fast_two_sum(double a, double b) {  // |a| >= |b|
  const double s = a + b;
  return {s, b - (s - a)};
}
MPASG_POW_HD DD two_prod(double a, double b) {
  const double p = a * b;
  return {p, fma_rn(a, b, -p)};
}

MPASG_POW_HD double pow_exner(double x, double y) {
  if (!(x >= 2.2250738585072014e-308 && x <= 1.7976931348623157e308) || !(fabs(y) <= 1.7976931348623157e308))
    return pow(x, y);
  // ---- ln x = lh + ll ----
  const int64_t b = bits_of(x);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  const int j = (int)((b >> 44) & 0xff);
  const double m = from_bits((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);  // [1, 2)
  const double c = 1.0 + (double)(2 * j + 1) * 0x1p-9;
  const double f = m - c;  // exact: |f| <= 2^-9, m and c share the binade
  const double* L = kPowLogTab[j];
  const DD fu = two_prod(f, tab(L + 0));
  const double uh = fu.hi, ul = fu.lo + f * tab(L + 1);  // u = f / c
  const DD sq = two_prod(uh, uh);
  double pl = kPowLogC10;
  pl = pl * uh + kPowLogC9;
  pl = pl * uh + kPowLogC8;
  pl = pl * uh + kPowLogC7;
  pl = pl * uh + kPowLogC6;
  pl = pl * uh + kPowLogC5;
  pl = pl * uh + kPowLogC4;
  pl = pl * uh + kPowLogC3;
  const double tail = (uh * sq.hi) * pl;          // u^3 (1/3 - u/4 + ...)
  const double ed = (double)e;
  const DD s1 = two_sum(ed * kPowLn2Hi, tab(L + 2));  // e * ln2_hi is exact
  const DD s2 = two_sum(s1.hi, uh);
  const DD s3 = two_sum(s2.hi, -0.5 * sq.hi);
  const double lo = ((s1.lo + s2.lo) + s3.lo) + (ed * kPowLn2Lo + tab(L + 3)) +
                    ((ul - uh * ul) - 0.5 * sq.lo) + tail;
  const DD ln = two_sum(s3.hi, lo);
  // ---- z = y ln x ----
  const DD zp = two_prod(y, ln.hi);
  const double zh = zp.hi, zl = zp.lo + y * ln.lo;
  if (!(fabs(zh) < 700.0)) return pow(x, y);
  // ---- exp(zh + zl) ----
  const double kf = rint(zh * kPowInvL256);
  const int k = (int)kf;
  const DD t = two_sum(zh - kf * kPowL256Hi, zl - kf * kPowL256Lo);  // first difference exact
  const double* T = kPowExpTab[k & 255];
  const double th = tab(T + 0), tl = tab(T + 1);
  const double t1 = t.hi, t2 = t.lo;
  const DD tsq = two_prod(t1, t1);
  double pe = kPowExpC7;
  pe = pe * t1 + kPowExpC6;
  pe = pe * t1 + kPowExpC5;
  pe = pe * t1 + kPowExpC4;
  pe = pe * t1 + kPowExpC3;
  const double p3 = (t1 * tsq.hi) * pe;           // t^3 (1/6 + t/24 + ...)
  const DD a = two_prod(th, t1);
  const DD h2 = two_prod(th, 0.5 * tsq.hi);
  const DD r1 = fast_two_sum(th, a.hi);
  const DD r2 = fast_two_sum(r1.hi, h2.hi);
  const double small = th * (((t2 + 0.5 * tsq.lo) + t1 * t2) + p3) + tl * ((1.0 + t1) + 0.5 * tsq.hi);
  const double r = r2.hi + ((((r1.lo + r2.lo) + a.lo) + h2.lo) + small);
  const int kk = (k - (k & 255)) / 256;  // floor(k / 256)
  return r * from_bits((int64_t)(kk + 1023) << 52);
}

}  // namespace mpasg_pow
