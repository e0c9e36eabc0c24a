// Host build of pow_exner (mpas_dycore_pytorch_gb300/csrc/pow_exner.cuh) for
// tests/test_pow_exner.py: the same source the kernels use, compiled without
// multiply-add contraction.
#include "../mpas_dycore_pytorch_gb300/csrc/pow_exner.cuh"

extern "C" void pow_exner_many(const double* x, const double* y, double* out, long n) {
  for (long i = 0; i < n; ++i) out[i] = mpasg_pow::pow_exner(x[i], y[i]);
}
