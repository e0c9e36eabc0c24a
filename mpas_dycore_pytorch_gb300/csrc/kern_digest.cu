// Value digest of device memory: binds a returned step boundary to the exact bytes of its
// tensors without copying them to the host (the reference keeps a host copy of every
// tensor's bytes, mpas_pytorch/state.py:72-141).
//
// The bytes are read as little-endian 8-byte words w_i (the last word zero-padded).  Each
// word is mixed with its index, h_i = mix(w_i ^ mix(i + 0x9e3779b97f4a7c15)), and two lanes
// are summed modulo 2^64: A = sum h_i and B = sum mix(h_i ^ 0x5851f42d4c957f2d).  mix is the
// SplitMix64 output function (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014; constants as published with Vigna's SplitMix64).  Integer sums
// do not depend on the order of summation, so the digest is the same for any grid and on
// the host (the package's numpy restatement); the caller folds in the byte count.  A single
// changed word changes both lanes unless the mixed words collide (about 2^-64 each).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace {

MPASG_D uint64_t smix(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

__global__ void __launch_bounds__(256) k_digest(const uint64_t* __restrict__ w, long long n8,
                                                const unsigned char* __restrict__ tail, int ntail,
                                                unsigned long long* __restrict__ out) {
  uint64_t a = 0, b = 0;
  const long long n = n8 + (ntail > 0 ? 1 : 0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    uint64_t v = 0;
    if (i < n8) {
      v = w[i];
    } else {
      for (int j = 0; j < ntail; ++j) v |= (uint64_t)tail[j] << (8 * j);
    }
    const uint64_t h = smix(v ^ smix((uint64_t)i + 0x9e3779b97f4a7c15ull));
    a += h;
    b += smix(h ^ 0x5851f42d4c957f2dull);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  __shared__ uint64_t sa[8], sb[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sa[warp] = a;
    sb[warp] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      a += sa[k];
      b += sb[k];
    }
    atomicAdd(out, (unsigned long long)a);
    atomicAdd(out + 1, (unsigned long long)b);
  }
}

}  // namespace

extern "C" int mpasg_digest(const void* p, long long nbytes, unsigned long long* out, void* stream) {
  if (!out || nbytes < 0 || (nbytes > 0 && !p)) return MPASG_E_ARG;
  if (((uintptr_t)p & 7u) != 0) return MPASG_E_ARG;  // word loads need 8-byte alignment
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), s) != cudaSuccess) return MPASG_E_CUDA;
  if (nbytes == 0) return MPASG_OK;
  const long long n8 = nbytes / 8;
  const int ntail = (int)(nbytes - 8 * n8);
  const long long words = n8 + (ntail > 0 ? 1 : 0);
  long long blocks = (words + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;  // grid-stride beyond 8 blocks per SM
  k_digest<<<(unsigned)blocks, 256, 0, s>>>((const uint64_t*)p, n8, (const unsigned char*)p + 8 * n8, ntail, out);
  MPASG_LAUNCH_CHECK();
  return MPASG_OK;
}
