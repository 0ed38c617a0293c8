// Checks div_rcp (mode 0: Markstein's correctly rounded division from a
// reciprocal) and div_faithful_fix (mode 1: from the approximate hardware
// reciprocal, in its operand range) against the correctly rounded division
// __fdiv_rn on hashed operand pairs:
// random a and b over a wide exponent range, b integral (1..2^24) and b of
// the form n0 + j with n0 a multiple of 1/4 (the running-mean counts).
#include <cuda_runtime.h>

#include <cstdint>

#include "pgl_math.cuh"

using namespace pgl;

__device__ uint32_t mix32(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return uint32_t(x);
}
__device__ float rand_float(uint64_t key, int emin, int emax) {
  uint32_t h = mix32(key);
  uint32_t e = uint32_t(emin + int(mix32(key * 3 + 1) % uint32_t(emax - emin + 1)) + 127);
  return __uint_as_float((h & 0x80000000u) | (e << 23) | (h & 0x7FFFFFu));
}

__global__ void div_check_kernel(uint64_t n, uint64_t seed, int mode, unsigned long long *mismatches, float *bad) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = seed * 0x9E3779B97F4A7C15ULL + i;
    float a = rand_float(key * 7 + 3, -40, 40);
    float b;
    switch (i % 3) {
      case 0: b = rand_float(key * 11 + 5, -40, 40); break;
      case 1: b = float(1 + mix32(key * 13 + 7) % (1u << 24)); break;
      default: b = float(mix32(key * 17 + 9) % 4096u) * 0.25f + float(1 + mix32(key * 19 + 11) % 65536u); break;
    }
    if (i % 5 == 0) a = float(int(mix32(key * 23 + 1) % 2001u) - 1000) * 0.001f;  // small chi-like values, zero included
    const float r = __fdiv_rn(a, b);
    float q = div_rcp(a, b, rcp_for_div(b));
    if (mode == 1) {
      // div_faithful_fix, used in its range only (the callers divide otherwise)
      const float aa = fabsf(a), ar = fabsf(r);
      if (!(aa >= 1e-30f && aa <= 1e30f && ar >= 1e-30f && ar <= 1e30f)) continue;
      q = div_faithful_fix(a, b, rcp_approx(b));
    }
    if (__float_as_uint(q) != __float_as_uint(r) && !(q != q && r != r)) {
      unsigned long long k = atomicAdd(mismatches, 1ULL);
      if (k < 8) {
        bad[3 * k] = a;
        bad[3 * k + 1] = b;
        bad[3 * k + 2] = q;
      }
    }
  }
}

extern "C" int div_check(uint64_t n, uint64_t seed, int mode, unsigned long long *hostMismatches, float *hostBad) {
  unsigned long long *dm = nullptr;
  float *db = nullptr;
  if (cudaMalloc(&dm, sizeof(unsigned long long)) != cudaSuccess) return 1;
  if (cudaMalloc(&db, 24 * sizeof(float)) != cudaSuccess) return 1;
  cudaMemset(dm, 0, sizeof(unsigned long long));
  cudaMemset(db, 0, 24 * sizeof(float));
  div_check_kernel<<<152 * 8, 256>>>(n, seed, mode, dm, db);
  cudaError_t e = cudaDeviceSynchronize();
  cudaMemcpy(hostMismatches, dm, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaMemcpy(hostBad, db, 24 * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dm);
  cudaFree(db);
  return e == cudaSuccess ? 0 : 2;
}
