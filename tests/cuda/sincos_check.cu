// Checks lib_sincosf (the float double-float evaluation where Ziv's test
// decides, else the double path) bit for bit against the double-precision
// sincos rounded once to float, on every float whose bit pattern lies in
// [begin, begin + count), and counts the inputs the float evaluation decided.
#include <cuda_runtime.h>

#include <cstdint>

#include "pgl_math.cuh"

using namespace pgl;

__global__ void sincos_check_kernel(uint32_t begin, uint64_t count, unsigned long long *counts, float *bad) {
  unsigned long long decided = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < count; i += uint64_t(gridDim.x) * blockDim.x) {
    const float x = __uint_as_float(uint32_t(uint64_t(begin) + i));
    float s, c;
    lib_sincosf(x, &s, &c);
    double sd, cd;
    sincos(double(x), &sd, &cd);
    const float rs = float(sd), rc = float(cd);
    float ts, tc;
    decided += sincos_df(x, &ts, &tc) ? 1u : 0u;
    const bool sameS = __float_as_uint(s) == __float_as_uint(rs) || (s != s && rs != rs);
    const bool sameC = __float_as_uint(c) == __float_as_uint(rc) || (c != c && rc != rc);
    if (!sameS || !sameC) {
      const unsigned long long k = atomicAdd(&counts[0], 1ULL);
      if (k < 8) bad[k] = x;
    }
  }
  atomicAdd(&counts[1], decided);
}

// hostCounts: mismatches, decided; hostBad: up to 8 mismatching inputs
extern "C" int sincos_check(uint32_t begin, uint64_t count, unsigned long long *hostCounts, float *hostBad) {
  if (uint64_t(begin) + count > (uint64_t(1) << 32)) return 1;
  unsigned long long *dc = nullptr;
  float *db = nullptr;
  if (cudaMalloc(&dc, 2 * sizeof(unsigned long long)) != cudaSuccess) return 1;
  if (cudaMalloc(&db, 8 * sizeof(float)) != cudaSuccess) {
    cudaFree(dc);
    return 1;
  }
  cudaMemset(dc, 0, 2 * sizeof(unsigned long long));
  cudaMemset(db, 0, 8 * sizeof(float));
  sincos_check_kernel<<<152 * 8, 256>>>(begin, count, dc, db);
  const cudaError_t e = cudaDeviceSynchronize();
  cudaMemcpy(hostCounts, dc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaMemcpy(hostBad, db, 8 * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dc);
  cudaFree(db);
  return e == cudaSuccess ? 0 : 2;
}
