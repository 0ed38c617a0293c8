// Training samples from many paths' segments at once on the device
// (PathSegmentDataStorage.h:161-316 per path): one thread per path counts
// its samples, an exclusive scan turns the counts into each path's first
// output slot, and a second pass writes the samples there, so the output is
// in path order and, within a path, in the reference's order.
#include <cuda_runtime.h>

#include <cub/device/device_scan.cuh>

#include "launch.h"
#include "path_samples.cuh"

namespace pgl {

__global__ void path_count_kernel(const PathSegmentRecord *seg, const uint32_t *begin, uint32_t numPaths,
                                  float maxDistance, PathFlags fl, uint32_t *counts) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > numPaths) return;
  if (p == numPaths) {  // the scan's last entry becomes the total
    counts[p] = 0;
    return;
  }
  const uint32_t b = begin[p], e = begin[p + 1];
  counts[p] = path_prepare_samples(seg + b, int(e - b), maxDistance, fl, nullptr, 0);
}

__global__ void path_write_kernel(const PathSegmentRecord *seg, const uint32_t *begin, uint32_t numPaths,
                                  float maxDistance, PathFlags fl, const uint32_t *offsets, PGLSampleRecord *out) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= numPaths) return;
  const uint32_t b = begin[p], e = begin[p + 1];
  path_prepare_samples(seg + b, int(e - b), maxDistance, fl, out + offsets[p], offsets[p + 1] - offsets[p]);
}

cudaError_t launch_path_samples(const PathSegmentRecord *seg, const uint32_t *begin, uint32_t numPaths,
                                float maxDistance, PathFlags fl, PGLSampleRecord *out, uint32_t *offsets,
                                Scratch &scratch, cudaStream_t s) {
  const unsigned threads = 128;
  const unsigned blocks = unsigned((uint64_t(numPaths) + 1 + threads - 1) / threads);
  count_launch();
  path_count_kernel<<<blocks, threads, 0, s>>>(seg, begin, numPaths, maxDistance, fl, offsets);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  size_t tempBytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tempBytes, offsets, offsets, int(numPaths + 1), s);
  e = scratch_reserve(scratch, tempBytes);
  if (e != cudaSuccess) return e;
  e = cub::DeviceScan::ExclusiveSum(scratch.ptr, tempBytes, offsets, offsets, int(numPaths + 1), s);
  if (e != cudaSuccess) return e;
  if (numPaths == 0) return cudaSuccess;
  count_launch();
  path_write_kernel<<<blocks, threads, 0, s>>>(seg, begin, numPaths, maxDistance, fl, offsets, out);
  return cudaGetLastError();
}

}  // namespace pgl
