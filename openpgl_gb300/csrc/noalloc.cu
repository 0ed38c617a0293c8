// Splitting a device batch of sample records into surface and volume records
// without allocating: the variant of the sample ingest (ingest_flag_kernel +
// scan + ingest_scatter_kernel, whose flags, ranks and scan storage come from
// a growable scratch buffer) whose scratch is a fixed array in device memory.
//
// Three kernels on the caller's stream: per tile of 1024 records the number
// of inside-volume records (flag bit 2, SampleData::EInsideVolume), an
// exclusive scan of those counts, then a stable scatter (records keep their
// order within each kind).  The tile counts are fully rewritten by every call,
// so nothing has to start at zero; two calls that overlap in time (different
// streams or threads) share the array and race.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "launch.h"
#include "pgl_internal.h"

namespace pgl {

constexpr uint32_t kSplitTile = 1024;           // records per block
constexpr uint32_t kSplitThreads = 256;
constexpr uint32_t kSplitMaxTiles = 65536;      // 67,108,864 records per call
constexpr uint32_t kSplitScanThreads = 1024;

static __device__ __align__(256) uint32_t g_split_scratch[kSplitMaxTiles];

__global__ void split_count_kernel(const PGLSampleRecord *in, uint32_t n, uint32_t *tileVol) {
  const uint32_t base = blockIdx.x * kSplitTile;
  uint32_t total = 0;
  for (uint32_t k = 0; k < kSplitTile / kSplitThreads; ++k) {
    const uint32_t i = base + k * kSplitThreads + threadIdx.x;
    const int vol = (i < n && (in[i].flags & 2u)) ? 1 : 0;
    total += uint32_t(__syncthreads_count(vol));
  }
  if (threadIdx.x == 0) tileVol[blockIdx.x] = total;
}

// Exclusive scan of the tile counts in place (one block); counts[0..1] =
// surface and volume totals.
__global__ void split_scan_kernel(uint32_t *tileVol, uint32_t tiles, uint32_t n, uint32_t *counts) {
  __shared__ uint32_t part[kSplitScanThreads];
  const uint32_t per = (tiles + kSplitScanThreads - 1) / kSplitScanThreads;
  const uint32_t b = threadIdx.x * per, e = min(tiles, b + per);
  uint32_t sum = 0;
  for (uint32_t t = b; t < e; ++t) sum += tileVol[t];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (uint32_t off = 1; off < kSplitScanThreads; off <<= 1) {  // inclusive Hillis-Steele scan
    const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - sum;
  for (uint32_t t = b; t < e; ++t) {
    const uint32_t c = tileVol[t];
    tileVol[t] = run;
    run += c;
  }
  if (threadIdx.x == kSplitScanThreads - 1) {
    counts[1] = part[threadIdx.x];
    counts[0] = n - part[threadIdx.x];
  }
}

__global__ void split_scatter_kernel(const PGLSampleRecord *in, uint32_t n, const uint32_t *tileVolBefore,
                                     PGLSampleRecord *surf, PGLSampleRecord *vol) {
  __shared__ uint32_t warpVol[kSplitThreads / 32];
  __shared__ uint32_t runVol;
  const uint32_t base = blockIdx.x * kSplitTile;
  const uint32_t volBefore = tileVolBefore[blockIdx.x];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) runVol = 0;
  __syncthreads();
  for (uint32_t k = 0; k < kSplitTile / kSplitThreads; ++k) {
    const uint32_t local = k * kSplitThreads + threadIdx.x;  // index within the tile
    const uint32_t i = base + local;
    PGLSampleRecord r;
    bool have = i < n, isVol = false;
    if (have) {
      r = in[i];
      isVol = (r.flags & 2u) != 0;
    }
    const unsigned ball = __ballot_sync(0xFFFFFFFFu, isVol);
    if (lane == 0) warpVol[warp] = uint32_t(__popc(ball));
    __syncthreads();
    uint32_t before = runVol;
    for (uint32_t w = 0; w < warp; ++w) before += warpVol[w];
    before += uint32_t(__popc(ball & ((1u << lane) - 1u)));
    if (have) {
      if (isVol) vol[volBefore + before] = r;
      else surf[(base - volBefore) + (local - before)] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (uint32_t w = 0; w < kSplitThreads / 32; ++w) t += warpVol[w];
      runVol += t;
    }
    __syncthreads();
  }
}

size_t split_max_records() { return size_t(kSplitMaxTiles) * kSplitTile; }

// The array's address on the current device, looked up once per device.
static cudaError_t split_scratch(uint32_t **out) {
  static std::mutex m;
  static uint32_t *ptrs[128] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(m);
  if (!ptrs[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_split_scratch);
    if (e != cudaSuccess) return e;
    ptrs[dev] = static_cast<uint32_t *>(p);
  }
  *out = ptrs[dev];
  return cudaSuccess;
}

cudaError_t split_samples_noalloc(const PGLSampleRecord *in, size_t n, PGLSampleRecord *surf, PGLSampleRecord *vol,
                                  uint32_t *counts, cudaStream_t s) {
  uint32_t *scratch = nullptr;
  cudaError_t e = split_scratch(&scratch);
  if (e != cudaSuccess) return e;
  const uint32_t tiles = uint32_t((n + kSplitTile - 1) / kSplitTile);
  if (tiles > 0) {
    count_launch();
    split_count_kernel<<<tiles, kSplitThreads, 0, s>>>(in, uint32_t(n), scratch);
  }
  count_launch();
  split_scan_kernel<<<1, kSplitScanThreads, 0, s>>>(scratch, tiles, uint32_t(n), counts);
  if (tiles > 0) {
    count_launch();
    split_scatter_kernel<<<tiles, kSplitThreads, 0, s>>>(in, uint32_t(n), scratch, surf, vol);
  }
  return cudaGetLastError();
}

}  // namespace pgl
