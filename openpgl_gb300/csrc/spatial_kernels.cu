// Sample ingest, scene bounds, kd-tree level passes, leaf gather, the
// deterministic per-leaf ordering and the region k-nearest-neighbour table.
//
// The kd-tree is built level by level.  Samples are kept as
// (position, original index) records and, at every level, stably partitioned
// inside their node's segment (< pivot to the left, KDTreeBuilder.h:193), so
// that a node's samples stay contiguous, as in the reference's in-place
// partition (embree parallel_partition.h).  While classifying, each block
// accumulates the integer position statistics of the children it sees
// (IntegerSampleStatistics::addSample, SampleStatistics.h:261-277) in shared
// memory; because segments are contiguous a block touches few children.  The
// integer sums are order-free, so the split decisions made from them on the
// host are bit-identical to the reference's.
#include <atomic>
#include <climits>
#include <cuda_runtime.h>
#include <cub/cub.cuh>

#include "launch.h"
#include "pgl_internal.h"

namespace pgl {

static std::atomic<unsigned long long> g_kernel_launches{0};
unsigned long long kernel_launches() { return g_kernel_launches.load(std::memory_order_relaxed); }
void count_launch() { g_kernel_launches.fetch_add(1, std::memory_order_relaxed); }



// ------------------------------------------------------------------ ingest
// Splits an AoS batch into surface / volume SoA arrays, stable within each
// class (SampleDataStorage.h:72-90).  isVol[i] is produced by pass 1.
__global__ void ingest_flag_kernel(const PGLSampleRecord *in, uint32_t n, uint32_t *isVol) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) isVol[i] = (in[i].flags & 2u) ? 1u : 0u;
}
// The same for records in host memory: each record is read once over the
// host link and kept in device memory for the scatter.
__global__ void ingest_flag_stage_kernel(const PGLSampleRecord *in, uint32_t n, uint32_t *isVol,
                                         PGLSampleRecord *stage) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PGLSampleRecord r = in[i];
  stage[i] = r;
  isVol[i] = (r.flags & 2u) ? 1u : 0u;
}
__global__ void ingest_scatter_kernel(const PGLSampleRecord *in, uint32_t n, const uint32_t *volRank,
                                      float4 *sP, float4 *sD, float *sPdf, uint32_t *sFlags, uint64_t sBase,
                                      float4 *vP, float4 *vD, float *vPdf, uint32_t *vFlags, uint64_t vBase) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PGLSampleRecord r = in[i];
  uint32_t vr = volRank[i];
  float4 p = make_float4(r.px, r.py, r.pz, r.distance);
  float4 d = make_float4(r.dx, r.dy, r.dz, r.weight);
  if (r.flags & 2u) {
    uint64_t o = vBase + vr;
    vP[o] = p; vD[o] = d; vPdf[o] = r.pdf; vFlags[o] = r.flags;
  } else {
    uint64_t o = sBase + (i - vr);
    sP[o] = p; sD[o] = d; sPdf[o] = r.pdf; sFlags[o] = r.flags;
  }
}
__global__ void export_kernel(const float4 *P, const float4 *D, const float *pdf, const uint32_t *flags, uint64_t n,
                              PGLSampleRecord *out) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = P[i], d = D[i];
  PGLSampleRecord r{p.x, p.y, p.z, d.x, d.y, d.z, d.w, pdf[i], p.w, flags[i]};
  out[i] = r;
}

// ------------------------------------------------------------------ bounds
// min/max of positions [0, n) (the caller passes n-1: Field.h:326-344 stops
// one short of the end).  Floats are mapped to order-preserving integers.
__device__ __forceinline__ uint32_t ford(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__global__ void bounds_kernel(const float4 *P, uint64_t n, uint32_t *out6) {
  uint32_t lo[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, hi[3] = {0, 0, 0};
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    float4 p = P[i];
    float c[3] = {p.x, p.y, p.z};
    for (int d = 0; d < 3; ++d) {
      uint32_t o = ford(c[d]);
      lo[d] = min(lo[d], o);
      hi[d] = max(hi[d], o);
    }
  }
  for (int d = 0; d < 3; ++d) {
    for (int off = 16; off > 0; off >>= 1) {
      lo[d] = min(lo[d], __shfl_xor_sync(0xFFFFFFFFu, lo[d], off));
      hi[d] = max(hi[d], __shfl_xor_sync(0xFFFFFFFFu, hi[d], off));
    }
  }
  if ((threadIdx.x & 31) == 0)
    for (int d = 0; d < 3; ++d) {
      atomicMin(&out6[d], lo[d]);
      atomicMax(&out6[3 + d], hi[d]);
    }
}

// ------------------------------------------------------------------ kd levels
// One job per inner node visited at the current level.

constexpr int kKdThreads = 256;
constexpr int kKdItems = 16;                      // samples per thread
constexpr int kKdTile = kKdThreads * kKdItems;    // samples per block
constexpr int kKdLocal = 16;                      // distinct jobs aggregated per block

__device__ __forceinline__ void quantize(const KdJob &j, float4 p, long long q[3], long long qv[3]) {
  float c[3] = {p.x, p.y, p.z};
  for (int d = 0; d < 3; ++d) {
    float t = (c[d] - j.c[d]) * j.inv[d];
    float tv = (t * t) * 4096.f;
    t *= 4096.f;
    q[d] = (long long)t;
    qv[d] = (long long)tv;
  }
}

// Adds one sample's integer statistics (or a warp's reduced ones) to an
// accumulator in shared or global memory.
__device__ __forceinline__ void acc_add(IStatsAcc *a, const long long m[3], const long long v[3], const long long lo[3],
                                        const long long hi[3], unsigned long long n) {
  for (int d = 0; d < 3; ++d) {
    atomicAdd(reinterpret_cast<unsigned long long *>(&a->m[d]), (unsigned long long)m[d]);
    atomicAdd(reinterpret_cast<unsigned long long *>(&a->v[d]), (unsigned long long)v[d]);
    atomicMin(&a->lo[d], lo[d]);
    atomicMax(&a->hi[d], hi[d]);
  }
  atomicAdd(&a->n, n);
}

// A warp's running integer statistics of one job's two children, per lane.
struct WarpSideAcc {
  long long m[2][3], v[2][3], lo[2][3], hi[2][3];
  unsigned long long n[2];
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
#pragma unroll
      for (int d = 0; d < 3; ++d) { m[sd][d] = 0; v[sd][d] = 0; lo[sd][d] = LLONG_MAX; hi[sd][d] = LLONG_MIN; }
      n[sd] = 0;
    }
  }
};
__device__ __forceinline__ long long warp_sum64(long long x) {
  for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, off);
  return x;
}
__device__ __forceinline__ long long warp_min64(long long x) {
  for (int off = 16; off > 0; off >>= 1) x = min(x, __shfl_xor_sync(0xFFFFFFFFu, x, off));
  return x;
}
__device__ __forceinline__ long long warp_max64(long long x) {
  for (int off = 16; off > 0; off >>= 1) x = max(x, __shfl_xor_sync(0xFFFFFFFFu, x, off));
  return x;
}
// Adds a warp's running statistics of job `job` to acc[2 job + side] (or to
// the block's shared copy) and clears them.
__device__ __forceinline__ void warp_flush(WarpSideAcc &w, uint32_t job, bool stats, IStatsAcc *acc,
                                           IStatsAcc *local, bool useLocal, uint32_t firstJob) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int sd = 0; sd < 2; ++sd) {
    unsigned long long cnt = (unsigned long long)warp_sum64((long long)w.n[sd]);
    if (cnt == 0) continue;
    const uint32_t slot = 2 * job + uint32_t(sd);
    if (stats) {
      long long sm[3], sv[3], lo[3], hi[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        sm[d] = warp_sum64(w.m[sd][d]);
        sv[d] = warp_sum64(w.v[sd][d]);
        lo[d] = warp_min64(w.lo[sd][d]);
        hi[d] = warp_max64(w.hi[sd][d]);
      }
      if (lane == 0) acc_add(useLocal ? &local[slot - 2 * firstJob] : &acc[slot], sm, sv, lo, hi, cnt);
    } else if (lane == 0) {
      atomicAdd(&acc[slot].n, cnt);
    }
  }
  w.clear();
}

// Classifies the samples of every job at this level: side flag (1 = left),
// child statistics into acc[2*job + side].  jobOf[i] is the job of sample i
// (or ~0 when the sample already sits in a finished leaf).  Samples of a job
// are contiguous, so a warp mostly meets one job: each lane keeps running
// statistics of the warp's current job in registers, and the warp reduces
// and adds them only when its job changes and at the end; a group of 32
// samples that mixes jobs adds per sample.
__global__ void __launch_bounds__(kKdThreads)
kd_classify_kernel(const float4 *pos, const uint32_t *jobOf, uint32_t n, const KdJob *jobs, uint32_t *isLeft,
                   IStatsAcc *acc) {
  __shared__ IStatsAcc local[2 * kKdLocal];
  __shared__ uint32_t firstJob, lastJob;
  const uint32_t tileBegin = blockIdx.x * kKdTile;
  if (tileBegin >= n) return;
  const uint32_t tileEnd = min(n, tileBegin + kKdTile);
  if (threadIdx.x == 0) {
    firstJob = ~0u;
    lastJob = 0;
  }
  for (int s = threadIdx.x; s < 2 * kKdLocal; s += blockDim.x) {
    IStatsAcc &a = local[s];
    for (int d = 0; d < 3; ++d) { a.m[d] = 0; a.v[d] = 0; a.lo[d] = LLONG_MAX; a.hi[d] = LLONG_MIN; }
    a.n = 0;
  }
  __syncthreads();
  // jobs are sorted by segment and samples of a job are contiguous, so the
  // tile's jobs form the range [min, max] of its job ids (~0: finished sample)
  {
    uint32_t f = ~0u, l = 0;
    for (uint32_t i = tileBegin + threadIdx.x; i < tileEnd; i += blockDim.x) {
      const uint32_t j = jobOf[i];
      if (j != ~0u) {
        f = min(f, j);
        l = max(l, j);
      }
    }
    if (f != ~0u) {
      atomicMin(&firstJob, f);
      atomicMax(&lastJob, l);
    }
  }
  __syncthreads();
  const bool useLocal = firstJob != ~0u && (lastJob - firstJob) < uint32_t(kKdLocal);
  const unsigned full = 0xFFFFFFFFu;
  WarpSideAcc w;
  w.clear();
  uint32_t cur = ~0u;  // the warp's current job
  bool curStats = false;
  for (uint32_t base = tileBegin; base < tileEnd; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t jid = i < tileEnd ? jobOf[i] : ~0u;
    KdJob j;
    uint32_t left = 0;
    long long q[3] = {0, 0, 0}, qv[3] = {0, 0, 0};
    bool stats = false;
    if (jid != ~0u) {
      j = jobs[jid];
      const float4 p = pos[i];
      const float coord = j.dim == 0 ? p.x : (j.dim == 1 ? p.y : p.z);
      left = coord < j.pos ? 1u : 0u;
      stats = j.needStats != 0;
      if (stats) quantize(j, p, q, qv);
    }
    if (i < tileEnd) isLeft[i] = left;
    const unsigned act = __ballot_sync(full, jid != ~0u);
    if (act == 0) continue;
    const uint32_t j0 = __shfl_sync(full, jid, __ffs(act) - 1);
    if (__all_sync(full, jid == ~0u || jid == j0)) {
      if (j0 != cur) {
        if (cur != ~0u) warp_flush(w, cur, curStats, acc, local, useLocal, firstJob);
        cur = j0;
        curStats = __shfl_sync(full, stats ? 1 : 0, __ffs(act) - 1) != 0;
      }
      // both sides with selects (fixed register indices)
#pragma unroll
      for (int sd = 0; sd < 2; ++sd) {
        const bool on = jid != ~0u && (left != 0u) == (sd == 0);
        w.n[sd] += on ? 1ull : 0ull;
        if (curStats) {
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            w.m[sd][d] += on ? q[d] : 0ll;
            w.v[sd][d] += on ? qv[d] : 0ll;
            w.lo[sd][d] = min(w.lo[sd][d], on ? q[d] : LLONG_MAX);
            w.hi[sd][d] = max(w.hi[sd][d], on ? q[d] : LLONG_MIN);
          }
        }
      }
    } else if (jid != ~0u) {
      const uint32_t side = left ? 0u : 1u;
      if (stats) {
        IStatsAcc *a = useLocal ? &local[2 * (jid - firstJob) + side] : &acc[2 * jid + side];
        acc_add(a, q, qv, q, q, 1ull);
      } else {
        atomicAdd(&acc[2 * jid + side].n, 1ull);
      }
    }
  }
  if (cur != ~0u) warp_flush(w, cur, curStats, acc, local, useLocal, firstJob);
  __syncthreads();
  if (useLocal) {
    for (int s = threadIdx.x; s < 2 * kKdLocal; s += blockDim.x) {
      const IStatsAcc &a = local[s];
      if (a.n == 0) continue;
      acc_add(&acc[2 * firstJob + s], a.m, a.v, a.lo, a.hi, a.n);
    }
  }
}

// Integer statistics of all samples relative to the root bounds (the root is
// a leaf: KDTreeBuilder.h:94-115).
__global__ void __launch_bounds__(kKdThreads)
kd_root_stats_kernel(const float4 *pos, uint32_t n, KdJob job, IStatsAcc *acc) {
  long long m[3] = {0, 0, 0}, v[3] = {0, 0, 0}, lo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX},
            hi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
  unsigned long long cnt = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    long long q[3], qv[3];
    quantize(job, pos[i], q, qv);
    for (int d = 0; d < 3; ++d) { m[d] += q[d]; v[d] += qv[d]; lo[d] = min(lo[d], q[d]); hi[d] = max(hi[d], q[d]); }
    cnt++;
  }
  for (int off = 16; off > 0; off >>= 1) {
    for (int d = 0; d < 3; ++d) {
      m[d] += __shfl_xor_sync(0xFFFFFFFFu, m[d], off);
      v[d] += __shfl_xor_sync(0xFFFFFFFFu, v[d], off);
      lo[d] = min(lo[d], __shfl_xor_sync(0xFFFFFFFFu, lo[d], off));
      hi[d] = max(hi[d], __shfl_xor_sync(0xFFFFFFFFu, hi[d], off));
    }
    cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, off);
  }
  if ((threadIdx.x & 31) == 0 && cnt > 0) acc_add(acc, m, v, lo, hi, cnt);
}

// One pass down an existing tree: the leaf every sample reaches, by the
// builder's rule (coord < split goes left, KDTreeBuilder.h:193), as the
// leaf's slot (key) beside the sample's index (val).
__global__ void kd_route_kernel(const float4 *pos, uint32_t n, const KDNode *nodes, const uint32_t *nodeSlot,
                                uint32_t *key, uint32_t *val) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i];
  uint32_t nd = 0;
  KDNode node = nodes[0];
  while ((node.bits >> 30) != 3u) {
    const uint32_t dim = node.bits >> 30;
    const float c = dim == 0 ? p.x : (dim == 1 ? p.y : p.z);
    nd = (node.bits & 0x3FFFFFFFu) + (c < node.split ? 0u : 1u);
    node = nodes[nd];
  }
  key[i] = nodeSlot[nd];
  val[i] = i;
}
// Samples in slot order: positions and their leaf nodes.
__global__ void kd_route_gather_kernel(const float4 *pos, const uint32_t *key, const uint32_t *val, uint32_t n,
                                       const uint32_t *slotNode, float4 *posOut, uint32_t *nodeOut) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  posOut[j] = pos[val[j]];
  nodeOut[j] = slotNode[key[j]];
}

// Stable partition inside each job's segment using the exclusive scan of the
// left flags; finished samples keep their place.
__global__ void kd_scatter_kernel(const float4 *pos, const uint32_t *jobOf, const uint32_t *isLeft,
                                  const uint32_t *scanLeft, uint32_t n, const KdJob *jobs, float4 *posOut,
                                  uint32_t *nodeOut) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t jid = jobOf[i];
  if (jid == ~0u) {
    posOut[i] = pos[i];
    nodeOut[i] = ~0u;
    return;
  }
  const KdJob j = jobs[jid];
  uint32_t leftBefore = scanLeft[i] - scanLeft[j.begin];
  uint32_t L = scanLeft[j.end - 1] + isLeft[j.end - 1] - scanLeft[j.begin];
  uint32_t dst;
  uint32_t child;
  if (isLeft[i]) {
    dst = j.begin + leftBefore;
    child = j.left;
  } else {
    dst = j.begin + L + (i - j.begin - leftBefore);
    child = j.left + 1;
  }
  posOut[dst] = pos[i];
  nodeOut[dst] = child;
}

// Maps each sample's node to the job index of the next level (~0 if the node
// is a finished leaf).
// The job of every sample of a level (~0 for samples in finished leaves), and
// the level's child accumulators cleared, in one launch.
__global__ void kd_job_of_kernel(const uint32_t *node, uint32_t n, const uint32_t *nodeToJob, uint32_t *jobOf,
                                 IStatsAcc *acc, uint32_t accCount) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < accCount) {
    IStatsAcc a;
    for (int d = 0; d < 3; ++d) { a.m[d] = 0; a.v[d] = 0; a.lo[d] = LLONG_MAX; a.hi[d] = LLONG_MIN; }
    a.n = 0;
    acc[i] = a;
  }
  if (i >= n) return;
  uint32_t nd = node[i];
  jobOf[i] = nd == ~0u ? ~0u : nodeToJob[nd];
}

// ------------------------------------------------------------------ gather + ordering
// Gathers full samples into leaf order and builds the sort keys.  The key is
// the weight's bits mapped to an order-preserving integer (-0 as +0), the
// first field of SampleDataLess (SampleData.h:82-93).
__global__ void gather_kernel(const float4 *posIdx, uint32_t n, const float4 *P, const float4 *D, const float *pdf,
                              float4 *oP, float4 *oD, float *oPdf, uint32_t *key, uint32_t *val) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t src = __float_as_uint(posIdx[i].w);
  float4 d = D[src];
  oP[i] = P[src];
  oD[i] = d;
  oPdf[i] = pdf[src];
  float w = d.w == 0.0f ? 0.0f : d.w;
  key[i] = ford(w);
  val[i] = i;
}
__device__ __forceinline__ bool sample_less(float4 pa, float4 da, float fa, float4 pb, float4 db, float fb) {
  if (da.w != db.w) return da.w < db.w;   // weight
  if (fa != fb) return fa < fb;           // pdf
  if (pa.w != pb.w) return pa.w < pb.w;   // distance
  if (pa.x != pb.x) return pa.x < pb.x;
  if (pa.y != pb.y) return pa.y < pb.y;
  if (pa.z != pb.z) return pa.z < pb.z;
  if (da.x != db.x) return da.x < db.x;
  if (da.y != db.y) return da.y < db.y;
  return da.z < db.z;
}
// Permutes the samples into the sorted order (all samples, one thread each).
__global__ void permute_kernel(const uint32_t *sortedVal, uint32_t n, const float4 *P, const float4 *D,
                               const float *pdf, float4 *oP, float4 *oD, float *oPdf) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = sortedVal[i];
  oP[i] = P[s];
  oD[i] = D[s];
  oPdf[i] = pdf[s];
}
// Ties of equal weight within a leaf (equal adjacent 64-bit keys: same leaf,
// same weight) are ordered by the full comparator.  Float weights collide by
// chance (a few percent of the samples of a 2M batch), in runs of a handful,
// so every run is sorted by the thread at its first sample, all runs at once.
__global__ void fix_ties_kernel(const unsigned long long *sortedKey, uint32_t n, float4 *oP, float4 *oD,
                                float *oPdf) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i + 1 >= n) return;
  const unsigned long long k = sortedKey[i];
  if (sortedKey[i + 1] != k || (i > 0 && sortedKey[i - 1] == k)) return;  // not the start of a run
  uint32_t j = i + 2;
  while (j < n && sortedKey[j] == k) ++j;
  for (uint32_t x = i + 1; x < j; ++x) {  // insertion sort of the run [i, j)
    float4 kp = oP[x], kd = oD[x];
    float kf = oPdf[x];
    uint32_t y = x;
    while (y > i && sample_less(kp, kd, kf, oP[y - 1], oD[y - 1], oPdf[y - 1])) {
      oP[y] = oP[y - 1];
      oD[y] = oD[y - 1];
      oPdf[y] = oPdf[y - 1];
      --y;
    }
    oP[y] = kp;
    oD[y] = kd;
    oPdf[y] = kf;
  }
}

// ------------------------------------------------------------------ regions
__global__ void copy_region_kernel(RegionDir *regions, const uint32_t *dst, const uint32_t *src, uint32_t n) {
  uint32_t k = blockIdx.x;
  if (k >= n) return;
  const uint32_t *s = reinterpret_cast<const uint32_t *>(&regions[src[k]]);
  uint32_t *d = reinterpret_cast<uint32_t *>(&regions[dst[k]]);
  for (uint32_t i = threadIdx.x; i < sizeof(RegionDir) / 4; i += blockDim.x) d[i] = s[i];
}

// 8 nearest region means per region (KNN.h:212-266); nanoflann's squared
// distance ((dx*dx + dy*dy) + dz*dz), ties by region index.
__global__ void knn_kernel(const float4 *means, uint32_t R, Neighbours *out) {
  uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  float4 q = means[r];
  float bd[8];
  uint32_t bi[8];
  int cnt = 0;
  for (uint32_t j = 0; j < R; ++j) {
    float4 p = means[j];
    float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
    float d = 0.0f;
    d += dx * dx;
    d += dy * dy;
    d += dz * dz;
    if (cnt < 8 || d < bd[cnt - 1]) {
      int k = cnt < 8 ? cnt : 7;
      while (k > 0 && bd[k - 1] > d) {
        if (k < 8) { bd[k] = bd[k - 1]; bi[k] = bi[k - 1]; }
        --k;
      }
      bd[k] = d;
      bi[k] = j;
      if (cnt < 8) cnt++;
    }
  }
  Neighbours nb;
  nb.size = uint32_t(cnt);
  for (int i = 0; i < 8; ++i) {
    if (i < cnt) {
      nb.ids[i] = bi[i];
      float4 p = means[bi[i]];
      nb.px[i] = p.x; nb.py[i] = p.y; nb.pz[i] = p.z;
    } else {
      nb.ids[i] = ~0u;
      nb.px[i] = nb.py[i] = nb.pz[i] = 0.0f;
    }
  }
  out[r] = nb;
}

// ------------------------------------------------------------------ launchers
PGL_DEFINE_TABLE_UPLOAD(spatial_upload_tables)

cudaError_t scratch_reserve(Scratch &s, size_t bytes) {
  if (bytes <= s.bytes && s.ptr) return cudaSuccess;
  if (s.ptr) cudaFree(s.ptr);
  s.ptr = nullptr;
  s.bytes = 0;
  size_t want = bytes < 256 ? 256 : bytes + bytes / 4;
  cudaError_t e = cudaMalloc(&s.ptr, want);
  if (e == cudaSuccess) s.bytes = want;
  return e;
}
void scratch_free(Scratch &s) {
  if (s.ptr) cudaFree(s.ptr);
  s.ptr = nullptr;
  s.bytes = 0;
}

static inline unsigned blocks_for(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

cudaError_t ingest_samples(const PGLSampleRecord *in, uint32_t n, Scratch &scratch, SoAView surf, SoAView vol,
                           uint32_t *numVolume, cudaStream_t s, PGLSampleRecord *stage) {
  if (n == 0) { *numVolume = 0; return cudaSuccess; }
  size_t tempBytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tempBytes, (uint32_t *)nullptr, (uint32_t *)nullptr, int(n), s);
  const size_t flagBytes = (size_t(n) + 1) * sizeof(uint32_t);
  const size_t off = (flagBytes * 2 + 255) / 256 * 256;
  cudaError_t e = scratch_reserve(scratch, off + tempBytes);
  if (e != cudaSuccess) return e;
  uint32_t *isVol = reinterpret_cast<uint32_t *>(scratch.ptr);
  uint32_t *rank = isVol + (n + 1);
  void *temp = static_cast<char *>(scratch.ptr) + off;
  count_launch();
  if (stage) {
    ingest_flag_stage_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in, n, isVol, stage);
    in = stage;
  } else {
    ingest_flag_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in, n, isVol);
  }
  cub::DeviceScan::ExclusiveSum(temp, tempBytes, isVol, rank, int(n), s);
  count_launch();
  ingest_scatter_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in, n, rank, surf.P, surf.D, surf.pdf, surf.flags, surf.base,
                                                          vol.P, vol.D, vol.pdf, vol.flags, vol.base);
  uint32_t last[2];
  cudaMemcpyAsync(&last[0], rank + n - 1, 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&last[1], isVol + n - 1, 4, cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  *numVolume = last[0] + last[1];
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t export_samples(const float4 *P, const float4 *D, const float *pdf, const uint32_t *flags, uint64_t n,
                           PGLSampleRecord *out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  export_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, D, pdf, flags, n, out);
  return cudaGetLastError();
}

cudaError_t scene_bounds(const float4 *P, uint64_t n, uint32_t *d6, cudaStream_t s) {
  uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
  cudaError_t e = cudaMemcpyAsync(d6, init, sizeof(init), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess || n == 0) return e;
  unsigned b = blocks_for(n, 256);
  if (b > 4096) b = 4096;
  count_launch();
  bounds_kernel<<<b, 256, 0, s>>>(P, n, d6);
  return cudaGetLastError();
}

__global__ void init_posidx_kernel(const float4 *P, uint32_t n, float4 *posIdx) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = P[i];
  posIdx[i] = make_float4(p.x, p.y, p.z, __uint_as_float(i));
}
cudaError_t init_posidx(const float4 *P, uint32_t n, float4 *posIdx, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  init_posidx_kernel<<<blocks_for(n, 256), 256, 0, s>>>(P, n, posIdx);
  return cudaGetLastError();
}

__global__ void init_acc_kernel(IStatsAcc *acc, uint32_t count) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  IStatsAcc a;
  for (int d = 0; d < 3; ++d) { a.m[d] = 0; a.v[d] = 0; a.lo[d] = LLONG_MAX; a.hi[d] = LLONG_MIN; }
  a.n = 0;
  acc[i] = a;
}
cudaError_t init_acc(IStatsAcc *acc, uint32_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  count_launch();
  init_acc_kernel<<<blocks_for(count, 128), 128, 0, s>>>(acc, count);
  return cudaGetLastError();
}

cudaError_t kd_root_stats(const float4 *pos, uint32_t n, const KdJob &job, IStatsAcc *acc, cudaStream_t s) {
  unsigned b = blocks_for(n, kKdThreads * 8);
  if (b < 1) b = 1;
  if (b > 2048) b = 2048;
  count_launch();
  kd_root_stats_kernel<<<b, kKdThreads, 0, s>>>(pos, n, job, acc);
  return cudaGetLastError();
}

cudaError_t kd_job_of(const uint32_t *node, uint32_t n, const uint32_t *nodeToJob, uint32_t *jobOf, IStatsAcc *acc,
                      uint32_t accCount, cudaStream_t s) {
  const uint32_t m = n > accCount ? n : accCount;
  if (m == 0) return cudaSuccess;
  count_launch();
  kd_job_of_kernel<<<blocks_for(m, 256), 256, 0, s>>>(node, n, nodeToJob, jobOf, acc, accCount);
  return cudaGetLastError();
}

cudaError_t kd_level(const float4 *pos, const uint32_t *jobOf, uint32_t n, const KdJob *jobs, uint32_t *isLeft,
                     uint32_t *scanLeft, IStatsAcc *acc, float4 *posOut, uint32_t *nodeOut, Scratch &scratch,
                     cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  kd_classify_kernel<<<blocks_for(n, kKdTile), kKdThreads, 0, s>>>(pos, jobOf, n, jobs, isLeft, acc);
  size_t tempBytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tempBytes, isLeft, scanLeft, int(n), s);
  cudaError_t e = scratch_reserve(scratch, tempBytes);
  if (e != cudaSuccess) return e;
  cub::DeviceScan::ExclusiveSum(scratch.ptr, tempBytes, isLeft, scanLeft, int(n), s);
  count_launch();
  kd_scatter_kernel<<<blocks_for(n, 256), 256, 0, s>>>(pos, jobOf, isLeft, scanLeft, n, jobs, posOut, nodeOut);
  return cudaGetLastError();
}

cudaError_t kd_route(const float4 *pos, uint32_t n, const KDNode *nodes, const uint32_t *nodeSlot, uint32_t numSlots,
                     const uint32_t *slotNode, uint32_t *keys, uint32_t *vals, uint32_t *keysB, uint32_t *valsB,
                     float4 *posOut, uint32_t *nodeOut, Scratch &scratch, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  kd_route_kernel<<<blocks_for(n, 256), 256, 0, s>>>(pos, n, nodes, nodeSlot, keys, vals);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int bits = 1;
  while (bits < 32 && (1u << bits) < numSlots) ++bits;
  cub::DoubleBuffer<uint32_t> k(keys, keysB), v(vals, valsB);
  size_t tempBytes = 0;
  e = cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, k, v, int(n), 0, bits, s);
  if (e != cudaSuccess) return e;
  e = scratch_reserve(scratch, tempBytes);
  if (e != cudaSuccess) return e;
  e = cub::DeviceRadixSort::SortPairs(scratch.ptr, tempBytes, k, v, int(n), 0, bits, s);
  if (e != cudaSuccess) return e;
  count_launch();
  kd_route_gather_kernel<<<blocks_for(n, 256), 256, 0, s>>>(pos, k.Current(), v.Current(), n, slotNode, posOut,
                                                              nodeOut);
  return cudaGetLastError();
}
cudaError_t kd_classify(const float4 *pos, const uint32_t *jobOf, uint32_t n, const KdJob *jobs, uint32_t *isLeft,
                        IStatsAcc *acc, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  kd_classify_kernel<<<blocks_for(n, kKdTile), kKdThreads, 0, s>>>(pos, jobOf, n, jobs, isLeft, acc);
  return cudaGetLastError();
}

// 64-bit sort keys: the leaf's ordinal above the 32-bit weight key.
__global__ void leaf_key_kernel(const uint32_t *leafBegin, const uint32_t *leafEnd, uint32_t numLeaves,
                                const uint32_t *key, unsigned long long *key64) {
  const uint32_t leaf = blockIdx.x;
  if (leaf >= numLeaves) return;
  const unsigned long long hi = (unsigned long long)leaf << 32;
  for (uint32_t i = leafBegin[leaf] + threadIdx.x; i < leafEnd[leaf]; i += blockDim.x) key64[i] = hi | key[i];
}

cudaError_t gather_and_order(const float4 *posIdx, uint32_t n, const float4 *P, const float4 *D, const float *pdf,
                             const uint32_t *leafBegin, const uint32_t *leafCount, uint32_t numLeaves, bool sorted,
                             float4 *tmpP, float4 *tmpD, float *tmpPdf, uint32_t *keys, uint32_t *vals,
                             unsigned long long *keys64, float4 *oP, float4 *oD, float *oPdf, Scratch &scratch,
                             cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (!sorted) {
    count_launch();
    gather_kernel<<<blocks_for(n, 256), 256, 0, s>>>(posIdx, n, P, D, pdf, oP, oD, oPdf, keys, vals);
    return cudaGetLastError();
  }
  count_launch();
  gather_kernel<<<blocks_for(n, 256), 256, 0, s>>>(posIdx, n, P, D, pdf, tmpP, tmpD, tmpPdf, keys, vals);
  // stable order by (leaf, weight key): one LSD radix sort over the bits in
  // use (the leaves' sample ranges are disjoint and cover [0, n))
  uint32_t *valsOut = vals + n;
  unsigned long long *keys64Out = keys64 + n;
  const uint32_t *ends = leafBegin + numLeaves;  // caller stores ends after begins
  count_launch();
  leaf_key_kernel<<<numLeaves, 256, 0, s>>>(leafBegin, ends, numLeaves, keys, keys64);
  int leafBits = 1;
  while (leafBits < 32 && (1u << leafBits) < numLeaves) ++leafBits;
  size_t tempBytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, keys64, keys64Out, vals, valsOut, int(n), 0, 32 + leafBits, s);
  cudaError_t e = scratch_reserve(scratch, tempBytes);
  if (e != cudaSuccess) return e;
  cub::DeviceRadixSort::SortPairs(scratch.ptr, tempBytes, keys64, keys64Out, vals, valsOut, int(n), 0, 32 + leafBits,
                                  s);
  count_launch();
  permute_kernel<<<blocks_for(n, 256), 256, 0, s>>>(valsOut, n, tmpP, tmpD, tmpPdf, oP, oD, oPdf);
  count_launch();
  fix_ties_kernel<<<blocks_for(n, 256), 256, 0, s>>>(keys64Out, n, oP, oD, oPdf);
  (void)leafCount;
  return cudaGetLastError();
}

cudaError_t copy_regions(RegionDir *regions, const uint32_t *dst, const uint32_t *src, uint32_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  copy_region_kernel<<<n, 256, 0, s>>>(regions, dst, src, n);
  return cudaGetLastError();
}

cudaError_t build_knn(const float4 *means, uint32_t R, Neighbours *out, cudaStream_t s) {
  if (R == 0) return cudaSuccess;
  count_launch();
  knn_kernel<<<blocks_for(R, 128), 128, 0, s>>>(means, R, out);
  return cudaGetLastError();
}

}  // namespace pgl
