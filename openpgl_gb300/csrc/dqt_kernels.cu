// Directional quadtree field type: the per-region fit and update of
// DirectionalQuadtreeFactory (directional/dqt/DQTFactory.h:149-324) on the
// device, one thread block per region, regions handed out by an atomic queue.
//
// An update (DQTFactory.h:199-281) splats every sample of the region, in the
// region's sample order, into the leaves of the current statistics tree: a
// box of footprintFactor times the size of the leaf the sample's point falls
// in, clipped to the unit square, gives each leaf it overlaps the overlap's
// share of the box.  Per chunk of 256 samples each thread maps one sample to
// the square and finds its box; then each thread walks the chunk's samples in
// order and adds their shares to the leaves it owns, so every leaf's sums are
// the reference's sequential sums.  A leaf's overlap with a box is non-zero
// exactly when every ancestor's is (an ancestor's rectangle contains the
// leaf's), so visiting the leaves directly finds the leaves that the
// reference's depth-first descent reaches.  The sample and split weights
// (bottom-up), and the depth-first rebuild of the tree, run on one thread.
#include <cuda_runtime.h>

#include <cstdint>

#include "dqt.cuh"
#include "launch.h"
#include "pgl_internal.h"

namespace pgl {

constexpr int kDqtThreads = 256;

// the statistics' decay (Statistics::decay, DQTFactory.h:109-116)
__device__ void dqt_decay(DqtHead &h, DqtStatsNode *S, float a) {
  if (threadIdx.x == 0) h.numSamples *= a;
  for (uint32_t i = threadIdx.x; i < h.numNodes; i += blockDim.x) {
    S[i].numSamples *= a;
    S[i].first *= a;
    S[i].second *= a;
  }
  __syncthreads();
}

struct DqtScratch {
  Box2 *rect;
  DqtStatsNode *build;
  uint32_t *leaves;
};

// One update of a region's statistics and quadtree with `n` samples.
__device__ void dqt_update(DqtHead &h, DqtStatsNode *S, DqtNode *N, uint32_t stride, const DqtScratch &X,
                           const float4 *dirw, const float *pdf, uint32_t n, const DqtArgs &cfg, int *err) {
  __shared__ float sBox[kDqtThreads][4];
  __shared__ float sArea[kDqtThreads], sFirst[kDqtThreads], sSecond[kDqtThreads];
  __shared__ uint32_t sLeaf[kDqtThreads];
  __shared__ uint32_t numLeaves, newSize;
  // the factory's dispatch runs no branch for other values (DQTFactory.h:168-185)
  if (!(cfg.footprintFactor >= 0.0f) || (cfg.leafEstimator != 0 && cfg.leafEstimator != 1) ||
      (cfg.splitMetric != 0 && cfg.splitMetric != 1))
    return;
  const float ff = cfg.footprintFactor;
  if (threadIdx.x == 0) {
    h.numSamples += float(n);
    // rectangles of the current tree (children follow their parents) and its leaves
    X.rect[0] = Box2{0.f, 0.f, 1.f, 1.f};
    uint32_t L = 0;
    for (uint32_t i = 0; i < h.numNodes; ++i) {
      const uint32_t c0 = S[i].child;
      if (c0 > 0) {
        for (uint32_t c = 0; c < 4; ++c) X.rect[c0 + c] = X.rect[i].child(c);
      } else {
        X.leaves[L++] = i;
      }
    }
    numLeaves = L;
  }
  __syncthreads();
  const uint32_t L = numLeaves;
  for (uint32_t base = 0; base < n; base += kDqtThreads) {
    const uint32_t cnt = min(uint32_t(kDqtThreads), n - base);
    if (threadIdx.x < cnt) {
      const float4 d = dirw[base + threadIdx.x];
      const float p = pdf[base + threadIdx.x];
      float first, second;
      if (cfg.leafEstimator == 0) {  // REJECTION_SAMPLING
        first = d.w;
        second = d.w * d.w * p;
      } else {  // PER_LEAF
        first = d.w * p;
        second = first * first;
      }
      float px, py;
      dqt_dir_to_point(d.x, d.y, d.z, px, py);
      Box2 leaf;
      const uint32_t li = dqt_query(S, px, py, leaf);
      Box2 filter{0.f, 0.f, 0.f, 0.f};
      if (ff > 0.0f) {
        const float hx = ff * (leaf.x1 - leaf.x0) / 2.0f, hy = ff * (leaf.y1 - leaf.y0) / 2.0f;
        filter = Box2{px - hx, py - hy, px + hx, py + hy}.intersect(Box2{0.f, 0.f, 1.f, 1.f});
      }
      sBox[threadIdx.x][0] = filter.x0;
      sBox[threadIdx.x][1] = filter.y0;
      sBox[threadIdx.x][2] = filter.x1;
      sBox[threadIdx.x][3] = filter.y1;
      sArea[threadIdx.x] = filter.area();
      sFirst[threadIdx.x] = first;
      sSecond[threadIdx.x] = second;
      sLeaf[threadIdx.x] = li;
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < L; k += blockDim.x) {
      const uint32_t l = X.leaves[k];
      const Box2 r = X.rect[l];
      DqtStatsNode &node = S[l];
      float ns = node.numSamples, fs = node.first, ss = node.second;
      for (uint32_t s = 0; s < cnt; ++s) {
        float w;
        if (ff > 0.0f) {
          const Box2 f{sBox[s][0], sBox[s][1], sBox[s][2], sBox[s][3]};
          const float a = f.intersect(r).area();
          if (a == 0.0f) continue;
          w = a / sArea[s];
        } else {
          if (sLeaf[s] != l) continue;
          w = 1.0f;
        }
        ns += w;
        fs += w * sFirst[s];
        ss += w * sSecond[s];
      }
      node.numSamples = ns;
      node.first = fs;
      node.second = ss;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // sample and split weights bottom-up (DQTFactory.h:232-263)
    for (uint32_t i = h.numNodes; i-- > 0;) {
      DqtStatsNode &m = S[i];
      if (m.child > 0) {
        m.sampleWeight = 0.0f;
        m.splitWeight = 0.0f;
        for (uint32_t c = 0; c < 4; ++c) {
          m.sampleWeight += S[m.child + c].sampleWeight;
          m.splitWeight += S[m.child + c].splitWeight;
        }
      } else {
        const float k = cfg.leafEstimator == 0 ? 1.0f / h.numSamples : dqt_area(X.rect[i]) / m.numSamples;
        const float first = m.first * k, second = m.second * k;
        m.sampleWeight = first;
        m.splitWeight = cfg.splitMetric == 0 ? first : sqrtf(dqt_area(X.rect[i]) * second);
      }
    }
    // buildRecursive (DQTFactory.h:283-311): the new tree in depth-first
    // order, a node's four children allocated together when it is reached;
    // a leaf that splits gives its children a quarter of its statistics
    // (DQTFactory.h:313-324)
    struct Frame {
      uint32_t i, j, level, oc, c0;
      int c;
    };
    Frame st[40];
    int sp = 0;
    st[0] = Frame{0, 0, 0, 0, 0, -1};
    uint32_t size = 1;
    const float limit = cfg.splitThreshold * S[0].splitWeight;
    bool over = false;
    while (sp >= 0) {
      Frame &F = st[sp];
      if (F.c < 0) {
        const DqtStatsNode on = S[F.i];
        X.build[F.j] = on;
        if (F.level < cfg.maxLevels && on.splitWeight > limit) {
          if (size + 4 > stride || sp + 1 >= 40) {
            over = true;
            break;
          }
          const uint32_t c0 = size;
          X.build[F.j].child = c0;
          size += 4;
          if (on.child > 0) {
            F.c = 0;
            F.oc = on.child;
            F.c0 = c0;
            continue;
          }
          const DqtStatsNode par = X.build[F.j];
          for (uint32_t c = 0; c < 4; ++c) {
            DqtStatsNode &nn = X.build[c0 + c];
            nn.child = 0;
            nn.numSamples = par.numSamples / 4;
            nn.first = par.first / 4;
            nn.second = par.second / 4;
            nn.sampleWeight = par.sampleWeight / 4;
            nn.splitWeight = par.splitWeight / 4;
          }
        } else {
          X.build[F.j].child = 0;
        }
        --sp;
      } else if (F.c < 4) {
        const Frame child{F.oc + uint32_t(F.c), F.c0 + uint32_t(F.c), F.level + 1, 0, 0, -1};
        ++F.c;
        st[++sp] = child;
      } else {
        --sp;
      }
    }
    // a tree over the node bound (not possible for the bound's arguments)
    // keeps its previous nodes and fails the launch
    if (over) atomicCAS(err, 0, 3);
    newSize = over ? 0u : size;
  }
  __syncthreads();
  const uint32_t sz = newSize;
  if (sz > 0) {
    for (uint32_t i = threadIdx.x; i < sz; i += blockDim.x) {
      const DqtStatsNode b = X.build[i];
      S[i] = b;
      N[i] = DqtNode{b.child, b.sampleWeight};
    }
    if (threadIdx.x == 0) h.numNodes = sz;
  }
  __syncthreads();
}

__device__ bool dqt_stats_ok(float v) { return !isnan(v) && !isinf(v) && v >= 0.0f; }

__global__ void __launch_bounds__(kDqtThreads)
dqt_update_kernel(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, DqtSides sides, Box2 *rects,
                  DqtStatsNode *builds, uint32_t *leaves, uint32_t scratchStride, int *err) {
  __shared__ uint32_t taskId;
  __shared__ uint32_t statsBad;
  const DqtScratch X{rects + size_t(blockIdx.x) * scratchStride, builds + size_t(blockIdx.x) * scratchStride,
                     leaves + size_t(blockIdx.x) * scratchStride};
  for (;;) {
    if (threadIdx.x == 0) taskId = atomicAdd(queue, 1u);
    __syncthreads();
    if (taskId >= numTasks) break;
    const LeafTask t = tasks[taskId];
    const DqtSide &D = sides.side[(t.flags & kTaskVolume) ? 1 : 0];
    DqtHead &h = D.heads[t.region];
    DqtStatsNode *S = D.stats + size_t(t.region) * D.stride;
    DqtNode *N = D.nodes + size_t(t.region) * D.stride;
    const bool fit = (t.flags & kTaskFit) != 0;
    if (fit) {
      if (t.count > 0) {  // fitRegions (Field.h:389-439 -> DQTFactory.h:149-155): five decayed passes
        for (int k = 0; k < 5; ++k) {
          dqt_decay(h, S, 0.25f);
          dqt_update(h, S, N, D.stride, X, D.dirw + t.begin, D.pdf + t.begin, t.count, D.args, err);
        }
        if (threadIdx.x == 0) {
          h.pivot[0] = t.mean[0];
          h.pivot[1] = t.mean[1];
          h.pivot[2] = t.mean[2];
          h.valid = (!isinf(N[0].weight) && N[0].weight > 0.0f) ? 1u : 0u;
        }
      } else if (threadIdx.x == 0) {
        h.valid = 0;
      }
    } else {
      if (t.flags & kTaskDecay) dqt_decay(h, S, D.decay);  // Field.h:457-461
      if (t.count > 0) {
        dqt_update(h, S, N, D.stride, X, D.dirw + t.begin, D.pdf + t.begin, t.count, D.args, err);
        // DirectionalQuadtree::isValid and Statistics::isValid (DQT.h:40-42, DQTFactory.h:95-107)
        if (threadIdx.x == 0) statsBad = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < h.numNodes; i += blockDim.x) {
          const DqtStatsNode &m = S[i];
          if (!dqt_stats_ok(m.sampleWeight) || !dqt_stats_ok(m.splitWeight) || !dqt_stats_ok(m.numSamples) ||
              !dqt_stats_ok(m.first) || !dqt_stats_ok(m.second))
            atomicOr(&statsBad, 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          const bool treeOk = !isinf(N[0].weight) && N[0].weight > 0.0f;
          const bool statsOk = !statsBad && S[0].sampleWeight > 0.0f && S[0].splitWeight > 0.0f;
          h.valid = (treeOk && statsOk) ? 1u : 0u;
        }
      }
    }
    __syncthreads();
  }
}

// New regions start as copies of the region they split from (head and both
// node arrays).
__global__ void dqt_copy_kernel(DqtHead *heads, DqtStatsNode *stats, DqtNode *nodes, uint32_t stride,
                                const uint32_t *dst, const uint32_t *src, uint32_t n) {
  const uint32_t k = blockIdx.x;
  if (k >= n) return;
  const uint32_t a = src[k], b = dst[k];
  if (threadIdx.x == 0) heads[b] = heads[a];
  const uint32_t m = heads[a].numNodes;
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
    stats[size_t(b) * stride + i] = stats[size_t(a) * stride + i];
    nodes[size_t(b) * stride + i] = nodes[size_t(a) * stride + i];
  }
}

// A region in the reference's initial state: one leaf, zero statistics.
__global__ void dqt_init_kernel(DqtHead *heads, DqtStatsNode *stats, DqtNode *nodes, uint32_t stride, uint32_t first,
                                uint32_t n) {
  const uint32_t r = first + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= first + n) return;
  heads[r] = DqtHead{{0.f, 0.f, 0.f}, 0.0f, 1u, 0u, {0u, 0u}};
  stats[size_t(r) * stride] = DqtStatsNode{0u, 0.f, 0.f, 0.f, 0.f, 0.f};
  nodes[size_t(r) * stride] = DqtNode{0u, 0.f};
}

cudaError_t launch_dqt_update(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, const DqtSides &sides,
                              Box2 *rects, DqtStatsNode *builds, uint32_t *leaves, uint32_t scratchStride, int blocks,
                              int *err, cudaStream_t s) {
  if (numTasks == 0) return cudaSuccess;
  count_launch();
  dqt_update_kernel<<<unsigned(blocks), kDqtThreads, 0, s>>>(tasks, numTasks, queue, sides, rects, builds, leaves,
                                                             scratchStride, err);
  return cudaGetLastError();
}
cudaError_t launch_dqt_copy(DqtHead *heads, DqtStatsNode *stats, DqtNode *nodes, uint32_t stride, const uint32_t *dst,
                            const uint32_t *src, uint32_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  dqt_copy_kernel<<<n, 256, 0, s>>>(heads, stats, nodes, stride, dst, src, n);
  return cudaGetLastError();
}
cudaError_t launch_dqt_init(DqtHead *heads, DqtStatsNode *stats, DqtNode *nodes, uint32_t stride, uint32_t first,
                            uint32_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  dqt_init_kernel<<<(n + 127) / 128, 128, 0, s>>>(heads, stats, nodes, stride, first, n);
  return cudaGetLastError();
}

}  // namespace pgl
