// Per-leaf directional fitting on the GPU: parallax-aware vMF mixtures fitted
// by weighted MAP-EM with chi-square split and merge, one thread block per
// leaf (region), leaves handed out by an atomic work queue.
//
// What it computes is Open PGL's AdaptiveSplitAndMergeFactory::fit/update
// (directional/vmm/AdaptiveSplitandMergeFactory.h:303-462) on a leaf's
// deterministically sorted, parallax-reprojected samples, with the weighted EM
// of ParallaxAwareVonMisesFisherWeightedEMFactory.h:717-1326 and the splitter
// and merger of VMMChiSquareComponentSplitter.h / VMMChiSquareComponentMerger.h.
//
// How it is laid out for the GPU: a pass over a leaf's samples (E-step,
// distance pass, split-statistics pass) streams the samples in chunks through
// a two-stage producer/consumer pipeline (see "sample passes" below):
// producer threads compute each sample's lobe terms and pdf, consumer threads
// (one per accumulator, e.g. the x component of lobe 7's weighted direction
// sum) add the chunk's terms in sample order.  That keeps the reference's
// summation order (sequential over samples within each SIMD lane), so every
// accumulator gets the reference's bits.  Scalar per-leaf logic (M step,
// split/merge bookkeeping) runs on thread 0 between passes.
#include <cuda_runtime.h>

#include <cstddef>

#include "launch.h"
#include "pgl_internal.h"

namespace pgl {

constexpr int kEmThreads = 512;
constexpr int kStageFloats = 19200;  // floats per pipeline stage (two stages, 150 KB)

// E-step passes shared between blocks.  Every block owns a board and a ring of
// chunk slots in global memory.  For each E-step pass the home block publishes
// the pass on its board (lobe parameters, sample range, chunk shape).  Its own
// producer warps take chunks from the board's grab word and write them
// straight into its shared-memory stages; a block that has run out of leaves
// (a helper) takes chunks from the same grab word and writes them into the
// ring, from where the home block's loader warp copies them into the stages
// with bulk copies.  The consumer warps add the chunks in chunk order.
constexpr int kMaxStages = 8;                          // consumer pipeline stages
constexpr int kMaxChunk = 768;                         // E-step samples per chunk at most (chunk divisor 1)
constexpr uint32_t kRingFloats = 65536;                // ring per block (256 KB)
constexpr uint32_t kRingMaxSlots = 64;
constexpr unsigned long long kWaitNs = 2000000000ull;  // longest wait before the launch fails
constexpr uint32_t kGrabIdxBits = 22;                  // grab word: generation | chunks | next chunk
constexpr uint32_t kGrabMask = (1u << kGrabIdxBits) - 1u;
constexpr uint32_t kGrabGenMask = (1u << 20) - 1u;
constexpr uint32_t kMaxSharedChunks = kGrabMask - 4096u;

enum EmError { kErrNone = 0, kErrChunkWait = 1, kErrSlotWait = 2, kErrCopyWait = 3, kErrLeafTooLarge = 4 };

struct __align__(16) BoardParams {  // one pass as its home block publishes it
  float4 lobeA[kMaxK + kMaxK / kLanes];
  float2 lobeB[kMaxK];
  const float4 *dirw;
  uint32_t count, seqBase, cnt, pad;
};
struct __align__(128) Board {
  unsigned long long grab;     // generation (bits 44..63), chunks (22..43), next chunk (0..21)
  uint32_t pad0[30];
  uint32_t consumed;           // chunks (sequence numbers) whose ring slots are free again
  uint32_t pad1[31];
  uint32_t helpers;            // helper blocks attached to the board (at most EmTuning::maxHelpers)
  uint32_t pad2[31];
  uint32_t ready[kRingMaxSlots];  // per ring slot: sequence number of the chunk it holds
  BoardParams params[2];          // by generation parity
};

struct Unassigned {
  float sw, dx, dy, dz;
};

struct EmShared {
  VMMState vmm;
  SuffState suff;     // training statistics ("previous" statistics of EM)
  SplitState split;   // training split statistics
  SuffState cur;      // statistics of the current EM iteration
  SuffState temp;     // statistics of a partial refit
  SplitState lsplit;  // split statistics used by the recursive splitting
  Frame invFrame[kMaxK];
  __align__(16) float pbuf[2 * kStageFloats];  // the two pipeline stages
  __align__(16) float4 lobeA[kMaxK + kMaxK / kLanes];  // mean direction, kappa (entry k + k / 8)
  float2 lobeB[kMaxK];                // normalisation, weight
  float lobeWInv[kMaxK];              // RN(1 / weight) for div_rcp
  float xch[2][kMaxK];
  uint32_t rcpTab[2048];
  float cost[kMaxK][kMaxK];  // merge cost of components i < j (cost[i][j])
  float ll;
  Unassigned un;
  int mask[kMaxK];
  int loopFlag;
  int splitCount;
  int candIdx[kMaxK];
  float candChi[kMaxK];
  int numCands;
  float mcEstimate;
  int iterations;
  LeafReport report;
  LeafProfile prof;
  unsigned long long full[kMaxStages];  // stage holds its chunk (bulk copy or own producers)
  uint32_t stageUses[kMaxStages];       // completed phases of a stage's barrier
  uint32_t warpDone[kEmThreads / 32];   // chunks of the pass each consumer warp has added
  uint32_t own[64];    // sequence numbers of chunks this block's producers took
  BoardParams hp;      // a helper's copy of the pass it produces for
  Board *board;        // this block's board and ring
  float *ring;
  int *err;            // EmError of the launch
  uint32_t gen, seqBase, abortAt;
  EmTuning tune;       // the launch's schedule parameters (the same in every block)
  int hgrab[2], grabbed, helpBoard, helpExit;
  uint32_t grabGen;
  int grabExact;                                  // the chunk taken is the one whose slot was checked
  int nextGrabbed, nextExact, hasNext;            // a helper's next chunk, taken while producing
  uint32_t nextGen;
  uint32_t scanRem[kEmThreads / 32];
  int scanIdx[kEmThreads / 32];
  uint32_t validPerWarp[kEmThreads / 32];  // split passes: valid samples per producer warp
  float splitN0[kMaxK];                     // split passes: chi-square counts at the pass start
};
static_assert(offsetof(EmShared, pbuf) % 16 == 0 && offsetof(EmShared, lobeA) % 16 == 0 &&
                  offsetof(EmShared, hp) % 16 == 0 && offsetof(EmShared, full) % 8 == 0,
              "128-bit shared loads");

// cycle accounting of thread 0 (LeafProfile)
#define PGL_PROF_BEGIN(t) const long long t = clock64();
#define PGL_PROF_END(t, field) \
  if (threadIdx.x == 0) S.prof.field += uint64_t(clock64() - (t));

// ---------------------------------------------------------------- scalar helpers (thread 0)

__device__ void vmm_calc_norm(VMMState &v) {  // PAVMM.h:852-863
  int c = vec_count(int(v.K));
  for (int k = 0; k < c * kLanes; ++k) {
    v.e2k[k] = fexp(-2.0f * v.kappa[k]);
    float nrm = v.kappa[k] / (kTwoPiF * (1.0f - v.e2k[k]));
    v.norm[k] = v.kappa[k] > 0.0f ? nrm : kInv4Pi;
  }
}
__device__ void vmm_calc_mean_cosines(VMMState &v) {  // PAVMM.h:866-877
  int c = vec_count(int(v.K));
  for (int k = 0; k < c * kLanes; ++k) {
    float th = 1.0f - 2.0f / (fexp(2.0f * v.kappa[k]) - 1.0f);
    float m = 1.0f / th - 1.0f / v.kappa[k];
    v.mc[k] = v.kappa[k] > 0.0f ? m : 0.0f;
  }
}
__device__ void vmm_init_uniform(VMMState &v, int K, float kappa, const float *dirs) {  // WEMFactory.h:633-664
  v.K = uint32_t(K);
  float weight = 1.0f / float(K);
  const float *d = dirs + (K - 1) * kMaxK * 3;
  for (int n = 0; n < kMaxK; ++n) {
    v.mx[n] = d[3 * n + 0];
    v.my[n] = d[3 * n + 1];
    v.mz[n] = d[3 * n + 2];
    if (n < K) {
      v.kappa[n] = kappa;
      v.w[n] = weight;
    } else {
      v.kappa[n] = 0.0f;
      v.w[n] = 0.0f;
      v.norm[n] = kInv4Pi;
      v.e2k[n] = 1.0f;
      v.mc[n] = 0.0f;
    }
  }
  vmm_calc_norm(v);
  vmm_calc_mean_cosines(v);
}
__device__ void vmm_swap(VMMState &v, int i, int j) {
  if (i == j) return;
#define PGL_SWAPF(a) { float t_ = v.a[i]; v.a[i] = v.a[j]; v.a[j] = t_; }
  PGL_SWAPF(w) PGL_SWAPF(kappa) PGL_SWAPF(e2k) PGL_SWAPF(mc) PGL_SWAPF(norm) PGL_SWAPF(mx) PGL_SWAPF(my) PGL_SWAPF(mz) PGL_SWAPF(dist)
#undef PGL_SWAPF
}
__device__ void vmm_clear(VMMState &v, int i) {
  v.w[i] = 0.0f; v.kappa[i] = 0.0f; v.e2k[i] = 1.0f; v.mc[i] = 0.0f; v.norm[i] = kInv4Pi;
  v.mx[i] = 0.0f; v.my[i] = 0.0f; v.mz[i] = 1.0f; v.dist[i] = 0.0f;
}
__device__ void vmm_merge(VMMState &v, int i0, int i1) {  // PAVMM.h:259-343
  if (i0 == i1) return;
  float w0 = v.w[i0], w1 = v.w[i1], mc0 = v.mc[i0], mc1 = v.mc[i1];
  float kappa = 0.0f, nrm = kInv4Pi, e2k = 1.0f, w = w0 + w1;
  float mx = (w0 * mc0) * v.mx[i0] + (w1 * mc1) * v.mx[i1];
  float my = (w0 * mc0) * v.my[i0] + (w1 * mc1) * v.my[i1];
  float mz = (w0 * mc0) * v.mz[i0] + (w1 * mc1) * v.mz[i1];
  mx /= w; my /= w; mz /= w;
  float mc = mx * mx + my * my + mz * mz;
  if (mc > 0.0f) {
    mc = sqrtf(mc);
    kappa = mean_cosine_to_kappa(mc);
    kappa = kappa < 1e-3f ? 0.f : kappa;
    e2k = lib_expf(-2.0f * kappa);
    nrm = vmf_norm_double(kappa, e2k);
    mx /= mc; my /= mc; mz /= mc;
  } else {
    mx = v.mx[i0]; my = v.my[i0]; mz = v.mz[i0];
  }
  v.w[i0] = w; v.kappa[i0] = kappa; v.mc[i0] = mc; v.norm[i0] = nrm; v.e2k[i0] = e2k;
  v.mx[i0] = mx; v.my[i0] = my; v.mz[i0] = mz;
  float nd = w0 * v.dist[i0] + w1 * v.dist[i1];
  nd /= (w0 + w1);
  v.dist[i0] = nd;
  vmm_swap(v, i1, int(v.K) - 1);
  vmm_clear(v, int(v.K) - 1);
  v.K -= 1;
}
__device__ void vmm_split(VMMState &v, int i0, int i1, float w0, float w1, V3 m0, V3 m1, float mc0, float mc1) {
  v.dist[i1] = v.dist[i0];  // PAVMM.h:225-255
  v.w[i0] = w0; v.mc[i0] = mc0; v.kappa[i0] = mean_cosine_to_kappa(mc0);
  v.mx[i0] = m0.x; v.my[i0] = m0.y; v.mz[i0] = m0.z;
  v.w[i1] = w1; v.mc[i1] = mc1; v.kappa[i1] = mean_cosine_to_kappa(mc1);
  v.mx[i1] = m1.x; v.my[i1] = m1.y; v.mz[i1] = m1.z;
  if (uint32_t(i1) == v.K) v.K++;
  vmm_calc_norm(v);
}
__device__ void vmm_parallax_shift(VMMState &v, V3 s) {  // PAVMM.h:809-831
  int c = vec_count(int(v.K));
  for (int k = 0; k < c * kLanes; ++k) {
    V3 p = mk(v.mx[k], v.my[k], v.mz[k]) * v.dist[k] + s;
    float len = length(p);
    p = p / len;
    bool cond = (v.dist[k] > 0.0f) && (v.dist[k] >= -FLT_MAX) && (v.dist[k] <= FLT_MAX);
    if (cond) { v.mx[k] = p.x; v.my[k] = p.y; v.mz[k] = p.z; }
    v.dist[k] = v.dist[k] > 0.0f ? len : 0.0f;
  }
  v.pivot[0] -= s.x; v.pivot[1] -= s.y; v.pivot[2] -= s.z;
}
__device__ bool vmm_is_valid(const VMMState &v) {  // PAVMM.h:422-513
  bool ok = true;
  for (uint32_t k = 0; k < v.K && k < kMaxK; ++k) {
    ok = ok && isvalidf(v.w[k]) && v.w[k] >= 0.0f && v.w[k] <= 1.0f + 1e-6f;
    ok = ok && isvalidf(v.kappa[k]) && v.kappa[k] >= 0.0f;
    ok = ok && isvalidf(v.mc[k]) && v.mc[k] >= 0.0f && v.mc[k] <= 1.0f;
    ok = ok && isvalidf(v.mx[k]) && v.mx[k] >= -1.0f && v.mx[k] <= 1.0f;
    ok = ok && isvalidf(v.my[k]) && v.my[k] >= -1.0f && v.my[k] <= 1.0f;
    ok = ok && isvalidf(v.mz[k]) && v.mz[k] >= -1.0f && v.mz[k] <= 1.0f;
    ok = ok && isvalidf(v.norm[k]) && v.norm[k] >= 0.0f && isvalidf(v.e2k[k]);
    ok = ok && isvalidf(v.dist[k]) && v.dist[k] >= 0.0f;
  }
  for (uint32_t k = v.K; k < kMaxK; ++k) {
    ok = ok && v.w[k] == 0.0f && v.kappa[k] == 0.0f && v.mx[k] == 0.0f && v.my[k] == 0.0f && v.mz[k] == 1.0f;
    ok = ok && v.mc[k] == 0.0f && fabsf(v.norm[k] - kInv4Pi) < 1e-6f && v.e2k[k] == 1.0f && v.dist[k] == 0.0f;
  }
  return ok;
}

__device__ void suff_clear(SuffState &s, uint32_t K) {
  s.K = K;
  int c = vec_count(int(K));
  for (int k = 0; k < c * kLanes; ++k) s.dx[k] = s.dy[k] = s.dz[k] = s.w[k] = s.dw[k] = 0.0f;
  s.sumWeights = 0.0f; s.numSamples = 0.0f; s.normalized = 0;
}
__device__ void suff_normalize(SuffState &s, float n) {  // WEMFactory.h:553-572
  int c = vec_count(int(s.K));
  s.numSamples = n;
  float sv[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < c * kLanes; ++k) sv[k % kLanes] += s.w[k];
  s.sumWeights = reduce8(sv);
  float nrm = n / s.sumWeights;
  for (int k = 0; k < c * kLanes; ++k) { s.dx[k] *= nrm; s.dy[k] *= nrm; s.dz[k] *= nrm; s.w[k] *= nrm; }
  s.normalized = 1;
}
__device__ void suff_add(SuffState &a, const SuffState &b) {  // WEMFactory.h:575-593
  int c = vec_count(int(a.K));
  a.sumWeights += b.sumWeights;
  a.numSamples += b.numSamples;
  a.overallNumSamples += b.numSamples;
  for (int k = 0; k < c * kLanes; ++k) {
    a.dx[k] += b.dx[k]; a.dy[k] += b.dy[k]; a.dz[k] += b.dz[k]; a.w[k] += b.w[k]; a.dw[k] += b.dw[k];
  }
}
__device__ void suff_masked_replace(SuffState &a, const int *mask, const SuffState &b) {  // WEMFactory.h:448-468
  float sv[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < kMaxK; ++k) {
    if (mask[k]) { a.dx[k] = b.dx[k]; a.dy[k] = b.dy[k]; a.dz[k] = b.dz[k]; a.w[k] = b.w[k]; a.dw[k] = b.dw[k]; }
    sv[k % kLanes] += a.w[k];
  }
  if (a.normalized) a.numSamples = reduce8(sv); else a.sumWeights = reduce8(sv);
}
__device__ void suff_decay(SuffState &s, float a) {
  for (int k = 0; k < kMaxK; ++k) { s.dx[k] *= a; s.dy[k] *= a; s.dz[k] *= a; s.w[k] *= a; s.dw[k] *= a; }
  s.numSamples *= a; s.sumWeights *= a;
}
__device__ void suff_parallax_shift(SuffState &s, const VMMState &v, V3 shift) {  // WEMFactory.h:265-283
  int c = vec_count(int(v.K));
  for (int k = 0; k < c * kLanes; ++k) {
    V3 d0 = mk(s.dx[k], s.dy[k], s.dz[k]);
    float smc = length(d0);
    V3 d = d0 / smc;
    d = d * v.dist[k];
    d = d + shift;
    d = d / length(d);
    d = d * smc;
    d = smc > 0.0f ? d : d0;
    if (v.dist[k] > 0.0f) { s.dx[k] = d.x; s.dy[k] = d.y; s.dz[k] = d.z; }
  }
}
__device__ void suff_split(SuffState &s, int i, int j, V3 m0, V3 m1, float mc0, float mc1) {  // WEMFactory.h:516-550
  float sw = s.w[i];
  sw /= 2.0f;
  s.w[i] = sw; s.dx[i] = (m0.x * mc0) * sw; s.dy[i] = (m0.y * mc0) * sw; s.dz[i] = (m0.z * mc0) * sw;
  s.w[j] = sw; s.dx[j] = (m1.x * mc1) * sw; s.dy[j] = (m1.y * mc1) * sw; s.dz[j] = (m1.z * mc1) * sw;
  float t = s.dw[i] * 0.5f;
  s.dw[i] = t; s.dw[j] = t;
  s.K += 1;
}
__device__ void suff_merge(SuffState &s, int i0, int i1) {  // WEMFactory.h:485-513
  int L = int(s.K) - 1;
  s.dx[i0] += s.dx[i1]; s.dy[i0] += s.dy[i1]; s.dz[i0] += s.dz[i1]; s.w[i0] += s.w[i1]; s.dw[i0] += s.dw[i1];
  s.dx[i1] = s.dx[L]; s.dy[i1] = s.dy[L]; s.dz[i1] = s.dz[L]; s.w[i1] = s.w[L]; s.dw[i1] = s.dw[L];
  s.dx[L] = s.dy[L] = s.dz[L] = s.w[L] = s.dw[L] = 0.0f;
  s.K--;
}
__device__ bool suff_is_valid(const SuffState &s) {
  bool ok = true;
  for (uint32_t k = 0; k < s.K && k < kMaxK; ++k)
    ok = ok && isvalidf(s.dx[k]) && isvalidf(s.dy[k]) && isvalidf(s.dz[k]) && isvalidf(s.w[k]) && s.w[k] >= 0.0f &&
         isvalidf(s.dw[k]) && s.dw[k] >= 0.0f;
  for (uint32_t k = s.K; k < kMaxK; ++k)
    ok = ok && s.dx[k] == 0.0f && s.dy[k] == 0.0f && s.dz[k] == 0.0f && s.w[k] == 0.0f && s.dw[k] == 0.0f;
  return ok && isvalidf(s.numSamples) && s.numSamples >= 0.0f && isvalidf(s.sumWeights) && s.sumWeights >= 0.0f;
}
__device__ void split_clear(SplitState &s, uint32_t K) {
  s.K = K;
  int c = vec_count(int(K));
  for (int k = 0; k < c * kLanes; ++k)
    s.chi2[k] = s.cx[k] = s.cy[k] = s.cz[k] = s.mx[k] = s.my[k] = s.n[k] = s.sw[k] = s.sa[k] = 0.0f;
}
__device__ void split_zero_lane(SplitState &s, int i) {
  s.chi2[i] = s.sa[i] = s.n[i] = s.sw[i] = s.mx[i] = s.my[i] = s.cx[i] = s.cy[i] = s.cz[i] = 0.0f;
}
__device__ void split_decay(SplitState &s, float a) {
  int c = vec_count(int(s.K));
  for (int k = 0; k < c * kLanes; ++k) { s.cx[k] *= a; s.cy[k] *= a; s.cz[k] *= a; s.n[k] *= a; s.sw[k] *= a; s.sa[k] *= a; }
}
__device__ bool split_is_valid(const SplitState &s) {
  bool lane[kLanes];
  for (int j = 0; j < kLanes; ++j) lane[j] = true;
  for (int k = 0; k < kMaxK; ++k) {
    bool ok = isvalidf(s.mx[k]) && isvalidf(s.my[k]) && isvalidf(s.cx[k]) && isvalidf(s.cy[k]) && isvalidf(s.cz[k]) &&
              isvalidf(s.chi2[k]) && s.chi2[k] >= 0.0f && isvalidf(s.sw[k]) && s.sw[k] >= 0.0f && isvalidf(s.sa[k]) &&
              s.sa[k] >= 0.0f && isvalidf(s.n[k]) && s.n[k] >= 0.0f;
    lane[k % kLanes] = lane[k % kLanes] && ok;
  }
  bool any = false;
  for (int j = 0; j < kLanes; ++j) any = any || lane[j];
  return any && s.K > 0 && s.K <= kMaxK;
}

// MAP M-step (WEMFactory.h:895-1148); mask == nullptr is the full step.
__device__ void map_step(VMMState &v, const SuffState &cur, const SuffState &prev, const FieldConfig &cfg, const int *mask) {
  int c = vec_count(int(v.K));
  float K = float(v.K);
  float N = cur.numSamples + prev.numSamples;
  int rem = int(v.K % kLanes);
  if (!mask) {
    for (int k = 0; k < c * kLanes; ++k) {
      float w = cur.w[k] + prev.w[k];
      v.w[k] = (cfg.weightPrior + w) / ((cfg.weightPrior * K) + N);
    }
  } else {
    float sw[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0}, sp[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < c * kLanes; ++k) {
      float w = cur.w[k] + prev.w[k];
      w = (cfg.weightPrior + w) / ((cfg.weightPrior * K) + N);
      sp[k % kLanes] += mask[k] ? w : 0.0f;
      sw[k % kLanes] += mask[k] ? 0.0f : v.w[k];
      v.w[k] = mask[k] ? w : v.w[k];
    }
    float inv = 1.0f / reduce8(sp);
    inv *= 1.0f - reduce8(sw);
    for (int k = 0; k < c * kLanes; ++k) v.w[k] = mask[k] ? v.w[k] * inv : v.w[k];
  }
  if (rem > 0)
    for (int i = rem; i < kLanes; ++i) v.w[(c - 1) * kLanes + i] = 0.0f;

  float curN = cur.numSamples, prevN = prev.numSamples, NN = curN + prevN;
  float overallN = cur.numSamples + prev.overallNumSamples;
  float curW = curN / NN, prevW = 1.0f - curW;
  for (int k = 0; k < c * kLanes; ++k) {
    float partialN = v.w[k] * overallN;
    V3 cm = cur.w[k] > 0.0f ? mk(cur.dx[k] / cur.w[k], cur.dy[k] / cur.w[k], cur.dz[k] / cur.w[k]) : mk(0, 0, 0);
    V3 pm = prev.w[k] > 0.0f ? mk(prev.dx[k] / prev.w[k], prev.dy[k] / prev.w[k], prev.dz[k] / prev.w[k]) : mk(0, 0, 0);
    V3 md = cm * curW + pm * prevW;
    float mc = length(md);
    bool upd = mask ? (mask[k] != 0) : true;
    if (upd && mc > 0.0f) { v.mx[k] = md.x / mc; v.my[k] = md.y / mc; v.mz[k] = md.z / mc; }
    mc = (cfg.mcPrior * cfg.mcPriorStrength + mc * partialN) / (cfg.mcPriorStrength + partialN);
    mc = emin(cfg.maxMeanCosine, mc);
    if (upd) { v.mc[k] = mc; v.kappa[k] = mean_cosine_to_kappa(mc); }
  }
  if (rem > 0)
    for (int i = rem; i < kLanes; ++i) {
      int k = (c - 1) * kLanes + i;
      v.mx[k] = 0.0f; v.my[k] = 0.0f; v.mz[k] = 1.0f; v.mc[k] = 0.0f; v.kappa[k] = 0.0f;
      if (!mask) { v.norm[k] = kInv4Pi; v.e2k[k] = 1.0f; }
    }
  vmm_calc_norm(v);
}

// suff_normalize and map_step by one warp, lane k doing lobe k: every lobe's
// arithmetic is the scalar functions' own; the sums over lobes keep the
// scalar order (vfloat8 lane sums over k, then the 8-lane reduction) on lane 0.
__device__ void suff_normalize_warp(SuffState &s, float n) {
  const unsigned full = 0xFFFFFFFFu;
  const int k = int(threadIdx.x & 31);
  const int Kp = vec_count(int(s.K)) * kLanes;
  float nrm = 0.0f;
  if (k == 0) {
    s.numSamples = n;
    float sv[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < Kp; ++j) sv[j % kLanes] += s.w[j];
    s.sumWeights = reduce8(sv);
    nrm = n / s.sumWeights;
    s.normalized = 1;
  }
  nrm = __shfl_sync(full, nrm, 0);  // lane 0 has read every weight
  if (k < Kp) {
    s.dx[k] *= nrm;
    s.dy[k] *= nrm;
    s.dz[k] *= nrm;
    s.w[k] *= nrm;
  }
  __syncwarp();
}
__device__ void map_step_warp(VMMState &v, const SuffState &cur, const SuffState &prev, const FieldConfig &cfg,
                              const int *mask) {
  const unsigned full = 0xFFFFFFFFu;
  const int k = int(threadIdx.x & 31);
  const int c = vec_count(int(v.K)), Kp = c * kLanes;
  const bool act = k < Kp;
  const float K = float(v.K);
  const float N = cur.numSamples + prev.numSamples;
  const int rem = int(v.K % kLanes);
  if (!mask) {
    if (act) {
      const float w = cur.w[k] + prev.w[k];
      v.w[k] = (cfg.weightPrior + w) / ((cfg.weightPrior * K) + N);
    }
  } else {
    float wNew = 0.0f, wOld = 0.0f;
    int m = 0;
    if (act) {
      const float w = cur.w[k] + prev.w[k];
      wNew = (cfg.weightPrior + w) / ((cfg.weightPrior * K) + N);
      wOld = v.w[k];
      m = mask[k];
    }
    // lane sums over the lobes in order, on lane 0
    float sw[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0}, sp[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < Kp; ++j) {
      const float pj = __shfl_sync(full, m ? wNew : 0.0f, j);
      const float wj = __shfl_sync(full, m ? 0.0f : wOld, j);
      sp[j % kLanes] += pj;
      sw[j % kLanes] += wj;
    }
    float inv = 0.0f;
    if (k == 0) {
      inv = 1.0f / reduce8(sp);
      inv *= 1.0f - reduce8(sw);
    }
    inv = __shfl_sync(full, inv, 0);
    if (act) v.w[k] = m ? wNew * inv : wOld;
  }
  if (rem > 0 && k >= (c - 1) * kLanes + rem && k < Kp) v.w[k] = 0.0f;

  const float curN = cur.numSamples, prevN = prev.numSamples, NN = curN + prevN;
  const float overallN = cur.numSamples + prev.overallNumSamples;
  const float curW = curN / NN, prevW = 1.0f - curW;
  if (act) {
    const float partialN = v.w[k] * overallN;
    const V3 cm = cur.w[k] > 0.0f ? mk(cur.dx[k] / cur.w[k], cur.dy[k] / cur.w[k], cur.dz[k] / cur.w[k]) : mk(0, 0, 0);
    const V3 pm =
        prev.w[k] > 0.0f ? mk(prev.dx[k] / prev.w[k], prev.dy[k] / prev.w[k], prev.dz[k] / prev.w[k]) : mk(0, 0, 0);
    const V3 md = cm * curW + pm * prevW;
    float mc = length(md);
    const bool upd = mask ? (mask[k] != 0) : true;
    if (upd && mc > 0.0f) {
      v.mx[k] = md.x / mc;
      v.my[k] = md.y / mc;
      v.mz[k] = md.z / mc;
    }
    mc = (cfg.mcPrior * cfg.mcPriorStrength + mc * partialN) / (cfg.mcPriorStrength + partialN);
    mc = emin(cfg.maxMeanCosine, mc);
    if (upd) {
      v.mc[k] = mc;
      v.kappa[k] = mean_cosine_to_kappa(mc);
    }
    if (rem > 0 && k >= (c - 1) * kLanes + rem) {
      v.mx[k] = 0.0f; v.my[k] = 0.0f; v.mz[k] = 1.0f; v.mc[k] = 0.0f; v.kappa[k] = 0.0f;
      if (!mask) { v.norm[k] = kInv4Pi; v.e2k[k] = 1.0f; }
    }
    // vmm_calc_norm for lobe k
    v.e2k[k] = fexp(-2.0f * v.kappa[k]);
    const float nrm = v.kappa[k] / (kTwoPiF * (1.0f - v.e2k[k]));
    v.norm[k] = v.kappa[k] > 0.0f ? nrm : kInv4Pi;
  }
  __syncwarp();
}

__device__ void map3d_to_2d(V3 d, float &x, float &y) {  // Splitter.h:161-171
  float alpha = facos(d.z);
  float inv_sinc = alpha / fsin(alpha);
  x = alpha > 0.0f ? d.x * inv_sinc : 0.0f;
  y = alpha > 0.0f ? d.y * inv_sinc : 0.0f;
}
__device__ V3 map2d_to_3d(float x, float y) {  // Splitter.h:174-186
  float len = sqrtf(x * x + y * y);
  float sinc = fsin(len) / len;
  V3 r;
  r.x = len > 0.0f ? x * sinc : 0.0f;
  r.y = len > 0.0f ? y * sinc : 0.0f;
  r.z = lib_cosf(len);
  return r;
}

// SplitComponent (Splitter.h:527-665)
__device__ bool split_component(VMMState &v, SplitState &sp, SuffState &suff, int idx, const FieldConfig &cfg) {
  float numAssigned = sp.sa[idx];
  float invSW = rcp_avx2(sp.sw[idx]);
  float meanx = sp.mx[idx], meany = sp.my[idx];
  float cx = sp.cx[idx] * invSW, cy = sp.cy[idx] * invSW, cz = sp.cz[idx] * invSW;
  float D = sqrtf((cx - cy) * (cx - cy) + ((cz * cz) * 4.0f)) * 0.5f;
  float ev0 = float(double(cx + cy) * 0.5);
  ev0 += D;
  float e0x = -cz, e0y = cx - ev0;
  float l0 = sqrtf(e0x * e0x + e0y * e0y);
  e0x /= l0;
  e0y /= l0;
  float w = v.w[idx], mc = v.mc[idx], kappa = v.kappa[idx];
  if (double(kappa) >= double(cfg.maxKappaSplit) * 0.9) return false;
  V3 mu = mk(v.mx[idx], v.my[idx], v.mz[idx]);
  float nw0 = w * 0.5f, nw1 = nw0;
  V3 m0 = mu, m1 = mu;
  float nmc0 = mc, nmc1 = mc * mc;
  if (D > 1e-8f) {
    float ax = (e0x * ev0) * 0.5f, ay = (e0y * ev0) * 0.5f;
    Frame fr = frame_of(mu, false);
    m0 = xfm(fr, map2d_to_3d(meanx + ax, meany + ay));
    nmc0 = mc / fabsf(dot(mu, m0));
    nmc0 = smin(nmc0, cfg.maxMeanCosineSplit);
    nmc1 = nmc0;
    m1 = xfm(fr, map2d_to_3d(meanx - ax, meany - ay));
  } else {
    if (numAssigned < 2.0f) return false;
  }
  int K = int(v.K);
  vmm_split(v, idx, K, nw0, nw1, m0, m1, nmc0, nmc1);
  suff_split(suff, idx, K, m0, m1, nmc0, nmc1);
  split_zero_lane(sp, idx);
  split_zero_lane(sp, K);
  sp.K = uint32_t(K + 1);
  return true;
}

// ---------------------------------------------------------------- merge cost (parallel over pairs)
__device__ float product_scale(V3 m0, float k0, float n0, V3 m1, float k1, float n1, V3 &pm, float &pk, float &pn) {
  pm = m0 * k0 + m1 * k1;  // Merger.h:368-396
  pk = sqrtf(dot(pm, pm));
  pn = float(1.0 / (4.0 * kPiD));
  if (pk > 1e-3f) {
    float pe = lib_expf(-2.0f * pk);
    pn = vmf_norm_double(pk, pe);
    pm = pm / pk;
  } else {
    pk = 0.0f;
    pm = m0;
  }
  float scale = (n0 * n1) / pn;
  float c0 = dot(m0, pm), c1 = dot(m1, pm);
  scale *= lib_expf(k0 * (c0 - 1.0f) + k1 * (c1 - 1.0f));
  return scale;
}
__device__ float integrated_division(V3 m0, float k0, float n0, V3 m1, float k1, float n1, float e2k1) {  // Merger.h:337-365
  V3 pm = m0 * k0 + m1 * k1;
  float pk = sqrtf(dot(pm, pm));
  float pn = float(1.0 / (4.0 * kPiD));
  if (pk > 1e-3f) {
    float pe = lib_expf(-2.0f * pk);
    pn = vmf_norm_double(pk, pe);
    pm = pm / pk;
  } else {
    pm = m0;
  }
  float scale = (n0 * n1) / pn;
  float c0 = dot(m0, pm), c1 = dot(m1, pm);
  scale = float(double(scale) * ((4.0 * kPiD * kPiD * double(1.0f - e2k1)) / double(k1 * k1)));
  scale *= lib_expf((k0 * (c0 - 1.0f) + k1 * (c1 - 1.0f)) + (2.0f * k1));
  return scale;
}
__device__ float merge_cost(const VMMState &v, int i0, int i1) {  // Merger.h:92-177
  float w0 = v.w[i0], k0 = v.kappa[i0], mc0 = v.mc[i0], n0 = v.norm[i0];
  float w1 = v.w[i1], k1 = v.kappa[i1], mc1 = v.mc[i1], n1 = v.norm[i1];
  V3 m0 = mk(v.mx[i0], v.my[i0], v.mz[i0]), m1 = mk(v.mx[i1], v.my[i1], v.mz[i1]);
  if (i0 == i1) { w0 /= 2.0f; w1 /= 2.0f; }
  float w = w0 + w1, kappa = 0.0f, nrm = kInv4Pi, e2k = 1.0f;
  V3 m = m0 * (w0 * mc0) + m1 * (w1 * mc1);
  m = m / w;
  float mc = m.x * m.x + m.y * m.y + m.z * m.z;
  if (mc > 0.f) {
    mc = sqrtf(mc);
    kappa = mean_cosine_to_kappa(mc);
    kappa = kappa < 1e-3f ? 0.f : kappa;
    e2k = lib_expf(-2.0f * kappa);
    nrm = vmf_norm_double(kappa, e2k);
    m = m / mc;
  } else {
    m = m0;
  }
  V3 nm = mk(-m.x, -m.y, -m.z);
  V3 m00, m11, m01;
  float k00, k11, k01, n00, n11, n01;
  float s00 = product_scale(m0, k0, n0, m0, k0, n0, m00, k00, n00);
  float s11 = product_scale(m1, k1, n1, m1, k1, n1, m11, k11, n11);
  float s01 = product_scale(m0, k0, n0, m1, k1, n1, m01, k01, n01);
  float w00 = w0 * w0, w11 = w1 * w1, w01 = w0 * w1;
  float chi = 0.0f;
  chi += (w00 / w) * (s00 * integrated_division(m00, k00, n00, nm, kappa, nrm, e2k));
  chi += (w11 / w) * (s11 * integrated_division(m11, k11, n11, nm, kappa, nrm, e2k));
  chi += 2.0f * (w01 / w) * (s01 * integrated_division(m01, k01, n01, nm, kappa, nrm, e2k));
  chi -= w;
  return chi;
}
// ComponentSplitStatistics::mergeComponentStats, zero-mean form (Splitter.h:994-1100)
__device__ void split_merge_stats(SplitState &s, int I, int J, float wI, V3 muI, float wJ, V3 muJ, float wK, V3 muK) {
  int L = int(s.K) - 1;
  Frame invK = inverse_of(frame_of(muK, false));
  float ix, iy, jx, jy;
  map3d_to_2d(xfm(invK, muI), ix, iy);
  map3d_to_2d(xfm(invK, muJ), jx, jy);
  float invWK = (wK > 0.f) ? rcp_avx2(wK) : 1.f;
  float swI = s.sw[I], swJ = s.sw[J], swK = swI + swJ;
  V3 cI = (swI > 0.f) ? mk(s.cx[I], s.cy[I], s.cz[I]) * rcp_avx2(swI) : mk(0, 0, 0);
  V3 cJ = (swJ > 0.f) ? mk(s.cx[J], s.cy[J], s.cz[J]) * rcp_avx2(swJ) : mk(0, 0, 0);
  V3 mII = mk(ix * ix, iy * iy, ix * iy), mJJ = mk(jx * jx, jy * jy, jx * jy);
  V3 cK = ((cI * wI + mII * wI) + cJ * wJ) + mJJ * wJ;
  cK = cK * invWK;
  V3 scK = cK * swK;
  float saK = s.sa[I] + s.sa[J];
  float nK = invWK * (wI * s.n[I] + wJ * s.n[J]);
  float chiK = s.chi2[I] + s.chi2[J];
  s.mx[I] = 0.0f; s.my[I] = 0.0f; s.cx[I] = scK.x; s.cy[I] = scK.y; s.cz[I] = scK.z;
  s.sw[I] = swK; s.n[I] = nK; s.sa[I] = saK; s.chi2[I] = chiK;
  s.mx[J] = s.mx[L]; s.my[J] = s.my[L]; s.cx[J] = s.cx[L]; s.cy[J] = s.cy[L]; s.cz[J] = s.cz[L];
  s.sw[J] = s.sw[L]; s.n[J] = s.n[L]; s.sa[J] = s.sa[L]; s.chi2[J] = s.chi2[L];
  split_zero_lane(s, L);
  s.K--;
}

// ---------------------------------------------------------------- sample passes
//
// Distance and split-statistics passes run in the home block as a two-stage
// pipeline over chunks of samples, with one __syncthreads per chunk and two
// shared-memory stages:
//   producers (threads [0, C * parts)): `parts` adjacent lanes per sample, one
//     SIMD vector of 8 lobes each; the lobe terms in registers, the sample pdf
//     (vfloat8 lane sums carried from part to part in lobe-vector order, then
//     the 8-lane reduction), then the finished term of every accumulator for
//     their lobes written to stage (c & 1);
//   consumers (threads [P, 512)): one thread per accumulator (for example the
//     x component of lobe 7's weighted direction sum), adding the chunk in
//     stage ((c - 1) & 1) in sample order.
// The consumers keep the reference's summation order (sequential over samples
// within each SIMD lane).  Samples that the reference skips (pdf <= 1e-16)
// contribute a term of exactly +-0, which leaves an accumulator unchanged:
// accumulators start at +0 and a round-to-nearest sum that starts at +0 never
// becomes -0.  Consumer lanes only load and add, so chain warps do not diverge
// (chi-square lanes have a warp of their own).  Each pass gives the consumers
// the warps its chains need and the producers the rest; the chunk size
// follows from the stage memory and the producer threads.  E-step passes
// (most of the work) use the same roles, with a loader warp besides, and can
// take chunks made by other blocks (below).

struct LeafSamples {
  const float4 *dirw;  // direction xyz, weight
  const float *pdf;
  const float *dist;
  uint32_t count;
};

enum PassKind { kPassDistance = 1, kPassSplit = 2 };  // in-block passes

// Thread roles and stage layout of one pass (the same in every thread).
struct PassShape {
  int P;        // threads [P, kEmThreads) consume
  int parts;    // producer lanes per sample (lobe vectors, 3 rounded to 4)
  int C;        // samples per chunk
  int threads;  // producer threads: C * parts, a multiple of 32
  int R;        // row stride of the per-(lobe, sample) rows: C + 2 floats
  int stage;    // floats per stage
};
template <PassKind kind>
__device__ __forceinline__ PassShape pass_shape(int Kp, int budget = kStageFloats) {
  // rows: one per (accumulator, lobe); extra: per-sample arrays
  int consWarps, rows, extra;
  if (kind == kPassDistance) {  // 2 Kp chains
    consWarps = (2 * Kp + 31) / 32;
    rows = 2 * Kp;
    extra = 0;
  } else {  // 5 Kp product chains, two per lane, then (from a warp boundary) Kp chi-square chains
    consWarps = (5 * Kp + 63) / 64 + 1;
    rows = 7 * Kp;  // a, a w, three covariance terms, chi, 1/n
    extra = 1;      // validity
  }
  PassShape p;
  const int cnt = Kp / kLanes;
  p.parts = cnt == 3 ? 4 : cnt;
  p.P = kEmThreads - 32 * consWarps;
  int c = (budget - 2 * rows) / (rows + extra);
  const int byThreads = p.P / p.parts;
  c = c < byThreads ? c : byThreads;
  // C * parts a multiple of 32 (whole warps) and C a multiple of 8.  Rows of
  // C + 2 floats: (C + 2) / 2 is odd, so the consumers' 64-bit loads of
  // consecutive rows fall in distinct banks, and rows 8 apart are 16 banks
  // apart, so two parts of a sample store to distinct banks.
  const int mult = 32 / p.parts > 8 ? 32 / p.parts : 8;
  p.C = c - c % mult;
  p.threads = p.C * p.parts;
  p.R = p.C + 2;
  p.stage = rows * p.R + extra * p.C;
  return p;
}

// x86 RCPSS from the block's shared copy of the table (per-lane gathers from
// constant memory would serialise)
__device__ __forceinline__ float rcp_avx2_tab(float a, const uint32_t *tab) {
  uint32_t u = f2u(a), s = u & 0x80000000u, e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  float r;
  if (e == 0) {
    r = u2f(s | 0x7F800000u);
  } else if (e == 255) {
    r = m ? a : u2f(s);
  } else {
    uint32_t t = tab[m >> 12];
    int re = int((t >> 23) & 0xFFu) - (int(e) - 127);
    r = re <= 0 ? u2f(s) : (re >= 255 ? u2f(s | 0x7F800000u) : u2f(s | (uint32_t(re) << 23) | (t & 0x7FFFFFu)));
  }
  return r * fmaf_(-r, a, 2.0f);
}

// Lobe parameters packed for the producers' broadcast loads.
__device__ void pack_lobes(EmShared &S, int Kp) {
  const int tid = threadIdx.x;
  if (tid < Kp) {
    const VMMState &v = S.vmm;
    // entry k + k / 8: the parts of a sample read lobes k and k + 8 at once
    S.lobeA[tid + (tid >> 3)] = make_float4(v.mx[tid], v.my[tid], v.mz[tid], v.kappa[tid]);
    S.lobeB[tid] = make_float2(v.norm[tid], v.w[tid]);
    S.lobeWInv[tid] = rcp_for_div(v.w[tid]);
  }
}

// One producer lane's view of a sample: the E-step terms of its 8 lobes
// (vector v), then the sample pdf and 1/pdf shared by all parts.
struct PartTerms {
  float t[kLanes];
  float pdf, inv;
  bool valid;
};
__device__ __forceinline__ void part_terms(const EmShared &S, int cnt, int parts, int v, bool have, V3 d,
                                           PartTerms &T) {
  const unsigned full = 0xFFFFFFFFu;
  if (have && v < cnt) {
#pragma unroll
    for (int j = 0; j < kLanes; ++j) {
      const int k = v * kLanes + j;
      const float4 A = S.lobeA[k + v];
      const float2 B = S.lobeB[k];
      float ct = dot(d, mk(A.x, A.y, A.z));
      float cm1 = emin(ct - 1.0f, 0.0f);
      float ev = B.x * fexp(A.w * cm1);
      T.t[j] = B.y * ev;
    }
  } else {
#pragma unroll
    for (int j = 0; j < kLanes; ++j) T.t[j] = 0.0f;
  }
  // lane sums over the lobe vectors in order: ((t0 + t1) + t2) + t3
  float p[kLanes];
#pragma unroll
  for (int j = 0; j < kLanes; ++j) p[j] = T.t[j];
  for (int step = 1; step < parts; ++step) {
#pragma unroll
    for (int j = 0; j < kLanes; ++j) {
      const float in = __shfl_up_sync(full, p[j], 1);
      if (v == step) p[j] = in + T.t[j];
    }
  }
  float pdf = 0.0f, inv = 0.0f;
  bool valid = false;
  if (v == parts - 1 && have) {
    pdf = reduce8(p);
    valid = pdf > 1e-16f;
    inv = valid ? rcp_avx2_tab(pdf, S.rcpTab) : 0.0f;
  }
  const int last = (int(threadIdx.x & 31) - v) + parts - 1;
  T.pdf = __shfl_sync(full, pdf, last);
  T.inv = __shfl_sync(full, inv, last);
  T.valid = __shfl_sync(full, valid ? 1 : 0, last) != 0;
}

struct SampleIn {
  float4 dw;
  float x;  // pdf (split pass) or distance (distance pass)
  bool have;
};
template <PassKind kind>
__device__ __forceinline__ SampleIn load_sample(const LeafSamples &L, uint32_t idx) {
  SampleIn r;
  r.have = idx < L.count;
  r.dw = make_float4(0.f, 0.f, 0.f, 0.f);
  r.x = 0.0f;
  if (r.have) {
    r.dw = L.dirw[idx];
    if constexpr (kind == kPassDistance) r.x = L.dist[idx];
    else if constexpr (kind == kPassSplit) r.x = L.pdf[idx];
  }
  return r;
}

// Producer: lane v of sample slot s fills its lobes' rows of stage B.  In
// split passes the running count of valid samples (for the chi-square means'
// 1/n) needs a prefix over the chunk: warp ballots, then a barrier among the
// producer threads only (named barrier 1), then `base` (valid samples of the
// earlier chunks) moves on by the chunk's total.
template <PassKind kind>
__device__ __forceinline__ void produce(EmShared &S, const PassShape &sh, int cnt, int Kp, int s, int v,
                                        const SampleIn &in, float *B, uint32_t &base) {
  PartTerms T;
  const V3 d = mk(in.dw.x, in.dw.y, in.dw.z);
  const float w = in.dw.w;
  part_terms(S, cnt, sh.parts, v, in.have, d, T);
  const bool valid = in.have && T.valid;
  const int R = sh.R;
  const bool mine = v < cnt;  // this lane has lobes
  if constexpr (kind == kPassDistance) {
    // rows k: wts * rcp(distance); rows Kp + k: wts
    if (mine) {
      const float sd = valid ? rcp_avx2_tab(in.x, S.rcpTab) : 0.0f;
#pragma unroll
      for (int j = 0; j < kLanes; ++j) {
        const int k = v * kLanes + j;
        float wts = 0.0f;
        if (valid) {
          const float a = T.t[j] * T.inv;
          wts = (w * a) * div_rcp(a * T.pdf, S.lobeB[k].y, S.lobeWInv[k]);
        }
        B[k * R + s] = wts * sd;
        B[(Kp + k) * R + s] = wts;
      }
    }
  } else {
    // count of valid samples up to and including this one
    const unsigned full = 0xFFFFFFFFu;
    const int lane = int(threadIdx.x & 31), warp = int(threadIdx.x >> 5);
    const unsigned b = __ballot_sync(full, v == 0 && valid);
    if (lane == 0) S.validPerWarp[warp] = uint32_t(__popc(b));
    asm volatile("bar.sync 1, %0;" ::"r"(sh.threads) : "memory");
    uint32_t before = 0, total = 0;
    for (int q = 0; q < sh.threads / 32; ++q) {
      const uint32_t n = S.validPerWarp[q];
      before += q < warp ? n : 0u;
      total += n;
    }
    const uint32_t count = base + before + uint32_t(__popc(b & ((1u << (lane - v)) - 1u))) + 1u;
    base += total;
    // rows r Kp + k: a, a w, (a w)(lx lx), (a w)(ly ly), (a w)(lx ly), chi,
    // RN(1 / n) with n = n0_k + count; then the validity per sample
    const float spdfv = in.x;
    const float value = w * spdfv;
    const float mcEst = S.mcEstimate;
    // the three divisors are per sample: one reciprocal each, then Markstein
    const float den1 = mcEst * T.pdf, den2 = ((mcEst * mcEst) * T.pdf) * T.pdf;
    const float y1 = rcp_for_div(den1), y2 = rcp_for_div(den2), y3 = rcp_for_div(spdfv);
    if (mine) {
#pragma unroll
      for (int j = 0; j < kLanes; ++j) {
        const int k = v * kLanes + j;
        float a = 0.0f, aw = 0.0f, cxx = 0.0f, cyy = 0.0f, cxy = 0.0f, chi = 0.0f, yn = 0.0f;
        if (valid) {
          a = T.t[j] * T.inv;
          float vmf = a * T.pdf;
          float pvp = vmf * value;
          pvp = div_rcp(pvp, den1, y1);
          chi = (value * value) * vmf;
          chi = div_rcp(chi, den2, y2);
          chi -= 2.0f * pvp;
          chi += vmf;
          chi = div_rcp(chi, spdfv, y3);
          chi = a > 0.0f ? chi : 0.0f;
          V3 ld = xfm(S.invFrame[k], d);
          aw = a * w;
          cxx = aw * (ld.x * ld.x);
          cyy = aw * (ld.y * ld.y);
          cxy = aw * (ld.x * ld.y);
          const float n = S.splitN0[k] + float(count);
          yn = (n >= 1e-30f && n <= 1e30f) ? rcp_rn(n) : 0.0f;
        }
        B[k * R + s] = a;
        B[(Kp + k) * R + s] = aw;
        B[(2 * Kp + k) * R + s] = cxx;
        B[(3 * Kp + k) * R + s] = cyy;
        B[(4 * Kp + k) * R + s] = cxy;
        B[(5 * Kp + k) * R + s] = chi;
        B[(6 * Kp + k) * R + s] = yn;
      }
    }
    if (v == 0) B[7 * Kp * R + s] = valid ? 1.0f : 0.0f;
  }
}

__device__ __forceinline__ float2 ld2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ float4 ld4(const float *p) {  // two 64-bit loads (rows are 8-byte aligned)
  const float2 a = ld2(p), b = ld2(p + 2);
  return make_float4(a.x, a.y, b.x, b.y);
}

// Sum of one row (the terms of one accumulator) in sample order; loads run 8
// samples ahead of the additions.
__device__ __forceinline__ void row_chain(const float *row, int n4, float &acc) {
  int s = 0;
  if (n4 >= 8) {
    float4 a = ld4(row), b = ld4(row + 4);
    for (; s + 8 <= n4; s += 8) {
      const int sn = s + 16 <= n4 ? s + 8 : s;
      const float4 a1 = ld4(row + sn), b1 = ld4(row + sn + 4);
      acc += a.x;
      acc += a.y;
      acc += a.z;
      acc += a.w;
      acc += b.x;
      acc += b.y;
      acc += b.z;
      acc += b.w;
      a = a1;
      b = b1;
    }
  }
  if (s < n4) {
    const float4 v = ld4(row + s);
    acc += v.x;
    acc += v.y;
    acc += v.z;
    acc += v.w;
  }
}

// Distance pass (WEMFactory.h:1199-1326): lanes c < Kp sum wts * rcp(distance),
// lanes Kp <= c < 2 Kp sum wts.
__device__ __forceinline__ void distance_chain(const float *B, const PassShape &sh, int c, int Kp, int n4,
                                               float &acc) {
  if (c < 2 * Kp) row_chain(B + c * sh.R, n4, acc);
}

// Split-statistics pass (Splitter.h:439-523).  Lanes c < 5 Kp sum row c
// (r = c / Kp: sumAssignedSamples a, sumWeights a w, then the 2D covariance
// sums (a w)(lx lx), (a w)(ly ly), (a w)(lx ly)).  Chi-square lanes start at
// the next warp: the running mean chi2 += (chi - chi2) / n over the valid
// samples, n counting from n0.  Markstein's steps with the producers'
// y = RN(1 / (n0 + count)) give (chi - chi2) / n exactly (a skipped sample,
// y = 0, adds +-0) when y belongs to the lane's own running count n (the
// usual case: n equals n0 + count) and the difference d and the quotient lie
// in [1e-30, 1e30] (or d is 0).  The chain checks this per group of four
// samples beside the additions, not between them: the counts, the largest
// |d| against 1e30 and the smallest non-zero |d| against 1e-30 times the
// group's last n (so every quotient of the group is in range).  From the
// first group that fails (rare) the chunk is summed again with divisions,
// which give the same bits wherever Markstein's steps were exact.
__device__ __forceinline__ int split_chi_base(int Kp) { return ((5 * Kp + 63) / 64) * 32; }
__device__ __forceinline__ void split_chain(const float *B, const PassShape &sh, int c, int Kp, int n4, float n0,
                                            float &acc, float &acc2, float &accN, float &cnt) {
  const int R = sh.R;
  const int chiBase = split_chi_base(Kp);
  if (c < chiBase) {  // rows c and c + chiBase (a row chain costs a few cycles per sample, the chi chain ~50)
    if (c < 5 * Kp) row_chain(B + c * R, n4, acc);
    if (c + chiBase < 5 * Kp) row_chain(B + (c + chiBase) * R, n4, acc2);
  } else if (c < chiBase + Kp) {
    const int k = c - chiBase;
    const float *xr = B + (5 * Kp + k) * R, *yr = B + (6 * Kp + k) * R, *vr = B + 7 * Kp * R;
    const float accStart = acc, nStart = accN;
    int redoAt = n4;  // first group that failed the range check
    float accRedo = 0.0f, nRedo = 0.0f;
    float4 x = ld4(xr), y = ld4(yr), v = ld4(vr);
    for (int s = 0; s < n4; s += 4) {
      const int sn = s + 4 < n4 ? s + 4 : s;
      const float4 x1 = ld4(xr + sn), y1 = ld4(yr + sn), v1 = ld4(vr + sn);
      const float accG = acc, nG = accN;
      const float n1 = accN + v.x, n2 = n1 + v.y, n3 = n2 + v.z, n4v = n3 + v.w;
      const float c1 = cnt + v.x, c2 = c1 + v.y, c3 = c2 + v.z, c4 = c3 + v.w;
      const bool same = (v.x == 0.0f || n1 == n0 + c1) & (v.y == 0.0f || n2 == n0 + c2) &
                        (v.z == 0.0f || n3 == n0 + c3) & (v.w == 0.0f || n4v == n0 + c4);
      const float d1 = x.x - acc;
      acc = acc + markstein_q(d1, n1, y.x);
      const float d2 = x.y - acc;
      acc = acc + markstein_q(d2, n2, y.y);
      const float d3 = x.z - acc;
      acc = acc + markstein_q(d3, n3, y.z);
      const float d4 = x.w - acc;
      acc = acc + markstein_q(d4, n4v, y.w);
      const float a1 = fabsf(d1), a2 = fabsf(d2), a3 = fabsf(d3), a4 = fabsf(d4);
      const float gMax = fmaxf(fmaxf(a1, a2), fmaxf(a3, a4));
      const float gMin = fminf(fminf(a1 == 0.0f ? INFINITY : a1, a2 == 0.0f ? INFINITY : a2),
                               fminf(a3 == 0.0f ? INFINITY : a3, a4 == 0.0f ? INFINITY : a4));
      if ((!same || !(gMax <= 1e30f) || gMin < 1.0000002e-30f * n4v) && redoAt == n4) {
        redoAt = s;
        accRedo = accG;
        nRedo = nG;
      }
      accN = n4v;
      cnt = c4;
      x = x1;
      y = y1;
      v = v1;
    }
    if (acc != acc) {
      redoAt = 0;
      accRedo = accStart;
      nRedo = nStart;
    }
    if (redoAt < n4) {
      acc = accRedo;
      accN = nRedo;
      for (int s = redoAt; s < n4; ++s) {
        const float vv = vr[s];
        accN += vv;
        if (vv != 0.0f) acc += (xr[s] - acc) / accN;
      }
    }
  }
}

// Runs one distance or split-statistics pass over the leaf's samples in the
// home block.  `acc`/`accN` are the consumer's accumulators (initialised by
// the caller); chunk c is made into stage (c & 1) while the consumers add
// chunk c - 1.
template <PassKind kind>
__device__ __noinline__ void run_pass(EmShared &S, const LeafSamples &L, const PassShape &sh, int cnt, float &accOut,
                                      float &acc2Out, float &accNOut) {
  const int tid = threadIdx.x;
  float acc = accOut, acc2 = acc2Out, accN = accNOut;  // the chains run on registers
  const int Kp = cnt * kLanes;
  const int C = sh.C;
  const uint32_t rounds = (L.count + C - 1) / C;
  const bool producer = tid < sh.threads;
  const int s = tid / sh.parts, v = tid % sh.parts;
  const bool consumer = tid >= sh.P;
  const int c = tid - sh.P;
  const int chiK = kind == kPassSplit ? c - split_chi_base(Kp) : -1;
  const float n0 = (chiK >= 0 && chiK < Kp) ? S.splitN0[chiK] : 0.0f;
  float count = 0.0f;
  uint32_t base = 0;
  SampleIn next;
  if (producer) next = load_sample<kind>(L, uint32_t(s));
  long long cycP = 0, cycC = 0;
  for (uint32_t it = 0; it <= rounds; ++it) {
    if (producer && it < rounds) {
      const long long t0 = clock64();
      const SampleIn cur = next;
      if (it + 1 < rounds) next = load_sample<kind>(L, (it + 1) * C + s);
      produce<kind>(S, sh, cnt, Kp, s, v, cur, S.pbuf + (it & 1) * kStageFloats, base);
      cycP += clock64() - t0;
    }
    if (consumer && it >= 1) {
      const long long t0 = clock64();
      const uint32_t chunk = it - 1;
      const int n = int(min(uint32_t(C), L.count - chunk * C));
      const int n4 = (n + 3) & ~3;
      const float *B = S.pbuf + (chunk & 1) * kStageFloats;
      if constexpr (kind == kPassDistance) distance_chain(B, sh, c, Kp, n4, acc);
      else split_chain(B, sh, c, Kp, n4, n0, acc, acc2, accN, count);
      cycC += clock64() - t0;
    }
    __syncthreads();
  }
  accOut = acc;
  acc2Out = acc2;
  accNOut = accN;
  const int probe = kind == kPassSplit ? split_chi_base(Kp) : 0;
  if (tid == 0 && kind == kPassSplit) S.prof.cycProdS += uint64_t(cycP);
  if (c == probe && kind == kPassSplit) S.prof.cycConsS += uint64_t(cycC);
}

// ---------------------------------------------------------------- shared E-step passes

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(unsigned long long *m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *m) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *m, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}
// whether phase `parity` has completed, without waiting
__device__ __forceinline__ bool mbar_test_wait(unsigned long long *m, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared bulk copy (16-byte aligned, a multiple of 16 bytes)
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, unsigned long long *m) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(m))
               : "memory");
}
// orders this thread's generic-proxy global accesses with bulk copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void bar_named(int id, int threads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}
__device__ __forceinline__ void set_error(int *err, int code) { atomicCAS(err, 0, code); }
__device__ __forceinline__ bool has_error(const int *err) { return *reinterpret_cast<const volatile int *>(err) != 0; }

// Spins until *p >= want (true) or the launch failed / the wait ran out
// (after limitNs; the launch's error word then holds kErrSlotWait).
__device__ bool wait_at_least(const uint32_t *p, uint32_t want, int *err, unsigned long long limitNs = kWaitNs) {
  unsigned long long t0 = 0;
  unsigned sleep = 64;
  for (uint32_t it = 0;; ++it) {
    if (ld_acquire(p) >= want) return true;
    if ((it & 31) == 31) {
      if (has_error(err)) return false;
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > limitNs) {
        set_error(err, kErrSlotWait);
        return false;
      }
    }
    __nanosleep(sleep);
    sleep = sleep < 1024 ? 2 * sleep : sleep;
  }
}
// Waits for phase `parity` of a stage barrier.  Consumers give up on chunks
// from *abortAt on (the loader gave up on them: nothing will arrive); every
// waiter gives up after kWaitNs.
__device__ bool mbar_wait(unsigned long long *m, uint32_t parity, const volatile uint32_t *abortAt, uint32_t k,
                          int *err) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(m, parity)) return true;
    if (abortAt && k >= *abortAt) return false;
    if ((it & 15) == 15) {
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kWaitNs) {
        set_error(err, kErrCopyWait);
        return false;
      }
    }
  }
}

__device__ __forceinline__ unsigned long long grab_word(uint32_t gen, uint32_t chunks, uint32_t next) {
  return (static_cast<unsigned long long>(gen) << (2 * kGrabIdxBits)) |
         (static_cast<unsigned long long>(chunks) << kGrabIdxBits) | next;
}
__device__ __forceinline__ uint32_t grab_gen(unsigned long long w) { return uint32_t(w >> (2 * kGrabIdxBits)); }
__device__ __forceinline__ uint32_t grab_chunks(unsigned long long w) { return uint32_t(w >> kGrabIdxBits) & kGrabMask; }
__device__ __forceinline__ uint32_t grab_next(unsigned long long w) { return uint32_t(w) & kGrabMask; }
// Chunk shape of an E-step pass with `cnt` lobe vectors: consumers need
// 4 Kp + 5 chains in three warps (chain_role), one warp loads
// chunks made by other blocks, producers get
// the remaining warps (P threads, one chunk of C = P / parts samples).  A
// chunk holds rows of RS = C + 4 floats (RS / 4 odd, so the consumers'
// 128-bit loads of 8 consecutive rows hit distinct banks): a_k for k < Kp
// (the soft assignment t_k / pdf of valid samples, 0 otherwise), the
// direction x, y, z, the weight of valid samples, then w log(pdf) and the
// four unassigned-sample terms.
struct EStepShape {
  int cnt, Kp, parts, P, cons0, consWarps, C, C0, RS, stageFloats, stages, slots;
};
// Chunk k of a pass covers samples [chunk_begin, chunk_begin + chunk_size):
// the first chunk is one producer round (the leaf's own producers make it
// while helper blocks are still picking up the pass, and the consumers wait
// for it), the others C samples.
__device__ __forceinline__ uint32_t chunk_begin(const EStepShape &e, uint32_t k) {
  return k == 0 ? 0u : uint32_t(e.C0) + (k - 1u) * uint32_t(e.C);
}
__device__ __forceinline__ int chunk_size(const EStepShape &e, uint32_t k) { return k == 0 ? e.C0 : e.C; }
__device__ __forceinline__ uint32_t chunk_count(const EStepShape &e, uint32_t count) {
  return count <= uint32_t(e.C0) ? 1u : 1u + (count - uint32_t(e.C0) + uint32_t(e.C) - 1u) / uint32_t(e.C);
}
__device__ __forceinline__ EStepShape estep_shape(int cnt, const EmTuning &tune) {
  EStepShape e;
  e.cnt = cnt;
  e.Kp = cnt * kLanes;
  e.parts = cnt == 3 ? 4 : cnt;
  e.consWarps = 3;  // a w and (d_x a) w | (d_y a) w and (d_z a) w | per-sample rows
  e.cons0 = kEmThreads - 32 * e.consWarps;  // consumers: threads [cons0, 512)
  e.P = e.cons0 - 32;                       // producers [0, P), then the loader warp
  // as many producer rounds per chunk as keep two stages in the pipeline
  // buffer, up to kMaxChunk samples: a consumer warp spends a few hundred
  // cycles per chunk outside its chains
  const int slots = e.P / e.parts;
  const int fit = (2 * kStageFloats / 2) / (e.Kp + 9) - 4;  // C + 4 floats per row, two stages
  int rounds = min(kMaxChunk, fit) / slots;
  rounds = rounds < 1 ? 1 : rounds;
  e.C = ((rounds * slots) / tune.chunkDiv) & ~7;
  e.C0 = min(e.C, slots & ~7);
  e.RS = e.C + 4;
  e.stageFloats = (e.Kp + 9) * e.RS;
  e.stages = min(min(kMaxStages, tune.stageCap), 2 * kStageFloats / e.stageFloats);
  e.slots = min(int(kRingMaxSlots), int(kRingFloats) / e.stageFloats);
  return e;
}

// Producers: `nthreads` threads (index t) fill chunk `chunk` into G (a stage
// or a ring slot).  A sample's `parts` lanes are adjacent, so every warp holds
// whole samples; rounds of nthreads / parts samples cover the chunk.
template <bool kRing>
__device__ void produce_estep_chunk(const EmShared &S, const EStepShape &e, const float4 *dirw, uint32_t count,
                                    uint32_t chunk, float *G, int t, int nthreads) {
  const int per = nthreads / e.parts;
  const int v = t % e.parts;
  const int RS = e.RS, Kp = e.Kp;
  const int size = chunk_size(e, chunk);
  const uint32_t first = chunk_begin(e, chunk);
  for (int base = 0; base < size; base += per) {
    const int s = base + t / e.parts;
    const uint32_t idx = first + uint32_t(s);
    const bool have = s < size && idx < count;
    const float4 dw = have ? __ldcg(dirw + idx) : make_float4(0.f, 0.f, 0.f, 0.f);
    const V3 d = mk(dw.x, dw.y, dw.z);
    PartTerms T;
    part_terms(S, e.cnt, e.parts, v, have, d, T);
    if (s < size) {
      const bool valid = have && T.valid;
      if (v < e.cnt) {
#pragma unroll
        for (int j = 0; j < kLanes; ++j) G[(v * kLanes + j) * RS + s] = valid ? T.t[j] * T.inv : 0.0f;
      }
      if (v == 0) {
        const float w = dw.w;
        const bool un = have && !T.valid;
        float *X = G + Kp * RS + s;
        X[0] = d.x;
        X[RS] = d.y;
        X[2 * RS] = d.z;
        X[3 * RS] = valid ? w : 0.0f;
        // the log-likelihood only drives the convergence test (its relative
        // change against 0.005); it is not stored, so the single-precision
        // logf (<= 1 ulp) stands in for the C library's here
        X[4 * RS] = valid ? w * logf(T.pdf) : 0.0f;
        X[5 * RS] = un ? w : 0.0f;
        X[6 * RS] = un ? d.x * w : 0.0f;
        X[7 * RS] = un ? d.y * w : 0.0f;
        X[8 * RS] = un ? d.z * w : 0.0f;
      }
    }
  }
  if (kRing) fence_proxy_async();  // the ring is read by bulk copies
}

// A helper takes the next chunk of board `b` (one thread): only when that
// chunk's ring slot is free (known once the pass's parameters are loaded; a
// chunk of a pass not loaded yet is taken anyway).  Returns the chunk, -1 when
// the pass has none left, -2 when the ring is full for now; `exact` says the
// chunk taken is the one whose slot was checked (others can take chunks
// between the check and the atomic).
__device__ int helper_take(EmShared &S, Board &b, bool paramsLoaded, uint32_t paramsGen, uint32_t &gen, int &exact) {
  const unsigned long long w = ld_relaxed64(&b.grab);
  const uint32_t consumed = ld_relaxed(&b.consumed);
  exact = 0;
  gen = 0;
  if (has_error(S.err) || grab_gen(w) == 0 || grab_next(w) >= grab_chunks(w)) return -1;
  const bool known = paramsLoaded && grab_gen(w) == paramsGen;
  if (known && S.hp.seqBase + grab_next(w) + 1u > consumed + uint32_t(estep_shape(int(S.hp.cnt), S.tune).slots)) return -2;
  const unsigned long long w2 = atomicAdd(&b.grab, 1ull);
  if (grab_gen(w2) == 0 || grab_next(w2) >= grab_chunks(w2)) return -1;
  gen = grab_gen(w2);
  exact = known && w2 == w;
  return int(grab_next(w2));
}

// A helper's chunk of board `b`: wait until its ring slot is free (unless
// its slot was checked), fill the slot, then publish its sequence number.
// Warp 15 holds no samples of a chunk (C <= 384 samples in lanes 0..479), so
// its lane 0 takes the helper's next chunk meanwhile.
__device__ void produce_for(EmShared &S, Board &b, float *ring, const EStepShape &e, const float4 *dirw,
                            uint32_t count, uint32_t seqBase, uint32_t chunk, bool exact, uint32_t paramsGen) {
  const int t = threadIdx.x;
  const uint32_t seq = seqBase + chunk + 1u, slot = (seqBase + chunk) % uint32_t(e.slots);
  // the slot's previous chunk (sequence number seq - slots) must have been copied out
  if (t == 0 && !exact && seq > uint32_t(e.slots)) wait_at_least(&b.consumed, seq - uint32_t(e.slots), S.err);
  __syncthreads();
  if (t == kEmThreads - 32) {
    uint32_t g = 0;
    int x = 0;
    S.nextGrabbed = helper_take(S, b, true, paramsGen, g, x);
    S.nextGen = g;
    S.nextExact = x;
    S.hasNext = 1;
  }
  produce_estep_chunk<true>(S, e, dirw, count, chunk, ring + size_t(slot) * e.stageFloats, t, kEmThreads);
  __syncthreads();
  if (t == 0) {
    __threadfence();
    st_release(&b.ready[slot], seq);
  }
}

// Consumer side of the sum: a_k w, (d_q a_k) w or a per-sample row, in
// sample order (the products are those of the reference's E-step).
// Each chain keeps three groups of four samples in registers: the loads of a
// group are issued two groups before it is added (a warp issues in order, so
// loads placed after the dependent adds would wait for them).  The products
// of two samples share one packed multiply (each component rounded as its
// own multiply).  The loop is inlined into the consumer's chunk loop (a call
// per chunk, with the registers it saves and restores, measured 4 % of the
// first Update's EM launch) and works on 32-bit shared-memory addresses.
__device__ __forceinline__ float4 lds4(uint32_t a) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
  return v;
}
template <int kKind>  // 0: a w, 1: (d a) w, 2: the value itself
__device__ __forceinline__ void add_group(float &acc, float4 a, float4 d, float4 w) {
  if (kKind == 2) {
    acc += a.x;
    acc += a.y;
    acc += a.z;
    acc += a.w;
  } else {
    float2 p0 = make_float2(a.x, a.y), p1 = make_float2(a.z, a.w);
    if (kKind == 1) {
      p0 = __fmul2_rn(make_float2(d.x, d.y), p0);
      p1 = __fmul2_rn(make_float2(d.z, d.w), p1);
    }
    p0 = __fmul2_rn(p0, make_float2(w.x, w.y));
    p1 = __fmul2_rn(p1, make_float2(w.z, w.w));
    acc += p0.x;
    acc += p0.y;
    acc += p1.x;
    acc += p1.y;
  }
}
template <int kKind>
__device__ __forceinline__ float4 lds_if(uint32_t a) {
  return kKind ? lds4(a) : make_float4(0.f, 0.f, 0.f, 0.f);
}
// Rows start at 32-bit shared addresses A, D, W (bytes); n4 samples.
template <int kKind>
__device__ __forceinline__ float chain_rows(uint32_t A, uint32_t D, uint32_t W, int n4, float acc) {
  constexpr int kD = kKind == 1, kW = kKind != 2;
  // rows hold C + 4 >= 12 floats: the first two groups can be read even
  // when n4 is smaller
  float4 a0 = lds4(A), d0 = lds_if<kD>(D), w0 = lds_if<kW>(W);
  float4 a1 = lds4(A + 16), d1 = lds_if<kD>(D + 16), w1 = lds_if<kW>(W + 16);
  int s = 0;
  for (; s + 12 <= n4; s += 12) {
    const uint32_t o2 = uint32_t(s + 8) * 4u;
    const float4 a2 = lds4(A + o2), d2 = lds_if<kD>(D + o2), w2 = lds_if<kW>(W + o2);
    add_group<kKind>(acc, a0, d0, w0);
    const uint32_t o3 = uint32_t(s + 12 < n4 ? s + 12 : 0) * 4u;
    a0 = lds4(A + o3);
    d0 = lds_if<kD>(D + o3);
    w0 = lds_if<kW>(W + o3);
    add_group<kKind>(acc, a1, d1, w1);
    const uint32_t o4 = uint32_t(s + 16 < n4 ? s + 16 : 0) * 4u;
    a1 = lds4(A + o4);
    d1 = lds_if<kD>(D + o4);
    w1 = lds_if<kW>(W + o4);
    add_group<kKind>(acc, a2, d2, w2);
  }
  if (s < n4) add_group<kKind>(acc, a0, d0, w0);
  if (s + 4 < n4) add_group<kKind>(acc, a1, d1, w1);
  if (s + 8 < n4) {
    const uint32_t o2 = uint32_t(s + 8) * 4u;
    add_group<kKind>(acc, lds4(A + o2), lds_if<kD>(D + o2), lds_if<kW>(W + o2));
  }
  return acc;
}
// Two chains of lobe k in one consumer thread, so that the thread reads the
// a_k row once for both: kind 0 sums a_k w and (d_x a_k) w, kind 1 sums
// (d_y a_k) w and (d_z a_k) w.  The two chains' additions alternate (each
// chain still adds its terms in sample order, one rounding per addition).
template <int kKind>
__device__ __forceinline__ void add_group2(float &acc0, float &acc1, float4 a, float4 d0, float4 d1, float4 w) {
  const float2 a01 = make_float2(a.x, a.y), a23 = make_float2(a.z, a.w);
  const float2 w01 = make_float2(w.x, w.y), w23 = make_float2(w.z, w.w);
  float2 p01, p23;
  if (kKind == 0) {
    p01 = __fmul2_rn(a01, w01);
    p23 = __fmul2_rn(a23, w23);
  } else {
    p01 = __fmul2_rn(__fmul2_rn(make_float2(d0.x, d0.y), a01), w01);
    p23 = __fmul2_rn(__fmul2_rn(make_float2(d0.z, d0.w), a23), w23);
  }
  const float2 q01 = __fmul2_rn(__fmul2_rn(make_float2(d1.x, d1.y), a01), w01);
  const float2 q23 = __fmul2_rn(__fmul2_rn(make_float2(d1.z, d1.w), a23), w23);
  acc0 += p01.x;
  acc1 += q01.x;
  acc0 += p01.y;
  acc1 += q01.y;
  acc0 += p23.x;
  acc1 += q23.x;
  acc0 += p23.y;
  acc1 += q23.y;
}
// Rows start at 32-bit shared addresses A, D0 (kind 1 only), D1, W (bytes);
// n4 samples; three groups of four samples in flight as in chain_rows.
template <int kKind>
__device__ __forceinline__ float2 chain_rows2(uint32_t A, uint32_t D0, uint32_t D1, uint32_t W, int n4, float2 acc) {
  constexpr int kD0 = kKind == 1;
  float a0c = acc.x, a1c = acc.y;
  float4 a0 = lds4(A), e0 = lds_if<kD0>(D0), f0 = lds4(D1), w0 = lds4(W);
  float4 a1 = lds4(A + 16), e1 = lds_if<kD0>(D0 + 16), f1 = lds4(D1 + 16), w1 = lds4(W + 16);
  int s = 0;
  for (; s + 12 <= n4; s += 12) {
    const uint32_t o2 = uint32_t(s + 8) * 4u;
    const float4 a2 = lds4(A + o2), e2 = lds_if<kD0>(D0 + o2), f2 = lds4(D1 + o2), w2 = lds4(W + o2);
    add_group2<kKind>(a0c, a1c, a0, e0, f0, w0);
    const uint32_t o3 = uint32_t(s + 12 < n4 ? s + 12 : 0) * 4u;
    a0 = lds4(A + o3);
    e0 = lds_if<kD0>(D0 + o3);
    f0 = lds4(D1 + o3);
    w0 = lds4(W + o3);
    add_group2<kKind>(a0c, a1c, a1, e1, f1, w1);
    const uint32_t o4 = uint32_t(s + 16 < n4 ? s + 16 : 0) * 4u;
    a1 = lds4(A + o4);
    e1 = lds_if<kD0>(D0 + o4);
    f1 = lds4(D1 + o4);
    w1 = lds4(W + o4);
    add_group2<kKind>(a0c, a1c, a2, e2, f2, w2);
  }
  if (s < n4) add_group2<kKind>(a0c, a1c, a0, e0, f0, w0);
  if (s + 4 < n4) add_group2<kKind>(a0c, a1c, a1, e1, f1, w1);
  if (s + 8 < n4) {
    const uint32_t o2 = uint32_t(s + 8) * 4u;
    add_group2<kKind>(a0c, a1c, lds4(A + o2), lds_if<kD0>(D0 + o2), lds4(D1 + o2), lds4(W + o2));
  }
  return make_float2(a0c, a1c);
}
// The chains of consumer thread c: three consumer warps, lane k of the first
// summing a_k w and (d_x a_k) w, lane k of the second (d_y a_k) w and
// (d_z a_k) w, lanes 0-4 of the third the five per-sample rows; other lanes
// are idle (kind -1).  Every a_k row is read by one lane only; the direction
// and weight rows are read by whole warps at one address (broadcasts).
struct ChainRole {
  int kind, k, q;
};
__device__ __forceinline__ ChainRole chain_role(const EStepShape &e, int c) {
  const int cw = c >> 5, lane = c & 31;
  ChainRole r{-1, 0, 0};
  if (cw < 2) {
    if (lane < e.Kp) r = ChainRole{cw, lane, 0};
  } else if (cw == 2 && lane < 5) {
    r = ChainRole{2, lane, 0};
  }
  return r;
}
__device__ __forceinline__ void estep_chunk_chain(const float *B, const EStepShape &e, const ChainRole &role, int n4,
                                                  float2 &acc) {
  const int Kp = e.Kp;
  const uint32_t base = smem_u32(B), row = uint32_t(e.RS) * 4u;
  const uint32_t A = base + uint32_t(role.k) * row, X = base + uint32_t(Kp) * row, W = base + uint32_t(Kp + 3) * row;
  if (role.kind == 0) {
    acc = chain_rows2<0>(A, X, X, W, n4, acc);
  } else if (role.kind == 1) {
    acc = chain_rows2<1>(A, X + row, X + 2u * row, W, n4, acc);
  } else if (role.kind == 2) {
    const uint32_t R = base + uint32_t(Kp + 4 + role.k) * row;
    acc.x = chain_rows<2>(R, R, R, n4, acc.x);
  }
}

// Barrier phase of chunk k: use k / stages of stage k % stages.
__device__ __forceinline__ uint32_t use_parity(const EmShared &S, const EStepShape &e, uint32_t k) {
  return (S.stageUses[k % uint32_t(e.stages)] + k / uint32_t(e.stages)) & 1u;
}
// Chunks that every consumer warp has added (they are added in order).
__device__ __forceinline__ uint32_t chunks_done(const EmShared &S, const EStepShape &e) {
  const volatile uint32_t *d = S.warpDone;
  uint32_t m = d[0];
  for (int w = 1; w < e.consWarps; ++w) m = min(m, d[w]);
  return m;
}

// Consumer warps (threads [cons0, 512)): chunk k is added once stage
// k % stages is full; each warp then records its progress.
__device__ __forceinline__ float2 consume_estep(EmShared &S, const EStepShape &e, uint32_t N, uint32_t count) {
  const int r = int(threadIdx.x) - e.cons0;
  const ChainRole role = chain_role(e, r);
  float2 acc = make_float2(0.0f, 0.0f);
  const int lane = int(threadIdx.x & 31);
  long long waited = 0;
  for (uint32_t k = 0; k < N; ++k) {
    const int st = int(k % uint32_t(e.stages));
    const long long w0 = clock64();
    if (!mbar_wait(&S.full[st], use_parity(S, e, k), &S.abortAt, k, S.err)) break;
    waited += clock64() - w0;
    const int n = int(min(uint32_t(chunk_size(e, k)), count - chunk_begin(e, k)));
    estep_chunk_chain(S.pbuf + st * e.stageFloats, e, role, (n + 3) & ~3, acc);
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();  // this warp's reads of the stage come first
      reinterpret_cast<volatile uint32_t *>(S.warpDone)[r >> 5] = k + 1u;
    }
  }
  if (r == 32) S.prof.cycWaitE += uint64_t(waited);
  return acc;
}

// Waits until the consumers are done with chunk `need - 1` (bounded).
__device__ void wait_done(const EmShared &S, const EStepShape &e, uint32_t need) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0; chunks_done(S, e) < need; ++it) {
    __nanosleep(64);
    if ((it & 31) == 31) {
      if (has_error(S.err)) return;
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kWaitNs) {
        set_error(S.err, kErrSlotWait);
        return;
      }
    }
  }
  __threadfence_block();
}

// Loader warp: the chunks of the pass, 32 at a time.  A chunk is settled
// when this block's producers took it (they fill its stage) or when its ring
// slot holds it and its stage is free (then a bulk copy brings it in, also
// ahead of a late chunk); the settled count advances in order.  Ring slots are handed back as the copies land (all of them at the
// end of the pass).
__device__ void load_chunks(EmShared &S, const EStepShape &e, uint32_t N, uint32_t seqBase) {
  Board &b = *S.board;
  const int lane = int(threadIdx.x & 31);
  const uint32_t bytes = uint32_t(e.stageFloats) * 4u;
  const uint32_t stages = uint32_t(e.stages);
  uint32_t issued = 0, released = 0;
  unsigned handled = 0;  // bit i: chunk issued + i is settled (own, or its copy issued)
  unsigned long long t0 = 0;
  while (issued < N) {
    const uint32_t done = chunks_done(S, e);
    // a chunk's ring slot is free once its copy has landed (its stage's
    // barrier phase completed); stages of chunks past `done` are not reused
    // yet, so their phases are still the ones to test
    uint32_t rel = released > done ? released : done;
    while (rel < issued && mbar_test_wait(&S.full[rel % stages], use_parity(S, e, rel))) ++rel;
    if (rel > released) {
      if (lane == 0) st_release(&b.consumed, seqBase + rel);
      released = rel;
    }
    const uint32_t j = issued + uint32_t(lane);
    bool ok = (handled >> lane) & 1u, copy = false;
    if (!ok && j < N && j < done + stages) {  // stage j % stages is free
      const uint32_t seq = seqBase + j + 1u;
      if (reinterpret_cast<volatile uint32_t *>(S.own)[j & 63u] == seq) ok = true;
      else if (ld_relaxed(&b.ready[(seqBase + j) % uint32_t(e.slots)]) == seq) ok = copy = true;
    }
    const unsigned okMask = __ballot_sync(0xFFFFFFFFu, ok);
    const uint32_t prefix = okMask == 0xFFFFFFFFu ? 32u : uint32_t(__ffs(~okMask)) - 1u;  // settled from `issued` on
    // copies may be issued out of order (only the summing is in order): a
    // chunk that is ready behind a late one is copied now
    if (copy) {
      // the relaxed read saw the producer's release: acquire before the copy
      fence_acquire();
      fence_proxy_async();
      const int st = int(j % stages);
      mbar_expect_tx(&S.full[st], bytes);
      bulk_load(S.pbuf + st * e.stageFloats, S.ring + size_t((seqBase + j) % uint32_t(e.slots)) * e.stageFloats,
                bytes, &S.full[st]);
    }
    issued += prefix;
    handled = prefix >= 32u ? 0u : (okMask >> prefix);
    if (prefix == 0) {
      if (has_error(S.err)) {
        if (lane == 0) S.abortAt = issued;
        return;
      }
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kWaitNs) {
        if (lane == 0) {
          set_error(S.err, kErrChunkWait);
          S.abortAt = issued;
        }
        return;
      }
      __nanosleep(200);
    } else {
      t0 = 0;
    }
    __syncwarp();
  }
}

// This block's producers (threads [0, P)): take chunks from their own board,
// write each into its stage once the consumers are done with the stage's
// previous chunk, and complete the stage's full barrier.  Producing a sample
// costs the SM several times the issue slots of adding it, so the producers
// step back while helpers supply the consumers: when the chunks they take
// are not consecutive (other blocks are taking chunks too), they take the
// next one only once the board's next free chunk is within `stages` of the
// consumers; while they are alone, the next grab overlaps the current
// chunk's production.
__device__ int take_own_chunk(EmShared &S, const EStepShape &e, Board &b, uint32_t gen) {
  unsigned long long t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (has_error(S.err)) return -1;
    const unsigned long long w = ld_relaxed64(&b.grab);
    if (grab_gen(w) != gen || grab_next(w) >= grab_chunks(w)) return -1;  // none left
    if (grab_next(w) < chunks_done(S, e) + uint32_t(e.stages)) {
      const unsigned long long w2 = atomicAdd(&b.grab, 1ull);
      return (grab_gen(w2) == gen && grab_next(w2) < grab_chunks(w2)) ? int(grab_next(w2)) : -1;
    }
    __nanosleep(256);
    if ((it & 15) == 15) {
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > kWaitNs) {
        set_error(S.err, kErrChunkWait);
        return -1;
      }
    }
  }
}
__device__ void produce_own(EmShared &S, const EStepShape &e, const LeafSamples &L, uint32_t seqBase) {
  Board &b = *S.board;
  const int t = threadIdx.x;
  const uint32_t gen = S.gen;  // read by thread 0 only, which wrote it
  bool alone = true;           // thread 0: the last two chunks taken were consecutive
  if (t == 0) {
    const unsigned long long w = atomicAdd(&b.grab, 1ull);
    S.hgrab[0] = (!has_error(S.err) && grab_gen(w) == gen && grab_next(w) < grab_chunks(w)) ? int(grab_next(w)) : -1;
  }
  uint32_t made = 0;
  for (uint32_t i = 0;; ++i) {
    if (t == 0) {
      const int c0 = S.hgrab[i & 1u];
      if (c0 >= 0) {
        // mark the chunk as this block's only once its stage is free: it is
        // then within `stages` chunks of the consumers, so the marker's slot
        // (chunk - 64) has been settled and consumed long ago
        const uint32_t k = uint32_t(c0);
        if (k >= uint32_t(e.stages)) wait_done(S, e, k - uint32_t(e.stages) + 1u);
        reinterpret_cast<volatile uint32_t *>(S.own)[k & 63u] = seqBase + k + 1u;
      }
    }
    bar_named(3, e.P);
    const int chunk = S.hgrab[i & 1u];
    if (chunk < 0) break;
    ++made;
    const uint32_t k = uint32_t(chunk);
    const int st = int(k % uint32_t(e.stages));
    unsigned long long w = 0;
    const bool early = t == 0 && alone && !has_error(S.err);
    if (early) w = atomicAdd(&b.grab, 1ull);
    produce_estep_chunk<false>(S, e, L.dirw, L.count, k, S.pbuf + st * e.stageFloats, t, e.P);
    bar_named(3, e.P);
    if (t == 0) {
      mbar_arrive(&S.full[st]);
      int nextChunk;
      if (early) {
        nextChunk = (grab_gen(w) == gen && grab_next(w) < grab_chunks(w)) ? int(grab_next(w)) : -1;
        alone = nextChunk == chunk + 1;
      } else {
        nextChunk = take_own_chunk(S, e, b, gen);
      }
      S.hgrab[(i + 1u) & 1u] = nextChunk;
    }
  }
  if (t == 0) S.prof.chunksOwn += made;
}

// E-step over all samples into S.cur, S.ll and S.un (WEMFactory.h:847-892).
__device__ void pass_estep(EmShared &S, const LeafSamples &L) {
  const int tid = threadIdx.x;
  const int cnt = vec_count(int(S.vmm.K));
  const EStepShape e = estep_shape(cnt, S.tune);
  const int Kp = e.Kp;
  uint32_t N = L.count == 0 ? 0u : chunk_count(e, L.count);
  if (N > kMaxSharedChunks) {
    if (tid == 0) set_error(S.err, kErrLeafTooLarge);
    N = 0;
  }
  if (tid == 0) {
    S.un = Unassigned{0.f, 0.f, 0.f, 0.f};
    suff_clear(S.cur, S.vmm.K);
    S.cur.K = S.vmm.K;
    S.cur.numSamples = float(L.count);
    S.abortAt = has_error(S.err) ? 0u : 0xFFFFFFFFu;
  }
  if (tid < kEmThreads / 32) S.warpDone[tid] = 0;
  pack_lobes(S, Kp);
  __syncthreads();
  const uint32_t seqBase = S.seqBase;
  if (tid == 0) {  // publish the pass on the board
    Board &b = *S.board;
    const uint32_t gen = S.gen % kGrabGenMask + 1u;
    S.gen = gen;
    BoardParams &bp = b.params[gen & 1u];
    for (int i = 0; i < Kp + Kp / kLanes; ++i) bp.lobeA[i] = S.lobeA[i];
    for (int i = 0; i < Kp; ++i) bp.lobeB[i] = S.lobeB[i];
    bp.dirw = L.dirw;
    bp.count = L.count;
    bp.seqBase = seqBase;
    bp.cnt = uint32_t(cnt);
    __threadfence();
    atomicExch(&b.grab, grab_word(gen, N, 0));
  }
  float2 acc = make_float2(0.0f, 0.0f);
  const long long t0 = clock64();
  if (tid < e.P) produce_own(S, e, L, seqBase);
  else if (tid < e.cons0) load_chunks(S, e, N, seqBase);
  else acc = consume_estep(S, e, N, L.count);
  const long long cyc = clock64() - t0;
  if (tid == 0) S.prof.cycProdE += uint64_t(cyc);
  if (tid == e.cons0 + 32) S.prof.cycConsE += uint64_t(cyc);
  __syncthreads();
  if (tid >= e.cons0) {
    const ChainRole role = chain_role(e, tid - e.cons0);
    if (role.kind == 0) {
      S.cur.w[role.k] = acc.x;
      S.cur.dx[role.k] = acc.y;
    } else if (role.kind == 1) {
      S.cur.dy[role.k] = acc.x;
      S.cur.dz[role.k] = acc.y;
    } else if (role.kind == 2) {
      const int x = role.k;
      if (x == 0) S.ll = acc.x;
      else if (x == 1) S.un.sw = acc.x;
      else if (x == 2) S.un.dx = acc.x;
      else if (x == 3) S.un.dy = acc.x;
      else S.un.dz = acc.x;
    }
  }
  if (tid == 0) {
    S.prof.chunks += N;
    for (int st = 0; st < e.stages; ++st)
      S.stageUses[st] += N > uint32_t(st) ? (N - uint32_t(st) + uint32_t(e.stages) - 1u) / uint32_t(e.stages) : 0u;
    S.seqBase = seqBase + N;
    st_release(&S.board->consumed, seqBase + N);
  }
  __syncthreads();
}

// A block without leaves produces chunks for other blocks' E-step passes:
// it picks the board with the most chunks left (among boards with fewer than
// EmTuning::maxHelpers helpers) and takes chunks from it while
// it has any (loading the pass parameters when the generation changes).  It
// leaves once every leaf of the launch is finished (or the launch failed).
__device__ void help_others(EmShared &S, Board *boards, float *rings, const uint32_t *finished, uint32_t numTasks) {
  const int tid = threadIdx.x;
  const int nb = int(gridDim.x);
  int cachedBoard = -1;
  uint32_t cachedGen = 0;
  for (;;) {
    // scan: the board with the most chunks left
    uint32_t bestRem = 0;
    int best = -1;
    for (int i = tid; i < nb; i += kEmThreads) {
      const unsigned long long w = ld_relaxed64(&boards[i].grab);
      const uint32_t n = grab_chunks(w), nx = grab_next(w);
      const bool open = ld_relaxed(&boards[i].helpers) < uint32_t(S.tune.maxHelpers);
      const uint32_t rem = (grab_gen(w) != 0 && nx < n && open) ? n - nx : 0u;
      if (rem > bestRem) {
        bestRem = rem;
        best = i;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const uint32_t r = __shfl_down_sync(0xFFFFFFFFu, bestRem, off);
      const int i = __shfl_down_sync(0xFFFFFFFFu, best, off);
      if (r > bestRem) {
        bestRem = r;
        best = i;
      }
    }
    if ((tid & 31) == 0) {
      S.scanRem[tid >> 5] = bestRem;
      S.scanIdx[tid >> 5] = best;
    }
    __syncthreads();
    if (tid == 0) {
      uint32_t r = 0;
      int bi = -1;
      for (int w = 0; w < kEmThreads / 32; ++w)
        if (S.scanRem[w] > r) {
          r = S.scanRem[w];
          bi = S.scanIdx[w];
        }
      S.helpBoard = bi;
      S.helpExit = has_error(S.err) || (bi < 0 && ld_acquire(finished) >= numTasks);
    }
    __syncthreads();
    if (S.helpExit) return;
    const int bi = S.helpBoard;
    if (bi < 0) {
      __nanosleep(1000);
      continue;
    }
    Board &b = boards[bi];
    // attach to the board while it has fewer than maxHelpers helpers: with
    // at most one chunk held per helper, the chunks taken stay close to the
    // ring's free slots, and the other helpers stay free for other boards
    if (tid == 0) {
      const uint32_t before = atomicAdd(&b.helpers, 1u);
      S.helpExit = before < uint32_t(S.tune.maxHelpers) ? 0 : 1;
      if (before >= uint32_t(S.tune.maxHelpers)) atomicSub(&b.helpers, 1u);
    }
    __syncthreads();
    if (S.helpExit) {
      __syncthreads();
      __nanosleep(500);
      continue;
    }
    if (tid == 0) S.hasNext = 0;
    for (int tries = 0;;) {
      if (tid == 0) {
        if (S.hasNext) {  // taken while the last chunk was produced
          S.grabbed = S.nextGrabbed;
          S.grabGen = S.nextGen;
          S.grabExact = S.nextExact;
          S.hasNext = 0;
        } else {
          uint32_t g = 0;
          int x = 0;
          S.grabbed = helper_take(S, b, bi == cachedBoard, cachedGen, g, x);
          if (S.grabbed != -2 && S.grabbed != -1) S.grabGen = g;
          S.grabExact = x;
        }
      }
      __syncthreads();
      const int chunk = S.grabbed;
      const uint32_t gen = S.grabGen;
      if (chunk == -2) {
        __syncthreads();  // everyone has read S.grabbed before thread 0 rewrites it
        if (++tries > 64) break;  // look at the other boards again
        __nanosleep(200);
        continue;
      }
      if (chunk < 0) break;
      tries = 0;
      if (bi != cachedBoard || gen != cachedGen) {
        // the generation was published (atomic exchange) after its parameters
        if (tid == 0) __threadfence();
        __syncthreads();
        const BoardParams &src = b.params[gen & 1u];
        for (int i = tid; i < kMaxK + kMaxK / kLanes; i += kEmThreads) S.lobeA[i] = __ldcg(&src.lobeA[i]);
        for (int i = tid; i < kMaxK; i += kEmThreads) S.lobeB[i] = __ldcg(&src.lobeB[i]);
        if (tid == 0) {
          S.hp.dirw = reinterpret_cast<const float4 *>(__ldcg(reinterpret_cast<const unsigned long long *>(&src.dirw)));
          S.hp.count = __ldcg(&src.count);
          S.hp.seqBase = __ldcg(&src.seqBase);
          S.hp.cnt = __ldcg(&src.cnt);
        }
        __syncthreads();
        cachedBoard = bi;
        cachedGen = gen;
      }
      const EStepShape e = estep_shape(int(S.hp.cnt), S.tune);
      produce_for(S, b, rings + size_t(bi) * kRingFloats, e, S.hp.dirw, S.hp.count, S.hp.seqBase, uint32_t(chunk),
                  S.grabExact != 0, cachedGen);
      __syncthreads();
    }
    if (tid == 0) atomicSub(&b.helpers, 1u);
  }
}

// init/updateComponentDistances (WEMFactory.h:1199-1326)
__device__ void pass_distances(EmShared &S, const LeafSamples &L, bool init) {
  const int tid = threadIdx.x;
  const int cnt = vec_count(int(S.vmm.K));
  const int Kp = cnt * kLanes;
  const PassShape sh = pass_shape<kPassDistance>(Kp);
  pack_lobes(S, Kp);
  __syncthreads();
  float acc = 0.0f, accN = 0.0f;
  float unused = 0.0f;
  run_pass<kPassDistance>(S, L, sh, cnt, acc, unused, accN);
  // exchange: bd in xch[0][k], bw in xch[1][k]
  const int c = tid - sh.P;
  if (c >= 0 && c < 2 * Kp) S.xch[c / Kp][c % Kp] = acc;
  __syncthreads();
  if (tid == 0) {
    VMMState &v = S.vmm;
    SuffState &s = S.suff;
    int cc = vec_count(int(v.K)), rem = int(v.K % kLanes);
    for (int kk = 0; kk < cc * kLanes; ++kk) {
      float bd = S.xch[0][kk], bw = S.xch[1][kk];
      if (init) {
        s.dw[kk] = bw;
        v.dist[kk] = s.dw[kk] / bd;
      } else {
        float inv = bd;
        inv += v.dist[kk] > 0.0f ? (s.dw[kk] / v.dist[kk]) : 0.0f;
        s.dw[kk] += bw;
        v.dist[kk] = s.dw[kk] / inv;
      }
    }
    if (rem > 0)
      for (int i = rem; i < kLanes; ++i) { v.dist[(cc - 1) * kLanes + i] = 0.0f; s.dw[(cc - 1) * kLanes + i] = 0.0f; }
  }
  __syncthreads();
}

// UpdateSplitStatistics (Splitter.h:439-523) into sp (S.split or S.lsplit).
__device__ void pass_split_stats(EmShared &S, const LeafSamples &L, SplitState &sp) {
  const int tid = threadIdx.x;
  const int cnt = vec_count(int(sp.K));
  const int Kp = cnt * kLanes;
  const PassShape sh = pass_shape<kPassSplit>(Kp);
  if (tid < Kp) {
    S.invFrame[tid] = inverse_of(frame_of(mk(S.vmm.mx[tid], S.vmm.my[tid], S.vmm.mz[tid]), true));
    S.splitN0[tid] = sp.n[tid];
  }
  pack_lobes(S, Kp);
  __syncthreads();
  const int c = tid - sh.P;
  const int chiBase = split_chi_base(Kp);
  // row q < 5 Kp: r = q / Kp selects sa, sw, cx, cy, cz of lobe k = q % Kp
  auto row_value = [&](int q) {
    const int r = q / Kp, k = q % Kp;
    return r == 0 ? sp.sa[k] : r == 1 ? sp.sw[k] : r == 2 ? sp.cx[k] : r == 3 ? sp.cy[k] : sp.cz[k];
  };
  auto row_store = [&](int q, float v) {
    const int r = q / Kp, k = q % Kp;
    if (r == 0) sp.sa[k] = v;
    else if (r == 1) sp.sw[k] = v;
    else if (r == 2) sp.cx[k] = v;
    else if (r == 3) sp.cy[k] = v;
    else sp.cz[k] = v;
  };
  float acc = 0.0f, acc2 = 0.0f, accN = 0.0f;
  if (c >= 0 && c < chiBase) {
    if (c < 5 * Kp) acc = row_value(c);
    if (c + chiBase < 5 * Kp) acc2 = row_value(c + chiBase);
  } else if (c >= chiBase && c < chiBase + Kp) {
    acc = sp.chi2[c - chiBase];
    accN = sp.n[c - chiBase];
  }
  run_pass<kPassSplit>(S, L, sh, cnt, acc, acc2, accN);
  if (c >= 0 && c < chiBase) {
    if (c < 5 * Kp) row_store(c, acc);
    if (c + chiBase < 5 * Kp) row_store(c + chiBase, acc2);
  } else if (c >= chiBase && c < chiBase + Kp) {
    sp.chi2[c - chiBase] = acc;
    sp.n[c - chiBase] = accN;
  }
  __syncthreads();
}

// updateMixture / partialUpdateMixture (WEMFactory.h:751-844).  prev is the
// "previous" statistics (S.suff or S.temp); partial uses S.mask.
__device__ int em_loop(EmShared &S, const LeafSamples &L, SuffState &prev, bool partial, const FieldConfig &cfg) {
  const int tid = threadIdx.x;
  __shared__ float prevLL, invPrevLL;
  if (tid == 0) {
    suff_clear(S.cur, kMaxK);
    S.cur.overallNumSamples = 0.0f;
    S.iterations = 0;
    S.loopFlag = 1;
    prevLL = 0.0f;
    invPrevLL = 1.0f;
  }
  __syncthreads();
  while (S.loopFlag) {
    PGL_PROF_BEGIN(t0)
    pass_estep(S, L);
    PGL_PROF_END(t0, cycEstep)
    PGL_PROF_BEGIN(t1)
    if (tid < 32) {  // the M-step by warp 0, lane k on lobe k
      if (tid == 0) {
        S.prof.estepPasses++;
        S.prof.estepLobes += S.vmm.K;
        if (S.un.sw > 0.0f && S.cur.K < kMaxK) {  // handleUnassignedSampleStats (WEMFactory.h:731-748)
          int t = int(S.cur.K);
          S.cur.K++;
          S.cur.w[t] = S.un.sw; S.cur.dx[t] = S.un.dx; S.cur.dy[t] = S.un.dy; S.cur.dz[t] = S.un.dz;
          prev.K++;
          prev.w[t] = 0.0f; prev.dx[t] = prev.dy[t] = prev.dz[t] = 0.0f;
          S.vmm.K++;
          if (partial) S.mask[S.vmm.K - 1] = 1;
        }
      }
      __syncwarp();
      suff_normalize_warp(S.cur, S.cur.numSamples);
      map_step_warp(S.vmm, S.cur, prev, cfg, partial ? S.mask : nullptr);
    }
    if (tid == 0) {
      S.iterations++;
      bool converged = false;
      if (S.iterations > 1) {
        float rel = fabsf(S.ll - prevLL) * invPrevLL;
        if (rel < cfg.convergence) converged = true;
        prevLL = S.ll;
        invPrevLL = 1.0f / fabsf(S.ll);
      }
      S.loopFlag = (!converged && uint32_t(S.iterations) < cfg.maxIter) ? 1 : 0;
    }
    PGL_PROF_END(t1, cycMstep)
    __syncthreads();
  }
  if (tid == 0) suff_add(prev, S.cur);
  __syncthreads();
  return S.iterations;
}

__device__ void sort_candidates(EmShared &S, const SplitState &sp) {
  // getSplitCandidates (Splitter.h:1103-1117): descending chi-square, equal
  // values keep index order
  int n = int(sp.K);
  for (int i = 0; i < n; ++i) { S.candIdx[i] = i; S.candChi[i] = sp.chi2[i]; }
  for (int i = 1; i < n; ++i) {
    int ci = S.candIdx[i];
    float cv = S.candChi[i];
    int j = i - 1;
    while (j >= 0 && cv > S.candChi[j]) { S.candIdx[j + 1] = S.candIdx[j]; S.candChi[j + 1] = S.candChi[j]; --j; }
    S.candIdx[j + 1] = ci;
    S.candChi[j + 1] = cv;
  }
  S.numCands = n;
}

// PerformMerging (Merger.h:67-89, 218-279): all pair costs in parallel, then
// the first minimum in (i, j) scan order below the threshold.
__device__ int perform_merging(EmShared &S, const FieldConfig &cfg) {
  const int tid = threadIdx.x;
  __shared__ int mergeAgain, total, lastI, lastJ;
  if (tid == 0) { total = 0; mergeAgain = S.vmm.K > cfg.laneWidth ? 1 : 0; lastI = -1; lastJ = -1; }
  __syncthreads();
  while (mergeAgain) {
    const int K = int(S.vmm.K);
    if (lastI < 0) {  // every pair
      const int pairs = K * (K - 1) / 2;
      for (int p = tid; p < pairs; p += kEmThreads) {
        // p -> (i, j), i < j
        int i = 0, rem = p;
        while (rem >= K - 1 - i) { rem -= K - 1 - i; ++i; }
        const int j = i + 1 + rem;
        S.cost[i][j] = merge_cost(S.vmm, i, j);
      }
    } else {
      // after merging lastJ into lastI (and moving the last component into
      // slot lastJ) only the pairs with those two slots have new operands; a
      // pair's cost depends on its two components alone, so the others keep
      // the bits a full recomputation would give
      const int moved = lastJ < K ? 1 : 0;  // lastJ was not the last slot
      for (int t = tid; t < (1 + moved) * K; t += kEmThreads) {
        const int a = t < K ? lastI : lastJ, b = t < K ? t : t - K;
        if (b == a || (a == lastJ && b == lastI)) continue;  // (lastI, lastJ) is in the first row
        const int i = a < b ? a : b, j = a < b ? b : a;
        S.cost[i][j] = merge_cost(S.vmm, i, j);
      }
    }
    __syncthreads();
    if (tid == 0) {
      int ci = 0, cj = 0;
      float minCost = FLT_MAX;
      bool found = false;
      for (int i = 0; i < K - 1; ++i)  // the reference's row-major double loop (Merger.h:67-90)
        for (int j = i + 1; j < K; ++j) {
          float cost = S.cost[i][j];
          if (cost < cfg.mergeThreshold && cost < minCost && S.split.n[i] > 0.0f && S.split.n[j] > 0.0f) {
            ci = i; cj = j; minCost = cost; found = true;
          }
        }
      if (found) {
        VMMState &v = S.vmm;
        V3 muI = mk(v.mx[ci], v.my[ci], v.mz[ci]), muJ = mk(v.mx[cj], v.my[cj], v.mz[cj]);
        float wI = v.w[ci], wJ = v.w[cj];
        vmm_merge(v, ci, cj);
        V3 muK = mk(v.mx[ci], v.my[ci], v.mz[ci]);
        split_merge_stats(S.split, ci, cj, wI, muI, wJ, muJ, v.w[ci], muK);
        suff_merge(S.suff, ci, cj);
        total++;
        lastI = ci;
        lastJ = cj;
      }
      mergeAgain = (found && S.vmm.K > cfg.laneWidth) ? 1 : 0;
    }
    __syncthreads();
  }
  return total;
}

// PerformRecursiveSplitting (Splitter.h:293-356) with temp = copy of suff.
__device__ void recursive_splitting(EmShared &S, const LeafSamples &L, const FieldConfig &cfg) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    S.temp = S.suff;
    S.splitCount = -1;
  }
  __syncthreads();
  while (S.vmm.K < kMaxK && S.splitCount != 0) {
    if (tid == 0) {
      S.splitCount = 0;
      split_clear(S.lsplit, kMaxK);
      split_clear(S.lsplit, S.vmm.K);
    }
    __syncthreads();
    {
      PGL_PROF_BEGIN(tp0)
      if (threadIdx.x == 0) { S.prof.splitPasses++; S.prof.splitLobes += S.lsplit.K; }
      pass_split_stats(S, L, S.lsplit);
      PGL_PROF_END(tp0, cycSplit)
    }
    if (tid == 0) {
      sort_candidates(S, S.lsplit);
      for (int k = 0; k < kMaxK; ++k) S.mask[k] = 0;
      int numComp = int(S.vmm.K);
      for (int k = 0; k < numComp; ++k) {
        if (S.candChi[k] > cfg.splitThreshold && S.vmm.K < kMaxK) {
          bool ok = split_component(S.vmm, S.lsplit, S.temp, S.candIdx[k], cfg);
          S.mask[S.candIdx[k]] = 1;
          S.mask[S.vmm.K - 1] = 1;
          if (ok) S.splitCount++;
        }
      }
      if (S.splitCount > 0) suff_clear(S.temp, S.vmm.K);
    }
    __syncthreads();
    if (S.splitCount > 0) {
      em_loop(S, L, S.temp, true, cfg);
      if (tid == 0) {
        S.suff.K = S.vmm.K;
        suff_masked_replace(S.suff, S.mask, S.temp);
      }
      __syncthreads();
    }
  }
}

// Fit (first frame) of one leaf (ASMF.h:303-347)
__device__ void asm_fit(EmShared &S, const LeafSamples &L, const FieldConfig &cfg, const float *uniformDirs) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    suff_clear(S.suff, cfg.initK);
    split_clear(S.split, cfg.initK);
    vmm_init_uniform(S.vmm, int(cfg.initK), cfg.initKappa, uniformDirs);
    suff_clear(S.suff, cfg.initK);
    S.suff.normalized = 1;
  }
  __syncthreads();
  S.report.emIterations += em_loop(S, L, S.suff, false, cfg);
  {
    PGL_PROF_BEGIN(tp0)
    if (threadIdx.x == 0) { S.prof.distPasses++; S.prof.distLobes += S.vmm.K; }
    pass_distances(S, L, true);
    PGL_PROF_END(tp0, cycDist)
  }
  if (cfg.useSplitMerge) {
    if (tid == 0) S.mcEstimate = S.suff.sumWeights / S.suff.numSamples;
    __syncthreads();
    recursive_splitting(S, L, cfg);
    if (tid == 0) split_clear(S.split, S.vmm.K);
    __syncthreads();
    {
      PGL_PROF_BEGIN(tp1)
      if (threadIdx.x == 0) { S.prof.splitPasses++; S.prof.splitLobes += S.split.K; }
      pass_split_stats(S, L, S.split);
      PGL_PROF_END(tp1, cycSplit)
    }
    PGL_PROF_BEGIN(tm)
    int m = perform_merging(S, cfg);
    PGL_PROF_END(tm, cycMerge)
    if (tid == 0) S.report.merges += uint32_t(m);
  }
  {
    PGL_PROF_BEGIN(tp1)
    if (threadIdx.x == 0) { S.prof.distPasses++; S.prof.distLobes += S.vmm.K; }
    pass_distances(S, L, true);
    PGL_PROF_END(tp1, cycDist)
  }
}

// Update (later frames) of one leaf (ASMF.h:352-462)
__device__ void asm_update(EmShared &S, const LeafSamples &L, const FieldConfig &cfg, uint64_t &afterSplit,
                           uint64_t &afterMerge) {
  const int tid = threadIdx.x;
  __shared__ uint32_t prevK;
  __shared__ int doRefit;
  if (tid == 0) prevK = S.vmm.K;
  __syncthreads();
  S.report.emIterations += em_loop(S, L, S.suff, false, cfg);
  if (tid == 0 && prevK < S.vmm.K) S.split.K = S.vmm.K;
  __syncthreads();
  if (cfg.useSplitMerge) {
    if (tid == 0) {
      S.mcEstimate = S.suff.sumWeights / S.suff.numSamples;
      afterSplit += L.count;
      afterMerge += L.count;
    }
    __syncthreads();
    {
      PGL_PROF_BEGIN(tp2)
      if (threadIdx.x == 0) { S.prof.splitPasses++; S.prof.splitLobes += S.split.K; }
      pass_split_stats(S, L, S.split);
      PGL_PROF_END(tp2, cycSplit)
    }
    if (afterSplit >= uint64_t(int64_t(cfg.minSplit))) {
      if (tid == 0) {
        for (int k = 0; k < kMaxK; ++k) S.mask[k] = 0;
        sort_candidates(S, S.split);
        int total = 0;
        for (int k = 0; k < S.numCands; ++k) {
          if (S.candChi[k] > cfg.splitThreshold && S.vmm.K < kMaxK) {
            split_component(S.vmm, S.split, S.suff, S.candIdx[k], cfg);
            S.mask[S.candIdx[k]] = 1;
            S.mask[S.vmm.K - 1] = 1;
            total++;
          }
        }
        S.report.splits += uint32_t(total);
        doRefit = (total > 0 && cfg.partialReFit && uint64_t(L.count) >= uint64_t(int64_t(cfg.minRefit))) ? 1 : 0;
        if (doRefit) {
          S.temp = S.suff;
          suff_clear(S.temp, S.vmm.K);
        }
      }
      __syncthreads();
      if (doRefit) {
        em_loop(S, L, S.temp, true, cfg);
        if (tid == 0) {
          S.suff.K = S.vmm.K;
          suff_masked_replace(S.suff, S.mask, S.temp);
          S.split.K = S.vmm.K;
        }
      }
      if (tid == 0) afterSplit = 0;
      __syncthreads();
    }
    if (afterMerge >= uint64_t(int64_t(cfg.minMerge))) {
      PGL_PROF_BEGIN(tm)
      int m = perform_merging(S, cfg);
      PGL_PROF_END(tm, cycMerge)
      if (tid == 0) { S.report.merges += uint32_t(m); afterMerge = 0; }
      __syncthreads();
    }
  }
  {
    PGL_PROF_BEGIN(tp2)
    if (threadIdx.x == 0) { S.prof.distPasses++; S.prof.distLobes += S.vmm.K; }
    pass_distances(S, L, false);
    PGL_PROF_END(tp2, cycDist)
  }
}

// Reprojection of a leaf's samples to the region's sample mean
// (WEMFactory.h:1151-1196); positions are not needed afterwards.
// WEMFactory::prepareSamples (WEMFactory.h:1183-1196): parallax-aware
// mixtures reproject the samples onto the region's mean; plain ones keep them
// (the distance passes still read each sample's distance).
__device__ void reproject_leaf(const LeafTask &t, float4 *pd, float4 *dirw, float *dist, bool parallax) {
  if (!parallax) {
    for (uint32_t i = threadIdx.x; i < t.count; i += blockDim.x) dist[t.begin + i] = pd[t.begin + i].w;
    return;
  }
  V3 var = mk(t.varOverN[0], t.varOverN[1], t.varOverN[2]);
  float minD = length(var);
  minD = 3.f * 3.f * sqrtf(minD);
  const V3 mean = mk(t.mean[0], t.mean[1], t.mean[2]);
  for (uint32_t i = threadIdx.x; i < t.count; i += blockDim.x) {
    uint32_t g = t.begin + i;
    float4 p = pd[g];
    float4 dw = dirw[g];
    float dd = p.w;
    if (isinf(dd) || !(dd > 0.0f)) { dist[g] = dd; continue; }
    float dm = fmaxf(minD, dd);
    V3 o = mk(p.x, p.y, p.z) + mk(dw.x, dw.y, dw.z) * dm;
    V3 nd = o - mean;
    float nl = length(nd);
    nd = nd / nl;
    dirw[g] = make_float4(nd.x, nd.y, nd.z, dw.w);
    dist[g] = nl;
  }
}

__global__ void __launch_bounds__(kEmThreads)
em_leaf_kernel(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, EmSides sides, LeafReport *reports,
               LeafProfile *profiles, Board *boards, float *rings, int *err, uint32_t *finished, EmTuning tune) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EmShared &S = *reinterpret_cast<EmShared *>(smem_raw);
  __shared__ uint32_t taskId;
  __shared__ uint64_t afterSplit, afterMerge;
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) S.rcpTab[i] = rcp_seed(uint32_t(i));
  for (int i = threadIdx.x; i < 64; i += blockDim.x) S.own[i] = 0;
  if (threadIdx.x == 0) {
    S.board = boards + blockIdx.x;
    S.ring = rings + size_t(blockIdx.x) * kRingFloats;
    S.err = err;
    S.tune = tune;
    S.gen = 0;
    S.seqBase = 0;
    for (int i = 0; i < kMaxStages; ++i) {
      mbar_init(&S.full[i], 1);
      S.stageUses[i] = 0;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  // the plain form: block b fits region task b and exits (no queue, no help)
  const bool plain = tune.plainLaunches != 0;
  for (uint32_t round = 0;; ++round) {
    if (threadIdx.x == 0) taskId = plain ? (round == 0 ? blockIdx.x : numTasks) : atomicAdd(queue, 1u);
    __syncthreads();
    if (taskId >= numTasks) break;
    const LeafTask t = tasks[taskId];
    const EmSide &E = sides.side[(t.flags & kTaskVolume) ? 1 : 0];
    const FieldConfig &cfg = E.cfg;
    RegionDir &R = E.regions[t.region];
    // load the region's directional state
    {
      const uint32_t *src = reinterpret_cast<const uint32_t *>(&R.vmm);
      uint32_t *dst = reinterpret_cast<uint32_t *>(&S.vmm);
      for (int i = threadIdx.x; i < int(sizeof(VMMState) / 4); i += blockDim.x) dst[i] = src[i];
      src = reinterpret_cast<const uint32_t *>(&R.suff);
      dst = reinterpret_cast<uint32_t *>(&S.suff);
      for (int i = threadIdx.x; i < int(sizeof(SuffState) / 4); i += blockDim.x) dst[i] = src[i];
      src = reinterpret_cast<const uint32_t *>(&R.split);
      dst = reinterpret_cast<uint32_t *>(&S.split);
      for (int i = threadIdx.x; i < int(sizeof(SplitState) / 4); i += blockDim.x) dst[i] = src[i];
    }
    const long long leafStart = clock64();
    if (threadIdx.x == 0) {
      S.prof = LeafProfile{};
      S.prof.count = t.count;
      S.prof.tBegin = global_ns();
      afterSplit = R.afterSplit;
      afterMerge = R.afterMerge;
      S.report = LeafReport{0, 0, 0, 0};
    }
    reproject_leaf(t, E.pd, E.dirw, E.dist, cfg.parallax != 0);
    __syncthreads();
    const bool fit = (t.flags & kTaskFit) != 0;
    if (!fit && (t.flags & kTaskDecay) && threadIdx.x == 0) {  // Field.h:457-461
      suff_decay(S.suff, cfg.decayOnSpatialSplit);
      split_decay(S.split, cfg.decayOnSpatialSplit);
    }
    __syncthreads();
    uint32_t valid = R.valid;
    if (t.count > 0) {
      LeafSamples L{E.dirw + t.begin, E.pdf + t.begin, E.dist + t.begin, t.count};
      if (fit) {
        asm_fit(S, L, cfg, E.uniformDirs);
        if (threadIdx.x == 0) {
          S.vmm.pivot[0] = t.mean[0]; S.vmm.pivot[1] = t.mean[1]; S.vmm.pivot[2] = t.mean[2];
          valid = vmm_is_valid(S.vmm) ? 1u : 0u;
          afterSplit = 0;
          afterMerge = 0;
        }
      } else {
        if (threadIdx.x == 0 && cfg.parallax) {  // Field.h:476-482
          V3 shift = mk(S.vmm.pivot[0] - t.mean[0], S.vmm.pivot[1] - t.mean[1], S.vmm.pivot[2] - t.mean[2]);
          suff_parallax_shift(S.suff, S.vmm, shift);
          vmm_parallax_shift(S.vmm, shift);
        }
        __syncthreads();
        asm_update(S, L, cfg, afterSplit, afterMerge);
        if (threadIdx.x == 0)
          valid = (vmm_is_valid(S.vmm) && suff_is_valid(S.suff) && split_is_valid(S.split)) ? 1u : 0u;
      }
    } else if (fit) {
      valid = 0;
    }
    __syncthreads();
    {
      uint32_t *dst = reinterpret_cast<uint32_t *>(&R.vmm);
      const uint32_t *src = reinterpret_cast<const uint32_t *>(&S.vmm);
      for (int i = threadIdx.x; i < int(sizeof(VMMState) / 4); i += blockDim.x) dst[i] = src[i];
      dst = reinterpret_cast<uint32_t *>(&R.suff);
      src = reinterpret_cast<const uint32_t *>(&S.suff);
      for (int i = threadIdx.x; i < int(sizeof(SuffState) / 4); i += blockDim.x) dst[i] = src[i];
      dst = reinterpret_cast<uint32_t *>(&R.split);
      src = reinterpret_cast<const uint32_t *>(&S.split);
      for (int i = threadIdx.x; i < int(sizeof(SplitState) / 4); i += blockDim.x) dst[i] = src[i];
    }
    if (threadIdx.x == 0) {
      R.afterSplit = afterSplit;
      R.afterMerge = afterMerge;
      R.valid = valid;
      S.report.K = S.vmm.K;
      if (reports) reports[taskId] = S.report;
      if (profiles) {
        S.prof.cycTotal = uint64_t(clock64() - leafStart);
        S.prof.tEnd = global_ns();
        profiles[taskId] = S.prof;
      }
      atomicAdd(finished, 1u);
    }
    __syncthreads();
  }
  // no leaves left: produce for the blocks still working on theirs
  if (!plain) help_others(S, boards, rings, finished, numTasks);
}

PGL_DEFINE_TABLE_UPLOAD(em_upload_tables)

// One thread waits, with the EM kernel's bounded wait, on a flag that nothing
// sets: the wait gives up after limitNs and records its error in *err.
__global__ void bounded_wait_probe_kernel(const uint32_t *flag, int *err, unsigned long long limitNs) {
  if (threadIdx.x == 0 && blockIdx.x == 0) wait_at_least(flag, 1u, err, limitNs);
}
cudaError_t em_bounded_wait_probe(unsigned long long limitNs, int *errOut, cudaStream_t s) {
  uint32_t *flag = nullptr;
  int *err = nullptr;
  cudaError_t e = cudaMalloc(&flag, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(flag, 0, sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), s);
  if (e == cudaSuccess) {
    bounded_wait_probe_kernel<<<1, 32, 0, s>>>(flag, err, limitNs);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(errOut, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (flag) cudaFree(flag);
  if (err) cudaFree(err);
  return e;
}

size_t em_shared_bytes() { return sizeof(EmShared); }

// Shared-pass memory of a launch with `blocks` blocks: the boards, the error
// word and the finished-leaf counter, then one chunk ring per block.
static size_t share_header_bytes(int blocks) {
  return (size_t(blocks) * sizeof(Board) + 2 * sizeof(int) + 255) & ~size_t(255);
}
bool em_tuning_valid(const EmTuning &t) {
  return t.maxHelpers >= 0 && t.maxHelpers <= 64 && t.chunkDiv >= 1 && t.chunkDiv <= 4 && t.stageCap >= 2 &&
         t.stageCap <= kMaxStages && (t.orderByCost == 0 || t.orderByCost == 1) &&
         (t.plainLaunches == 0 || t.plainLaunches == 1) && t.reservedSMs >= 0 && t.reservedSMs < 4096;
}
size_t em_share_bytes(int blocks) { return share_header_bytes(blocks) + size_t(blocks) * kRingFloats * sizeof(float); }
size_t em_share_bytes_plain(int blocks) { return share_header_bytes(blocks); }
size_t em_share_error_offset(int blocks) { return size_t(blocks) * sizeof(Board); }

cudaError_t launch_em(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, const EmSides &sides,
                      LeafReport *reports, LeafProfile *profiles, void *share, int blocks, const EmTuning &tune,
                      cudaStream_t stream) {
  const size_t smem = sizeof(EmShared);
  // once per process (thread-safe static initialisation)
  static const cudaError_t attr =
      cudaFuncSetAttribute(em_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (attr != cudaSuccess) return attr;
  if (numTasks == 0) return cudaSuccess;
  if (blocks < 1 || share == nullptr || !em_tuning_valid(tune)) return cudaErrorInvalidValue;
  // boards start empty (generation 0, no chunk ready); error word and counter 0
  unsigned char *base = static_cast<unsigned char *>(share);
  cudaError_t e = cudaMemsetAsync(base, 0, share_header_bytes(blocks), stream);
  if (e != cudaSuccess) return e;
  Board *boards = reinterpret_cast<Board *>(base);
  int *err = reinterpret_cast<int *>(base + em_share_error_offset(blocks));
  uint32_t *finished = reinterpret_cast<uint32_t *>(base + em_share_error_offset(blocks) + sizeof(int));
  float *rings = reinterpret_cast<float *>(base + share_header_bytes(blocks));
  // persistent blocks (one per SM: shared memory bound) take leaves from the
  // queue; blocks without a leaf help the others' E-step passes.  The plain
  // form launches one block per region (blocks == numTasks); its blocks use
  // their own boards only, never a chunk ring.
  count_launch();
  em_leaf_kernel<<<unsigned(blocks), kEmThreads, smem, stream>>>(tasks, numTasks, queue, sides, reports, profiles,
                                                                 boards, rings, err, finished, tune);
  return cudaGetLastError();
}

}  // namespace pgl
