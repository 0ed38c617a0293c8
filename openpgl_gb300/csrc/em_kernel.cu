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
// distance pass, split-statistics pass) streams the samples in chunks of
// kChunk.  Phase A computes every per-(sample, lobe) term in parallel (4 threads
// per sample, one per group of 8 lobes) into shared memory; phase B runs one
// thread per accumulator (for example the x component of lobe 7's weighted
// direction sum) that adds the chunk's terms in sample order.  That keeps the
// reference's summation order (sequential over samples within each SIMD
// lane), so every accumulator gets the reference's bits, while the 4K+1 to
// 6K accumulators of many leaves keep the SM busy.  Scalar per-leaf logic (M
// step, split/merge bookkeeping) runs on thread 0 between passes.
#include <cuda_runtime.h>

#include "launch.h"
#include "pgl_internal.h"

namespace pgl {

constexpr int kEmThreads = 256;
constexpr int kChunk = 64;
constexpr int kTermStride = kChunk + 1;  // pad: conflict-free for both phases
constexpr int kMaxPairs = kMaxK * (kMaxK - 1) / 2;

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
  float term[6][kMaxK][kTermStride];
  float sdx[kChunk], sdy[kChunk], sdz[kChunk], sw[kChunk], spdf[kChunk], sinv[kChunk], lterm[kChunk], ssd[kChunk],
      sSamplePdf[kChunk];
  int svalid[kChunk];
  float cost[kMaxPairs];
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
};

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

struct LeafSamples {
  const float4 *dirw;  // direction xyz, weight
  const float *pdf;
  const float *dist;
  uint32_t count;
};

enum PassKind { kPassEStep = 0, kPassDistance = 1, kPassSplit = 2 };

// Phase A for one chunk: responsibilities (and pass-specific terms) of sample
// s = tid % kChunk for lobes [8v, 8v+8), v = tid / kChunk.
__device__ void phase_a(EmShared &S, const LeafSamples &L, uint32_t base, int nIn, PassKind kind) {
  const int tid = threadIdx.x;
  const int s = tid % kChunk, v = tid / kChunk;
  const VMMState &vm = S.vmm;
  const int cnt = vec_count(int(vm.K));
  bool have = s < nIn;
  float4 dw = make_float4(0.f, 0.f, 0.f, 0.f);
  if (have) dw = L.dirw[base + s];
  if (v == 0) {
    S.sdx[s] = dw.x; S.sdy[s] = dw.y; S.sdz[s] = dw.z; S.sw[s] = dw.w;
    if (have && kind != kPassEStep) {
      if (kind == kPassDistance) S.ssd[s] = rcp_avx2(L.dist[base + s]);
      else S.sSamplePdf[s] = L.pdf[base + s];
    }
  }
  const V3 d = mk(dw.x, dw.y, dw.z);
  if (have && v < cnt) {
#pragma unroll
    for (int j = 0; j < kLanes; ++j) {
      int k = v * kLanes + j;
      float ct = dot(d, mk(vm.mx[k], vm.my[k], vm.mz[k]));
      float cm1 = emin(ct - 1.0f, 0.0f);
      float ev = vm.norm[k] * fexp(vm.kappa[k] * cm1);
      S.term[0][k][s] = vm.w[k] * ev;
    }
  }
  __syncthreads();
  if (v == 0) {
    int valid = 0;
    float pdf = 0.0f, inv = 0.0f, lt = 0.0f;
    if (have) {
      float pv[kLanes];
#pragma unroll
      for (int j = 0; j < kLanes; ++j) pv[j] = 0.0f;
      for (int vv = 0; vv < cnt; ++vv)
#pragma unroll
        for (int j = 0; j < kLanes; ++j) pv[j] += S.term[0][vv * kLanes + j][s];
      pdf = reduce8(pv);
      if (pdf > 1e-16f) {
        valid = 1;
        inv = rcp_avx2(pdf);
        lt = dw.w * lib_logf(pdf);
      }
    }
    S.svalid[s] = valid;
    S.spdf[s] = pdf;
    S.sinv[s] = inv;
    S.lterm[s] = lt;
  }
  __syncthreads();
  if (have && v < cnt && S.svalid[s]) {
    const float inv = S.sinv[s], pdf = S.spdf[s];
#pragma unroll
    for (int j = 0; j < kLanes; ++j) {
      int k = v * kLanes + j;
      float a = S.term[0][k][s] * inv;
      if (kind == kPassEStep) {
        S.term[0][k][s] = a;
      } else if (kind == kPassDistance) {
        float wts = (dw.w * a) * ((a * pdf) / vm.w[k]);
        S.term[0][k][s] = wts;
        S.term[1][k][s] = wts * S.ssd[s];
      } else {
        float spdfv = S.sSamplePdf[s];
        float value = dw.w * spdfv;
        float mcEst = S.mcEstimate;
        float vmf = a * pdf;
        float pvp = vmf * value;
        pvp /= (mcEst * pdf);
        float chi = (value * value) * vmf;
        chi /= ((mcEst * mcEst) * pdf) * pdf;
        chi -= 2.0f * pvp;
        chi += vmf;
        chi /= spdfv;
        chi = a > 0.0f ? chi : 0.0f;
        V3 ld = xfm(S.invFrame[k], d);
        float aw = a * dw.w;
        S.term[0][k][s] = a;
        S.term[1][k][s] = chi;
        S.term[2][k][s] = aw;
        S.term[3][k][s] = aw * (ld.x * ld.x);
        S.term[4][k][s] = aw * (ld.y * ld.y);
        S.term[5][k][s] = aw * (ld.x * ld.y);
      }
    }
  }
  __syncthreads();
}

// E-step (WEMFactory.h:847-892).  Accumulators: t < 128 -> (component t/32,
// lobe t%32) of the weighted direction/weight sums, 128 -> log-likelihood,
// 129..132 -> unassigned weight and direction.
__device__ void pass_estep(EmShared &S, const LeafSamples &L) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    S.un = Unassigned{0.f, 0.f, 0.f, 0.f};
    suff_clear(S.cur, S.vmm.K);
    S.cur.K = S.vmm.K;
    S.cur.numSamples = float(L.count);
  }
  __syncthreads();
  const int cnt = vec_count(int(S.vmm.K));
  const int q = tid / kMaxK, k = tid % kMaxK;
  const bool lobeChain = tid < 4 * kMaxK && k < cnt * kLanes;
  float acc = 0.0f;
  for (uint32_t base = 0; base < L.count; base += kChunk) {
    int nIn = int(min(uint32_t(kChunk), L.count - base));
    phase_a(S, L, base, nIn, kPassEStep);
    if (lobeChain) {
      for (int s = 0; s < nIn; ++s) {
        if (!S.svalid[s]) continue;
        float a = S.term[0][k][s], w = S.sw[s];
        if (q == 0) acc += (S.sdx[s] * a) * w;
        else if (q == 1) acc += (S.sdy[s] * a) * w;
        else if (q == 2) acc += (S.sdz[s] * a) * w;
        else acc += a * w;
      }
    } else if (tid == 128) {
      for (int s = 0; s < nIn; ++s)
        if (S.svalid[s]) acc += S.lterm[s];
    } else if (tid >= 129 && tid <= 132) {
      for (int s = 0; s < nIn; ++s) {
        if (S.svalid[s]) continue;
        float w = S.sw[s];
        if (tid == 129) acc += w;
        else if (tid == 130) acc = acc + (S.sdx[s] * w);
        else if (tid == 131) acc = acc + (S.sdy[s] * w);
        else acc = acc + (S.sdz[s] * w);
      }
    }
    __syncthreads();
  }
  if (lobeChain) {
    if (q == 0) S.cur.dx[k] = acc;
    else if (q == 1) S.cur.dy[k] = acc;
    else if (q == 2) S.cur.dz[k] = acc;
    else S.cur.w[k] = acc;
  } else if (tid == 128) {
    S.ll = acc;
  } else if (tid == 129) {
    S.un.sw = acc;
  } else if (tid == 130) {
    S.un.dx = acc;
  } else if (tid == 131) {
    S.un.dy = acc;
  } else if (tid == 132) {
    S.un.dz = acc;
  }
  __syncthreads();
}

// init/updateComponentDistances (WEMFactory.h:1199-1326)
__device__ void pass_distances(EmShared &S, const LeafSamples &L, bool init) {
  const int tid = threadIdx.x;
  const int cnt = vec_count(int(S.vmm.K));
  const int q = tid / kMaxK, k = tid % kMaxK;
  const bool chain = tid < 2 * kMaxK && k < cnt * kLanes;
  float acc = 0.0f;
  for (uint32_t base = 0; base < L.count; base += kChunk) {
    int nIn = int(min(uint32_t(kChunk), L.count - base));
    phase_a(S, L, base, nIn, kPassDistance);
    if (chain)
      for (int s = 0; s < nIn; ++s)
        if (S.svalid[s]) acc += S.term[q == 0 ? 1 : 0][k][s];  // q0: distances, q1: weights
    __syncthreads();
  }
  // exchange: bd in term[0][k][0], bw in term[1][k][0]
  if (chain) S.term[q][k][0] = acc;
  __syncthreads();
  if (tid == 0) {
    VMMState &v = S.vmm;
    SuffState &s = S.suff;
    int c = vec_count(int(v.K)), rem = int(v.K % kLanes);
    for (int kk = 0; kk < c * kLanes; ++kk) {
      float bd = S.term[0][kk][0], bw = S.term[1][kk][0];
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
      for (int i = rem; i < kLanes; ++i) { v.dist[(c - 1) * kLanes + i] = 0.0f; s.dw[(c - 1) * kLanes + i] = 0.0f; }
  }
  __syncthreads();
}

// UpdateSplitStatistics (Splitter.h:439-523) into sp (S.split or S.lsplit).
__device__ void pass_split_stats(EmShared &S, const LeafSamples &L, SplitState &sp) {
  const int tid = threadIdx.x;
  const int cnt = vec_count(int(sp.K));
  if (tid < cnt * kLanes) S.invFrame[tid] = inverse_of(frame_of(mk(S.vmm.mx[tid], S.vmm.my[tid], S.vmm.mz[tid]), true));
  __syncthreads();
  const int q = tid / kMaxK, k = tid % kMaxK;
  const bool chain = tid < 6 * kMaxK && k < cnt * kLanes;
  float acc = 0.0f, accN = 0.0f;
  if (chain) {
    switch (q) {
      case 0: acc = sp.sa[k]; break;
      case 1: acc = sp.chi2[k]; accN = sp.n[k]; break;
      case 2: acc = sp.sw[k]; break;
      case 3: acc = sp.cx[k]; break;
      case 4: acc = sp.cy[k]; break;
      default: acc = sp.cz[k]; break;
    }
  }
  for (uint32_t base = 0; base < L.count; base += kChunk) {
    int nIn = int(min(uint32_t(kChunk), L.count - base));
    phase_a(S, L, base, nIn, kPassSplit);
    if (chain) {
      for (int s = 0; s < nIn; ++s) {
        if (!S.svalid[s]) continue;
        if (q == 1) {
          accN += 1.0f;
          acc += (S.term[1][k][s] - acc) / accN;
        } else {
          acc += S.term[q == 0 ? 0 : q][k][s];
        }
      }
    }
    __syncthreads();
  }
  if (chain) {
    switch (q) {
      case 0: sp.sa[k] = acc; break;
      case 1: sp.chi2[k] = acc; sp.n[k] = accN; break;
      case 2: sp.sw[k] = acc; break;
      case 3: sp.cx[k] = acc; break;
      case 4: sp.cy[k] = acc; break;
      default: sp.cz[k] = acc; break;
    }
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
    pass_estep(S, L);
    if (tid == 0) {
      if (S.un.sw > 0.0f && S.cur.K < kMaxK) {  // handleUnassignedSampleStats (WEMFactory.h:731-748)
        int t = int(S.cur.K);
        S.cur.K++;
        S.cur.w[t] = S.un.sw; S.cur.dx[t] = S.un.dx; S.cur.dy[t] = S.un.dy; S.cur.dz[t] = S.un.dz;
        prev.K++;
        prev.w[t] = 0.0f; prev.dx[t] = prev.dy[t] = prev.dz[t] = 0.0f;
        S.vmm.K++;
        if (partial) S.mask[S.vmm.K - 1] = 1;
      }
      suff_normalize(S.cur, S.cur.numSamples);
      map_step(S.vmm, S.cur, prev, cfg, partial ? S.mask : nullptr);
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
  __shared__ int mergeAgain, total;
  if (tid == 0) { total = 0; mergeAgain = S.vmm.K > cfg.laneWidth ? 1 : 0; }
  __syncthreads();
  while (mergeAgain) {
    const int K = int(S.vmm.K);
    const int pairs = K * (K - 1) / 2;
    for (int p = tid; p < pairs; p += kEmThreads) {
      // p -> (i, j), i < j, in row-major order of the reference's double loop
      int i = 0, rem = p;
      while (rem >= K - 1 - i) { rem -= K - 1 - i; ++i; }
      int j = i + 1 + rem;
      S.cost[p] = merge_cost(S.vmm, i, j);
    }
    __syncthreads();
    if (tid == 0) {
      int ci = 0, cj = 0, p = 0;
      float minCost = FLT_MAX;
      bool found = false;
      for (int i = 0; i < K - 1; ++i)
        for (int j = i + 1; j < K; ++j, ++p) {
          float cost = S.cost[p];
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
    pass_split_stats(S, L, S.lsplit);
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
  pass_distances(S, L, true);
  if (cfg.useSplitMerge) {
    if (tid == 0) S.mcEstimate = S.suff.sumWeights / S.suff.numSamples;
    __syncthreads();
    recursive_splitting(S, L, cfg);
    if (tid == 0) split_clear(S.split, S.vmm.K);
    __syncthreads();
    pass_split_stats(S, L, S.split);
    int m = perform_merging(S, cfg);
    if (tid == 0) S.report.merges += uint32_t(m);
  }
  pass_distances(S, L, true);
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
    pass_split_stats(S, L, S.split);
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
      int m = perform_merging(S, cfg);
      if (tid == 0) { S.report.merges += uint32_t(m); afterMerge = 0; }
      __syncthreads();
    }
  }
  pass_distances(S, L, false);
}

// Reprojection of a leaf's samples to the region's sample mean
// (WEMFactory.h:1151-1196); positions are not needed afterwards.
__device__ void reproject_leaf(const LeafTask &t, float4 *pd, float4 *dirw, float *dist) {
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
em_leaf_kernel(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, RegionDir *regions, float4 *pd,
               float4 *dirw, const float *pdf, float *dist, FieldConfig cfg, const float *uniformDirs,
               LeafReport *reports) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EmShared &S = *reinterpret_cast<EmShared *>(smem_raw);
  __shared__ uint32_t taskId;
  __shared__ uint64_t afterSplit, afterMerge;
  for (;;) {
    if (threadIdx.x == 0) taskId = atomicAdd(queue, 1u);
    __syncthreads();
    if (taskId >= numTasks) return;
    const LeafTask t = tasks[taskId];
    RegionDir &R = regions[t.region];
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
    if (threadIdx.x == 0) {
      afterSplit = R.afterSplit;
      afterMerge = R.afterMerge;
      S.report = LeafReport{0, 0, 0, 0};
    }
    reproject_leaf(t, pd, dirw, dist);
    __syncthreads();
    const bool fit = (t.flags & kTaskFit) != 0;
    if (!fit && (t.flags & kTaskDecay) && threadIdx.x == 0) {  // Field.h:457-461
      suff_decay(S.suff, cfg.decayOnSpatialSplit);
      split_decay(S.split, cfg.decayOnSpatialSplit);
    }
    __syncthreads();
    uint32_t valid = R.valid;
    if (t.count > 0) {
      LeafSamples L{dirw + t.begin, pdf + t.begin, dist + t.begin, t.count};
      if (fit) {
        asm_fit(S, L, cfg, uniformDirs);
        if (threadIdx.x == 0) {
          S.vmm.pivot[0] = t.mean[0]; S.vmm.pivot[1] = t.mean[1]; S.vmm.pivot[2] = t.mean[2];
          valid = vmm_is_valid(S.vmm) ? 1u : 0u;
          afterSplit = 0;
          afterMerge = 0;
        }
      } else {
        if (threadIdx.x == 0) {  // Field.h:476-482
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
    }
    __syncthreads();
  }
}

PGL_DEFINE_TABLE_UPLOAD(em_upload_tables)

size_t em_shared_bytes() { return sizeof(EmShared); }

cudaError_t launch_em(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, RegionDir *regions, float4 *pd,
                      float4 *dirw, const float *pdf, float *dist, const FieldConfig &cfg, const float *uniformDirs,
                      LeafReport *reports, int numBlocks, cudaStream_t stream) {
  static bool attrSet = false;
  const size_t smem = sizeof(EmShared);
  if (!attrSet) {
    cudaError_t e = cudaFuncSetAttribute(em_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    attrSet = true;
  }
  em_leaf_kernel<<<numBlocks, kEmThreads, smem, stream>>>(tasks, numTasks, queue, regions, pd, dirw, pdf, dist, cfg,
                                                          uniformDirs, reports);
  return cudaGetLastError();
}

}  // namespace pgl
