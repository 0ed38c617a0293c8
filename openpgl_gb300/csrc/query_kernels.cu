// Guided queries: kd lookup, stochastic nearest-region choice, parallax shift
// of the region's mixture to the query point, cosine product, sampling and
// pdf evaluation (Field.h:109-145, KNN.h:22-28,134-148,
// VMMSurfaceSamplingDistribution.h:37-108, PAVMM.h:609-831).
//
// One warp per query, lane k owning mixture lobe k, which mirrors the
// reference's 8-wide SIMD lanes: per-lane arithmetic is the reference's, and
// horizontal sums use shuffles in the vfloat8 reduce order (lanes j, j+8, j+16,
// j+24 summed in vector order, then the 8-lane tree).
#include <cuda_runtime.h>

#include "dqt.cuh"
#include "hg_table.h"
#include "launch.h"
#include "pgl_internal.h"

namespace pgl {




// (p[dim] >= pivot) goes right (KDTree.h:390-393); treelets give the same leaf.
__device__ __forceinline__ uint32_t kd_leaf(const FieldView &f, float p0, float p1, float p2) {
  uint32_t i = 0;
  KDNode n = f.nodes[0];
  while ((n.bits >> 30) != 3u) {
    uint32_t dim = n.bits >> 30;
    float c = dim == 0 ? p0 : (dim == 1 ? p1 : p2);
    i = (n.bits & 0x3FFFFFFFu) + (c >= n.split ? 1u : 0u);
    n = f.nodes[i];
  }
  return n.bits & 0x3FFFFFFFu;
}

// Returns the region to use, updating s1d (KNN.h:22-28, 134-148).
__device__ uint32_t choose_region(const FieldView &f, uint32_t leaf, float p0, float p1, float p2, float &s1d,
                                  int lane) {
  const Neighbours &nb = f.nbrs[leaf];
  uint32_t size = min(4u, nb.size);
  uint32_t sel = uint32_t(s1d * float(size));
  s1d = (s1d - float(sel) / float(size)) * float(size);
  sel = min(sel, size - 1);
  uint32_t key = 0xFFFFFFFFu;
  if (lane < 8) {
    V3 d = mk(nb.px[lane] - p0, nb.py[lane] - p1, nb.pz[lane] - p2);
    float dd = dot(d, d);
    key = (f2u(dd) & ~7u) | uint32_t(lane);
    if (nb.ids[lane] == ~0u) key = f2u(INFINITY);
  }
  // rank among the 8 keys (all finite keys are distinct)
  uint32_t rank = 0;
  for (int j = 0; j < 8; ++j) {
    uint32_t kj = __shfl_sync(0xFFFFFFFFu, key, j);
    float fj = u2f(kj), fk = u2f(key);
    rank += (fj < fk) ? 1u : 0u;
  }
  uint32_t hit = __ballot_sync(0xFFFFFFFFu, lane < 8 && rank == sel && key != f2u(INFINITY));
  int src = __ffs(hit) - 1;
  uint32_t chosenKey = __shfl_sync(0xFFFFFFFFu, key, src < 0 ? 0 : src);
  return nb.ids[chosenKey & 7u];
}

// The same choice by one thread (quadtree fields: a thread per query): the
// lowest neighbour slot whose key has rank `sel`, else slot 0's.
__device__ uint32_t choose_region_1(const FieldView &f, uint32_t leaf, float p0, float p1, float p2, float &s1d) {
  const Neighbours &nb = f.nbrs[leaf];
  uint32_t size = min(4u, nb.size);
  uint32_t sel = uint32_t(s1d * float(size));
  s1d = (s1d - float(sel) / float(size)) * float(size);
  sel = min(sel, size - 1);
  uint32_t key[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    V3 d = mk(nb.px[j] - p0, nb.py[j] - p1, nb.pz[j] - p2);
    float dd = dot(d, d);
    key[j] = (f2u(dd) & ~7u) | uint32_t(j);
    if (nb.ids[j] == ~0u) key[j] = f2u(INFINITY);
  }
  for (int j = 0; j < 8; ++j) {
    uint32_t rank = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) rank += (u2f(key[k]) < u2f(key[j])) ? 1u : 0u;
    if (rank == sel && key[j] != f2u(INFINITY)) return nb.ids[key[j] & 7u];
  }
  return nb.ids[key[0] & 7u];
}

// vfloat8 horizontal sum of lane values over the mixture: per group lane j
// sums lanes j, j+8, ... over cnt vectors, then the 8-lane tree.
__device__ __forceinline__ float lane_sum(float v, int cnt, int lane) {
  float acc = 0.0f;
  for (int q = 0; q < cnt; ++q) acc += __shfl_sync(0xFFFFFFFFu, v, (q * kLanes + (lane & 7)) & 31);
  acc += __shfl_xor_sync(0xFFFFFFFFu, acc, 1);
  acc += __shfl_xor_sync(0xFFFFFFFFu, acc, 2);
  acc += __shfl_xor_sync(0xFFFFFFFFu, acc, 4);
  return __shfl_sync(0xFFFFFFFFu, acc, 0);
}

// Copy of the region's lobe with the parallax shift to the query point
// (parallax-aware mixtures only: VMMSurfaceSamplingDistribution.h:41-46).
__device__ __forceinline__ Lobe load_shifted(const VMMState &v, int lane, float p0, float p1, float p2,
                                             bool parallax) {
  Lobe L;
  L.w = v.w[lane]; L.kappa = v.kappa[lane]; L.norm = v.norm[lane]; L.e2k = v.e2k[lane];
  float dist = v.dist[lane];
  V3 mu = mk(v.mx[lane], v.my[lane], v.mz[lane]);
  V3 s = mk(v.pivot[0] - p0, v.pivot[1] - p1, v.pivot[2] - p2);
  V3 p = mu * dist + s;
  float len = length(p);
  p = p / len;
  bool cond = (dist > 0.0f) && (dist >= -FLT_MAX) && (dist <= FLT_MAX);
  if (cond && parallax) mu = p;
  L.mx = mu.x; L.my = mu.y; L.mz = mu.z;
  return L;
}

// the phase function fits (VMMPhaseFunctions.cpp), uploaded with the seed tables
static_assert(kHgLobes == kMaxProducts, "a distribution holds one product per lobe of the fit");
static __constant__ HgLobeFit c_hg[kHgFits][kHgLobes];

// PAVMM::product with a single lobe of weight `weight` (the cosine lobe, or a
// lobe of the phase function's fit), before the normalisation by the
// product's integral
__device__ __forceinline__ Lobe product_terms(const Lobe &L, V3 n, float kappa, float normalization, float weight) {
  V3 mu = mk(L.mx, L.my, L.mz);
  V3 nm = mu * L.kappa + n * kappa;
  float nk = sqrtf(dot(nm, nm));
  bool chk = nk > 1e-3f;
  nk = chk ? nk : 0.0f;
  nm = chk ? nm / nk : mu;
  float ne = fexp(-2.0f * nk);
  float nn = nk / (kTwoPiF * (1.0f - ne));
  nn = chk ? nn : kInv4Pi;
  float scale = (L.norm * normalization) / nn;
  float c0 = dot(mu, nm), c1 = dot(n, nm);
  float ev = fexp(L.kappa * (c0 - 1.0f) + kappa * (c1 - 1.0f));
  scale *= ev;
  scale *= L.w * weight;
  Lobe R;
  R.w = scale; R.kappa = nk; R.mx = nm.x; R.my = nm.y; R.mz = nm.z; R.norm = nn; R.e2k = ne;
  return R;
}
// the product; integral = the product's integral
__device__ __forceinline__ Lobe product_lobe(Lobe L, V3 n, float kappa, float normalization, float weight, int cnt,
                                             int lane, float &integral) {
  Lobe R = product_terms(L, n, kappa, normalization, weight);
  integral = lane_sum(lane < cnt * kLanes ? R.w : 0.0f, cnt, lane);
  R.w /= integral;
  return R;
}

// one lobe's term of the mixture's pdf in direction d
__device__ __forceinline__ float mixture_term(const Lobe &L, V3 d) {
  float ct = dot(d, mk(L.mx, L.my, L.mz));
  float cm1 = emin(ct - 1.0f, 0.0f);
  float ev = L.norm * fexp(L.kappa * cm1);
  return L.w * ev;
}
__device__ __forceinline__ float mixture_pdf(const Lobe &L, V3 d, int cnt, int lane) {
  const float t = mixture_term(L, d);
  return lane_sum(lane < cnt * kLanes ? t : 0.0f, cnt, lane);
}

__device__ V3 lobe_direction(float k, float e2k, V3 mu, float ux, float u1);
// PAVMM::sample (PAVMM.h:737-806)
__device__ V3 mixture_sample(const Lobe &L, int K, float ux, float uy, int lane) {
  // per-vector sums of the weights
  float g = L.w;
  g += __shfl_xor_sync(0xFFFFFFFFu, g, 1);
  g += __shfl_xor_sync(0xFFFFFFFFu, g, 2);
  g += __shfl_xor_sync(0xFFFFFFFFu, g, 4);
  float vecSum[4];
  for (int q = 0; q < 4; ++q) vecSum[q] = __shfl_sync(0xFFFFFFFFu, g, q * kLanes);
  uint32_t sv = 0, sc = 0;
  float searched = uy, sumW = 0.0f, cdf = 0.0f;
  uint32_t quot = uint32_t((K - 1) / kLanes), rem = uint32_t((K - 1) % kLanes);
  for (;;) {
    cdf = vecSum[sv];
    if (sumW + cdf >= searched || sv + 1 >= quot + 1) break;
    sumW += cdf;
    sv++;
  }
  uint32_t maxSel = (sv == quot) ? rem + 1 : kLanes;
  for (;;) {
    cdf = __shfl_sync(0xFFFFFFFFu, L.w, int(sv * kLanes + sc));
    if (sumW + cdf >= searched || sc + 1 >= maxSel) break;
    sumW += cdf;
    sc++;
  }
  float u1 = smin(1.0f - FLT_EPSILON, (searched - sumW) / cdf);
  int s = int(sv * kLanes + sc);
  float k = __shfl_sync(0xFFFFFFFFu, L.kappa, s), e2k = __shfl_sync(0xFFFFFFFFu, L.e2k, s);
  V3 mu = mk(__shfl_sync(0xFFFFFFFFu, L.mx, s), __shfl_sync(0xFFFFFFFFu, L.my, s), __shfl_sync(0xFFFFFFFFu, L.mz, s));
  return lobe_direction(k, e2k, mu, ux, u1);
}
// A direction of the chosen lobe (kappa k, e^{-2k}, mean mu) from the
// rescaled uniform u1 and ux (PAVMM.h:779-806)
__device__ V3 lobe_direction(float k, float e2k, V3 mu, float ux, float u1) {
  V3 d;
  if (k == 0.0f) {
    float z = 1.0f - 2.0f * u1;
    float r = sqrtf(smax(0.f, (1.0f - z * z)));
    float sp, cp;
    lib_sincosf(float(2.0 * kPiD * double(ux)), &sp, &cp);
    d = mk(r * cp, r * sp, z);
  } else {
    float ct = 1.f + (flog(1.0f + ((e2k - 1.f) * ux))) / k;
    ct = smin(1.0f, smax(ct, -1.f));
    float st = sqrtf(1.f - ct * ct);
    float phi = float(2.0 * kPiD * double(u1));
    float sp, cp;
    lib_sincosf(phi, &sp, &cp);
    d = mk(st * cp, st * sp, ct);
  }
  return xfm(frame_of(mu, false), d);
}


// The Henyey-Greenstein product (VMMVolumeSamplingDistribution.h:54-80,
// VMMPhaseFunctions.h:45-57): the fit for |meanCosine|, li times each of its
// lobes (lobes of the fit's sign facing dir, else -dir); w = the products'
// integrals over their sum.
__device__ __forceinline__ void hg_products(const Lobe &li, V3 dir, float meanCosine, int cnt, int lane,
                                            Lobe h[kHgLobes], float w[kHgLobes]) {
  const float absG = fabsf(meanCosine);
  const float step = (kHgMaxMeanCosine - kHgMinMeanCosine) / float(kHgFits);
  int idx = int(floorf((absG - kHgMinMeanCosine) / step));
  idx = idx < kHgFits - 1 ? idx : kHgFits - 1;
  float sum = 0.0f;
#pragma unroll
  for (int i = 0; i < kHgLobes; ++i) {
    const HgLobeFit fit = c_hg[idx][i];
    const V3 out = meanCosine * fit.meanCosine > 0.f ? dir : mk(-dir.x, -dir.y, -dir.z);
    h[i] = product_lobe(li, out, fit.kappa, fit.normalization, fit.weight, cnt, lane, w[i]);
    sum += w[i];
  }
#pragma unroll
  for (int i = 0; i < kHgLobes; ++i) w[i] /= sum;
}
// Sample of a weighted set of products: the first product whose running
// weight passes u.x, sampled with u.x rescaled into it
// (VMMVolumeSamplingDistribution.h:87-105); pdf = the weighted sum.
__device__ __forceinline__ V3 products_sample(const Lobe h[kHgLobes], const float w[kHgLobes], int np, int K, float ux,
                                              float uy, int lane, float &pdf) {
  float acc = 0.0f;
  int i = 0;
  for (; i < np - 1; ++i) {
    const float next = acc + w[i];
    if (next > ux) break;
    acc = next;
  }
  const Lobe g = i == 0 ? h[0] : (i == 1 ? h[1] : h[2]);
  const float wi = i == 0 ? w[0] : (i == 1 ? w[1] : w[2]);
  const V3 d = mixture_sample(g, K, (ux - acc) / wi, uy, lane);
  const int cnt = vec_count(K);
  pdf = 0.0f;
  for (int k = 0; k < np; ++k) pdf += w[k] * mixture_pdf(h[k], d, cnt, lane);
  return d;
}

// ---------------------------------------------------------------- quadtree regions
// SphereToSquareCylindrical::pointToDirection (SphereToSquare.h:40-55), with
// the host C library's cosf and sinf of the azimuth
__device__ V3 dqt_point_to_dir(float px, float py) {
  px = dqt_clamp(px, 0.f, 1.f);
  py = dqt_clamp(py, 0.f, 1.f);
  const float cosTheta = 2.0f * px - 1.0f;
  const float sinTheta = sqrtf(1.0f - cosTheta * cosTheta);
  const float phi = float((double(py) - 0.5) * 2.0 * kPiD);
  return mk(dqt_clamp(sinTheta * lib_cosf_any(phi), -1.f, 1.f), dqt_clamp(sinTheta * lib_sinf(phi), -1.f, 1.f),
            dqt_clamp(cosTheta, -1.f, 1.f));
}
// samplePdf (DQT.h:62-72, :115-153): a stochastic descent that picks the
// left or right half by u.x and the lower or upper half by u.y, each
// rescaled into the chosen part; pdf = leaf weight / (root weight x leaf
// area) / 4 pi
__device__ float dqt_sample_pdf(const DqtNode *N, float ux, float uy, V3 &dir) {
  float span = 1.0f, x = 0.0f, y = 0.0f;
  auto rescale = [](float t, float &u) {
    if (u < t) {
      u /= t;
      return true;
    }
    u -= t;
    u /= 1.0f - t;
    return false;
  };
  uint32_t idx = 0;
  while (N[idx].child > 0) {
    span /= 2.0f;
    uint32_t off = 0;
    const DqtNode *c = &N[N[idx].child];
    const float wl = c[0].weight + c[2].weight, wr = c[1].weight + c[3].weight;
    if (!rescale(wl / (wl + wr), ux)) {
      off += 1;
      x += span;
    }
    const float wt = c[off].weight, wb = c[off + 2].weight;
    if (!rescale(wt / (wt + wb), uy)) {
      off += 2;
      y += span;
    }
    idx = N[idx].child + off;
  }
  float pdf = N[idx].weight / (N[0].weight * span * span);
  const float px = x + ux * span, py = y + uy * span;
  pdf /= kDqtJacobian;
  dir = dqt_point_to_dir(px, py);
  return pdf;
}
// pdf (DQT.h:53-60, :155-159)
__device__ float dqt_pdf(const DqtNode *N, V3 d) {
  float px, py;
  dqt_dir_to_point(d.x, d.y, d.z, px, py);
  Box2 rect;
  const uint32_t i = dqt_query(N, px, py, rect);
  const float p = N[i].weight / (N[0].weight * rect.area()) / kDqtJacobian;
  return smin(FLT_MAX, p);
}
// A guided query on a quadtree region (DQTSurfaceSamplingDistribution.h /
// DQTVolumeSamplingDistribution.h: no products, pdfLi = pdf); lane 0 writes.
__device__ void dqt_query_out(const FieldView &f, uint32_t reg, uint32_t leaf, float ux, float uy, QueryOut &o) {
  if (!f.dqtHeads[reg].valid) return;
  const DqtNode *N = f.dqtNodes + size_t(reg) * f.dqtStride;
  V3 d;
  o.pdf = dqt_sample_pdf(N, ux, uy, d);
  o.ok = 1;
  o.id = leaf;
  o.dx = d.x;
  o.dy = d.y;
  o.dz = d.z;
  o.pdfLi = dqt_pdf(N, d);
}

// ---------------------------------------------------------------- four queries per warp
// A group of eight lanes per query: lane j of a group holds lobes j, j + 8,
// j + 16 and j + 24 (the vfloat8 lane j of each lobe vector), so the sums over
// the mixture keep the warp-per-query order (per lane over the vectors, then
// the 8-lane tree) and mixtures of up to eight lobes keep every lane busy.
// Shuffles stay inside the group (width 8, the group's lane mask): groups of
// one warp may take different paths.
struct LobeSet {
  Lobe l[4];
};
__device__ __forceinline__ float group_sum(const float v[4], int cnt, unsigned gm) {
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < cnt) acc += v[q];
  acc += __shfl_xor_sync(gm, acc, 1, 8);
  acc += __shfl_xor_sync(gm, acc, 2, 8);
  acc += __shfl_xor_sync(gm, acc, 4, 8);
  return __shfl_sync(gm, acc, 0, 8);
}
__device__ __forceinline__ Lobe pick(const LobeSet &L, uint32_t q) {  // q uniform in the group
  Lobe r = L.l[0];
  if (q == 1) r = L.l[1];
  if (q == 2) r = L.l[2];
  if (q == 3) r = L.l[3];
  return r;
}
// the lobe vectors q < cnt of the mixture (the others are never read)
__device__ __forceinline__ LobeSet load_shifted_g(const VMMState &v, int j, float p0, float p1, float p2,
                                                  bool parallax, int cnt) {
  LobeSet L;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < cnt) L.l[q] = load_shifted(v, q * kLanes + j, p0, p1, p2, parallax);
  return L;
}
__device__ __forceinline__ LobeSet product_lobe_g(const LobeSet &L, V3 n, float kappa, float normalization,
                                                  float weight, int cnt, unsigned gm) {
  LobeSet R;
  float w[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (q < cnt) R.l[q] = product_terms(L.l[q], n, kappa, normalization, weight);
    w[q] = q < cnt ? R.l[q].w : 0.0f;
  }
  const float integral = group_sum(w, cnt, gm);
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < cnt) R.l[q].w /= integral;
  return R;
}
__device__ __forceinline__ float mixture_pdf_g(const LobeSet &L, V3 d, int cnt, unsigned gm) {
  float t[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) t[q] = q < cnt ? mixture_term(L.l[q], d) : 0.0f;
  return group_sum(t, cnt, gm);
}
// PAVMM::sample (PAVMM.h:737-806) by a group
__device__ V3 mixture_sample_g(const LobeSet &L, int K, float ux, float uy, unsigned gm) {
  // per-vector sums of the weights (vectors past the mixture's last are never searched)
  const int cnt = vec_count(K);
  float vecSum[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float g = q < cnt ? L.l[q].w : 0.0f;
    if (q < cnt) {
      g += __shfl_xor_sync(gm, g, 1, 8);
      g += __shfl_xor_sync(gm, g, 2, 8);
      g += __shfl_xor_sync(gm, g, 4, 8);
      g = __shfl_sync(gm, g, 0, 8);
    }
    vecSum[q] = g;
  }
  uint32_t sv = 0, sc = 0;
  float searched = uy, sumW = 0.0f, cdf = 0.0f;
  uint32_t quot = uint32_t((K - 1) / kLanes), rem = uint32_t((K - 1) % kLanes);
  for (;;) {
    cdf = sv == 0 ? vecSum[0] : sv == 1 ? vecSum[1] : sv == 2 ? vecSum[2] : vecSum[3];
    if (sumW + cdf >= searched || sv + 1 >= quot + 1) break;
    sumW += cdf;
    sv++;
  }
  const Lobe V = pick(L, sv);
  uint32_t maxSel = (sv == quot) ? rem + 1 : kLanes;
  for (;;) {
    cdf = __shfl_sync(gm, V.w, int(sc), 8);
    if (sumW + cdf >= searched || sc + 1 >= maxSel) break;
    sumW += cdf;
    sc++;
  }
  float u1 = smin(1.0f - FLT_EPSILON, (searched - sumW) / cdf);
  const int s = int(sc);
  float k = __shfl_sync(gm, V.kappa, s, 8), e2k = __shfl_sync(gm, V.e2k, s, 8);
  V3 mu = mk(__shfl_sync(gm, V.mx, s, 8), __shfl_sync(gm, V.my, s, 8), __shfl_sync(gm, V.mz, s, 8));
  return lobe_direction(k, e2k, mu, ux, u1);
}
// choose_region by a group: lane j ranks neighbour j
__device__ uint32_t choose_region_g(const FieldView &f, uint32_t leaf, float p0, float p1, float p2, float &s1d,
                                    int j, int lane, unsigned gm) {
  const Neighbours &nb = f.nbrs[leaf];
  uint32_t size = min(4u, nb.size);
  uint32_t sel = uint32_t(s1d * float(size));
  s1d = (s1d - float(sel) / float(size)) * float(size);
  sel = min(sel, size - 1);
  V3 d = mk(nb.px[j] - p0, nb.py[j] - p1, nb.pz[j] - p2);
  float dd = dot(d, d);
  uint32_t key = (f2u(dd) & ~7u) | uint32_t(j);
  if (nb.ids[j] == ~0u) key = f2u(INFINITY);
  uint32_t rank = 0;
  for (int jj = 0; jj < 8; ++jj) {
    uint32_t kj = __shfl_sync(gm, key, jj, 8);
    rank += (u2f(kj) < u2f(key)) ? 1u : 0u;
  }
  const uint32_t hit = (__ballot_sync(gm, rank == sel && key != f2u(INFINITY)) >> (lane & 24)) & 0xFFu;
  int src = __ffs(hit) - 1;
  uint32_t chosenKey = __shfl_sync(gm, key, src < 0 ? 0 : src, 8);
  return nb.ids[chosenKey & 7u];
}

// Batched volume guided queries with the Henyey-Greenstein product, a warp
// per query: Init + product with the phase function's fit + SamplePDF (+
// pdfLi).  The three products of a mixture need three times the registers
// of the cosine product, so a lane keeps one lobe here.
__global__ void query_hg_kernel(QueryParams P, const QueryIn *in, QueryOut *out, uint32_t n) {
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= n) return;
  const QueryIn q = in[gw];
  const FieldView &f = P.f;
  QueryOut o;
  o.ok = 0; o.id = 0; o.s1d = q.s1d; o.dx = o.dy = o.dz = 0.0f; o.pdf = 0.0f; o.pdfLi = 0.0f;
  bool inside = f.iteration > 0 && q.px >= f.bounds[0] && q.px <= f.bounds[3] && q.py >= f.bounds[1] &&
                q.py <= f.bounds[4] && q.pz >= f.bounds[2] && q.pz <= f.bounds[5];
  if (inside) {
    uint32_t leaf = kd_leaf(f, q.px, q.py, q.pz);
    uint32_t reg = leaf;
    float s1d = q.s1d;
    if (f.knn && s1d >= 0.f) reg = choose_region(f, leaf, q.px, q.py, q.pz, s1d, lane);
    o.s1d = s1d;
    const RegionDir &R = f.regions[reg];
    if (R.valid) {
      const int K = int(R.vmm.K), cnt = vec_count(K);
      Lobe li = load_shifted(R.vmm, lane, q.px, q.py, q.pz, f.parallax != 0);
      Lobe h[kHgLobes];
      float w[kHgLobes];
      hg_products(li, mk(q.nx, q.ny, q.nz), P.hgMeanCosine[gw], cnt, lane, h, w);
      const V3 d = products_sample(h, w, kHgLobes, K, q.ux, q.uy, lane, o.pdf);
      o.ok = 1;
      o.id = leaf;
      o.dx = d.x; o.dy = d.y; o.dz = d.z;
      o.pdfLi = mixture_pdf(li, d, cnt, lane);
    }
  }
  if (lane == 0) out[gw] = o;
}

// Batched guided queries, four per warp: Init + optional cosine product
// (surface) + SamplePDF (+ pdfLi).
__global__ void query_g_kernel(QueryParams P, const QueryIn *in, QueryOut *out, uint32_t n) {
  const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int lane = threadIdx.x & 31, j = lane & 7;
  const unsigned gm = 0xFFu << (lane & 24);
  if (gid >= n) return;
  const QueryIn q = in[gid];
  const FieldView &f = P.f;
  QueryOut o;
  o.ok = 0; o.id = 0; o.s1d = q.s1d; o.dx = o.dy = o.dz = 0.0f; o.pdf = 0.0f; o.pdfLi = 0.0f;
  bool inside = f.iteration > 0 && q.px >= f.bounds[0] && q.px <= f.bounds[3] && q.py >= f.bounds[1] &&
                q.py <= f.bounds[4] && q.pz >= f.bounds[2] && q.pz <= f.bounds[5];
  if (inside) {
    uint32_t leaf = kd_leaf(f, q.px, q.py, q.pz);
    uint32_t reg = leaf;
    float s1d = q.s1d;
    if (f.knn && s1d >= 0.f) reg = choose_region_g(f, leaf, q.px, q.py, q.pz, s1d, j, lane, gm);
    o.s1d = s1d;
    const RegionDir &R = f.regions[reg];
    if (R.valid) {
      const int K = int(R.vmm.K), cnt = vec_count(K);
      const LobeSet li = load_shifted_g(R.vmm, j, q.px, q.py, q.pz, f.parallax != 0, cnt);
      V3 d;
      if (P.cosine) {
        const LobeSet g = product_lobe_g(li, mk(q.nx, q.ny, q.nz), P.cosKappa, P.cosNorm, 1.0f, cnt, gm);
        d = mixture_sample_g(g, K, (q.ux - 0.0f) / 1.0f, q.uy, gm);
        o.pdf = 0.0f + 1.0f * mixture_pdf_g(g, d, cnt, gm);
      } else {
        d = mixture_sample_g(li, K, (q.ux - 0.0f) / 1.0f, q.uy, gm);
        o.pdf = 0.0f + 1.0f * mixture_pdf_g(li, d, cnt, gm);
      }
      o.ok = 1;
      o.id = leaf;
      o.dx = d.x; o.dy = d.y; o.dz = d.z;
      o.pdfLi = mixture_pdf_g(li, d, cnt, gm);
    }
  }
  if (j == 0) out[gid] = o;
}
// Batched path-vertex query, four per warp: Init + cosine product once, then
// one SamplePDF per 2D random number on the same distribution (the sampled
// distribution is not changed by sampling: VMMSurfaceSamplingDistribution.h:67-103),
// as a renderer does per vertex and openpgl_bench's lookup loop does per
// initialised distribution (openpgl_bench.cpp:343-362).
__global__ void query_s4_g_kernel(QueryParams P, const QueryInS4 *in, QueryOutS4 *out, uint32_t n) {
  const uint32_t gid = (blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const int lane = threadIdx.x & 31, j = lane & 7;
  const unsigned gm = 0xFFu << (lane & 24);
  if (gid >= n) return;
  const QueryInS4 q = in[gid];
  const FieldView &f = P.f;
  QueryOutS4 o;
  o.ok = 0;
  o.id = 0;
  o.s1d = q.s1d;
#pragma unroll
  for (int k = 0; k < kVertexSamples; ++k) o.s[k][0] = o.s[k][1] = o.s[k][2] = o.s[k][3] = 0.0f;
  bool inside = f.iteration > 0 && q.px >= f.bounds[0] && q.px <= f.bounds[3] && q.py >= f.bounds[1] &&
                q.py <= f.bounds[4] && q.pz >= f.bounds[2] && q.pz <= f.bounds[5];
  if (inside) {
    uint32_t leaf = kd_leaf(f, q.px, q.py, q.pz);
    uint32_t reg = leaf;
    float s1d = q.s1d;
    if (f.knn && s1d >= 0.f) reg = choose_region_g(f, leaf, q.px, q.py, q.pz, s1d, j, lane, gm);
    o.s1d = s1d;
    const RegionDir &R = f.regions[reg];
    if (R.valid) {
      const int K = int(R.vmm.K), cnt = vec_count(K);
      LobeSet g = load_shifted_g(R.vmm, j, q.px, q.py, q.pz, f.parallax != 0, cnt);
      if (P.cosine) g = product_lobe_g(g, mk(q.nx, q.ny, q.nz), P.cosKappa, P.cosNorm, 1.0f, cnt, gm);
#pragma unroll
      for (int k = 0; k < kVertexSamples; ++k) {
        const V3 d = mixture_sample_g(g, K, (q.u[k][0] - 0.0f) / 1.0f, q.u[k][1], gm);
        o.s[k][0] = d.x;
        o.s[k][1] = d.y;
        o.s[k][2] = d.z;
        o.s[k][3] = 0.0f + 1.0f * mixture_pdf_g(g, d, cnt, gm);
      }
      o.ok = 1;
      o.id = leaf;
    }
  }
  if (j == 0) out[gid] = o;
}


// Batched guided queries on a quadtree field: a thread per query (a
// quadtree's descent has no lobes to spread over a warp).
__global__ void query_dqt_kernel(QueryParams P, const QueryIn *in, QueryOut *out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const QueryIn q = in[i];
  const FieldView &f = P.f;
  QueryOut o;
  o.ok = 0; o.id = 0; o.s1d = q.s1d; o.dx = o.dy = o.dz = 0.0f; o.pdf = 0.0f; o.pdfLi = 0.0f;
  const bool inside = f.iteration > 0 && q.px >= f.bounds[0] && q.px <= f.bounds[3] && q.py >= f.bounds[1] &&
                      q.py <= f.bounds[4] && q.pz >= f.bounds[2] && q.pz <= f.bounds[5];
  if (inside) {
    const uint32_t leaf = kd_leaf(f, q.px, q.py, q.pz);
    uint32_t reg = leaf;
    float s1d = q.s1d;
    if (f.knn && s1d >= 0.f) reg = choose_region_1(f, leaf, q.px, q.py, q.pz, s1d);
    o.s1d = s1d;
    dqt_query_out(f, reg, leaf, q.ux, q.uy, o);
  }
  out[i] = o;
}
__global__ void query_s4_dqt_kernel(QueryParams P, const QueryInS4 *in, QueryOutS4 *out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const QueryInS4 q = in[i];
  const FieldView &f = P.f;
  QueryOutS4 o;
  o.ok = 0;
  o.id = 0;
  o.s1d = q.s1d;
#pragma unroll
  for (int k = 0; k < kVertexSamples; ++k) o.s[k][0] = o.s[k][1] = o.s[k][2] = o.s[k][3] = 0.0f;
  const bool inside = f.iteration > 0 && q.px >= f.bounds[0] && q.px <= f.bounds[3] && q.py >= f.bounds[1] &&
                      q.py <= f.bounds[4] && q.pz >= f.bounds[2] && q.pz <= f.bounds[5];
  if (inside) {
    const uint32_t leaf = kd_leaf(f, q.px, q.py, q.pz);
    uint32_t reg = leaf;
    float s1d = q.s1d;
    if (f.knn && s1d >= 0.f) reg = choose_region_1(f, leaf, q.px, q.py, q.pz, s1d);
    o.s1d = s1d;
    if (f.dqtHeads[reg].valid) {
      const DqtNode *N = f.dqtNodes + size_t(reg) * f.dqtStride;
      for (int k = 0; k < kVertexSamples; ++k) {
        V3 d;
        o.s[k][3] = dqt_sample_pdf(N, q.u[k][0], q.u[k][1], d);
        o.s[k][0] = d.x;
        o.s[k][1] = d.y;
        o.s[k][2] = d.z;
      }
      o.ok = 1;
      o.id = leaf;
    }
  }
  out[i] = o;
}

// ---------------------------------------------------------------- per-object path
// State of one SurfaceSamplingDistribution / VolumeSamplingDistribution on the
// device: the shifted mixture (for IncomingRadiancePDF) and the product one.

__global__ void ssd_init_kernel(FieldView f, float px, float py, float pz, float s1dIn, SSDState *st, SSDResult *res) {
  const int lane = threadIdx.x & 31;
  SSDResult r{0, 0, s1dIn, 0, 0, 0, 0};
  bool inside = f.iteration > 0 && px >= f.bounds[0] && px <= f.bounds[3] && py >= f.bounds[1] && py <= f.bounds[4] &&
                pz >= f.bounds[2] && pz <= f.bounds[5];
  if (inside) {
    uint32_t leaf = kd_leaf(f, px, py, pz);
    uint32_t reg = leaf;
    float s1d = s1dIn;
    if (f.knn && s1d >= 0.f) reg = choose_region(f, leaf, px, py, pz, s1d, lane);
    r.s1d = s1d;
    const RegionDir &R = f.regions[reg];
    if (f.dqt) {  // the quadtree is read from the field when sampled
      if (f.dqtHeads[reg].valid) {
        if (lane == 0) st->region = reg;
        r.ok = 1;
        r.id = leaf;
      }
    } else if (R.valid) {
      Lobe li = load_shifted(R.vmm, lane, px, py, pz, f.parallax != 0);
      st->li[lane] = li;
      st->g[lane] = li;
      if (lane == 0) {
        st->K = R.vmm.K;
        st->numProducts = 0;
      }
      r.ok = 1;
      r.id = leaf;
    }
  }
  if (lane == 0) *res = r;
}
__global__ void ssd_cosine_kernel(SSDState *st, float nx, float ny, float nz, float cosKappa, float cosNorm) {
  const int lane = threadIdx.x & 31;
  const int cnt = vec_count(int(st->K));
  float integral;
  Lobe g = product_lobe(st->g[lane], mk(nx, ny, nz), cosKappa, cosNorm, 1.0f, cnt, lane, integral);
  __syncwarp();
  st->g[lane] = g;
}
__global__ void ssd_hg_kernel(SSDState *st, float dx, float dy, float dz, float meanCosine) {
  const int lane = threadIdx.x & 31;
  const int cnt = vec_count(int(st->K));
  Lobe h[kHgLobes];
  float w[kHgLobes];
  hg_products(st->li[lane], mk(dx, dy, dz), meanCosine, cnt, lane, h, w);
#pragma unroll
  for (int i = 0; i < kHgLobes; ++i) st->h[i][lane] = h[i];
  if (lane == 0) {
    for (int i = 0; i < kHgLobes; ++i) st->hw[i] = w[i];
    st->numProducts = kHgLobes;
  }
}
__global__ void ssd_sample_kernel(const SSDState *st, float ux, float uy, int withPdf, SSDResult *res) {
  const int lane = threadIdx.x & 31;
  const int K = int(st->K), cnt = vec_count(K);
  V3 d;
  float pdf = 0.0f;
  if (st->numProducts > 0) {
    Lobe h[kHgLobes];
    float w[kHgLobes];
#pragma unroll
    for (int i = 0; i < kHgLobes; ++i) {
      h[i] = st->h[i][lane];
      w[i] = st->hw[i];
    }
    d = products_sample(h, w, int(st->numProducts), K, ux, uy, lane, pdf);
  } else {
    Lobe g = st->g[lane];
    d = mixture_sample(g, K, (ux - 0.0f) / 1.0f, uy, lane);
    pdf = withPdf ? 0.0f + 1.0f * mixture_pdf(g, d, cnt, lane) : 0.0f;
  }
  if (lane == 0) {
    res->dx = d.x; res->dy = d.y; res->dz = d.z; res->pdf = pdf;
  }
}
__global__ void ssd_pdf_kernel(const SSDState *st, float dx, float dy, float dz, int li, SSDResult *res) {
  const int lane = threadIdx.x & 31;
  const int cnt = vec_count(int(st->K));
  const V3 d = mk(dx, dy, dz);
  float pdf;
  if (li) {
    pdf = mixture_pdf(st->li[lane], d, cnt, lane);
  } else if (st->numProducts > 0) {
    pdf = 0.0f;
    for (uint32_t k = 0; k < st->numProducts; ++k) pdf += st->hw[k] * mixture_pdf(st->h[k][lane], d, cnt, lane);
  } else {
    pdf = 0.0f + 1.0f * mixture_pdf(st->g[lane], d, cnt, lane);
  }
  if (lane == 0) res->pdf = pdf;
}

// Per-object Sample / SamplePDF / PDF / IncomingRadiancePDF of a quadtree
// region (DQTSurfaceSamplingDistribution.h:28-45: pdfLi is the pdf).
__global__ void ssd_dqt_sample_kernel(FieldView f, const SSDState *st, float ux, float uy, SSDResult *res) {
  const DqtNode *N = f.dqtNodes + size_t(st->region) * f.dqtStride;
  V3 d;
  const float pdf = dqt_sample_pdf(N, ux, uy, d);
  res->dx = d.x;
  res->dy = d.y;
  res->dz = d.z;
  res->pdf = pdf;
}
__global__ void ssd_dqt_pdf_kernel(FieldView f, const SSDState *st, float dx, float dy, float dz, SSDResult *res) {
  const DqtNode *N = f.dqtNodes + size_t(st->region) * f.dqtStride;
  res->pdf = dqt_pdf(N, mk(dx, dy, dz));
}

// ---------------------------------------------------------------- launchers
PGL_DEFINE_TABLE_UPLOAD(query_upload_seed_tables)
cudaError_t query_upload_tables(const LibmTables &libm) {
  cudaError_t e = query_upload_seed_tables(libm);
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_hg, kHgTable, sizeof(kHgTable));
}

cudaError_t launch_query(const QueryParams &p, const QueryIn *in, QueryOut *out, uint32_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned threads = 256;
  count_launch();
  if (p.f.dqt) {
    query_dqt_kernel<<<unsigned((uint64_t(n) + threads - 1) / threads), threads, 0, s>>>(p, in, out, n);
    return cudaGetLastError();
  }
  if (p.hgMeanCosine) {
    query_hg_kernel<<<unsigned((uint64_t(n) * 32 + threads - 1) / threads), threads, 0, s>>>(p, in, out, n);
    return cudaGetLastError();
  }
  query_g_kernel<<<unsigned((uint64_t(n) * 8 + threads - 1) / threads), threads, 0, s>>>(p, in, out, n);
  return cudaGetLastError();
}
cudaError_t launch_query_s4(const QueryParams &p, const QueryInS4 *in, QueryOutS4 *out, uint32_t n,
                            cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned threads = 256;
  count_launch();
  if (p.f.dqt) {
    query_s4_dqt_kernel<<<unsigned((uint64_t(n) + threads - 1) / threads), threads, 0, s>>>(p, in, out, n);
    return cudaGetLastError();
  }
  query_s4_g_kernel<<<unsigned((uint64_t(n) * 8 + threads - 1) / threads), threads, 0, s>>>(p, in, out, n);
  return cudaGetLastError();
}
cudaError_t launch_ssd_init(const FieldView &f, float px, float py, float pz, float s1d, SSDState *st, SSDResult *res,
                            cudaStream_t s) {
  count_launch();
  ssd_init_kernel<<<1, 32, 0, s>>>(f, px, py, pz, s1d, st, res);
  return cudaGetLastError();
}
cudaError_t launch_ssd_cosine(SSDState *st, float nx, float ny, float nz, float ck, float cn, cudaStream_t s) {
  count_launch();
  ssd_cosine_kernel<<<1, 32, 0, s>>>(st, nx, ny, nz, ck, cn);
  return cudaGetLastError();
}
cudaError_t launch_ssd_hg(SSDState *st, float dx, float dy, float dz, float meanCosine, cudaStream_t s) {
  count_launch();
  ssd_hg_kernel<<<1, 32, 0, s>>>(st, dx, dy, dz, meanCosine);
  return cudaGetLastError();
}
cudaError_t launch_ssd_sample(const SSDState *st, float ux, float uy, int withPdf, SSDResult *res, cudaStream_t s) {
  count_launch();
  ssd_sample_kernel<<<1, 32, 0, s>>>(st, ux, uy, withPdf, res);
  return cudaGetLastError();
}
cudaError_t launch_ssd_pdf(const SSDState *st, float dx, float dy, float dz, int li, SSDResult *res, cudaStream_t s) {
  count_launch();
  ssd_pdf_kernel<<<1, 32, 0, s>>>(st, dx, dy, dz, li, res);
  return cudaGetLastError();
}

}  // namespace pgl

namespace pgl {
cudaError_t launch_ssd_dqt_sample(const FieldView &f, const SSDState *st, float ux, float uy, SSDResult *res,
                                  cudaStream_t s) {
  count_launch();
  ssd_dqt_sample_kernel<<<1, 1, 0, s>>>(f, st, ux, uy, res);
  return cudaGetLastError();
}
cudaError_t launch_ssd_dqt_pdf(const FieldView &f, const SSDState *st, float dx, float dy, float dz, SSDResult *res,
                               cudaStream_t s) {
  count_launch();
  ssd_dqt_pdf_kernel<<<1, 1, 0, s>>>(f, st, dx, dy, dz, res);
  return cudaGetLastError();
}
}  // namespace pgl
