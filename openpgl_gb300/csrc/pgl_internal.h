// Internal data layouts of the GPU guiding field (host and device).
#pragma once

#include <cstdint>

#include "dqt.cuh"
#include "pgl_math.cuh"

namespace pgl {

// Effective configuration of FieldConfig::Init(KDTREE, PARALLAX_AWARE_VMM,
// deterministic, maxSamplesPerLeaf) (api.cpp:755-787 -> Device.h:99-136 in the
// reference).  maxMeanCosine is KappaToMeanCosine(maxKappa), computed on the
// host with libm's tanhf as the reference does.
struct FieldConfig {
  uint64_t maxSamples = 32000, maxDepth = 32, minSamples = 100;
  uint32_t deterministic = 1, knn = 1, fitRegions = 1;
  float decayOnSpatialSplit = 0.25f;
  uint32_t initK = 16;
  float initKappa = 0.5f;
  uint32_t maxK = 32, maxIter = 100;
  float maxKappa = 320000.f, maxMeanCosine = 0.0f, convergence = 0.005f, weightPrior = 0.01f;
  float mcPriorStrength = 0.2f, mcPrior = 0.0f;
  float splitThreshold = 0.5f, mergeThreshold = 0.025f;
  uint32_t useSplitMerge = 1, partialReFit = 1;
  int32_t maxSplitItr = 1, minSplit = 4000, minRefit = 4000, minMerge = 8000;
  float maxKappaSplit = 32000.0f;    // OPENPGL_MAX_KAPPA, hard-coded in the splitter
  float maxMeanCosineSplit = 0.0f;   // KappaToMeanCosine(32000)
  uint32_t laneWidth = 8;            // merging stops at K <= lane width (CPU_8)
  uint32_t parallax = 1;             // PARALLAX_AWARE_VMM (1) or VMM (0): reprojection and shifts
  uint32_t dqt = 0;                  // QUADTREE (Device.h:185-210): quadtrees instead of mixtures
  DqtArgs dqtArgs;                   // the quadtree factory's arguments
};

// Parallax-aware vMF mixture, lane-major (lobe k at index k), as
// ParallaxAwareVonMisesFisherMixture<8,32,true> (PAVMM.h:60-72).
struct VMMState {
  float w[kMaxK], kappa[kMaxK], mx[kMaxK], my[kMaxK], mz[kMaxK], norm[kMaxK], e2k[kMaxK], mc[kMaxK], dist[kMaxK];
  uint32_t K;
  float pivot[3];
};
// Weighted-EM sufficient statistics (WEMFactory.h:93-168).
struct SuffState {
  float dx[kMaxK], dy[kMaxK], dz[kMaxK], w[kMaxK], dw[kMaxK];
  float sumWeights, numSamples, overallNumSamples;
  uint32_t K;
  uint32_t normalized;
};
// Chi-square split statistics (VMMChiSquareComponentSplitter.h:66-118).
struct SplitState {
  float chi2[kMaxK], mx[kMaxK], my[kMaxK], cx[kMaxK], cy[kMaxK], cz[kMaxK], n[kMaxK], sw[kMaxK], sa[kMaxK];
  uint32_t K;
};
// Directional half of a region (Region.h: distribution + training statistics).
struct RegionDir {
  VMMState vmm;
  SuffState suff;
  SplitState split;
  uint64_t afterSplit, afterMerge;
  uint32_t valid;
  uint32_t pad;
};

// Float sample statistics (SampleStatistics.h:12-193); host side of a region.
struct Stats {
  float mean[3] = {0, 0, 0}, var[3] = {0, 0, 0}, n = 0;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
};

struct KDNode {  // 8 bytes, as KDTree.h:21-170: top 2 bits dim (3 = leaf), low 30 child/data index
  float split;
  uint32_t bits;
};

struct Neighbours {  // RegionNeighbours<8> (KNN.h:116-149)
  uint32_t ids[8];
  float px[8], py[8], pz[8];
  uint32_t size;
};

// One unit of directional work: a region and its samples in the sorted arrays.
struct LeafTask {
  uint32_t region;
  uint32_t begin;
  uint32_t count;
  uint32_t flags;      // kTaskFit | kTaskDecay | kTaskVolume
  float mean[3];       // region sample mean (reprojection pivot, new VMM pivot)
  float varOverN[3];   // getVariance() (reprojection distance)
};
constexpr uint32_t kTaskFit = 1u, kTaskDecay = 2u, kTaskVolume = 4u;  // kTaskVolume: a volume leaf

// Per-leaf counters written by the EM kernel (fit statistics, for tests and
// the statistics API).
struct LeafReport {
  uint32_t emIterations, splits, merges, K;
};
// Where the EM kernel spent its time on one region: passes over the leaf's
// samples by kind and SM clock cycles (clock64 of thread 0) per phase.
struct LeafProfile {
  uint32_t count;                      // samples of the leaf
  uint32_t estepPasses, distPasses, splitPasses;
  uint64_t cycEstep, cycDist, cycSplit, cycMerge, cycMstep, cycTotal;
  // inside the passes: cycles thread 0 spent producing, and cycles of the
  // slowest consumer role (E-step: lobe chain 0; split: chi-square chain 0)
  uint64_t cycProdE, cycConsE, cycProdS, cycConsS;
  // E-step chunks of the leaf, those its own block produced (the rest came
  // from helper blocks), and the cycles a summing thread waited for chunks
  uint64_t chunks, chunksOwn, cycWaitE;
  // lobes summed over the passes of each kind (sum of K per pass): the
  // algorithmic work of a pass is samples x lobes
  uint64_t estepLobes, distLobes, splitLobes;
  // the device's global timer (ns) when the block took the region and when
  // it was done with it
  uint64_t tBegin, tEnd;
};

// Integer position statistics of one kd child (IntegerSampleStatistics).
struct IStatsAcc {
  long long m[3], v[3], lo[3], hi[3];
  unsigned long long n;
};


struct PGLSampleRecord {  // PGLSampleData, 40 bytes (data.h:21-49)
  float px, py, pz, dx, dy, dz, weight, pdf, distance;
  uint32_t flags;
};

struct KdJob {
  uint32_t begin, end;       // segment of the node's samples (current order)
  uint32_t dim, left;        // split axis, index of the left child node
  float pos;                 // split position
  uint32_t needStats;        // a child is a leaf: compute integer statistics
  float c[3], inv[3];        // quantisation frame of the node's bounds
};

struct QueryIn {  // 36 bytes: position, normal, sample1D, u
  float px, py, pz, nx, ny, nz, s1d, ux, uy;
};

struct QueryOut {  // 32 bytes
  uint32_t ok, id;
  float s1d, dx, dy, dz, pdf, pdfLi;
};

// A path vertex with several SamplePDF calls on one initialised
// distribution (76 bytes): position, normal, outgoing direction and
// roughness (carried; the surface distribution consumes only the normal,
// through the cosine product), the region-choice random number and one 2D
// random number per sample.
constexpr int kVertexSamples = 4;
struct QueryInS4 {
  float px, py, pz, nx, ny, nz, wox, woy, woz, roughness, s1d;
  float u[kVertexSamples][2];
};
struct QueryOutS4 {  // 76 bytes
  uint32_t ok, id;
  float s1d;
  float s[kVertexSamples][4];  // direction xyz, pdf of each SamplePDF
};

struct FieldView {
  const KDNode *nodes;
  const RegionDir *regions;
  const Neighbours *nbrs;
  float bounds[6];
  uint32_t iteration;
  uint32_t knn;
  uint32_t numNodes;
  uint32_t parallax;  // shift the region's mixture to the query point
  // the quadtree field type: per region a head and `dqtStride` tree nodes
  const DqtHead *dqtHeads;
  const DqtNode *dqtNodes;
  uint32_t dqtStride;
  uint32_t dqt;
};

struct Lobe {
  float w, kappa, mx, my, mz, norm, e2k;
};

// Up to three products (the Henyey-Greenstein fit's lobes) per distribution.
constexpr int kMaxProducts = 3;
struct SSDState {
  Lobe li[kMaxK];                 // the region's mixture shifted to the query point
  Lobe g[kMaxK];                  // it times the cosine lobe (surface), or li
  Lobe h[kMaxProducts][kMaxK];    // li times each lobe of the phase function's fit (volume)
  float hw[kMaxProducts];         // the products' weights (their integrals, normalised)
  uint32_t K;
  uint32_t numProducts;           // 0: sample and evaluate g; else h[0, numProducts)
  uint32_t region;                // the region chosen at Init (quadtree fields sample its tree)
};

struct SSDResult {
  uint32_t ok, id;
  float s1d;
  float dx, dy, dz, pdf;
};

struct QueryParams {
  FieldView f;
  float cosKappa, cosNorm;
  int cosine;
  int samplesPerQuery;  // SamplePDF calls per query (u re-used per call index)
  const float *hgMeanCosine;  // volume queries: per-query mean cosine of the
                              // Henyey-Greenstein product (the query's normal is
                              // its direction), or null for no product
};

}  // namespace pgl
