// Host side of the GPU guiding field: device-resident sample storage, the
// surface/volume sub-fields and their Update and query paths.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "launch.h"
#include "pgl_internal.h"

namespace pgl {

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string &m) : std::runtime_error(m) {}
};
void check(cudaError_t e, const char *what);

// Process-wide CUDA state: the stream every object uses, constant tables.
struct Context {
  cudaStream_t stream = nullptr;
  int device = 0;
  int numSMs = 0;
  static Context &get();
};

template <typename T>
struct DevArray {
  T *p = nullptr;
  size_t cap = 0;
  void reserve(size_t n, bool keep = false);
  void release();
  size_t bytes() const { return cap * sizeof(T); }
  ~DevArray() { release(); }
  DevArray() = default;
  DevArray(const DevArray &) = delete;
  DevArray &operator=(const DevArray &) = delete;
};

// Page-locked host memory (grows; the caller makes sure no copy from or to the
// old block is in flight when it grows).
struct HostPinned {
  unsigned char *p = nullptr;
  size_t cap = 0;
  void reserve(size_t bytes);
  ~HostPinned();
  HostPinned() = default;
  HostPinned(const HostPinned &) = delete;
  HostPinned &operator=(const HostPinned &) = delete;
};

struct SampleSide {
  DevArray<float4> P, D;
  DevArray<float> pdf;
  DevArray<uint32_t> flags;
  uint64_t n = 0;
  void reserve(uint64_t count);
  size_t deviceBytes() const { return P.bytes() + D.bytes() + pdf.bytes() + flags.bytes(); }
};

// SampleDataStorage on the device (SampleDataStorage.h:18-324): surface and
// volume samples as structure-of-arrays.  Samples added one by one are kept
// in a host buffer and moved to the device in one copy when needed.
// The device address of page-locked host memory that the device addresses
// over the host link, or null (ordinary host memory: copy it).
void *device_address(const void *host);

class Storage {
 public:
  SampleSide surf, vol;
  void add(const PGLSampleRecord *s, size_t n);
  void flush();
  void ingest(const PGLSampleRecord *src, size_t count);
  void ingestDevice(const PGLSampleRecord *dsrc, size_t count, PGLSampleRecord *stage = nullptr);
  void flushIfPending();
  void reserve(size_t ns, size_t nv);
  void clearSurface() { flush(); surf.n = 0; }
  void clearVolume() { flush(); vol.n = 0; }
  uint64_t sizeSurface() { flush(); return surf.n; }
  uint64_t sizeVolume() { flush(); return vol.n; }
  PGLSampleRecord get(bool volume, uint64_t idx);
  std::vector<PGLSampleRecord> download(bool volume);
  bool validate();
  size_t deviceBytes() const { return surf.deviceBytes() + vol.deviceBytes() + staging_.bytes() + scratch_.bytes; }
  uint64_t lastH2DBytes = 0;

 private:
  std::vector<PGLSampleRecord> pending_;
  DevArray<PGLSampleRecord> staging_;
  Scratch scratch_;
};

struct RegionHost {
  Stats stats;
  float bounds[6] = {0, 0, 0, 0, 0, 0};
  bool splitFlag = false;
  uint64_t rb = 0, re = 0;
  uint64_t lastCost = 0;  // SM cycles of the region's last directional update (queue order)
};

// Per-phase timings of the last Update (FieldStatistics, Field.h:153-216).
struct UpdateTimings {
  float total = 0, copy = 0, spatial = 0, directional = 0;
  float gather = 0, emKernel = 0;  // the two parts of `directional`
  uint64_t samples = 0, regions = 0;
};

class SubField {
 public:
  // The stream this field's Update runs on (created on first use).
  cudaStream_t stream() {
    if (!stream_) check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "field stream");
    return stream_;
  }
  ~SubField() {
    for (cudaEvent_t e : events)
      if (e) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
  }
  SubField() = default;
  SubField(const SubField &) = delete;
  SubField &operator=(const SubField &) = delete;
  FieldConfig cfg;
  bool isSurface = true;
  uint64_t iteration = 0, totalSPP = 0;
  bool boundsSet = false, initialized = false, kdInit = false;
  float sceneBounds[6] = {0, 0, 0, 0, 0, 0};
  float kdBounds[6] = {0, 0, 0, 0, 0, 0};
  std::vector<KDNode> nodes;
  std::vector<RegionHost> regions;
  UpdateTimings timings;
  std::vector<LeafReport> lastReports;
  std::vector<LeafProfile> lastProfiles;
  cudaStream_t stream_ = nullptr;
  std::vector<uint32_t> lastReportRegion;

  DevArray<RegionDir> dRegions;
  DevArray<KDNode> dNodes;
  DevArray<Neighbours> dNbrs;
  DevArray<float> dUniformDirs;
  // the quadtree field type: per region a head and dqtStride node slots
  DevArray<DqtHead> dDqtHeads;
  DevArray<DqtStatsNode> dDqtStats;
  DevArray<DqtNode> dDqtNodes;
  uint32_t dqtStride = 0;
  void dqtReserve(uint32_t regions);  // keeps the existing regions' quadtrees
  DqtSide dqtSide();

  // An Update runs in three steps so that one EM launch serves both
  // sub-fields: prepare() builds the tree, gathers the samples in leaf order
  // and lists the leaf tasks (false when there are no samples); the EM launch
  // (GpuField::runEm); finish() keeps the per-leaf counters and timings.
  bool prepare(SampleSide &in);
  EmSide emSide();
  void finish(std::vector<LeafReport> reports, std::vector<LeafProfile> profiles, std::vector<uint32_t> regionOf,
              cudaEvent_t emStart, cudaEvent_t emEnd);
  std::vector<LeafTask> pending;  // leaf tasks of the prepared update, by region
  uint32_t pendingSamples() const { return pendingSamples_; }
  cudaEvent_t events[4] = {};     // start, samples copied, tree built, tasks ready
  void reset();
  FieldView view() const;
  std::vector<RegionDir> downloadRegions() const;
  void uploadRegions(const std::vector<RegionDir> &r);
  void uploadTree();
  bool valid() const;
  // device memory the sub-field holds: its state (regions, nodes,
  // neighbours) and, separately, its Update working set
  size_t stateBytes() const {
    return dRegions.bytes() + dNodes.bytes() + dNbrs.bytes() + dUniformDirs.bytes() + dDqtHeads.bytes() +
           dDqtStats.bytes() + dDqtNodes.bytes();
  }
  size_t workBytes() const;

 private:
  void buildTree(uint32_t n, const float4 *P);
  void renumber(uint32_t oldNodes, uint32_t oldRegions);
  void ensureUniformDirs();
  uint32_t pendingSamples_ = 0;

  // working buffers (sized to the largest update seen)
  DevArray<float4> posA_, posB_, sP_, sD_, tmpP_, tmpD_;
  DevArray<float> sPdf_, tmpPdf_, dist_;
  DevArray<uint32_t> node_, nodeB_, jobOf_, isLeft_, scanLeft_, keys_, vals_, nodeToJob_, leafSeg_, copyIdx_;
  DevArray<uint32_t> keysB_, valsB_;  // second buffers of the one-pass descent's sort
  DevArray<KDNode> routeNodes_;       // the tree as it stands at the start of an Update
  DevArray<unsigned long long> keys64_;
  DevArray<KdJob> jobs_;
  DevArray<IStatsAcc> acc_;
  HostPinned kdStage_;  // a kd level's jobs and node map going up, its child statistics coming back
  DevArray<float4> means_;
  DevArray<uint32_t> bounds6_;
  Scratch scratch_;
  std::vector<uint32_t> splitNodes_;        // nodes split in this update (creation order)
  std::vector<uint32_t> regionOrigin_;      // origin region of every region created in this update
};

class GpuField {
 public:
  explicit GpuField(const FieldConfig &cfg);
  SubField surface, volume;
  uint64_t iteration = 0, totalSPP = 0;
  void update(Storage &s, bool doSurface, bool doVolume);
  void setSceneBounds(const float b[6]);
  void sceneBounds(float out[6]) const;
  void reset();
  // device memory of both sub-fields' state and working sets and of the EM launch
  size_t deviceBytes() const;
  std::string serialize() const;  // byte layout of pglFieldStoreToFile (CPU_8 lanes)
  void deserialize(const std::string &bytes);  // the same layout (pglDeviceNewFieldFromFile)
  bool equals(const GpuField &o) const;

  // EM schedule parameters (never the result): set directly, or chosen by
  // timing the candidates on the next Update (autotuneNext).
  EmTuning tuning;
  bool autotuneNext = false;
  struct TuneTrial {
    EmTuning t;
    float ms;
  };
  std::vector<TuneTrial> lastTuneTrials;

 private:
  void runEm(SubField *const *sides, int count);
  void runDqt(SubField *const *sides, int count);  // the quadtree field type's fit / update
  DevArray<Box2> dqtRects_;                      // per block of the quadtree launch: scratch
  DevArray<DqtStatsNode> dqtBuild_;
  DevArray<uint32_t> dqtLeaves_;
  std::vector<LeafTask> emOrder(SubField *const *sides, int count, bool byCost) const;
  void autotuneEm(SubField *const *sides, int count, cudaStream_t s);
  DevArray<unsigned char> tuneSnap_;  // state an EM launch changes, kept while trials run
  // the EM launch of both sub-fields: leaf tasks, per-leaf counters, queue,
  // boards and chunk rings
  DevArray<LeafTask> tasks_;
  DevArray<LeafReport> reports_;
  DevArray<LeafProfile> profiles_;
  DevArray<unsigned int> queue_;
  DevArray<unsigned char> emShare_;
};

// Per-object sampling distribution (plain drop-in path).
struct GpuSamplingDistribution {
  GpuField *field = nullptr;
  bool volume = false;
  SSDState *dState = nullptr;
  SSDResult *hRes = nullptr;  // pinned
  uint32_t numDistributions = 0;
  uint32_t id = 0;
  const void *regionTag = nullptr;
  GpuSamplingDistribution(GpuField *f, bool vol);
  ~GpuSamplingDistribution();
};

// Host reproductions of the reference's scalar statistics code.
Stats stats_from_acc(const IStatsAcc &a, const float bounds[6]);
void stats_merge(Stats &a, const Stats &b);
void stats_split(Stats &s, int dim, float pos, float decay, bool lower);
void quant_frame(const float bounds[6], float c[3], float inv[3]);
float kappa_to_mean_cosine(float k);
float cosine_lobe_normalization();

}  // namespace pgl
