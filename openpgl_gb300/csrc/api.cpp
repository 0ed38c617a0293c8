// The Open PGL C API (extern "C", plain pointers) implemented on the GPU field.
// Every function replaces the reference function of the same name in
// openpgl/api/api.cpp; error handling follows api.cpp:33-72: exceptions never
// cross the ABI, the message is printed and a neutral value returned.  The
// message is also kept for pglGetLastError (appended symbol).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <iterator>
#include <memory>
#include <sstream>
#include <string>

#include "../../include/openpgl_gb300.h"
#include "field.h"
#include "serve.h"

using namespace pgl;

namespace {
thread_local std::string g_lastError;

struct DeviceImpl {
  PGL_DEVICE_TYPE type;
  size_t numThreads;
};

struct StatsImpl {
  size_t numRegions = 0, numNodes = 0, maxDepth = 0;
  size_t sizePerRegion = 0;
  float timeUpdate = 0, timeCopy = 0, timeSpatial = 0, timeDirectional = 0;
  float minK = 0, maxK = 0, avgK = 0, secondMomentK = 0;
};

PGLString make_string(const std::string &s) {
  PGLString p;
  p.m_size = s.size() + 1;
  p.m_str = new char[p.m_size];
  std::memcpy(p.m_str, s.c_str(), p.m_size);
  return p;
}

void fail(const char *fn, const std::exception &e) {
  g_lastError = std::string(fn) + ": " + e.what();
  std::cout << g_lastError << std::endl;
}
}  // namespace

// The error convention of the C API for entry points defined in other files.
namespace pgl {
void api_error(const char *fn, const std::exception &e) { fail(fn, e); }
void api_clear_error() { g_lastError.clear(); }
}  // namespace pgl

namespace {

GpuField *F(PGLField f) { return reinterpret_cast<GpuField *>(f); }
Storage *S(PGLSampleStorage s) { return reinterpret_cast<Storage *>(s); }
GpuSamplingDistribution *D(void *d) { return reinterpret_cast<GpuSamplingDistribution *>(d); }

static_assert(sizeof(PGLSampleData) == sizeof(PGLSampleRecord), "sample record layout");
static_assert(sizeof(PGLGuidedQuery) == sizeof(QueryIn), "query layout");
static_assert(sizeof(PGLGuidedQueryResult) == sizeof(QueryOut), "query result layout");
static_assert(sizeof(PGLGuidedVertex) == sizeof(QueryInS4) && sizeof(PGLGuidedVertex) == 76, "vertex layout");
static_assert(sizeof(PGLGuidedVertexResult) == sizeof(QueryOutS4) && sizeof(PGLGuidedVertexResult) == 76,
              "vertex result layout");

#define PGL_TRY \
  try {         \
    g_lastError.clear();
// As the reference's catch blocks (api/api.cpp:33-72): a failed allocation,
// any std::exception and anything else are caught; none crosses the ABI.
#define PGL_CATCH(ret)                                                              \
  }                                                                                 \
  catch (const std::bad_alloc &) {                                                  \
    fail(__func__, std::runtime_error("unable to allocate memory"));                \
    return ret;                                                                     \
  }                                                                                 \
  catch (const std::exception &e) {                                                 \
    fail(__func__, e);                                                              \
    return ret;                                                                     \
  }                                                                                 \
  catch (...) {                                                                     \
    fail(__func__, std::runtime_error("an unrecognized exception was caught"));     \
    return ret;                                                                     \
  }
#define PGL_CATCH_VOID                                                              \
  }                                                                                 \
  catch (const std::bad_alloc &) {                                                  \
    fail(__func__, std::runtime_error("unable to allocate memory"));                \
    return;                                                                         \
  }                                                                                 \
  catch (const std::exception &e) {                                                 \
    fail(__func__, e);                                                              \
    return;                                                                         \
  }                                                                                 \
  catch (...) {                                                                     \
    fail(__func__, std::runtime_error("an unrecognized exception was caught"));     \
    return;                                                                         \
  }

FieldConfig config_from(const PGLFieldArguments &args) {  // Device.h:99-136
  if (args.spatialStructureType != PGL_SPATIAL_STRUCTURE_KDTREE ||
      (args.directionalDistributionType != PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM &&
       args.directionalDistributionType != PGL_DIRECTIONAL_DISTRIBUTION_VMM &&
       args.directionalDistributionType != PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE)) {
    // the field takes ownership of the argument structs (Device.h:109,136,184-207), refused or not
    delete static_cast<PGLKDTreeArguments *>(args.spatialSturctureArguments);
    throw std::runtime_error("only kd-tree fields (parallax-aware VMM, VMM, quadtree) run on the GPU");
  }
  if (args.directionalDistributionType == PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE) {  // Device.h:185-210
    std::unique_ptr<PGLKDTreeArguments> kd(static_cast<PGLKDTreeArguments *>(args.spatialSturctureArguments));
    std::unique_ptr<PGLDQTFactoryArguments> dq(
        static_cast<PGLDQTFactoryArguments *>(args.directionalDistributionArguments));
    if (!kd || !dq) throw std::runtime_error("null field arguments");
    FieldConfig c;
    c.dqt = 1;
    c.parallax = 0;  // a quadtree has no parallax compensation (DQT.h:28-30)
    c.deterministic = args.deterministic ? 1u : 0u;
    c.fitRegions = args.debugArguments.fitRegions ? 1u : 0u;
    c.knn = kd->knnLookup ? 1u : 0u;
    c.minSamples = kd->minSamples;
    c.maxSamples = kd->maxSamples;
    c.maxDepth = kd->maxDepth;
    c.dqtArgs.leafEstimator = int32_t(dq->leafEstimator);
    c.dqtArgs.splitMetric = int32_t(dq->splitMetric);
    c.dqtArgs.splitThreshold = dq->splitThreshold;
    c.dqtArgs.footprintFactor = dq->footprintFactor;
    c.dqtArgs.maxLevels = dq->maxLevels;
    if (dqt_max_nodes(c.dqtArgs) > (uint64_t(1) << 18))
      throw std::runtime_error("quadtree factory arguments allow trees of more than 262144 nodes");
    return c;
  }
  FieldConfig c;
  // Device.h:139-178: the plain VMM is the same mixture without parallax compensation
  c.parallax = args.directionalDistributionType == PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM ? 1u : 0u;
  const PGLKDTreeArguments *kd = static_cast<const PGLKDTreeArguments *>(args.spatialSturctureArguments);
  const PGLVMMFactoryArguments *vm = static_cast<const PGLVMMFactoryArguments *>(args.directionalDistributionArguments);
  if (!kd || !vm) throw std::runtime_error("null field arguments");
  c.deterministic = args.deterministic ? 1u : 0u;
  c.fitRegions = args.debugArguments.fitRegions ? 1u : 0u;
  c.knn = kd->knnLookup ? 1u : 0u;
  c.minSamples = kd->minSamples;
  c.maxSamples = kd->maxSamples;
  c.maxDepth = kd->maxDepth;
  c.initK = uint32_t(vm->initK);
  c.initKappa = vm->initKappa;
  c.maxK = uint32_t(vm->maxK);
  c.maxIter = uint32_t(vm->maxEMIterrations);
  c.maxKappa = vm->maxKappa;
  c.maxMeanCosine = kappa_to_mean_cosine(c.maxKappa);
  c.convergence = vm->convergenceThreshold;
  c.weightPrior = vm->weightPrior;
  c.mcPriorStrength = vm->meanCosinePriorStrength;
  c.mcPrior = vm->meanCosinePrior;
  c.splitThreshold = vm->splittingThreshold;
  c.mergeThreshold = vm->mergingThreshold;
  c.partialReFit = vm->partialReFit ? 1u : 0u;
  c.maxSplitItr = vm->maxSplitItr;
  c.useSplitMerge = vm->useSplitAndMerge ? 1u : 0u;
  c.minSplit = vm->minSamplesForSplitting;
  c.minRefit = vm->minSamplesForPartialRefitting;
  c.minMerge = vm->minSamplesForMerging;
  c.maxKappaSplit = 32000.0f;
  c.maxMeanCosineSplit = kappa_to_mean_cosine(32000.0f);
  c.laneWidth = 8;
  // the reference takes ownership of the argument structs (Device.h:109,136)
  delete kd;
  delete vm;
  return c;
}

StatsImpl *make_stats(const SubField &f) {  // Field::getStatistics (Field.h:604-638)
  StatsImpl *s = new StatsImpl();
  s->numRegions = f.regions.size();
  s->numNodes = f.nodes.size();
  s->sizePerRegion = sizeof(RegionDir) + sizeof(RegionHost);
  s->timeUpdate = f.timings.total;
  s->timeCopy = f.timings.copy;
  s->timeSpatial = f.timings.spatial;
  s->timeDirectional = f.timings.directional;
  // depth
  std::vector<std::pair<uint32_t, uint32_t>> st;
  if (!f.nodes.empty()) st.push_back({0, 1});
  while (!st.empty()) {
    auto it = st.back();
    st.pop_back();
    s->maxDepth = std::max<size_t>(s->maxDepth, it.second);
    const KDNode &n = f.nodes[it.first];
    if ((n.bits >> 30) != 3u) {
      st.push_back({(n.bits & 0x3FFFFFFFu), it.second + 1});
      st.push_back({(n.bits & 0x3FFFFFFFu) + 1, it.second + 1});
    }
  }
  std::vector<RegionDir> r = f.downloadRegions();
  if (!r.empty()) {
    s->minK = 1e10f;
    for (const RegionDir &d : r) {
      float k = float(d.vmm.K);
      s->minK = std::min(s->minK, k);
      s->maxK = std::max(s->maxK, k);
      s->avgK += k;
      s->secondMomentK += k * k;
    }
    s->avgK /= float(r.size());
    s->secondMomentK = std::sqrt(s->secondMomentK / float(r.size()));
  }
  return s;
}
}  // namespace

extern "C" {

// ------------------------------------------------------------------ device (api.cpp:83-114)
OPENPGL_CORE_INTERFACE PGLDevice pglNewDevice(PGL_DEVICE_TYPE deviceType, size_t numThreads) {
  PGL_TRY
  Context::get();  // fails loudly without a usable GPU
  return reinterpret_cast<PGLDevice>(new DeviceImpl{deviceType, numThreads});
  PGL_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE void pglReleaseDevice(PGLDevice device) { delete reinterpret_cast<DeviceImpl *>(device); }

OPENPGL_CORE_INTERFACE PGLField pglDeviceNewField(PGLDevice device, PGLFieldArguments args) {
  PGL_TRY
  if (!device) throw std::runtime_error("null handle provided to pglDeviceNewField");
  return reinterpret_cast<PGLField>(new GpuField(config_from(args)));
  PGL_CATCH(nullptr)
}
// Device::newFieldFromFile (Device.h:217-260): the reference's file layout
// (VecSize 8 lanes), kd-tree fields with parallax-aware VMMs.
OPENPGL_CORE_INTERFACE PGLField pglDeviceNewFieldFromFile(PGLDevice device, const char *fieldFileName) {
  PGL_TRY
  if (!device) throw std::runtime_error("null handle provided to pglDeviceNewFieldFromFile");
  if (!fieldFileName) throw std::runtime_error("null string provided to pglDeviceNewFieldFromFile");
  std::ifstream in(fieldFileName, std::ios::binary);
  if (!in) throw std::runtime_error("error: couldn't open file");
  std::string bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  // settings the file does not hold keep the defaults of a new field
  FieldConfig c;
  c.maxKappaSplit = 32000.0f;
  c.maxMeanCosineSplit = kappa_to_mean_cosine(32000.0f);
  c.laneWidth = 8;
  std::unique_ptr<GpuField> f(new GpuField(c));
  f->deserialize(bytes);
  return reinterpret_cast<PGLField>(f.release());
  PGL_CATCH(nullptr)
}

OPENPGL_CORE_INTERFACE void pglFieldArgumentsSetDefaults(PGLFieldArguments &a, const PGL_SPATIAL_STRUCTURE_TYPE,
                                                         const PGL_DIRECTIONAL_DISTRIBUTION_TYPE directionalType,
                                                         const bool deterministic, const size_t maxSamplesPerLeaf) {
  // api.cpp:755-787
  a.spatialStructureType = PGL_SPATIAL_STRUCTURE_KDTREE;
  PGLKDTreeArguments *kd = new PGLKDTreeArguments();
  kd->maxSamples = maxSamplesPerLeaf;
  a.spatialSturctureArguments = kd;
  a.deterministic = deterministic;
  a.debugArguments.fitRegions = true;
  if (directionalType == PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE) {
    a.directionalDistributionType = PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE;
    a.directionalDistributionArguments = new PGLDQTFactoryArguments();
  } else {
    a.directionalDistributionType = directionalType == PGL_DIRECTIONAL_DISTRIBUTION_VMM
                                        ? PGL_DIRECTIONAL_DISTRIBUTION_VMM
                                        : PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM;
    a.directionalDistributionArguments = new PGLVMMFactoryArguments(maxSamplesPerLeaf);
  }
}

// ------------------------------------------------------------------ field (api.cpp:115-280)
OPENPGL_CORE_INTERFACE void pglReleaseField(PGLField field) {
  PGL_TRY
  delete F(field);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE bool pglFieldStoreToFile(PGLField field, const char *fieldFileName) {
  PGL_TRY
  if (!field || !fieldFileName) throw std::runtime_error("null handle or file name");
  std::string b = F(field)->serialize();
  std::ofstream os(fieldFileName, std::ios::binary);
  if (!os) throw std::runtime_error("error: couldn't open file!");
  os.write(b.data(), std::streamsize(b.size()));
  return bool(os);
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE size_t pglFieldGetIteration(PGLField field) {
  PGL_TRY
  return F(field)->iteration;
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE void pglFieldSetSceneBounds(PGLField field, pgl_box3f bounds) {
  PGL_TRY
  float b[6] = {bounds.lower.x, bounds.lower.y, bounds.lower.z, bounds.upper.x, bounds.upper.y, bounds.upper.z};
  F(field)->setSceneBounds(b);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE pgl_box3f pglFieldGetSceneBounds(PGLField field) {
  pgl_box3f r{};
  PGL_TRY
  float b[6];
  F(field)->sceneBounds(b);
  r.lower = pgl_vec3f{b[0], b[1], b[2]};
  r.upper = pgl_vec3f{b[3], b[4], b[5]};
  return r;
  PGL_CATCH(r)
}
OPENPGL_CORE_INTERFACE void pglFieldUpdate(PGLField field, PGLSampleStorage sampleStorage) {
  PGL_TRY
  F(field)->update(*S(sampleStorage), true, true);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglFieldUpdateSurface(PGLField field, PGLSampleStorage sampleStorage) {
  PGL_TRY
  F(field)->update(*S(sampleStorage), true, false);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglFieldUpdateVolume(PGLField field, PGLSampleStorage sampleStorage) {
  PGL_TRY
  F(field)->update(*S(sampleStorage), false, true);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglFieldReset(PGLField field) {
  PGL_TRY
  F(field)->reset();
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE bool pglFieldValidate(PGLField field) {
  PGL_TRY
  GpuField *f = F(field);
  bool v = true;
  if (f->surface.initialized) v = v && f->surface.valid();
  if (f->volume.initialized) v = v && f->volume.valid();
  return v;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldCompare(PGLField a, PGLField b) {
  PGL_TRY
  return F(a)->equals(*F(b));
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE PGLFieldStatistics pglFieldGetSurfaceStatistics(PGLField field) {
  PGL_TRY
  return reinterpret_cast<PGLFieldStatistics>(make_stats(F(field)->surface));
  PGL_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE PGLFieldStatistics pglFieldGetVolumeStatistics(PGLField field) {
  PGL_TRY
  return reinterpret_cast<PGLFieldStatistics>(make_stats(F(field)->volume));
  PGL_CATCH(nullptr)
}

// ------------------------------------------------------------------ per-object sampling distributions
OPENPGL_CORE_INTERFACE PGLSurfaceSamplingDistribution pglFieldNewSurfaceSamplingDistribution(PGLField field) {
  PGL_TRY
  return reinterpret_cast<PGLSurfaceSamplingDistribution>(new GpuSamplingDistribution(F(field), false));
  PGL_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE PGLVolumeSamplingDistribution pglFieldNewVolumeSamplingDistribution(PGLField field) {
  PGL_TRY
  return reinterpret_cast<PGLVolumeSamplingDistribution>(new GpuSamplingDistribution(F(field), true));
  PGL_CATCH(nullptr)
}
static bool init_distribution(GpuField *f, GpuSamplingDistribution *d, bool volume, pgl_point3f p, float *s1d) {
  // SurfaceVolumeField::init{Surface,Volume}SamplingDistribution (SurfaceVolumeField.h:50-85)
  Context &c = Context::get();
  const SubField &sf = volume ? f->volume : f->surface;
  float in = s1d ? *s1d : -1.0f;
  check(launch_ssd_init(sf.view(), p.x, p.y, p.z, in, d->dState, d->hRes, c.stream), "init");
  check(cudaStreamSynchronize(c.stream), "init");
  if (s1d) *s1d = d->hRes->s1d;
  if (!d->hRes->ok) return false;
  d->numDistributions = 1;
  d->id = d->hRes->id;
  d->regionTag = reinterpret_cast<const void *>(uintptr_t(d->hRes->id) + 1u);
  return true;
}
OPENPGL_CORE_INTERFACE bool pglFieldInitSurfaceSamplingDistribution(PGLField field, PGLSurfaceSamplingDistribution d,
                                                                    pgl_point3f position, float *sample1D) {
  PGL_TRY
  return init_distribution(F(field), D(d), false, position, sample1D);
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldInitVolumeSamplingDistribution(PGLField field, PGLVolumeSamplingDistribution d,
                                                                   pgl_point3f position, float *sample1D) {
  PGL_TRY
  return init_distribution(F(field), D(d), true, position, sample1D);
  PGL_CATCH(false)
}
static bool dist_dqt(const GpuSamplingDistribution *d) { return d->field->surface.cfg.dqt != 0; }
static FieldView dist_view(const GpuSamplingDistribution *d) {
  return (d->volume ? d->field->volume : d->field->surface).view();
}
static pgl_vec3f dist_sample(GpuSamplingDistribution *d, pgl_point2f u, float *pdf) {
  Context &c = Context::get();
  if (dist_dqt(d))
    check(launch_ssd_dqt_sample(dist_view(d), d->dState, u.x, u.y, d->hRes, c.stream), "sample");
  else
    check(launch_ssd_sample(d->dState, u.x, u.y, pdf ? 1 : 0, d->hRes, c.stream), "sample");
  check(cudaStreamSynchronize(c.stream), "sample");
  if (pdf) *pdf = d->hRes->pdf;
  return pgl_vec3f{d->hRes->dx, d->hRes->dy, d->hRes->dz};
}
static float dist_pdf(GpuSamplingDistribution *d, pgl_vec3f dir, bool li) {
  Context &c = Context::get();
  if (dist_dqt(d))  // a quadtree's incoming-radiance pdf is its pdf
    check(launch_ssd_dqt_pdf(dist_view(d), d->dState, dir.x, dir.y, dir.z, d->hRes, c.stream), "pdf");
  else
    check(launch_ssd_pdf(d->dState, dir.x, dir.y, dir.z, li ? 1 : 0, d->hRes, c.stream), "pdf");
  check(cudaStreamSynchronize(c.stream), "pdf");
  return d->hRes->pdf;
}
OPENPGL_CORE_INTERFACE void pglReleaseSurfaceSamplingDistribution(PGLSurfaceSamplingDistribution d) {
  PGL_TRY
  delete D(d);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglReleaseVolumeSamplingDistribution(PGLVolumeSamplingDistribution d) {
  PGL_TRY
  delete D(d);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglSurfaceSamplingDistributionApplyCosineProduct(PGLSurfaceSamplingDistribution d,
                                                                             pgl_vec3f normal) {
  PGL_TRY
  if (D(d)->numDistributions == 0) return;  // VMMSurfaceSamplingDistribution.h:52-60
  if (dist_dqt(D(d))) return;                // not supported by quadtrees (DQTSurfaceSamplingDistribution.h:20-27)
  Context &c = Context::get();
  check(launch_ssd_cosine(D(d)->dState, normal.x, normal.y, normal.z, 2.18853f, cosine_lobe_normalization(), c.stream),
        "cosine product");
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE bool pglSurfaceSamplingDistributionSupportsApplyCosineProduct(PGLSurfaceSamplingDistribution d) {
  return d && !dist_dqt(D(d));
}
OPENPGL_CORE_INTERFACE pgl_vec3f pglSurfaceSamplingDistributionSample(PGLSurfaceSamplingDistribution d,
                                                                      pgl_point2f sample) {
  PGL_TRY
  return dist_sample(D(d), sample, nullptr);
  PGL_CATCH(pgl_vec3f{})
}
OPENPGL_CORE_INTERFACE float pglSurfaceSamplingDistributionPDF(PGLSurfaceSamplingDistribution d, pgl_vec3f direction) {
  PGL_TRY
  return dist_pdf(D(d), direction, false);
  PGL_CATCH(0.0f)
}
OPENPGL_CORE_INTERFACE float pglSurfaceSamplingDistributionSamplePDF(PGLSurfaceSamplingDistribution d,
                                                                     pgl_point2f sample, pgl_vec3f &direction) {
  PGL_TRY
  float pdf = 0.0f;
  direction = dist_sample(D(d), sample, &pdf);
  return pdf;
  PGL_CATCH(0.0f)
}
OPENPGL_CORE_INTERFACE float pglSurfaceSamplingDistributionIncomingRadiancePDF(PGLSurfaceSamplingDistribution d,
                                                                               pgl_vec3f direction) {
  PGL_TRY
  return dist_pdf(D(d), direction, true);
  PGL_CATCH(0.0f)
}
OPENPGL_CORE_INTERFACE uint32_t pglSurfaceSamplingDistributionGetId(PGLSurfaceSamplingDistribution d) {
  return D(d)->id;
}
OPENPGL_CORE_INTERFACE bool pglSurfaceSamplingDistributionValidate(PGLSurfaceSamplingDistribution d) {
  return D(d)->numDistributions > 0;
}
OPENPGL_CORE_INTERFACE void pglSurfaceSamplingDistributionClear(PGLSurfaceSamplingDistribution d) {
  D(d)->numDistributions = 0;
}
OPENPGL_CORE_INTERFACE PGLRegion pglSurfaceSamplingGetRegion(PGLSurfaceSamplingDistribution d) {
  return reinterpret_cast<PGLRegion>(const_cast<void *>(D(d)->regionTag));
}
OPENPGL_CORE_INTERFACE pgl_vec3f pglVolumeSamplingDistributionSample(PGLVolumeSamplingDistribution d,
                                                                     pgl_point2f sample) {
  PGL_TRY
  return dist_sample(D(d), sample, nullptr);
  PGL_CATCH(pgl_vec3f{})
}
OPENPGL_CORE_INTERFACE float pglVolumeSamplingDistributionPDF(PGLVolumeSamplingDistribution d, pgl_vec3f direction) {
  PGL_TRY
  return dist_pdf(D(d), direction, false);
  PGL_CATCH(0.0f)
}
OPENPGL_CORE_INTERFACE float pglVolumeSamplingDistributionSamplePDF(PGLVolumeSamplingDistribution d,
                                                                    pgl_point2f sample, pgl_vec3f &direction) {
  PGL_TRY
  float pdf = 0.0f;
  direction = dist_sample(D(d), sample, &pdf);
  return pdf;
  PGL_CATCH(0.0f)
}
OPENPGL_CORE_INTERFACE float pglVolumeSamplingDistributionIncomingRadiancePDF(PGLVolumeSamplingDistribution d,
                                                                              pgl_vec3f direction) {
  PGL_TRY
  return dist_pdf(D(d), direction, true);
  PGL_CATCH(0.0f)
}
OPENPGL_CORE_INTERFACE uint32_t pglVolumeSamplingDistributionGetId(PGLVolumeSamplingDistribution d) {
  return D(d)->id;
}
OPENPGL_CORE_INTERFACE bool pglVolumeSamplingDistributionValidate(PGLVolumeSamplingDistribution d) {
  return D(d)->numDistributions > 0;
}
OPENPGL_CORE_INTERFACE void pglVolumeSamplingDistributionClear(PGLVolumeSamplingDistribution d) {
  D(d)->numDistributions = 0;
}
// VMMVolumeSamplingDistribution::applySingleLobeHenyeyGreensteinProduct
// (VMMVolumeSamplingDistribution.h:54-80; api.cpp:742-747)
OPENPGL_CORE_INTERFACE void pglVolumeSamplingDistributionApplySingleLobeHenyeyGreensteinProduct(
    PGLVolumeSamplingDistribution d, pgl_vec3f dir, const float meanCosine) {
  PGL_TRY
  if (D(d)->numDistributions == 0) return;
  if (dist_dqt(D(d))) return;  // not supported by quadtrees
  Context &c = Context::get();
  check(launch_ssd_hg(D(d)->dState, dir.x, dir.y, dir.z, meanCosine, c.stream), "Henyey-Greenstein product");
  D(d)->numDistributions = kMaxProducts;
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE bool pglVolumeSamplingDistributionSupportsApplySingleLobeHenyeyGreensteinProduct(
    PGLVolumeSamplingDistribution d) {
  return d && !dist_dqt(D(d));
}
OPENPGL_CORE_INTERFACE PGLRegion pglVolumeSamplingGetRegion(PGLVolumeSamplingDistribution d) {
  return reinterpret_cast<PGLRegion>(const_cast<void *>(D(d)->regionTag));
}

// ------------------------------------------------------------------ sample storage (api.cpp:328-400)
OPENPGL_CORE_INTERFACE PGLSampleStorage pglNewSampleStorage() {
  PGL_TRY
  Context::get();
  return reinterpret_cast<PGLSampleStorage>(new Storage());
  PGL_CATCH(nullptr)
}
static const char kStorageHeader[] = "OPENPGL_0.6.0_SAMPLE_STORAGE";
OPENPGL_CORE_INTERFACE PGLSampleStorage pglNewSampleStorageFromFile(const char *fileName) {
  PGL_TRY
  if (!fileName) throw std::runtime_error("null string provided to pglNewSampleStorageFromFile");
  std::ifstream is(fileName, std::ios::binary);
  if (!is) throw std::runtime_error("error: couldn't open file");
  char hdr[sizeof(kStorageHeader)];
  is.read(hdr, sizeof(hdr));
  if (!is) throw std::runtime_error("error: invalid file header");
  Storage *s = new Storage();
  for (int side = 0; side < 2; ++side) {  // SampleDataStorage.h:176-216
    uint64_t n = 0;
    is.read(reinterpret_cast<char *>(&n), 8);
    std::vector<PGLSampleRecord> v(n);
    is.read(reinterpret_cast<char *>(v.data()), std::streamsize(n * sizeof(PGLSampleRecord)));
    s->add(v.data(), v.size());
  }
  s->flush();
  return reinterpret_cast<PGLSampleStorage>(s);
  PGL_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE void pglReleaseSampleStorage(PGLSampleStorage s) {
  PGL_TRY
  delete S(s);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE bool pglSampleStorageStoreToFile(PGLSampleStorage s, const char *fileName) {
  PGL_TRY
  if (!s || !fileName) throw std::runtime_error("null handle or file name");
  std::ofstream os(fileName, std::ios::binary);
  if (!os) throw std::runtime_error("error: couldn't open file!");
  os.write(kStorageHeader, sizeof(kStorageHeader));
  for (bool vol : {false, true}) {
    std::vector<PGLSampleRecord> v = S(s)->download(vol);
    uint64_t n = v.size();
    os.write(reinterpret_cast<const char *>(&n), 8);
    os.write(reinterpret_cast<const char *>(v.data()), std::streamsize(n * sizeof(PGLSampleRecord)));
  }
  return bool(os);
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE void pglSampleStorageAddSample(PGLSampleStorage s, PGLSampleData &sample) {
  PGL_TRY
  S(s)->add(reinterpret_cast<const PGLSampleRecord *>(&sample), 1);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglSampleStorageAddSamples(PGLSampleStorage s, const PGLSampleData *samples, size_t n) {
  PGL_TRY
  S(s)->add(reinterpret_cast<const PGLSampleRecord *>(samples), n);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglSampleStorageReserve(PGLSampleStorage s, const size_t ns, const size_t nv) {
  PGL_TRY
  S(s)->reserve(ns, nv);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglSampleStorageClear(PGLSampleStorage s) {
  PGL_TRY
  S(s)->clearSurface();
  S(s)->clearVolume();
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglSampleStorageClearSurface(PGLSampleStorage s) {
  PGL_TRY
  S(s)->clearSurface();
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE void pglSampleStorageClearVolume(PGLSampleStorage s) {
  PGL_TRY
  S(s)->clearVolume();
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE size_t pglSampleStorageGetSizeSurface(PGLSampleStorage s) {
  PGL_TRY
  return S(s)->sizeSurface();
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE size_t pglSampleStorageGetSizeVolume(PGLSampleStorage s) {
  PGL_TRY
  return S(s)->sizeVolume();
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE PGLSampleData pglSampleStorageGetSampleSurface(PGLSampleStorage s, const int idx) {
  PGLSampleData d{};
  PGL_TRY
  PGLSampleRecord r = S(s)->get(false, uint64_t(idx));
  std::memcpy(&d, &r, sizeof(d));
  return d;
  PGL_CATCH(d)
}
OPENPGL_CORE_INTERFACE PGLSampleData pglSampleStorageGetSampleVolume(PGLSampleStorage s, const int idx) {
  PGLSampleData d{};
  PGL_TRY
  PGLSampleRecord r = S(s)->get(true, uint64_t(idx));
  std::memcpy(&d, &r, sizeof(d));
  return d;
  PGL_CATCH(d)
}
OPENPGL_CORE_INTERFACE bool pglSampleStorageValidate(PGLSampleStorage s) {
  PGL_TRY
  return S(s)->validate();
  PGL_CATCH(false)
}
static bool sample_less(const PGLSampleRecord &a, const PGLSampleRecord &b) {  // SampleData.h:82-93
  if (a.weight != b.weight) return a.weight < b.weight;
  if (a.pdf != b.pdf) return a.pdf < b.pdf;
  if (a.distance != b.distance) return a.distance < b.distance;
  if (a.px != b.px) return a.px < b.px;
  if (a.py != b.py) return a.py < b.py;
  if (a.pz != b.pz) return a.pz < b.pz;
  if (a.dx != b.dx) return a.dx < b.dx;
  if (a.dy != b.dy) return a.dy < b.dy;
  return a.dz < b.dz;
}
OPENPGL_CORE_INTERFACE bool pglSampleStorageCompare(PGLSampleStorage a, PGLSampleStorage b) {
  // SampleDataStorage::operator== (SampleDataStorage.h:230-279): both sides
  // sorted, compared over the first storage's size (its size check is missing)
  PGL_TRY
  // SampleDataEqual (SampleData.h:69-80): member-wise float comparison
  // (+0 equals -0, a NaN equals nothing) and equal flags
  auto equal = [](const PGLSampleRecord &p, const PGLSampleRecord &q) {
    return p.px == q.px && p.py == q.py && p.pz == q.pz && p.dx == q.dx && p.dy == q.dy && p.dz == q.dz &&
           p.weight == q.weight && p.pdf == q.pdf && p.distance == q.distance && p.flags == q.flags;
  };
  bool same = true;
  for (bool vol : {false, true}) {
    std::vector<PGLSampleRecord> x = S(a)->download(vol), y = S(b)->download(vol);
    std::sort(x.begin(), x.end(), sample_less);
    std::sort(y.begin(), y.end(), sample_less);
    for (size_t i = 0; i < x.size() && i < y.size(); ++i)
      if (!equal(x[i], y[i])) same = false;
  }
  return same;
  PGL_CATCH(false)
}

// ------------------------------------------------------------------ statistics strings (api.cpp:788-846)
OPENPGL_CORE_INTERFACE void pglReleaseFieldStatistics(PGLFieldStatistics s) {
  delete reinterpret_cast<StatsImpl *>(s);
}
OPENPGL_CORE_INTERFACE PGLString pglFieldStatisticsToString(PGLFieldStatistics p) {
  const StatsImpl &s = *reinterpret_cast<StatsImpl *>(p);
  std::stringstream ss;
  ss << "FieldStatistics:\n  numCacheRegions = " << s.numRegions << "\n  sizePerCacheRegions = " << s.sizePerRegion
     << "\n  timeLastUpdate = " << s.timeUpdate << " ms\n  timeLastUpdateCopySamples = " << s.timeCopy
     << " ms\n  timeLastUpdateSpatialStructureUpdate = " << s.timeSpatial
     << " ms\n  timeLastUpdateDirectionalDistriubtionUpdate = " << s.timeDirectional
     << " ms\nKDTreeStatistics:\n  numberOfNodes = " << s.numNodes << "\n  maxDepth = " << s.maxDepth
     << "\nDirectionalDistributionStatistics:\n  minNumberOfComponents = " << s.minK
     << "\n  maxNumberOfComponents = " << s.maxK << "\n  averageNumberOfComponents = " << s.avgK
     << "\n  secondMomentNumberOfComponents = " << s.secondMomentK << "\n";
  return make_string(ss.str());
}
OPENPGL_CORE_INTERFACE PGLString pglFieldStatisticsHeaderCSVString(PGLFieldStatistics) {
  return make_string(
      "FieldStatistics: , numCacheRegions , sizePerCacheRegions(bs) , timeUpdate(ms) , timeCopySamples(ms) , "
      "timeSpatialStructureUpdate(ms) , timeDirectionalDistriubtionUpdate(ms) , KDTreeStatistics: , numberOfNodes , "
      "maxDepth , DirectionalDistributionStatistics: , minNumberOfComponents , maxNumberOfComponents , "
      "averageNumberOfComponents , secondMomentNumberOfComponents , ");
}
OPENPGL_CORE_INTERFACE PGLString pglFieldStatisticsToCSVString(PGLFieldStatistics p) {
  const StatsImpl &s = *reinterpret_cast<StatsImpl *>(p);
  std::stringstream ss;
  ss << "  , " << s.numRegions << " , " << s.sizePerRegion << " , " << s.timeUpdate << " , " << s.timeCopy << " , "
     << s.timeSpatial << " , " << s.timeDirectional << " ,   , " << s.numNodes << " , " << s.maxDepth << " ,   , "
     << s.minK << " , " << s.maxK << " , " << s.avgK << " , " << s.secondMomentK << " , ";
  return make_string(ss.str());
}
OPENPGL_CORE_INTERFACE void pglReleaseString(PGLString str) { delete[] str.m_str; }

// ------------------------------------------------------------------ appended entry points (openpgl_gb300.h)
static void launch_batch(PGLField field, bool volume, const PGLGuidedQuery *dQueries, size_t n,
                         PGLGuidedQueryResult *dResults, bool cosineProduct, const float *dMeanCosines,
                         cudaStream_t s) {
  const SubField &sf = volume ? F(field)->volume : F(field)->surface;
  QueryParams p{};
  p.f = sf.view();
  p.cosKappa = 2.18853f;
  p.cosNorm = cosine_lobe_normalization();
  p.cosine = cosineProduct ? 1 : 0;
  p.samplesPerQuery = 1;
  p.hgMeanCosine = dMeanCosines;
  check(launch_query(p, reinterpret_cast<const QueryIn *>(dQueries), reinterpret_cast<QueryOut *>(dResults),
                     uint32_t(n), s),
        "query");
}
OPENPGL_CORE_INTERFACE bool pglFieldSampleBatchDevice(PGLField field, bool volume, const PGLGuidedQuery *dQueries,
                                                      size_t n, PGLGuidedQueryResult *dResults, bool cosineProduct,
                                                      void *cudaStream) {
  PGL_TRY
  Context &c = Context::get();
  launch_batch(field, volume, dQueries, n, dResults, cosineProduct, nullptr,
               cudaStream ? static_cast<cudaStream_t>(cudaStream) : c.stream);
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldSampleVolumeBatchHGDevice(PGLField field, const PGLGuidedQuery *dQueries,
                                                              const float *dMeanCosines, size_t n,
                                                              PGLGuidedQueryResult *dResults, void *cudaStream) {
  PGL_TRY
  if (n > 0 && dMeanCosines == nullptr) throw std::runtime_error("Henyey-Greenstein batch without mean cosines");
  Context &c = Context::get();
  launch_batch(field, true, dQueries, n, dResults, false, dMeanCosines,
               cudaStream ? static_cast<cudaStream_t>(cudaStream) : c.stream);
  return true;
  PGL_CATCH(false)
}
// Queries and results in page-locked host memory are read and written in
// place by the query kernel over the host link; others are copied.
static bool sample_batch_host(PGLField field, bool volume, const PGLGuidedQuery *q, size_t n, PGLGuidedQueryResult *r,
                              bool cosine) {
  Context &c = Context::get();
  static thread_local DevArray<QueryIn> dq;
  static thread_local DevArray<QueryOut> dr;
  const void *qin = device_address(q);
  void *rout = device_address(r);
  if (!qin) {
    dq.reserve(n);
    check(cudaMemcpyAsync(dq.p, q, n * sizeof(QueryIn), cudaMemcpyHostToDevice, c.stream), "H2D queries");
    qin = dq.p;
  }
  if (!rout) {
    dr.reserve(n);
    rout = dr.p;
  }
  if (!pglFieldSampleBatchDevice(field, volume, static_cast<const PGLGuidedQuery *>(qin), n,
                                 static_cast<PGLGuidedQueryResult *>(rout), cosine, c.stream))
    return false;
  if (rout == dr.p) check(cudaMemcpyAsync(r, dr.p, n * sizeof(QueryOut), cudaMemcpyDeviceToHost, c.stream), "D2H results");
  check(cudaStreamSynchronize(c.stream), "queries");
  return true;
}
OPENPGL_CORE_INTERFACE bool pglFieldSampleSurfaceBatch(PGLField field, const PGLGuidedQuery *queries, size_t n,
                                                       PGLGuidedQueryResult *results, bool cosineProduct) {
  PGL_TRY
  return sample_batch_host(field, false, queries, n, results, cosineProduct);
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldSampleVolumeBatch(PGLField field, const PGLGuidedQuery *queries, size_t n,
                                                      PGLGuidedQueryResult *results) {
  PGL_TRY
  return sample_batch_host(field, true, queries, n, results, false);
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldSampleVolumeBatchHG(PGLField field, const PGLGuidedQuery *queries,
                                                        const float *meanCosines, size_t n,
                                                        PGLGuidedQueryResult *results) {
  PGL_TRY
  if (n > 0 && meanCosines == nullptr) throw std::runtime_error("Henyey-Greenstein batch without mean cosines");
  Context &c = Context::get();
  static thread_local DevArray<QueryIn> dq;
  static thread_local DevArray<QueryOut> dr;
  static thread_local DevArray<float> dg;
  dq.reserve(n);
  dr.reserve(n);
  dg.reserve(n);
  check(cudaMemcpyAsync(dq.p, queries, n * sizeof(QueryIn), cudaMemcpyHostToDevice, c.stream), "H2D queries");
  check(cudaMemcpyAsync(dg.p, meanCosines, n * sizeof(float), cudaMemcpyHostToDevice, c.stream), "H2D mean cosines");
  launch_batch(field, true, reinterpret_cast<const PGLGuidedQuery *>(dq.p), n,
               reinterpret_cast<PGLGuidedQueryResult *>(dr.p), false, dg.p, c.stream);
  check(cudaMemcpyAsync(results, dr.p, n * sizeof(QueryOut), cudaMemcpyDeviceToHost, c.stream), "D2H results");
  check(cudaStreamSynchronize(c.stream), "queries");
  return true;
  PGL_CATCH(false)
}
static void launch_vertices(PGLField field, const PGLGuidedVertex *dv, size_t n, PGLGuidedVertexResult *dr,
                            cudaStream_t s) {
  if (!field) throw std::runtime_error("null field");
  if (n > 0 && (!dv || !dr)) throw std::runtime_error("null buffer");
  if (n > 0xFFFFFFFFull) throw std::runtime_error("at most 2^32 - 1 vertices per call");
  QueryParams p{};
  p.f = F(field)->surface.view();
  p.cosKappa = 2.18853f;
  p.cosNorm = cosine_lobe_normalization();
  p.cosine = 1;
  p.samplesPerQuery = kVertexSamples;
  check(launch_query_s4(p, reinterpret_cast<const QueryInS4 *>(dv), reinterpret_cast<QueryOutS4 *>(dr), uint32_t(n),
                        s),
        "vertex queries");
}
OPENPGL_CORE_INTERFACE bool pglFieldSampleSurfaceVerticesDevice(PGLField field, const PGLGuidedVertex *dVertices,
                                                                size_t n, PGLGuidedVertexResult *dResults,
                                                                void *cudaStream) {
  PGL_TRY
  Context &c = Context::get();
  launch_vertices(field, dVertices, n, dResults, cudaStream ? static_cast<cudaStream_t>(cudaStream) : c.stream);
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldSampleSurfaceVertices(PGLField field, const PGLGuidedVertex *vertices, size_t n,
                                                          PGLGuidedVertexResult *results) {
  PGL_TRY
  Context &c = Context::get();
  if (n == 0) return true;
  static thread_local DevArray<QueryInS4> dv;
  static thread_local DevArray<QueryOutS4> dr;
  // page-locked host buffers are read and written in place (as for queries)
  const void *vin = device_address(vertices);
  void *rout = device_address(results);
  if (!vin) {
    dv.reserve(n);
    check(cudaMemcpyAsync(dv.p, vertices, n * sizeof(QueryInS4), cudaMemcpyHostToDevice, c.stream), "H2D vertices");
    vin = dv.p;
  }
  if (!rout) {
    dr.reserve(n);
    rout = dr.p;
  }
  launch_vertices(field, static_cast<const PGLGuidedVertex *>(vin), n, static_cast<PGLGuidedVertexResult *>(rout),
                  c.stream);
  if (rout == dr.p)
    check(cudaMemcpyAsync(results, dr.p, n * sizeof(QueryOutS4), cudaMemcpyDeviceToHost, c.stream), "D2H results");
  check(cudaStreamSynchronize(c.stream), "vertex queries");
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE void pglSampleStorageAddSamplesDevice(PGLSampleStorage s, const PGLSampleData *d, size_t n) {
  PGL_TRY
  S(s)->ingestDevice(reinterpret_cast<const PGLSampleRecord *>(d), n);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE size_t pglFieldStoreToBuffer(PGLField field, char *buffer, size_t capacity) {
  PGL_TRY
  std::string b = F(field)->serialize();
  if (buffer && capacity >= b.size()) std::memcpy(buffer, b.data(), b.size());
  return b.size();
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE bool pglFieldGetLastUpdateTimings(PGLField field, int volume, float out4[4]) {
  PGL_TRY
  const UpdateTimings &t = volume ? F(field)->volume.timings : F(field)->surface.timings;
  out4[0] = t.total;
  out4[1] = t.copy;
  out4[2] = t.spatial;
  out4[3] = t.directional;
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE size_t pglFieldGetLastUpdatePhases(PGLField field, int volume, double *out, size_t cap) {
  PGL_TRY
  const UpdateTimings &t = volume ? F(field)->volume.timings : F(field)->surface.timings;
  const double v[8] = {t.total, t.copy, t.spatial, t.directional, t.gather, t.emKernel, double(t.samples),
                       double(t.regions)};
  if (out && cap >= 8)
    for (int i = 0; i < 8; ++i) out[i] = v[i];
  return 8;
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE bool pglSplitSamplesDeviceNoAlloc(const PGLSampleData *dSamples, size_t numSamples,
                                                         PGLSampleData *dSurface, PGLSampleData *dVolume,
                                                         uint32_t *dCounts, void *cudaStream) {
  PGL_TRY
  if (numSamples > split_max_records())
    throw std::runtime_error("pglSplitSamplesDeviceNoAlloc: at most 67108864 samples per call, got " +
                             std::to_string(numSamples));
  if (!dCounts || (numSamples > 0 && (!dSamples || !dSurface || !dVolume)))
    throw std::runtime_error("pglSplitSamplesDeviceNoAlloc: null device pointer");
  check(split_samples_noalloc(reinterpret_cast<const PGLSampleRecord *>(dSamples), numSamples,
                              reinterpret_cast<PGLSampleRecord *>(dSurface), reinterpret_cast<PGLSampleRecord *>(dVolume),
                              dCounts, static_cast<cudaStream_t>(cudaStream)),
        "pglSplitSamplesDeviceNoAlloc");
  return true;
  PGL_CATCH(false)
}
// ---- serving a field (appended; no reference counterpart)
OPENPGL_CORE_INTERFACE PGLGuidingServer pglNewGuidingServer(PGLField field, size_t hbmBudgetBytes) {
  PGL_TRY
  if (!field) throw std::runtime_error("null field provided to pglNewGuidingServer");
  return reinterpret_cast<PGLGuidingServer>(new pgl::GuidingServer(F(field), hbmBudgetBytes));
  PGL_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE PGLGuidingServer pglNewGuidingServerEx(PGLField field, size_t hbmBudgetBytes,
                                                              int reservedSMs) {
  PGL_TRY
  if (!field) throw std::runtime_error("null field provided to pglNewGuidingServerEx");
  if (reservedSMs < 0) throw std::runtime_error("negative SM reservation");
  return reinterpret_cast<PGLGuidingServer>(new pgl::GuidingServer(F(field), hbmBudgetBytes, reservedSMs));
  PGL_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE void pglReleaseGuidingServer(PGLGuidingServer server) {
  PGL_TRY
  delete reinterpret_cast<pgl::GuidingServer *>(server);
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE uint64_t pglGuidingServerSubmit(PGLGuidingServer server, const PGLGuidedQuery *queries,
                                                       size_t n, PGLGuidedQueryResult *results, bool volume,
                                                       bool cosineProduct) {
  PGL_TRY
  if (!server || (n > 0 && (!queries || !results))) throw std::runtime_error("null pointer");
  return reinterpret_cast<pgl::GuidingServer *>(server)->submit(reinterpret_cast<const QueryIn *>(queries),
                                                           reinterpret_cast<QueryOut *>(results), n, volume,
                                                           cosineProduct);
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE bool pglGuidingServerWait(PGLGuidingServer server, uint64_t ticket, double *latencyMs,
                                                 uint64_t *fieldVersion) {
  PGL_TRY
  if (!server) throw std::runtime_error("null server");
  reinterpret_cast<pgl::GuidingServer *>(server)->wait(ticket, latencyMs, fieldVersion);
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglGuidingServerAddSamples(PGLGuidingServer server, const PGLSampleData *samples,
                                                       size_t n) {
  PGL_TRY
  if (!server || (n > 0 && !samples)) throw std::runtime_error("null pointer");
  reinterpret_cast<pgl::GuidingServer *>(server)->addSamples(reinterpret_cast<const PGLSampleRecord *>(samples), n);
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglGuidingServerAddSamplesDevice(PGLGuidingServer server, const PGLSampleData *dSamples,
                                                             size_t n) {
  PGL_TRY
  if (!server || (n > 0 && !dSamples)) throw std::runtime_error("null pointer");
  reinterpret_cast<pgl::GuidingServer *>(server)->addSamplesDevice(
      reinterpret_cast<const PGLSampleRecord *>(dSamples), n);
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE uint64_t pglGuidingServerUpdate(PGLGuidingServer server) {
  PGL_TRY
  if (!server) throw std::runtime_error("null server");
  return reinterpret_cast<pgl::GuidingServer *>(server)->update();
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE bool pglGuidingServerWaitUpdate(PGLGuidingServer server, uint64_t ticket) {
  PGL_TRY
  if (!server) throw std::runtime_error("null server");
  reinterpret_cast<pgl::GuidingServer *>(server)->waitUpdate(ticket);
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglGuidingServerStats(PGLGuidingServer server, double out8[8]) {
  PGL_TRY
  if (!server || !out8) throw std::runtime_error("null pointer");
  double all[11];
  reinterpret_cast<pgl::GuidingServer *>(server)->stats(all);
  std::memcpy(out8, all, 8 * sizeof(double));
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE size_t pglGuidingServerStatsEx(PGLGuidingServer server, double *out, size_t count) {
  PGL_TRY
  if (!server) throw std::runtime_error("null pointer");
  double all[11];
  reinterpret_cast<pgl::GuidingServer *>(server)->stats(all);
  if (out) std::memcpy(out, all, std::min<size_t>(count, 11) * sizeof(double));
  return 11;
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE bool pglGuidingServerResetStats(PGLGuidingServer server) {
  PGL_TRY
  if (!server) throw std::runtime_error("null pointer");
  reinterpret_cast<pgl::GuidingServer *>(server)->resetStats();
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE uint64_t pglGuidingServerSubmitVertices(PGLGuidingServer server,
                                                               const PGLGuidedVertex *vertices, size_t n,
                                                               PGLGuidedVertexResult *results) {
  PGL_TRY
  if (!server || (n > 0 && (!vertices || !results))) throw std::runtime_error("null pointer");
  return reinterpret_cast<pgl::GuidingServer *>(server)->submitVertices(
      reinterpret_cast<const QueryInS4 *>(vertices), reinterpret_cast<QueryOutS4 *>(results), n);
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE uint64_t pglGetKernelLaunchCount() { return kernel_launches(); }
OPENPGL_CORE_INTERFACE int pglDebugBoundedWaitRunsOut(uint64_t limitNs) {
  PGL_TRY
  if (limitNs > 10000000000ull) throw std::runtime_error("pglDebugBoundedWaitRunsOut: limit above 10 s");
  int code = 0;
  check(em_bounded_wait_probe(limitNs, &code, Context::get().stream), "bounded wait probe");
  return code;
  PGL_CATCH(-1)
}
OPENPGL_CORE_INTERFACE void *pglDeviceGetCudaStream(PGLDevice device) {
  PGL_TRY
  (void)device;
  return static_cast<void *>(Context::get().stream);
  PGL_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE size_t pglFieldGetLastUpdateProfile(PGLField field, int volume, uint64_t *out, size_t cap) {
  PGL_TRY
  const SubField &sf = volume ? F(field)->volume : F(field)->surface;
  size_t n = sf.lastProfiles.size();
  if (out && cap >= 23 * n)
    for (size_t i = 0; i < n; ++i) {
      const LeafProfile &p = sf.lastProfiles[i];
      uint64_t *o = out + 23 * i;
      o[0] = sf.lastReportRegion[i];
      o[1] = p.count;
      o[2] = p.estepPasses;
      o[3] = p.distPasses;
      o[4] = p.splitPasses;
      o[5] = p.cycEstep;
      o[6] = p.cycDist;
      o[7] = p.cycSplit;
      o[8] = p.cycMerge;
      o[9] = p.cycMstep;
      o[10] = p.cycTotal;
      o[11] = p.cycProdE;
      o[12] = p.cycConsE;
      o[13] = p.cycProdS;
      o[14] = p.cycConsS;
      o[15] = p.chunks;
      o[16] = p.chunksOwn;
      o[17] = p.cycWaitE;
      o[18] = p.estepLobes;
      o[19] = p.distLobes;
      o[20] = p.splitLobes;
      o[21] = p.tBegin;
      o[22] = p.tEnd;
    }
  return n;
  PGL_CATCH(0)
}
// EM schedule parameters of a field: helper blocks per region, chunk size
// divisor, pipeline stages, queue order by measured cost (int[4]).
OPENPGL_CORE_INTERFACE bool pglFieldSetEmTuning(PGLField field, const int *tuning) {
  PGL_TRY
  if (!field || !tuning) throw std::runtime_error("null argument");
  EmTuning t{tuning[0], tuning[1], tuning[2], tuning[3]};
  t.plainLaunches = F(field)->tuning.plainLaunches;
  t.reservedSMs = F(field)->tuning.reservedSMs;
  if (!em_tuning_valid(t)) throw std::runtime_error("EM tuning out of range");
  F(field)->tuning = t;
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldSetPlainUpdate(PGLField field, bool plain) {
  PGL_TRY
  if (!field) throw std::runtime_error("null field");
  F(field)->tuning.plainLaunches = plain ? 1 : 0;
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglFieldGetEmTuning(PGLField field, int *tuning) {
  PGL_TRY
  if (!field || !tuning) throw std::runtime_error("null argument");
  const EmTuning &t = F(field)->tuning;
  tuning[0] = t.maxHelpers;
  tuning[1] = t.chunkDiv;
  tuning[2] = t.stageCap;
  tuning[3] = t.orderByCost;
  return true;
  PGL_CATCH(false)
}
OPENPGL_CORE_INTERFACE void pglFieldAutotuneNextUpdate(PGLField field) {
  PGL_TRY
  if (!field) throw std::runtime_error("null field");
  F(field)->autotuneNext = true;
  PGL_CATCH_VOID
}
OPENPGL_CORE_INTERFACE size_t pglFieldGetEmTuningTrials(PGLField field, int *tunings, float *ms, size_t cap) {
  PGL_TRY
  const auto &trials = F(field)->lastTuneTrials;
  if (tunings && ms && cap >= trials.size())
    for (size_t i = 0; i < trials.size(); ++i) {
      const EmTuning &t = trials[i].t;
      tunings[4 * i] = t.maxHelpers;
      tunings[4 * i + 1] = t.chunkDiv;
      tunings[4 * i + 2] = t.stageCap;
      tunings[4 * i + 3] = t.orderByCost;
      ms[i] = trials[i].ms;
    }
  return trials.size();
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE size_t pglFieldGetLastUpdateReports(PGLField field, int volume, uint32_t *out, size_t cap) {
  PGL_TRY
  const SubField &sf = volume ? F(field)->volume : F(field)->surface;
  size_t n = sf.lastReports.size();
  if (out && cap >= 5 * n)
    for (size_t i = 0; i < n; ++i) {
      out[5 * i + 0] = sf.lastReportRegion[i];
      out[5 * i + 1] = sf.lastReports[i].emIterations;
      out[5 * i + 2] = sf.lastReports[i].splits;
      out[5 * i + 3] = sf.lastReports[i].merges;
      out[5 * i + 4] = sf.lastReports[i].K;
    }
  return n;
  PGL_CATCH(0)
}
OPENPGL_CORE_INTERFACE const char *pglGetLastError() { return g_lastError.c_str(); }

}  // extern "C"
