// Path segment storage (api.cpp:445-567, PathSegmentDataStorage.h): the
// reference's per-path host object, and the appended device batch that turns
// many paths' segments into samples without a host round trip.  The
// arithmetic is path_samples.cuh, shared with the device kernel.
#include <cstddef>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/openpgl_gb300.h"
#include "field.h"
#include "launch.h"
#include "path_samples.cuh"

namespace pgl {

static_assert(sizeof(PGLPathSegmentData) == sizeof(PathSegmentRecord), "path segment layout");
static_assert(offsetof(PGLPathSegmentData, volumeScatter) == offsetof(PathSegmentRecord, volumeScatter) &&
                  offsetof(PGLPathSegmentData, pdfDirectionIn) == offsetof(PathSegmentRecord, pdfDirectionIn) &&
                  offsetof(PGLPathSegmentData, isDelta) == offsetof(PathSegmentRecord, isDelta) &&
                  offsetof(PGLPathSegmentData, scatteringWeight) == offsetof(PathSegmentRecord, sw) &&
                  offsetof(PGLPathSegmentData, miWeight) == offsetof(PathSegmentRecord, miWeight) &&
                  offsetof(PGLPathSegmentData, russianRouletteProbability) == offsetof(PathSegmentRecord, rr) &&
                  offsetof(PGLPathSegmentData, roughness) == offsetof(PathSegmentRecord, roughness) &&
                  offsetof(PGLPathSegmentData, regionPtr) == offsetof(PathSegmentRecord, regionPtr),
              "path segment fields");
static_assert(sizeof(PGLSampleData) == sizeof(PGLSampleRecord), "sample layout");

// PathSegmentDataStorage with OPENPGL_PATHSEGMENT_STORAGE_USE_ARRAY: fixed
// arrays of the reserved size.  Where the reference writes one element past
// them (its bounds test is `index + 1 <= size`), this one stops at the size.
struct PathStore {
  float maxDistance = 1e6f;
  std::vector<PGLPathSegmentData> seg;
  std::vector<PGLSampleData> smp;
  int segIdx = -1, smpIdx = -1;
  void reserve(size_t size) {
    if (smp.size() == size && seg.size() == size) return;
    seg.assign(size, PGLPathSegmentData());
    smp.assign(size, PGLSampleData());
    segIdx = -1;
    smpIdx = -1;
  }
  void clear() {
    segIdx = -1;
    smpIdx = -1;
  }
  PGLPathSegmentData *next() {
    if (size_t(segIdx + 1) >= seg.size()) return nullptr;
    ++segIdx;
    seg[segIdx] = PGLPathSegmentData();
    return &seg[segIdx];
  }
  void addSegment(const PGLPathSegmentData &s) {
    if (size_t(segIdx + 1) >= seg.size()) return;
    seg[++segIdx] = s;
  }
  void addSample(const PGLSampleData &s) {
    if (size_t(smpIdx + 1) >= smp.size()) return;
    smp[++smpIdx] = s;
  }
  size_t prepare(bool useNEEMiWeights, bool guideDirectLight, bool rrAffectsDirectContribution) {
    const PathFlags fl{useNEEMiWeights, guideDirectLight, rrAffectsDirectContribution};
    const uint32_t room = uint32_t(smp.size() - size_t(smpIdx + 1));
    const uint32_t made = path_prepare_samples(reinterpret_cast<const PathSegmentRecord *>(seg.data()), segIdx + 1,
                                               maxDistance, fl,
                                               reinterpret_cast<PGLSampleRecord *>(smp.data() + (smpIdx + 1)), room);
    smpIdx += int(made < room ? made : room);
    return size_t(smpIdx + 1);
  }
};

PathStore *PS(PGLPathSegmentStorage s) {
  if (!s) throw std::runtime_error("null path segment storage");
  return reinterpret_cast<PathStore *>(s);
}

void api_error(const char *fn, const std::exception &e);  // api.cpp: the C API's error convention
void api_clear_error();

}  // namespace pgl

using namespace pgl;

#define PGL_PS_TRY \
  try {            \
    api_clear_error();
#define PGL_PS_CATCH(ret)                                                           \
  }                                                                                 \
  catch (const std::bad_alloc &) {                                                  \
    api_error(__func__, std::runtime_error("unable to allocate memory"));           \
    return ret;                                                                     \
  }                                                                                 \
  catch (const std::exception &e) {                                                 \
    api_error(__func__, e);                                                         \
    return ret;                                                                     \
  }                                                                                 \
  catch (...) {                                                                     \
    api_error(__func__, std::runtime_error("an unrecognized exception was caught")); \
    return ret;                                                                     \
  }

extern "C" {

// api.cpp:448-460
OPENPGL_CORE_INTERFACE PGLPathSegmentStorage pglNewPathSegmentStorage() {
  PGL_PS_TRY
  return reinterpret_cast<PGLPathSegmentStorage>(new PathStore());
  PGL_PS_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE void pglReleasePathSegmentStorage(PGLPathSegmentStorage s) {
  delete reinterpret_cast<PathStore *>(s);
}
// api.cpp:462-496
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageReserve(PGLPathSegmentStorage s, size_t size) {
  PGL_PS_TRY
  PS(s)->reserve(size);
  PGL_PS_CATCH()
}
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageClear(PGLPathSegmentStorage s) {
  PGL_PS_TRY
  PS(s)->clear();
  PGL_PS_CATCH()
}
OPENPGL_CORE_INTERFACE void pglPathSegmentSetMaxDistance(PGLPathSegmentStorage s, float maxDistance) {
  PGL_PS_TRY
  PS(s)->maxDistance = maxDistance;
  PGL_PS_CATCH()
}
OPENPGL_CORE_INTERFACE float pglPathSegmentGetMaxDistance(PGLPathSegmentStorage s) {
  PGL_PS_TRY
  return PS(s)->maxDistance;
  PGL_PS_CATCH(0.0f)
}
OPENPGL_CORE_INTERFACE int pglPathSegmentGetNumSegments(PGLPathSegmentStorage s) {
  PGL_PS_TRY
  return PS(s)->segIdx + 1;
  PGL_PS_CATCH(0)
}
OPENPGL_CORE_INTERFACE int pglPathSegmentGetNumSamples(PGLPathSegmentStorage s) {
  PGL_PS_TRY
  return PS(s)->smpIdx + 1;
  PGL_PS_CATCH(0)
}
// api.cpp:498-508
OPENPGL_CORE_INTERFACE size_t pglPathSegmentStoragePrepareSamples(PGLPathSegmentStorage s, const bool useNEEMiWeights,
                                                                  const bool guideDirectLight,
                                                                  const bool rrAffectsDirectContribution) {
  PGL_PS_TRY
  return PS(s)->prepare(useNEEMiWeights, guideDirectLight, rrAffectsDirectContribution);
  PGL_PS_CATCH(0)
}
OPENPGL_CORE_INTERFACE pgl_vec3f pglPathSegmentStorageCalculatePixelEstimate(PGLPathSegmentStorage s,
                                                                            const bool rrAffectsDirectContribution) {
  PGL_PS_TRY
  PathStore *p = PS(s);
  float c[3];
  path_pixel_estimate(reinterpret_cast<const PathSegmentRecord *>(p->seg.data()), p->segIdx + 1,
                      rrAffectsDirectContribution, c);
  return pgl_vec3f{c[0], c[1], c[2]};
  PGL_PS_CATCH(pgl_vec3f{})
}
// api.cpp:510-567
OPENPGL_CORE_INTERFACE const PGLSampleData *pglPathSegmentStorageGetSamples(PGLPathSegmentStorage s, size_t &n) {
  n = 0;
  PGL_PS_TRY
  PathStore *p = PS(s);
  n = size_t(p->smpIdx + 1);
  return p->smp.data();
  PGL_PS_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageAddSample(PGLPathSegmentStorage s, PGLSampleData sample) {
  PGL_PS_TRY
  PS(s)->addSample(sample);
  PGL_PS_CATCH()
}
OPENPGL_CORE_INTERFACE PGLPathSegmentData *pglPathSegmentStorageNextSegment(PGLPathSegmentStorage s) {
  PGL_PS_TRY
  return PS(s)->next();
  PGL_PS_CATCH(nullptr)
}
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageAddSegment(PGLPathSegmentStorage s, PGLPathSegmentData segment) {
  PGL_PS_TRY
  PS(s)->addSegment(segment);
  PGL_PS_CATCH()
}
OPENPGL_CORE_INTERFACE bool pglPathSegmentStorageValidateSamples(PGLPathSegmentStorage s) {
  PGL_PS_TRY
  PathStore *p = PS(s);
  bool valid = true;
  for (int i = 0; i <= p->smpIdx; ++i)
    valid = valid && sample_record_valid(*reinterpret_cast<const PGLSampleRecord *>(&p->smp[i]));
  return valid;
  PGL_PS_CATCH(false)
}
OPENPGL_CORE_INTERFACE bool pglPathSegmentStorageValidateSegments(PGLPathSegmentStorage s) {
  PGL_PS_TRY
  PathStore *p = PS(s);
  bool valid = true;
  for (int i = 0; i <= p->segIdx; ++i)
    valid = valid && path_segment_valid(*reinterpret_cast<const PathSegmentRecord *>(&p->seg[i]));
  return valid;
  PGL_PS_CATCH(false)
}
// propagateSamples (PathSegmentDataStorage.h:503-513): prepare, hand the
// samples to the sample storage, clear
OPENPGL_CORE_INTERFACE void pglPathSegmentStoragePropagateSamples(PGLPathSegmentStorage s,
                                                                  PGLSampleStorage sampleStorage,
                                                                  bool guideDirectLight, bool useNEEMiWeights,
                                                                  bool rrAffectsDirectContribution) {
  PGL_PS_TRY
  PathStore *p = PS(s);
  p->prepare(useNEEMiWeights, guideDirectLight, rrAffectsDirectContribution);
  if (!sampleStorage) throw std::runtime_error("null sample storage");
  reinterpret_cast<Storage *>(sampleStorage)
      ->add(reinterpret_cast<const PGLSampleRecord *>(p->smp.data()), size_t(p->smpIdx + 1));
  p->clear();
  PGL_PS_CATCH()
}

// ---- appended: many paths at once on the device
OPENPGL_CORE_INTERFACE bool pglPathSegmentsPrepareSamplesDevice(const PGLPathSegmentData *dSegments,
                                                                const uint32_t *dPathBegin, size_t numPaths,
                                                                float maxDistance, bool useNEEMiWeights,
                                                                bool guideDirectLight,
                                                                bool rrAffectsDirectContribution,
                                                                PGLSampleData *dSamples, uint32_t *dSampleBegin,
                                                                void *cudaStream) {
  PGL_PS_TRY
  if (numPaths >= 0xFFFFFFFFull) throw std::runtime_error("too many paths for one call");
  Context &c = Context::get();
  cudaStream_t st = cudaStream ? static_cast<cudaStream_t>(cudaStream) : c.stream;
  static thread_local Scratch scratch;
  check(launch_path_samples(reinterpret_cast<const PathSegmentRecord *>(dSegments), dPathBegin, uint32_t(numPaths),
                            maxDistance, PathFlags{useNEEMiWeights, guideDirectLight, rrAffectsDirectContribution},
                            reinterpret_cast<PGLSampleRecord *>(dSamples), dSampleBegin, scratch, st),
        "path samples");
  return true;
  PGL_PS_CATCH(false)
}
OPENPGL_CORE_INTERFACE size_t pglPathSegmentsPropagateSamplesDevice(const PGLPathSegmentData *dSegments,
                                                                    const uint32_t *dPathBegin, size_t numPaths,
                                                                    float maxDistance, PGLSampleStorage sampleStorage,
                                                                    bool guideDirectLight, bool useNEEMiWeights,
                                                                    bool rrAffectsDirectContribution) {
  PGL_PS_TRY
  if (!sampleStorage) throw std::runtime_error("null sample storage");
  Context &c = Context::get();
  uint32_t numSegments = 0;
  if (numPaths > 0)
    check(cudaMemcpyAsync(&numSegments, dPathBegin + numPaths, 4, cudaMemcpyDeviceToHost, c.stream), "path count");
  static thread_local DevArray<PGLSampleRecord> out;
  static thread_local DevArray<uint32_t> offsets;
  check(cudaStreamSynchronize(c.stream), "path count");
  out.reserve(numSegments > 0 ? numSegments : 1);
  offsets.reserve(numPaths + 1);
  if (!pglPathSegmentsPrepareSamplesDevice(dSegments, dPathBegin, numPaths, maxDistance, useNEEMiWeights,
                                           guideDirectLight, rrAffectsDirectContribution,
                                           reinterpret_cast<PGLSampleData *>(out.p), offsets.p, c.stream))
    return 0;
  uint32_t total = 0;
  check(cudaMemcpyAsync(&total, offsets.p + numPaths, 4, cudaMemcpyDeviceToHost, c.stream), "sample count");
  check(cudaStreamSynchronize(c.stream), "path samples");
  reinterpret_cast<Storage *>(sampleStorage)->ingestDevice(out.p, total);
  return total;
  PGL_PS_CATCH(0)
}

}  // extern "C"
