// Host-callable launchers of the library's CUDA kernels (defined next to the
// kernels in em_kernel.cu, spatial_kernels.cu, query_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "pgl_internal.h"

namespace pgl {

// Growable device scratch buffer.
struct Scratch {
  void *ptr = nullptr;
  size_t bytes = 0;
};
cudaError_t scratch_reserve(Scratch &s, size_t bytes);
void scratch_free(Scratch &s);

struct SoAView {
  float4 *P;       // position xyz, distance
  float4 *D;       // direction xyz, weight
  float *pdf;
  uint32_t *flags;
  uint64_t base;   // append offset
};

// Number of this library's own kernels launched so far in the process (CUB's
// scan and sort kernels not included).
unsigned long long kernel_launches();
void count_launch();

// Stable split of a device batch into caller buffers with a fixed device
// scratch array (noalloc.cu); at most split_max_records() records per call.
size_t split_max_records();
cudaError_t split_samples_noalloc(const PGLSampleRecord *in, size_t n, PGLSampleRecord *surf, PGLSampleRecord *vol,
                                  uint32_t *counts, cudaStream_t s);

cudaError_t em_upload_tables(const LibmTables &libm);
// The directional quadtree field type (dqt_kernels.cu): one sub-field's
// quadtrees (a head per region, `stride` node slots per region), its
// sorted samples and its factory arguments.
struct DqtSide {
  DqtHead *heads;
  DqtStatsNode *stats;
  DqtNode *nodes;
  uint32_t stride;
  const float4 *dirw;
  const float *pdf;
  DqtArgs args;
  float decay;  // on a spatial split
};
struct DqtSides {
  DqtSide side[2];
};
// Fit or update of every task's region (persistent blocks on a queue; per
// block `scratchStride` rectangles, build nodes and leaf indices of scratch);
// *err becomes non-zero when a tree outgrows its node slots.
cudaError_t launch_dqt_update(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, const DqtSides &sides,
                              Box2 *rects, DqtStatsNode *builds, uint32_t *leaves, uint32_t scratchStride, int blocks,
                              int *err, cudaStream_t s);
cudaError_t launch_dqt_copy(DqtHead *heads, DqtStatsNode *stats, DqtNode *nodes, uint32_t stride, const uint32_t *dst,
                            const uint32_t *src, uint32_t n, cudaStream_t s);
cudaError_t launch_dqt_init(DqtHead *heads, DqtStatsNode *stats, DqtNode *nodes, uint32_t stride, uint32_t first,
                            uint32_t n, cudaStream_t s);
// Path-vertex queries: Init + cosine product, then kVertexSamples SamplePDF calls.
cudaError_t launch_query_s4(const QueryParams &p, const QueryInS4 *in, QueryOutS4 *out, uint32_t n,
                            cudaStream_t s);
// Launches one thread that waits, with the EM kernel's bounded wait, on a flag
// nothing sets; *errOut receives the error the wait recorded (2: it ran out).
cudaError_t em_bounded_wait_probe(unsigned long long limitNs, int *errOut, cudaStream_t s);
cudaError_t spatial_upload_tables(const LibmTables &libm);
cudaError_t query_upload_tables(const LibmTables &libm);

// ingest: AoS batch (device, or host memory the device addresses when
// `stage` is given: the records are then read once into stage) -> surface /
// volume SoA, stable per class.
cudaError_t ingest_samples(const PGLSampleRecord *in, uint32_t n, Scratch &scratch, SoAView surf, SoAView vol,
                           uint32_t *numVolume, cudaStream_t s, PGLSampleRecord *stage = nullptr);
cudaError_t export_samples(const float4 *P, const float4 *D, const float *pdf, const uint32_t *flags, uint64_t n,
                           PGLSampleRecord *out, cudaStream_t s);
// min/max over positions [0, n) as order-preserving integers (6 x u32, device)
cudaError_t scene_bounds(const float4 *P, uint64_t n, uint32_t *d6, cudaStream_t s);

cudaError_t init_posidx(const float4 *P, uint32_t n, float4 *posIdx, cudaStream_t s);
cudaError_t init_acc(IStatsAcc *acc, uint32_t count, cudaStream_t s);
cudaError_t kd_root_stats(const float4 *pos, uint32_t n, const KdJob &job, IStatsAcc *acc, cudaStream_t s);
// One pass down an existing tree (the root is not a leaf): every sample goes
// to the leaf it reaches; the samples come out in leaf-slot order
// (nodeSlot: node -> slot, slotNode: slot -> node), positions into posOut and
// leaf nodes into nodeOut.  keys/vals/keysB/valsB: n entries each.
cudaError_t kd_route(const float4 *pos, uint32_t n, const KDNode *nodes, const uint32_t *nodeSlot, uint32_t numSlots,
                     const uint32_t *slotNode, uint32_t *keys, uint32_t *vals, uint32_t *keysB, uint32_t *valsB,
                     float4 *posOut, uint32_t *nodeOut, Scratch &scratch, cudaStream_t s);
// The classification and child statistics of one level alone (no partition).
cudaError_t kd_classify(const float4 *pos, const uint32_t *jobOf, uint32_t n, const KdJob *jobs, uint32_t *isLeft,
                        IStatsAcc *acc, cudaStream_t s);
// jobOf[i] = nodeToJob[node[i]] (~0 for finished samples); clears acc[0, accCount)
cudaError_t kd_job_of(const uint32_t *node, uint32_t n, const uint32_t *nodeToJob, uint32_t *jobOf, IStatsAcc *acc,
                      uint32_t accCount, cudaStream_t s);
cudaError_t kd_level(const float4 *pos, const uint32_t *jobOf, uint32_t n, const KdJob *jobs, uint32_t *isLeft,
                     uint32_t *scanLeft, IStatsAcc *acc, float4 *posOut, uint32_t *nodeOut, Scratch &scratch,
                     cudaStream_t s);
// Gathers samples into leaf order and applies the deterministic per-leaf
// order (SampleDataLess) when `sorted`; leafBegin/leafCount are device arrays.
cudaError_t gather_and_order(const float4 *posIdx, uint32_t n, const float4 *P, const float4 *D, const float *pdf,
                             const uint32_t *leafBegin, const uint32_t *leafCount, uint32_t numLeaves, bool sorted,
                             float4 *tmpP, float4 *tmpD, float *tmpPdf, uint32_t *keys, uint32_t *vals,
                             unsigned long long *keys64, float4 *oP, float4 *oD, float *oPdf, Scratch &scratch,
                             cudaStream_t s);
cudaError_t copy_regions(RegionDir *regions, const uint32_t *dst, const uint32_t *src, uint32_t n, cudaStream_t s);
cudaError_t build_knn(const float4 *means, uint32_t R, Neighbours *out, cudaStream_t s);

size_t em_shared_bytes();
// One sub-field (surface or volume) of an EM launch: its regions, its
// samples in leaf order (position and distance, direction and weight, pdf,
// reprojected distance), the uniform directions of first fits and its
// configuration.  Tasks flagged kTaskVolume belong to side[1].
struct EmSide {
  RegionDir *regions;
  float4 *pd;
  float4 *dirw;
  const float *pdf;
  float *dist;
  const float *uniformDirs;
  FieldConfig cfg;
};
struct EmSides {
  EmSide side[2];
};
// Schedule parameters of an EM launch (they change the speed, never the
// result): helper blocks per region at a time, the E-step chunk size
// divisor (samples per chunk = the producers' sample slots / chunkDiv), the
// consumers' pipeline stages, and whether leaves go to the queue by the
// previous Update's measured cost (else by sample count), largest first.
struct EmTuning {
  int maxHelpers = 4;
  int chunkDiv = 1;
  int stageCap = 8;
  int orderByCost = 0;
  int plainLaunches = 0;  // 1: the plain form (one launch per sub-field, one block per region,
                          // no queue and no helper blocks), same results
  int reservedSMs = 0;    // SMs the batched launch leaves free (for queries on other streams
                          // while a served field trains), same results
};
bool em_tuning_valid(const EmTuning &t);
// Device memory through which the EM launch's blocks share E-step passes
// (boards, an error word, chunk rings): em_share_bytes(blocks) bytes; after
// the launch the int at em_share_error_offset(blocks) is non-zero if a wait
// of the launch ran out (its results are then not valid).
size_t em_share_bytes(int blocks);
size_t em_share_bytes_plain(int blocks);  // the plain form: boards and error word only
size_t em_share_error_offset(int blocks);
cudaError_t launch_em(const LeafTask *tasks, uint32_t numTasks, unsigned int *queue, const EmSides &sides,
                      LeafReport *reports, LeafProfile *profiles, void *share, int blocks, const EmTuning &tune,
                      cudaStream_t stream);

cudaError_t launch_query(const QueryParams &p, const QueryIn *in, QueryOut *out, uint32_t n, cudaStream_t s);
// Samples of numPaths paths (path p = seg[begin[p], begin[p + 1])): offsets
// (numPaths + 1 entries) gets each path's first sample slot and the total;
// out needs room for the total (at most begin[numPaths]).
struct PathSegmentRecord;
struct PathFlags;
cudaError_t launch_path_samples(const PathSegmentRecord *seg, const uint32_t *begin, uint32_t numPaths,
                                float maxDistance, PathFlags fl, PGLSampleRecord *out, uint32_t *offsets,
                                Scratch &scratch, cudaStream_t s);
cudaError_t launch_ssd_init(const FieldView &f, float px, float py, float pz, float s1d, SSDState *st, SSDResult *res,
                            cudaStream_t s);
cudaError_t launch_ssd_cosine(SSDState *st, float nx, float ny, float nz, float ck, float cn, cudaStream_t s);
// The single-lobe Henyey-Greenstein product of an initialised distribution
// (VMMVolumeSamplingDistribution.h:54-80).
cudaError_t launch_ssd_hg(SSDState *st, float dx, float dy, float dz, float meanCosine, cudaStream_t s);
cudaError_t launch_ssd_sample(const SSDState *st, float ux, float uy, int withPdf, SSDResult *res, cudaStream_t s);
cudaError_t launch_ssd_pdf(const SSDState *st, float dx, float dy, float dz, int li, SSDResult *res, cudaStream_t s);
// the same for a quadtree region (the region Init chose, read from the field)
cudaError_t launch_ssd_dqt_sample(const FieldView &f, const SSDState *st, float ux, float uy, SSDResult *res,
                                  cudaStream_t s);
cudaError_t launch_ssd_dqt_pdf(const FieldView &f, const SSDState *st, float dx, float dy, float dz, SSDResult *res,
                               cudaStream_t s);

}  // namespace pgl
