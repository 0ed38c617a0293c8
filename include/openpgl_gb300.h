// Entry points appended to the Open PGL C API by the GB300 library.  They have
// no counterpart in the reference; they expose the batched GPU forms of the
// guided query and of the sample ingest, and diagnostics.
#pragma once

#include "openpgl/openpgl.h"

#ifdef __cplusplus
extern "C" {
#endif

// One guided query: position, normal (for the cosine product), the 1D random
// number of the stochastic region choice, and the 2D random number of the
// direction sample (36 bytes).
typedef struct {
  pgl_point3f position;
  pgl_vec3f normal;
  float sample1D;
  pgl_point2f sample2D;
} PGLGuidedQuery;

// Result of Init + (cosine product) + SamplePDF + IncomingRadiancePDF (32 bytes).
typedef struct {
  uint32_t valid;     // Init succeeded
  uint32_t id;        // kd leaf (GetId)
  float sample1D;     // sample1D after the region choice rescaled it
  pgl_vec3f direction;
  float pdf;          // SamplePDF
  float pdfLi;        // IncomingRadiancePDF(direction)
} PGLGuidedQueryResult;

// A path vertex with four SamplePDF calls on one initialised distribution
// (76 bytes): position, normal (for the cosine product), outgoing direction
// and roughness (carried for the caller; the reference's surface
// distribution uses neither), the 1D random number of the region choice and
// one 2D random number per sample.
typedef struct {
  pgl_point3f position;
  pgl_vec3f normal;
  pgl_vec3f wo;
  float roughness;
  float sample1D;
  pgl_point2f sample2D[4];
} PGLGuidedVertex;

// Result of Init + cosine product + four SamplePDF calls (76 bytes): the
// sampled direction and its pdf per 2D random number.
typedef struct {
  uint32_t valid;     // Init succeeded
  uint32_t id;        // kd leaf (GetId)
  float sample1D;     // sample1D after the region choice rescaled it
  struct {
    pgl_vec3f direction;
    float pdf;
  } sample[4];
} PGLGuidedVertexResult;

// Guided queries on host buffers: runs one kernel and returns with the
// results written.  Page-locked buffers (cudaHostAlloc, cudaHostRegister) are
// read and written in place by the kernel; other host memory is copied in
// and out.  Same results as the per-object calls.
OPENPGL_CORE_INTERFACE bool pglFieldSampleSurfaceBatch(PGLField field, const PGLGuidedQuery *queries, size_t n,
                                                       PGLGuidedQueryResult *results, bool cosineProduct);
OPENPGL_CORE_INTERFACE bool pglFieldSampleVolumeBatch(PGLField field, const PGLGuidedQuery *queries, size_t n,
                                                      PGLGuidedQueryResult *results);
// Guided queries on device buffers, enqueued on `cudaStream` (a cudaStream_t,
// or null for the library's stream); does not synchronise.
OPENPGL_CORE_INTERFACE bool pglFieldSampleBatchDevice(PGLField field, bool volume, const PGLGuidedQuery *dQueries,
                                                      size_t n, PGLGuidedQueryResult *dResults, bool cosineProduct,
                                                      void *cudaStream);
// Volume guided queries with the single-lobe Henyey-Greenstein product
// (what pglVolumeSamplingDistributionApplySingleLobeHenyeyGreensteinProduct
// does per object): query i's normal is the phase function's direction and
// meanCosines[i] its mean cosine g; results as the per-object calls (Init +
// product + SamplePDF + IncomingRadiancePDF).  Host buffers, or device
// buffers enqueued on `cudaStream` (null: the library's stream; does not
// synchronise).
OPENPGL_CORE_INTERFACE bool pglFieldSampleVolumeBatchHG(PGLField field, const PGLGuidedQuery *queries,
                                                        const float *meanCosines, size_t n,
                                                        PGLGuidedQueryResult *results);
OPENPGL_CORE_INTERFACE bool pglFieldSampleVolumeBatchHGDevice(PGLField field, const PGLGuidedQuery *dQueries,
                                                              const float *dMeanCosines, size_t n,
                                                              PGLGuidedQueryResult *dResults, void *cudaStream);
// Path-vertex queries (no reference counterpart; what a renderer does per
// vertex with SurfaceSamplingDistribution: Init, ApplyCosineProduct, then
// SamplePDF for each of the vertex's four 2D random numbers,
// VMMSurfaceSamplingDistribution.h:67-103), in one kernel: host buffers
// (page-locked ones used in place, others copied in and out; synchronises)
// or device buffers enqueued on `cudaStream` (null: the library's stream;
// does not synchronise).
OPENPGL_CORE_INTERFACE bool pglFieldSampleSurfaceVertices(PGLField field, const PGLGuidedVertex *vertices, size_t n,
                                                          PGLGuidedVertexResult *results);
OPENPGL_CORE_INTERFACE bool pglFieldSampleSurfaceVerticesDevice(PGLField field, const PGLGuidedVertex *dVertices,
                                                                size_t n, PGLGuidedVertexResult *dResults,
                                                                void *cudaStream);
// Adds samples that already live in device memory.
OPENPGL_CORE_INTERFACE void pglSampleStorageAddSamplesDevice(PGLSampleStorage sampleStorage,
                                                             const PGLSampleData *dSamples, size_t numSamples);
// Serialised field (the bytes pglFieldStoreToFile writes); returns the size,
// copies when buffer holds at least that many bytes.
OPENPGL_CORE_INTERFACE size_t pglFieldStoreToBuffer(PGLField field, char *buffer, size_t capacity);
// Milliseconds of the last Update of the surface (0) or volume (1) field:
// total, sample copy, spatial structure, directional fitting.
OPENPGL_CORE_INTERFACE bool pglFieldGetLastUpdateTimings(PGLField field, int volume, float out4[4]);
// Phases of the last Update of the surface (0) or volume (1) field, from CUDA
// events on the library's stream: total, sample copy, spatial structure,
// directional (= gather + EM kernel), gather, EM kernel (ms), then the number
// of samples and of regions.  Returns 8; writes when capacity >= 8.
OPENPGL_CORE_INTERFACE size_t pglFieldGetLastUpdatePhases(PGLField field, int volume, double *out, size_t capacity);
// The cudaStream_t every kernel of the library is launched on (one per
// process), for callers that order their own work or events against it.
OPENPGL_CORE_INTERFACE void *pglDeviceGetCudaStream(PGLDevice device);
// Number of the library's own CUDA kernels launched so far by this process
// (the scan and sort kernels of CUB that it calls are not counted).
OPENPGL_CORE_INTERFACE uint64_t pglGetKernelLaunchCount();
// Failure detection without a GPU fault: one device thread waits, with the
// EM kernel's bounded wait, on a flag that nothing sets; the wait gives up
// after limitNs (at most 10 s) and records its error.  Returns that error
// code (2: the wait ran out) or -1 on a CUDA error (pglGetLastError()).
OPENPGL_CORE_INTERFACE int pglDebugBoundedWaitRunsOut(uint64_t limitNs);
// Per-region counters of the last Update: region, EM iterations, splits,
// merges, components (5 x u32 per region); returns the region count, writes
// when capacity >= 5 x count.
OPENPGL_CORE_INTERFACE size_t pglFieldGetLastUpdateReports(PGLField field, int volume, uint32_t *out, size_t capacity);
// Where the EM kernel spent the last Update, per region (23 x u64 each):
// region, samples, E-step passes, distance passes, split-statistics passes,
// then SM clock cycles in E-steps, distance passes, split-statistics passes,
// merging, M-steps and in total, then inside the passes the cycles of the
// producing threads and of the slowest summing thread, for E-steps and for
// split-statistics passes, then the E-step chunks of the region, those made
// by its own block (the others by blocks that had no region left), and the
// cycles a summing thread waited for chunks, then the lobes summed over the
// E-step, distance and split-statistics passes (the sum of the mixture's
// lobe count over the passes of each kind), then the device's global timer
// (ns) when a block took the region and when it was done with it.  Returns
// the region count; writes when capacity >= 23 x count.
OPENPGL_CORE_INTERFACE size_t pglFieldGetLastUpdateProfile(PGLField field, int volume, uint64_t *out,
                                                           size_t capacity);
// Schedule parameters of the field's EM launch (no reference counterpart;
// they change the Update's speed, never its result), as int[4]: helper
// blocks that may work on one region at a time (0-64, default 4), the E-step
// chunk-size divisor (1-4, default 1), the pipeline stages of the summing
// warps (2-8, default 8), and 1 to queue regions by their previous Update's
// measured cost instead of by sample count (default 0).  Set returns false
// (and records the error) for values out of range.
OPENPGL_CORE_INTERFACE bool pglFieldSetEmTuning(PGLField field, const int *tuning);
OPENPGL_CORE_INTERFACE bool pglFieldGetEmTuning(PGLField field, int *tuning);
// The plain form of the Update's directional fit (no reference counterpart;
// for comparisons): one single-block EM launch per region, one after the
// other, instead of one persistent launch for all regions of both
// sub-fields with E-step passes shared between blocks.  Same results.
OPENPGL_CORE_INTERFACE bool pglFieldSetPlainUpdate(PGLField field, bool plain);
// The next Update first times candidate schedules (helper blocks 2/4/8 x
// chunk divisor 1/2, x queue order when costs are known) on its own regions,
// restoring the state they change after each trial, keeps the fastest and
// then runs; its result is the same as without tuning.
OPENPGL_CORE_INTERFACE void pglFieldAutotuneNextUpdate(PGLField field);
// The trials of the last tuning: int[4] schedule and milliseconds each;
// returns their count, writes when capacity >= count.
OPENPGL_CORE_INTERFACE size_t pglFieldGetEmTuningTrials(PGLField field, int *tunings, float *ms, size_t capacity);
// Training samples from many paths at once on the device (what
// pglPathSegmentStoragePrepareSamples does for one path in host memory):
// path p is dSegments[dPathBegin[p], dPathBegin[p + 1]) (numPaths + 1 offsets
// in device memory).  Writes the samples to dSamples (device memory with room
// for dPathBegin[numPaths] records, the segment count, which bounds the
// sample count) in path order, each path's in the reference's order, and
// path p's first slot to dSampleBegin[p] (numPaths + 1 entries, the last is
// the total).  Enqueued on cudaStream (null: the library's stream); does not
// synchronise.
OPENPGL_CORE_INTERFACE bool pglPathSegmentsPrepareSamplesDevice(const PGLPathSegmentData *dSegments,
                                                                const uint32_t *dPathBegin, size_t numPaths,
                                                                float maxDistance, bool useNEEMiWeights,
                                                                bool guideDirectLight,
                                                                bool rrAffectsDirectContribution,
                                                                PGLSampleData *dSamples, uint32_t *dSampleBegin,
                                                                void *cudaStream);
// The same for pglPathSegmentStoragePropagateSamples: the paths' samples go
// into sampleStorage without leaving the device.  Returns their count;
// synchronises with the library's stream.
OPENPGL_CORE_INTERFACE size_t pglPathSegmentsPropagateSamplesDevice(const PGLPathSegmentData *dSegments,
                                                                    const uint32_t *dPathBegin, size_t numPaths,
                                                                    float maxDistance, PGLSampleStorage sampleStorage,
                                                                    bool guideDirectLight, bool useNEEMiWeights,
                                                                    bool rrAffectsDirectContribution);
// Splits numSamples sample records that live in device memory into the
// surface records and the inside-volume records (flags & EInsideVolume), each
// kind in its original order, written to dSurface and dVolume (device
// buffers with room for numSamples records each); the two counts go to
// dCounts[0] (surface) and dCounts[1] (volume) in device memory.  Work is
// enqueued on cudaStream (null: the legacy default stream) and not waited for.
// No reference counterpart.  Unlike pglSampleStorageAddSamplesDevice it
// allocates nothing, neither device memory nor library scratch: for callers
// that must not allocate, such as a renderer that reserves all of its device
// memory up front, or one that cannot afford the device-wide synchronisation
// that cudaFree implies in the middle of a frame.
// Its scratch is one fixed array in device memory: at most 67,108,864 records
// per call (larger batches are rejected with an error), and calls that may
// overlap in time (other threads or streams) must be serialised by the caller.
// The first call on each device looks the array up (cudaGetSymbolAddress);
// make it before any stream capture.  The address found is kept for the
// life of the process, so do not use this entry point on a device after
// cudaDeviceReset (the array's storage is then gone).
OPENPGL_CORE_INTERFACE bool pglSplitSamplesDeviceNoAlloc(const PGLSampleData *dSamples, size_t numSamples,
                                                         PGLSampleData *dSurface, PGLSampleData *dVolume,
                                                         uint32_t *dCounts, void *cudaStream);
// ---- Serving a field (no reference counterpart).  A server answers guided
// queries against a resident field while it keeps training it: requests of
// any size from any thread are batched continuously into kernel launches on
// the server's stream, against a snapshot of the field; an Update runs in the
// background on the field's own streams and its result replaces the snapshot
// when it is done (two snapshots: requests already started finish on the one
// they started on).  While a server serves a field, use the field only through
// the server; release the server before the field.
#ifdef __cplusplus
struct GuidingServer;
#endif
typedef struct GuidingServer *PGLGuidingServer;
// hbmBudgetBytes bounds the device memory that the server and its field use:
// the field's state and Update working set, two snapshots of it that queries
// read, the samples of the next Update (AddSamples refuses a batch whose
// Update would not fit) and the buffers of two query launches in flight
// (given at most a quarter of what the field leaves; larger requests run in
// several launches).  While the server runs, the field's EM launches leave 8
// SMs to the query launches, so queries keep being answered during an Update.
OPENPGL_CORE_INTERFACE PGLGuidingServer pglNewGuidingServer(PGLField field, size_t hbmBudgetBytes);
// The same with the number of SMs the field's EM launches leave to queries
// (default 8; at most all but one): more keeps query latency low under a
// heavy query load while the field trains, fewer lets Updates finish sooner.
OPENPGL_CORE_INTERFACE PGLGuidingServer pglNewGuidingServerEx(PGLField field, size_t hbmBudgetBytes,
                                                              int reservedSMs);
OPENPGL_CORE_INTERFACE void pglReleaseGuidingServer(PGLGuidingServer server);
// Queues n queries; `queries` and `results` (host memory) must stay valid until
// the request is waited for.  When both are page-locked, the server's launches
// read and write them in place (no staging copies).  Returns a ticket (0 on
// error).
OPENPGL_CORE_INTERFACE uint64_t pglGuidingServerSubmit(PGLGuidingServer server, const PGLGuidedQuery *queries,
                                                       size_t n, PGLGuidedQueryResult *results, bool volume,
                                                       bool cosineProduct);
// Blocks until the request is done; reports its latency (submit to results)
// and the field iteration its results come from.
OPENPGL_CORE_INTERFACE bool pglGuidingServerWait(PGLGuidingServer server, uint64_t ticket, double *latencyMs,
                                                 uint64_t *fieldVersion);
// Training samples for the next Update (copied).
OPENPGL_CORE_INTERFACE bool pglGuidingServerAddSamples(PGLGuidingServer server, const PGLSampleData *samples,
                                                       size_t n);
// Training samples in device memory (copied into the server's own device
// buffer before the call returns).
OPENPGL_CORE_INTERFACE bool pglGuidingServerAddSamplesDevice(PGLGuidingServer server, const PGLSampleData *dSamples,
                                                             size_t n);
// Starts an Update with the samples added so far; returns a ticket.
OPENPGL_CORE_INTERFACE uint64_t pglGuidingServerUpdate(PGLGuidingServer server);
OPENPGL_CORE_INTERFACE bool pglGuidingServerWaitUpdate(PGLGuidingServer server, uint64_t ticket);
// Queues n path vertices (Init, cosine product, four SamplePDF calls each;
// buffers as for pglGuidingServerSubmit).  Returns a ticket (0 on error).
OPENPGL_CORE_INTERFACE uint64_t pglGuidingServerSubmitVertices(PGLGuidingServer server,
                                                               const PGLGuidedVertex *vertices, size_t n,
                                                               PGLGuidedVertexResult *results);
// queries served, requests done, latency p50 / p99 / p99.9 (ms), launches,
// updates done, field iteration being served
OPENPGL_CORE_INTERFACE bool pglGuidingServerStats(PGLGuidingServer server, double out8[8]);
// The same eight values, then the device bytes the server and its field hold,
// the budget and the queries one launch takes at most; writes min(count, 11)
// values and returns 11.
OPENPGL_CORE_INTERFACE size_t pglGuidingServerStatsEx(PGLGuidingServer server, double *out, size_t count);
// Starts a new measurement window (latencies, queries and launches counted
// from here on).
OPENPGL_CORE_INTERFACE bool pglGuidingServerResetStats(PGLGuidingServer server);
// Message of the error raised by the last library call on this thread ("" if
// that call succeeded).
OPENPGL_CORE_INTERFACE const char *pglGetLastError();

#ifdef __cplusplus
}
#endif
