// Serving a resident guiding field: guided-query requests of any size and
// training batches arrive concurrently; queries are batched continuously into
// launches on their own stream, against a snapshot of the field that is
// swapped after each Update, so retraining overlaps answering.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "field.h"

namespace pgl {

// Read-only copy of what guided queries read from a field (both kinds).
struct Snapshot {
  DevArray<RegionDir> regions[2];
  DevArray<KDNode> nodes[2];
  DevArray<Neighbours> nbrs[2];
  DevArray<DqtHead> dqtHeads[2];  // quadtree fields: the regions' heads and trees
  DevArray<DqtNode> dqtNodes[2];
  FieldView view[2];
  uint64_t version = 0;  // field updates folded in
  cudaEvent_t lastRead = nullptr;  // the last query launch that read it
};

// Kinds of request: single-sample guided queries (QueryIn/QueryOut) and
// path vertices with several SamplePDF calls (QueryInS4/QueryOutS4).
enum class RequestKind { Query, Vertex };

class GuidingServer {
 public:
  // `budgetBytes` bounds the device memory the server and its field use:
  // the field's own state and Update working set, the two snapshots that
  // queries read, the sample storage of the next Update and the buffers of
  // the queries in flight.  `reservedSMs` SMs are left out of the field's
  // EM launches so that queries keep running while the field trains.
  GuidingServer(GpuField *field, size_t budgetBytes, int reservedSMs = 8);
  ~GuidingServer();
  GuidingServer(const GuidingServer &) = delete;
  GuidingServer &operator=(const GuidingServer &) = delete;

  // Queue n queries (host buffers that stay valid until the request is
  // done); returns a ticket.
  uint64_t submit(const QueryIn *in, QueryOut *out, size_t n, bool volume, bool cosine);
  // Queue n path vertices (surface, cosine product, kVertexSamples samples each).
  uint64_t submitVertices(const QueryInS4 *in, QueryOutS4 *out, size_t n);
  // Wait for a request: its latency (submit to results in `out`) and the
  // field version its results come from.
  void wait(uint64_t ticket, double *latencyMs, uint64_t *version);
  // Training samples for the next Update (host records); throws when the
  // next Update would not fit in the budget.
  void addSamples(const PGLSampleRecord *s, size_t n);
  // The same for records in device memory (copied before the call returns).
  void addSamplesDevice(const PGLSampleRecord *d, size_t n);
  // Update the field with the samples added so far, in the background;
  // returns a ticket.
  uint64_t update();
  void waitUpdate(uint64_t ticket);
  // queries served, requests done, p50 / p99 / p99.9 latency (ms), launches,
  // updates done, current snapshot version, device bytes in use, budget,
  // queries per launch at most
  void stats(double out[11]);
  // forget the latencies recorded so far (a new measurement window)
  void resetStats();

 private:
  struct Request {
    uint64_t id;
    RequestKind kind;
    const void *in;
    void *out;
    const void *inDev = nullptr;  // device addresses of page-locked request buffers (read and written in place)
    void *outDev = nullptr;
    size_t n, sent = 0, done = 0;
    bool volume, cosine;
    int snap = -1;  // snapshot pinned at the first launch
    std::chrono::steady_clock::time_point t0;
    double latencyMs = 0.0;
    uint64_t version = 0;
    bool finished = false;
  };
  struct Seg {
    Request *r;
    size_t off, cnt, pos;
  };
  // one launch in flight: its device buffers, the requests' pieces, the
  // event after its results are back in host memory
  struct Slot {
    DevArray<unsigned char> dIn, dOut;
    std::vector<Seg> segs;
    cudaStream_t stream = nullptr;  // copies and kernel of the slot's launches
    cudaEvent_t done = nullptr;
    bool busy = false;
    size_t queries = 0;
  };
  void dispatchLoop();
  void trainLoop();
  void dispatch();
  void train();
  void complete(Slot &slot);
  void fail(const std::exception &e);
  void takeSnapshot(int slot);
  size_t fieldBytes() const;       // device state of the live field (regions, nodes, neighbours)
  size_t deviceBytesInUse() const;  // everything the budget counts
  // device bytes once an Update of `samples` samples has allocated what it
  // needs (it reuses the field's and the storage's buffers where they suffice)
  size_t projectedBytes(size_t samples) const;

  GpuField *field_;
  Storage storage_;
  Snapshot snap_[2];
  int active_ = 0;
  size_t budget_;
  size_t capacity_;  // queries per launch (of the largest kind)
  Slot slots_[2];

  std::mutex m_;
  std::condition_variable cvWork_, cvDone_, cvTrain_;
  std::deque<Request *> pending_;
  std::unordered_map<uint64_t, Request *> requests_;
  int pinned_[2] = {0, 0};  // unfinished requests pinned to each snapshot
  uint64_t nextId_ = 1;
  bool stop_ = false;
  std::vector<double> latencies_;
  uint64_t served_ = 0, launches_ = 0;

  std::mutex incomingMutex_;  // training samples that arrived since the last Update
  std::vector<PGLSampleRecord> incoming_;
  DevArray<PGLSampleRecord> incomingDev_;  // device records that arrived since the last Update
  size_t incomingDevN_ = 0;
  cudaStream_t copyStream_ = nullptr;
  uint64_t updatesAsked_ = 0, updatesDone_ = 0;
  std::string error_;  // a failure of the dispatcher or trainer, reported to waiters
  std::thread dispatcher_, trainer_;
};

// Device bytes of an Update's working set per sample of the frame (sorted
// copies, partition buffers, keys; see SubField) plus the sample itself.
constexpr size_t kUpdateBytesPerSample = 130 + 40;

}  // namespace pgl
