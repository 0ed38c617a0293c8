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
  FieldView view[2];
  uint64_t version = 0;  // field updates folded in
  cudaEvent_t lastRead = nullptr;  // the last query launch that read it
};

class GuidingServer {
 public:
  // `budgetBytes` bounds the device memory of in-flight query data
  // (68 bytes per query: input and result).
  GuidingServer(GpuField *field, size_t budgetBytes);
  ~GuidingServer();
  GuidingServer(const GuidingServer &) = delete;
  GuidingServer &operator=(const GuidingServer &) = delete;

  // Queue n queries (host buffers that stay valid until the request is
  // done); returns a ticket.
  uint64_t submit(const QueryIn *in, QueryOut *out, size_t n, bool volume, bool cosine);
  // Wait for a request: its latency (submit to results in `out`) and the
  // field version its results come from.
  void wait(uint64_t ticket, double *latencyMs, uint64_t *version);
  // Training samples for the next Update (host records).
  void addSamples(const PGLSampleRecord *s, size_t n);
  // Update the field with the samples added so far, in the background;
  // returns a ticket.
  uint64_t update();
  void waitUpdate(uint64_t ticket);
  // queries served, requests done, p50 / p99 / p99.9 latency (ms), launches,
  // updates done, current snapshot version
  void stats(double out[8]);

 private:
  struct Request {
    uint64_t id;
    const QueryIn *in;
    QueryOut *out;
    size_t n, sent = 0, done = 0;
    bool volume, cosine;
    int snap = -1;  // snapshot pinned at the first launch
    std::chrono::steady_clock::time_point t0;
    double latencyMs = 0.0;
    uint64_t version = 0;
    bool finished = false;
  };
  void dispatchLoop();
  void trainLoop();
  void dispatch();
  void train();
  void fail(const std::exception &e);
  void takeSnapshot(int slot);

  GpuField *field_;
  Storage storage_;
  Snapshot snap_[2];
  int active_ = 0;
  size_t capacity_;  // queries per launch
  DevArray<QueryIn> dIn_;
  DevArray<QueryOut> dOut_;
  cudaStream_t qstream_ = nullptr;

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
  uint64_t updatesAsked_ = 0, updatesDone_ = 0;
  std::string error_;  // a failure of the dispatcher or trainer, reported to waiters
  std::thread dispatcher_, trainer_;
};

}  // namespace pgl
