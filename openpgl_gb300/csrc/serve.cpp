// GuidingServer: continuous batching of guided queries against a double-
// buffered snapshot of a field that a background thread keeps training.
#include "serve.h"

#include <algorithm>
#include <cstring>
#include <stdexcept>

namespace pgl {

namespace {
// bytes of a path vertex in flight (input and result; the larger kind)
constexpr size_t kVertexBytes = sizeof(QueryInS4) + sizeof(QueryOutS4);
constexpr size_t kMaxLaunch = size_t(1) << 24;  // queries per launch at most
}  // namespace

size_t GuidingServer::fieldBytes() const {
  return field_->surface.stateBytes() + field_->volume.stateBytes();
}

size_t GuidingServer::deviceBytesInUse() const {
  size_t b = field_->deviceBytes() + storage_.deviceBytes();
  for (const Snapshot &s : snap_)
    for (int k = 0; k < 2; ++k) b += s.regions[k].bytes() + s.nodes[k].bytes() + s.nbrs[k].bytes();
  for (const Slot &s : slots_) b += s.dIn.bytes() + s.dOut.bytes();
  return b + incomingDev_.bytes();
}

size_t GuidingServer::projectedBytes(size_t samples) const {
  const size_t training = field_->deviceBytes() + storage_.deviceBytes();
  const size_t others = deviceBytesInUse() - training;
  return others + std::max(training, fieldBytes() + samples * kUpdateBytesPerSample);
}

GuidingServer::GuidingServer(GpuField *field, size_t budgetBytes, int reservedSMs)
    : field_(field), budget_(budgetBytes) {
  if (!field) throw std::runtime_error("null field");
  Context &c = Context::get();
  // the field's EM launches leave these SMs to the query stream
  field_->tuning.reservedSMs = std::max(0, std::min(reservedSMs, c.numSMs - 1));
  // query buffers: two launches in flight, each of up to capacity_ queries of
  // the largest kind; they take at most a quarter of what the budget leaves
  // after the field and its two snapshots (the rest is for training)
  const size_t fixed = 3 * fieldBytes() + field_->deviceBytes();
  if (budgetBytes <= fixed + 2 * 1024 * kVertexBytes)
    throw std::runtime_error("HBM budget of the guiding server is below the field's own memory");
  capacity_ = std::min<size_t>(std::max<size_t>((budgetBytes - fixed) / 4 / (2 * kVertexBytes), 1024), kMaxLaunch);
  for (Slot &s : slots_) {
    s.dIn.reserve(capacity_ * sizeof(QueryInS4));
    s.dOut.reserve(capacity_ * sizeof(QueryOutS4));
    check(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "event");
    check(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "query stream");
  }
  for (Snapshot &s : snap_) check(cudaEventCreateWithFlags(&s.lastRead, cudaEventDisableTiming), "event");
  takeSnapshot(0);
  active_ = 0;
  const int device = c.device;
  dispatcher_ = std::thread([this, device] {
    cudaSetDevice(device);
    dispatchLoop();
  });
  trainer_ = std::thread([this, device] {
    cudaSetDevice(device);
    trainLoop();
  });
}

GuidingServer::~GuidingServer() {
  {
    std::lock_guard<std::mutex> lk(m_);
    stop_ = true;
  }
  cvWork_.notify_all();
  cvTrain_.notify_all();
  cvDone_.notify_all();
  if (dispatcher_.joinable()) dispatcher_.join();
  if (trainer_.joinable()) trainer_.join();
  for (auto &kv : requests_) delete kv.second;
  for (Slot &s : slots_) {
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  for (Snapshot &s : snap_)
    if (s.lastRead) cudaEventDestroy(s.lastRead);
  if (copyStream_) cudaStreamDestroy(copyStream_);
  field_->tuning.reservedSMs = 0;
}

// Copies what queries read (regions, nodes, neighbours of both kinds) into
// snapshot `slot`; the caller makes sure no query launch uses the slot.
void GuidingServer::takeSnapshot(int slot) {
  Snapshot &s = snap_[slot];
  SubField *sides[2] = {&field_->surface, &field_->volume};
  for (int k = 0; k < 2; ++k) {
    SubField &f = *sides[k];
    cudaStream_t st = f.stream();
    const size_t R = f.regions.size(), N = f.nodes.size();
    FieldView v = f.view();
    if (R > 0 && N > 0) {
      s.regions[k].reserve(R);
      s.nodes[k].reserve(N);
      check(cudaMemcpyAsync(s.regions[k].p, f.dRegions.p, R * sizeof(RegionDir), cudaMemcpyDeviceToDevice, st),
            "snapshot regions");
      check(cudaMemcpyAsync(s.nodes[k].p, f.nodes.data(), N * sizeof(KDNode), cudaMemcpyHostToDevice, st),
            "snapshot nodes");
      v.regions = s.regions[k].p;
      v.nodes = s.nodes[k].p;
      if (f.cfg.knn && f.dNbrs.p) {
        s.nbrs[k].reserve(R);
        check(cudaMemcpyAsync(s.nbrs[k].p, f.dNbrs.p, R * sizeof(Neighbours), cudaMemcpyDeviceToDevice, st),
              "snapshot neighbours");
        v.nbrs = s.nbrs[k].p;
      } else {
        v.nbrs = nullptr;
      }
      if (f.cfg.dqt) {
        const size_t nodes = R * size_t(f.dqtStride);
        s.dqtHeads[k].reserve(R);
        s.dqtNodes[k].reserve(nodes);
        check(cudaMemcpyAsync(s.dqtHeads[k].p, f.dDqtHeads.p, R * sizeof(DqtHead), cudaMemcpyDeviceToDevice, st),
              "snapshot quadtree heads");
        check(cudaMemcpyAsync(s.dqtNodes[k].p, f.dDqtNodes.p, nodes * sizeof(DqtNode), cudaMemcpyDeviceToDevice, st),
              "snapshot quadtrees");
        v.dqtHeads = s.dqtHeads[k].p;
        v.dqtNodes = s.dqtNodes[k].p;
      }
      check(cudaStreamSynchronize(st), "snapshot");
    } else {
      v.iteration = 0;  // nothing to query yet: Init fails, as on an untrained field
      v.numNodes = 0;
    }
    s.view[k] = v;
  }
  s.version = field_->iteration;
}

uint64_t GuidingServer::submit(const QueryIn *in, QueryOut *out, size_t n, bool volume, bool cosine) {
  Request *r = new Request();
  r->kind = RequestKind::Query;
  r->in = in;
  r->out = out;
  r->inDev = device_address(in);
  r->outDev = r->inDev ? device_address(out) : nullptr;
  r->n = n;
  r->volume = volume;
  r->cosine = cosine && !volume;
  r->t0 = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lk(m_);
    if (stop_) {
      delete r;
      throw std::runtime_error("server is shutting down");
    }
    r->id = nextId_++;
    requests_[r->id] = r;
    if (n == 0) {
      r->finished = true;
      r->version = snap_[active_].version;
    } else {
      pending_.push_back(r);
    }
  }
  if (n == 0) cvDone_.notify_all();
  else cvWork_.notify_one();
  return r->id;
}

uint64_t GuidingServer::submitVertices(const QueryInS4 *in, QueryOutS4 *out, size_t n) {
  Request *r = new Request();
  r->kind = RequestKind::Vertex;
  r->in = in;
  r->out = out;
  r->inDev = device_address(in);
  r->outDev = r->inDev ? device_address(out) : nullptr;
  r->n = n;
  r->volume = false;
  r->cosine = true;
  r->t0 = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lk(m_);
    if (stop_) {
      delete r;
      throw std::runtime_error("server is shutting down");
    }
    r->id = nextId_++;
    requests_[r->id] = r;
    if (n == 0) {
      r->finished = true;
      r->version = snap_[active_].version;
    } else {
      pending_.push_back(r);
    }
  }
  if (n == 0) cvDone_.notify_all();
  else cvWork_.notify_one();
  return r->id;
}

void GuidingServer::wait(uint64_t ticket, double *latencyMs, uint64_t *version) {
  std::unique_lock<std::mutex> lk(m_);
  auto it = requests_.find(ticket);
  if (it == requests_.end()) throw std::runtime_error("unknown request ticket");
  Request *r = it->second;
  cvDone_.wait(lk, [&] { return r->finished || stop_; });
  if (!error_.empty()) throw std::runtime_error("guiding server failed: " + error_);
  if (!r->finished) throw std::runtime_error("server stopped before the request finished");
  if (latencyMs) *latencyMs = r->latencyMs;
  if (version) *version = r->version;
  requests_.erase(it);
  delete r;
}

void GuidingServer::fail(const std::exception &e) {
  {
    std::lock_guard<std::mutex> lk(m_);
    if (error_.empty()) error_ = e.what();
    for (auto &kv : requests_) kv.second->finished = true;
    pending_.clear();
    updatesDone_ = updatesAsked_;
    stop_ = true;
  }
  cvDone_.notify_all();
  cvWork_.notify_all();
  cvTrain_.notify_all();
}

void GuidingServer::dispatchLoop() {
  try {
    dispatch();
  } catch (const std::exception &e) {
    fail(e);
  } catch (...) {
    fail(std::runtime_error("an unrecognized exception was caught"));
  }
}

// Results of a finished launch: its requests' pieces are done.
void GuidingServer::complete(Slot &slot) {
  check(cudaEventSynchronize(slot.done), "queries");
  {
    std::lock_guard<std::mutex> lk(m_);
    const auto now = std::chrono::steady_clock::now();
    for (const Seg &g : slot.segs) {
      Request *r = g.r;
      r->done += g.cnt;
      if (r->done == r->n) {
        r->finished = true;
        r->latencyMs = std::chrono::duration<double, std::milli>(now - r->t0).count();
        latencies_.push_back(r->latencyMs);
        served_ += r->n;
        pinned_[r->snap]--;
      }
    }
    launches_++;
  }
  slot.segs.clear();
  slot.busy = false;
  cvDone_.notify_all();
  cvTrain_.notify_all();
}

// Continuous batching with two launches in flight: while one launch runs,
// the next is formed from whatever requests are pending (first come, first
// served, of the head request's kind, up to the launch capacity) and its
// copies and kernel are enqueued behind it; a launch's requests complete when
// its results are back in their host buffers.
void GuidingServer::dispatch() {
  int next = 0;
  for (;;) {
    Slot &slot = slots_[next];
    Slot &other = slots_[1 - next];
    if (slot.busy) complete(slot);
    std::unique_lock<std::mutex> lk(m_);
    cvWork_.wait(lk, [&] { return stop_ || !pending_.empty() || other.busy; });
    if (stop_) return;
    if (pending_.empty()) {  // nothing new: finish the launch in flight
      lk.unlock();
      complete(other);
      continue;
    }
    Request *head = pending_.front();
    const RequestKind kind = head->kind;
    const int snap = head->snap >= 0 ? head->snap : active_;
    size_t total = 0;
    for (Request *r : pending_) {
      if (total >= capacity_) break;
      if (r->kind != kind || r->volume != head->volume || r->cosine != head->cosine) continue;
      if ((r->snap >= 0 ? r->snap : active_) != snap) continue;
      const size_t take = std::min(r->n - r->sent, capacity_ - total);
      if (r->snap < 0) {
        r->snap = snap;
        r->version = snap_[snap].version;
        pinned_[snap]++;
      }
      slot.segs.push_back(Seg{r, r->sent, take, total});
      r->sent += take;
      total += take;
    }
    pending_.erase(std::remove_if(pending_.begin(), pending_.end(), [](Request *r) { return r->sent == r->n; }),
                   pending_.end());
    const FieldView view = snap_[snap].view[head->volume ? 1 : 0];
    const bool cosine = head->cosine;
    lk.unlock();

    const size_t inBytes = kind == RequestKind::Vertex ? sizeof(QueryInS4) : sizeof(QueryIn);
    const size_t outBytes = kind == RequestKind::Vertex ? sizeof(QueryOutS4) : sizeof(QueryOut);
    QueryParams p{};
    p.f = view;
    p.cosKappa = 2.18853f;
    p.cosNorm = cosine_lobe_normalization();
    p.cosine = cosine ? 1 : 0;
    p.samplesPerQuery = kind == RequestKind::Vertex ? kVertexSamples : 1;
    auto launch = [&](const unsigned char *in, unsigned char *out, size_t n) {
      if (kind == RequestKind::Vertex)
        check(launch_query_s4(p, reinterpret_cast<const QueryInS4 *>(in), reinterpret_cast<QueryOutS4 *>(out),
                              uint32_t(n), slot.stream),
              "vertex query launch");
      else
        check(launch_query(p, reinterpret_cast<const QueryIn *>(in), reinterpret_cast<QueryOut *>(out), uint32_t(n),
                           slot.stream),
              "query launch");
    };
    // requests in page-locked host memory are read and written in place, a
    // launch per piece; the others go through the slot's device buffers
    bool inPlace = true;
    for (const Seg &g : slot.segs) inPlace = inPlace && g.r->inDev && g.r->outDev;
    if (inPlace) {
      for (const Seg &g : slot.segs)
        launch(static_cast<const unsigned char *>(g.r->inDev) + g.off * inBytes,
               static_cast<unsigned char *>(g.r->outDev) + g.off * outBytes, g.cnt);
      check(cudaEventRecord(snap_[snap].lastRead, slot.stream), "event");
    } else {
      for (const Seg &g : slot.segs)
        check(cudaMemcpyAsync(slot.dIn.p + g.pos * inBytes, static_cast<const unsigned char *>(g.r->in) + g.off * inBytes,
                              g.cnt * inBytes, cudaMemcpyHostToDevice, slot.stream),
              "H2D queries");
      launch(slot.dIn.p, slot.dOut.p, total);
      check(cudaEventRecord(snap_[snap].lastRead, slot.stream), "event");
      for (const Seg &g : slot.segs)
        check(cudaMemcpyAsync(static_cast<unsigned char *>(g.r->out) + g.off * outBytes, slot.dOut.p + g.pos * outBytes,
                              g.cnt * outBytes, cudaMemcpyDeviceToHost, slot.stream),
              "D2H results");
    }
    check(cudaEventRecord(slot.done, slot.stream), "event");
    slot.busy = true;
    slot.queries = total;
    next = 1 - next;
  }
}

void GuidingServer::addSamplesDevice(const PGLSampleRecord *d, size_t n) {
  std::lock_guard<std::mutex> lk(incomingMutex_);
  // the server's own copy of the records grows (by at most its reserve's headroom)
  const size_t grow = incomingDev_.cap < incomingDevN_ + n
                          ? (incomingDevN_ + n + (incomingDevN_ + n) / 4) * sizeof(PGLSampleRecord) - incomingDev_.bytes()
                          : 0;
  const size_t projected = projectedBytes(incoming_.size() + incomingDevN_ + n) + grow;
  if (projected > budget_)
    throw std::runtime_error("training batch over the guiding server's HBM budget (" + std::to_string(projected) +
                             " > " + std::to_string(budget_) + " bytes)");
  if (!copyStream_) check(cudaStreamCreateWithFlags(&copyStream_, cudaStreamNonBlocking), "copy stream");
  incomingDev_.reserve(incomingDevN_ + n, true);
  check(cudaMemcpyAsync(incomingDev_.p + incomingDevN_, d, n * sizeof(PGLSampleRecord), cudaMemcpyDeviceToDevice,
                        copyStream_),
        "training samples");
  check(cudaStreamSynchronize(copyStream_), "training samples");
  incomingDevN_ += n;
}

void GuidingServer::addSamples(const PGLSampleRecord *s, size_t n) {
  std::lock_guard<std::mutex> lk(incomingMutex_);
  // admission by the HBM budget: the next Update's samples and working set
  // beside what the field's snapshots and the query buffers hold
  const size_t projected = projectedBytes(incoming_.size() + incomingDevN_ + n);
  if (projected > budget_)
    throw std::runtime_error("training batch over the guiding server's HBM budget (" + std::to_string(projected) +
                             " > " + std::to_string(budget_) + " bytes)");
  incoming_.insert(incoming_.end(), s, s + n);
}

uint64_t GuidingServer::update() {
  uint64_t ticket;
  {
    std::lock_guard<std::mutex> lk(m_);
    ticket = ++updatesAsked_;
  }
  cvTrain_.notify_all();
  return ticket;
}

void GuidingServer::waitUpdate(uint64_t ticket) {
  std::unique_lock<std::mutex> lk(m_);
  cvDone_.wait(lk, [&] { return updatesDone_ >= ticket || stop_; });
  if (!error_.empty()) throw std::runtime_error("guiding server failed: " + error_);
}

void GuidingServer::trainLoop() {
  try {
    train();
  } catch (const std::exception &e) {
    fail(e);
  } catch (...) {
    fail(std::runtime_error("an unrecognized exception was caught"));
  }
}

void GuidingServer::train() {
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(m_);
      cvTrain_.wait(lk, [&] { return stop_ || updatesAsked_ > updatesDone_; });
      if (stop_) return;
    }
    std::vector<PGLSampleRecord> batch;
    {
      std::lock_guard<std::mutex> lk(incomingMutex_);
      batch.swap(incoming_);
      if (incomingDevN_ > 0) {
        storage_.ingestDevice(incomingDev_.p, incomingDevN_);
        // the ingest has read the buffer before the next addSamplesDevice may write it
        check(cudaStreamSynchronize(Context::get().stream), "training samples");
      }
      incomingDevN_ = 0;
    }
    if (!batch.empty()) storage_.add(batch.data(), batch.size());
    field_->update(storage_, true, true);
    storage_.clearSurface();
    storage_.clearVolume();
    int slot;
    {
      // the other snapshot: wait until no unfinished request uses it
      std::unique_lock<std::mutex> lk(m_);
      slot = 1 - active_;
      cvTrain_.wait(lk, [&] { return stop_ || pinned_[slot] == 0; });
      if (stop_) return;
    }
    check(cudaEventSynchronize(snap_[slot].lastRead), "snapshot reader");  // its last launch is done
    takeSnapshot(slot);
    {
      std::lock_guard<std::mutex> lk(m_);
      active_ = slot;
      updatesDone_++;
    }
    cvDone_.notify_all();
  }
}

void GuidingServer::stats(double out[11]) {
  std::lock_guard<std::mutex> lk(m_);
  std::vector<double> l = latencies_;
  std::sort(l.begin(), l.end());
  auto q = [&](double f) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, size_t(f * double(l.size())))]; };
  out[0] = double(served_);
  out[1] = double(l.size());
  out[2] = q(0.5);
  out[3] = q(0.99);
  out[4] = q(0.999);
  out[5] = double(launches_);
  out[6] = double(updatesDone_);
  out[7] = double(snap_[active_].version);
  out[8] = double(deviceBytesInUse());
  out[9] = double(budget_);
  out[10] = double(capacity_);
}

void GuidingServer::resetStats() {
  std::lock_guard<std::mutex> lk(m_);
  latencies_.clear();
  served_ = 0;
  launches_ = 0;
}

}  // namespace pgl
