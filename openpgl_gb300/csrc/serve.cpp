// GuidingServer: continuous batching of guided queries against a double-
// buffered snapshot of a field that a background thread keeps training.
#include "serve.h"

#include <algorithm>
#include <cstring>
#include <stdexcept>

namespace pgl {

namespace {
constexpr size_t kQueryBytes = sizeof(QueryIn) + sizeof(QueryOut);
}

GuidingServer::GuidingServer(GpuField *field, size_t budgetBytes) : field_(field) {
  if (!field) throw std::runtime_error("null field");
  Context &c = Context::get();
  capacity_ = std::min<size_t>(std::max<size_t>(budgetBytes / kQueryBytes, 1024), size_t(1) << 24);
  dIn_.reserve(capacity_);
  dOut_.reserve(capacity_);
  check(cudaStreamCreateWithFlags(&qstream_, cudaStreamNonBlocking), "query stream");
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
  for (Snapshot &s : snap_)
    if (s.lastRead) cudaEventDestroy(s.lastRead);
  if (qstream_) cudaStreamDestroy(qstream_);
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
  r->in = in;
  r->out = out;
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

void GuidingServer::dispatch() {
  struct Seg {
    Request *r;
    size_t off, cnt, pos;
  };
  std::vector<Seg> segs;
  for (;;) {
    std::unique_lock<std::mutex> lk(m_);
    cvWork_.wait(lk, [&] { return stop_ || !pending_.empty(); });
    if (stop_) return;
    // one launch: the queries of the head request's kind, first come first
    // served, up to the launch capacity; each request stays on the snapshot
    // its first queries used
    Request *head = pending_.front();
    const int snap = head->snap >= 0 ? head->snap : active_;
    segs.clear();
    size_t total = 0;
    for (Request *r : pending_) {
      if (total >= capacity_) break;
      if (r->volume != head->volume || r->cosine != head->cosine) continue;
      if ((r->snap >= 0 ? r->snap : active_) != snap) continue;
      const size_t take = std::min(r->n - r->sent, capacity_ - total);
      if (r->snap < 0) {
        r->snap = snap;
        r->version = snap_[snap].version;
        pinned_[snap]++;
      }
      segs.push_back(Seg{r, r->sent, take, total});
      r->sent += take;
      total += take;
    }
    pending_.erase(std::remove_if(pending_.begin(), pending_.end(), [](Request *r) { return r->sent == r->n; }),
                   pending_.end());
    const FieldView view = snap_[snap].view[head->volume ? 1 : 0];
    const bool cosine = head->cosine;
    lk.unlock();

    for (const Seg &g : segs)
      check(cudaMemcpyAsync(dIn_.p + g.pos, g.r->in + g.off, g.cnt * sizeof(QueryIn), cudaMemcpyHostToDevice,
                            qstream_),
            "H2D queries");
    QueryParams p{};
    p.f = view;
    p.cosKappa = 2.18853f;
    p.cosNorm = cosine_lobe_normalization();
    p.cosine = cosine ? 1 : 0;
    p.samplesPerQuery = 1;
    check(launch_query(p, dIn_.p, dOut_.p, uint32_t(total), qstream_), "query launch");
    check(cudaEventRecord(snap_[snap].lastRead, qstream_), "event");
    for (const Seg &g : segs)
      check(cudaMemcpyAsync(g.r->out + g.off, dOut_.p + g.pos, g.cnt * sizeof(QueryOut), cudaMemcpyDeviceToHost,
                            qstream_),
            "D2H results");
    check(cudaStreamSynchronize(qstream_), "queries");

    lk.lock();
    const auto now = std::chrono::steady_clock::now();
    for (const Seg &g : segs) {
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
    lk.unlock();
    cvDone_.notify_all();
    cvTrain_.notify_all();
  }
}

void GuidingServer::addSamples(const PGLSampleRecord *s, size_t n) {
  std::lock_guard<std::mutex> lk(incomingMutex_);
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
    check(cudaEventSynchronize(snap_[slot].lastRead), "snapshot reader");
    takeSnapshot(slot);
    {
      std::lock_guard<std::mutex> lk(m_);
      active_ = slot;
      updatesDone_++;
    }
    cvDone_.notify_all();
  }
}

void GuidingServer::stats(double out[8]) {
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
}

}  // namespace pgl
