// Host orchestration of the GPU guiding field.  Compiled with
// -ffp-contract=off: the float code here (statistics merge/split, split
// decisions, quantisation frames) must produce the reference's bits.
#include "field.h"

#include <dlfcn.h>

#include <algorithm>
#include <cstdlib>
#include <fstream>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <exception>
#include <numeric>
#include <thread>

namespace pgl {

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// The host C library's expf/cosf/sinf exception table (gen_libm_exceptions.cpp),
// written by the build next to this library as libm_exceptions.bin, copied
// to device memory that lives until the process exits.
static LibmTables load_libm_tables() {
  Dl_info info{};
  if (!dladdr(reinterpret_cast<void *>(&load_libm_tables), &info) || !info.dli_fname)
    throw std::runtime_error("cannot locate the library to find libm_exceptions.bin");
  std::string path = info.dli_fname;
  const size_t slash = path.rfind('/');
  path = (slash == std::string::npos ? std::string(".") : path.substr(0, slash)) + "/libm_exceptions.bin";
  std::ifstream is(path, std::ios::binary);
  char magic[8];
  uint32_t n[3] = {0, 0, 0};
  if (!is.read(magic, 8) || std::memcmp(magic, "PGLLIBM2", 8) != 0 || !is.read(reinterpret_cast<char *>(n), 12))
    throw std::runtime_error("missing or bad " + path + " (the build writes it)");
  std::vector<float2> v(size_t(n[0]) + n[1] + n[2]);
  if (!is.read(reinterpret_cast<char *>(v.data()), std::streamsize(v.size() * sizeof(float2))))
    throw std::runtime_error("truncated " + path);
  float2 *d = nullptr;
  if (!v.empty()) {
    check(cudaMalloc(&d, v.size() * sizeof(float2)), "libm table");
    check(cudaMemcpy(d, v.data(), v.size() * sizeof(float2), cudaMemcpyHostToDevice), "libm table");
  }
  LibmTables t;
  t.expf = d;
  t.cosf = d ? d + n[0] : nullptr;
  t.sinf = d ? d + n[0] + n[1] : nullptr;
  t.numExpf = n[0];
  t.numCosf = n[1];
  t.numSinf = n[2];
  return t;
}

Context &Context::get() {
  // thread-safe one-time set-up (C++ static initialisation)
  static Context c = [] {
    Context x;
    check(cudaGetDevice(&x.device), "cudaGetDevice");
    check(cudaDeviceGetAttribute(&x.numSMs, cudaDevAttrMultiProcessorCount, x.device), "SM count");
    check(cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking), "stream");
    const LibmTables libm = load_libm_tables();
    check(em_upload_tables(libm), "tables (em)");
    check(spatial_upload_tables(libm), "tables (spatial)");
    check(query_upload_tables(libm), "tables (query)");
    return x;
  }();
  return c;
}

template <typename T>
void DevArray<T>::reserve(size_t n, bool keep) {
  if (n <= cap && p) return;
  size_t want = std::max<size_t>(n + n / 4, 64);
  T *np = nullptr;
  check(cudaMalloc(&np, want * sizeof(T)), "cudaMalloc");
  if (keep && p && cap) check(cudaMemcpy(np, p, cap * sizeof(T), cudaMemcpyDeviceToDevice), "grow copy");
  if (p) cudaFree(p);
  p = np;
  cap = want;
}
void HostPinned::reserve(size_t bytes) {
  if (bytes <= cap && p) return;
  const size_t want = std::max<size_t>(bytes + bytes / 4, 4096);
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  check(cudaMallocHost(reinterpret_cast<void **>(&p), want), "cudaMallocHost");
  cap = want;
}
HostPinned::~HostPinned() {
  if (p) cudaFreeHost(p);
}

template <typename T>
void DevArray<T>::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}
template struct DevArray<float4>;
template struct DevArray<float>;
template struct DevArray<uint32_t>;
template struct DevArray<RegionDir>;
template struct DevArray<KDNode>;
template struct DevArray<Neighbours>;
template struct DevArray<PGLSampleRecord>;
template struct DevArray<KdJob>;
template struct DevArray<LeafTask>;
template struct DevArray<LeafReport>;
template struct DevArray<LeafProfile>;
template struct DevArray<IStatsAcc>;
template struct DevArray<QueryIn>;
template struct DevArray<QueryOut>;
template struct DevArray<QueryInS4>;
template struct DevArray<DqtHead>;
template struct DevArray<DqtStatsNode>;
template struct DevArray<DqtNode>;
template struct DevArray<Box2>;
template struct DevArray<QueryOutS4>;
template struct DevArray<unsigned long long>;
template struct DevArray<unsigned char>;

// ------------------------------------------------------------------ statistics (host)
// IntegerSampleStatistics frame (SampleStatistics.h:227-241), SSE rcp form.
void quant_frame(const float b[6], float c[3], float inv[3]) {
  for (int d = 0; d < 3; ++d) {
    float ext = b[3 + d] - b[d];
    float half = ext * 0.5f;
    inv[d] = rcp_sse(half);
    c[d] = b[d] + half;
  }
}
// IntegerSampleStatistics::getSampleStatistics (SampleStatistics.h:297-340)
Stats stats_from_acc(const IStatsAcc &a, const float b[6]) {
  Stats s;
  if (a.n == 0) return s;
  float half[3], center[3];
  for (int d = 0; d < 3; ++d) {
    float ext = b[3 + d] - b[d];
    half[d] = ext * 0.5f;
    center[d] = b[d] + half[d];
  }
  uint32_t n = uint32_t(a.n);
  float invN = 1.f / float(n);
  float mean[3], var[3];
  for (int d = 0; d < 3; ++d) {
    mean[d] = (float(a.m[d]) / 4096.f) * invN;
    var[d] = (float(a.v[d]) / 4096.f) * invN;
  }
  for (int d = 0; d < 3; ++d) var[d] -= mean[d] * mean[d];
  for (int d = 0; d < 3; ++d) var[d] = std::fabs(var[d]);
  for (int d = 0; d < 3; ++d) {
    mean[d] = mean[d] * half[d];
    mean[d] += center[d];
    var[d] = var[d] * (half[d] * half[d]);
  }
  for (int d = 0; d < 3; ++d) {
    s.mean[d] = mean[d];
    s.var[d] = var[d] * float(n);
    float lw = (float(a.lo[d]) - 0.0f) / 4096.f;
    lw = lw * half[d];
    lw = lw + center[d];
    float up = (float(a.hi[d]) + 0.0f) / 4096.f;
    up = up * half[d];
    up = up + center[d];
    s.lo[d] = lw;
    s.hi[d] = up;
  }
  s.n = float(n);
  return s;
}
// SampleStatistics::merge (SampleStatistics.h:101-118)
void stats_merge(Stats &a, const Stats &b) {
  float mA[3], mB[3], vA[3], vB[3];
  std::memcpy(mA, a.mean, 12);
  std::memcpy(mB, b.mean, 12);
  std::memcpy(vA, a.var, 12);
  std::memcpy(vB, b.var, 12);
  float nA = a.n, nB = b.n;
  for (int d = 0; d < 3; ++d) a.mean[d] = mA[d] * nA + mB[d] * nB;
  a.n += nB;
  for (int d = 0; d < 3; ++d) a.mean[d] /= a.n;
  for (int d = 0; d < 3; ++d)
    a.var[d] = (((vA[d] + (nA * mA[d]) * mA[d]) + vB[d]) + (nB * mB[d]) * mB[d]) - (a.n * a.mean[d]) * a.mean[d];
  for (int d = 0; d < 3; ++d) {
    a.lo[d] = emin(a.lo[d], b.lo[d]);
    a.hi[d] = emax(a.hi[d], b.hi[d]);
  }
}
// SampleStatistics::split (SampleStatistics.h:68-99)
void stats_split(Stats &s, int dim, float pos, float decay, bool lower) {
  if (s.n > 0.f) {
    float variance = s.var[dim] / s.n;
    float sd = std::sqrt(variance);
    float nv = variance - variance / 4.0f;
    s.var[dim] = nv * s.n;
    if (lower) {
      s.lo[dim] = smax(pos, s.lo[dim]);
      s.mean[dim] = smin(s.hi[dim], s.mean[dim] + sd / 2.0f);
    } else {
      s.hi[dim] = smin(pos, s.hi[dim]);
      s.mean[dim] = smax(s.lo[dim], s.mean[dim] - sd / 2.0f);
    }
    s.n *= decay;
    for (int d = 0; d < 3; ++d) s.var[d] *= decay;
  }
}
float kappa_to_mean_cosine(float k) {  // PAVMM.h:910-918 (scalar, libm tanhf)
  float m = 1.0f / std::tanh(k) - 1.0f / k;
  return k > 0.0f ? m : 0.0f;
}
float cosine_lobe_normalization() {  // VMMSurfaceSamplingDistribution.h:52-60
  return float(double(2.18853f) / (2.0 * kPiD * double(1.0f - std::exp(-2.0f * 2.18853f))));
}

// ------------------------------------------------------------------ storage
void SampleSide::reserve(uint64_t count) {
  P.reserve(count, true);
  D.reserve(count, true);
  pdf.reserve(count, true);
  flags.reserve(count, true);
}

void Storage::add(const PGLSampleRecord *s, size_t n) {
  if (n >= (1u << 16)) {  // large batches go to the device straight from the caller's buffer
    flush();
    ingest(s, n);
    return;
  }
  pending_.insert(pending_.end(), s, s + n);
  if (pending_.size() >= (1u << 16)) flush();
}

void Storage::reserve(size_t ns, size_t nv) {
  flush();
  if (ns > surf.n) surf.reserve(ns);
  if (nv > vol.n) vol.reserve(nv);
}

void Storage::flush() {
  if (pending_.empty()) return;
  std::vector<PGLSampleRecord> p;
  p.swap(pending_);
  ingest(p.data(), p.size());
}
void Storage::flushIfPending() {
  if (!pending_.empty()) flush();
}

void *device_address(const void *host) {
  cudaPointerAttributes a{};
  if (host && cudaPointerGetAttributes(&a, host) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer)
    return a.devicePointer;
  (void)cudaGetLastError();  // an address unknown to CUDA is not an error here
  return nullptr;
}

// Copies n host records to the device and splits them into the surface and
// volume arrays.  Returns after the records have been read (ingest_samples
// synchronises), so the caller may reuse its buffer.  Records in page-locked
// host memory that the device addresses are read in place by the split
// kernels over the host link; other host memory is staged by a copy.
void Storage::ingest(const PGLSampleRecord *src, size_t count) {
  Context &c = Context::get();
  const uint32_t n = uint32_t(count);
  if (const void *dsrc = device_address(src)) {
    lastH2DBytes += uint64_t(n) * sizeof(PGLSampleRecord);
    staging_.reserve(n);
    ingestDevice(static_cast<const PGLSampleRecord *>(dsrc), count, staging_.p);
    return;
  }
  staging_.reserve(n);
  check(cudaMemcpyAsync(staging_.p, src, size_t(n) * sizeof(PGLSampleRecord), cudaMemcpyHostToDevice, c.stream),
        "H2D samples");
  lastH2DBytes += uint64_t(n) * sizeof(PGLSampleRecord);
  ingestDevice(staging_.p, count);
}

// Splits n device-resident records (or host records the device addresses,
// read once into `stage`) into the surface and volume arrays.
void Storage::ingestDevice(const PGLSampleRecord *dsrc, size_t count, PGLSampleRecord *stage) {
  flushIfPending();
  Context &c = Context::get();
  const uint32_t n = uint32_t(count);
  // worst case: every sample in one class
  surf.reserve(surf.n + n);
  vol.reserve(vol.n + n);
  SoAView sv{surf.P.p, surf.D.p, surf.pdf.p, surf.flags.p, surf.n};
  SoAView vv{vol.P.p, vol.D.p, vol.pdf.p, vol.flags.p, vol.n};
  uint32_t numVol = 0;
  check(ingest_samples(dsrc, n, scratch_, sv, vv, &numVol, c.stream, stage), "ingest");
  vol.n += numVol;
  surf.n += n - numVol;
}

std::vector<PGLSampleRecord> Storage::download(bool volume) {
  flush();
  SampleSide &s = volume ? vol : surf;
  std::vector<PGLSampleRecord> out(s.n);
  if (s.n == 0) return out;
  Context &c = Context::get();
  DevArray<PGLSampleRecord> tmp;
  tmp.reserve(s.n);
  check(export_samples(s.P.p, s.D.p, s.pdf.p, s.flags.p, s.n, tmp.p, c.stream), "export");
  check(cudaMemcpyAsync(out.data(), tmp.p, s.n * sizeof(PGLSampleRecord), cudaMemcpyDeviceToHost, c.stream), "D2H");
  check(cudaStreamSynchronize(c.stream), "sync");
  return out;
}

PGLSampleRecord Storage::get(bool volume, uint64_t idx) {
  flush();
  SampleSide &s = volume ? vol : surf;
  PGLSampleRecord r{};
  if (idx >= s.n) return r;
  Context &c = Context::get();
  float4 p, d;
  float pdf;
  uint32_t fl;
  check(cudaMemcpyAsync(&p, s.P.p + idx, sizeof(p), cudaMemcpyDeviceToHost, c.stream), "D2H");
  check(cudaMemcpyAsync(&d, s.D.p + idx, sizeof(d), cudaMemcpyDeviceToHost, c.stream), "D2H");
  check(cudaMemcpyAsync(&pdf, s.pdf.p + idx, sizeof(pdf), cudaMemcpyDeviceToHost, c.stream), "D2H");
  check(cudaMemcpyAsync(&fl, s.flags.p + idx, sizeof(fl), cudaMemcpyDeviceToHost, c.stream), "D2H");
  check(cudaStreamSynchronize(c.stream), "sync");
  r = PGLSampleRecord{p.x, p.y, p.z, d.x, d.y, d.z, d.w, pdf, p.w, fl};
  return r;
}

static bool valid_sample(const PGLSampleRecord &s) {  // SampleData.h:25-46
  bool v = isvalidf(s.px) && isvalidf(s.py) && isvalidf(s.pz);
  v = v && isvalidf(s.dx) && isvalidf(s.dy) && isvalidf(s.dz);
  v = v && isvalidf(s.weight) && s.weight >= 0.f;
  v = v && isvalidf(s.pdf) && s.pdf > 0.f;
  v = v && isvalidf(s.distance) && s.distance > 0.f;
  return v;
}
bool Storage::validate() {
  for (bool v : {false, true})
    for (const PGLSampleRecord &s : download(v))
      if (!valid_sample(s)) return false;
  return true;
}

// ------------------------------------------------------------------ sub-field
void SubField::ensureUniformDirs() {
  if (dUniformDirs.p) return;
  // Spherical Fibonacci directions (WEMFactory.h:668-700), with libm as in the reference
  std::vector<float> d(kMaxK * kMaxK * 3);
  const float gr = 1.618033988749895f;
  for (uint32_t l = 0; l < uint32_t(kMaxK); ++l)
    for (uint32_t n = 0; n < uint32_t(kMaxK); ++n) {
      float *o = &d[(l * kMaxK + n) * 3];
      if (n < l + 1) {
        float phi = float(2.0 * kPiD * double(float(n) / gr));
        float z = 1.0f - ((2.0f * float(n) + 1.0f) / float(l + 1));
        float theta = std::acos(z);
        float ct = std::cos(theta), st = std::sin(theta), cp = std::cos(phi), sp = std::sin(phi);
        o[0] = st * cp;
        o[1] = st * sp;
        o[2] = ct;
      } else {
        o[0] = 0.0f;
        o[1] = 0.0f;
        o[2] = 1.0f;
      }
    }
  dUniformDirs.reserve(d.size());
  check(cudaMemcpy(dUniformDirs.p, d.data(), d.size() * sizeof(float), cudaMemcpyHostToDevice), "uniform dirs");
}

static inline bool is_leaf(const KDNode &n) { return (n.bits >> 30) == 3u; }
static inline uint32_t child_of(const KDNode &n) { return n.bits & 0x3FFFFFFFu; }

void SubField::buildTree(uint32_t n, const float4 *P) {
  struct Front {
    uint32_t node, depth;
    float b[6];
    uint32_t begin, end;
    Stats st;
  };
  std::vector<Front> front;
  Stats rootStats;
  if (is_leaf(nodes[0])) {  // KDTreeBuilder.h:94-115
    KdJob j{};
    quant_frame(kdBounds, j.c, j.inv);
    acc_.reserve(1);
    check(init_acc(acc_.p, 1, stream()), "init acc");
    check(kd_root_stats(posA_.p, n, j, acc_.p, stream()), "root stats");
    IStatsAcc a;
    check(cudaMemcpyAsync(&a, acc_.p, sizeof(a), cudaMemcpyDeviceToHost, stream()), "D2H");
    check(cudaStreamSynchronize(stream()), "sync");
    rootStats = stats_from_acc(a, kdBounds);
  }
  if (!is_leaf(nodes[0]) && n > 0) {
    // One pass down the existing tree instead of one level at a time: each
    // sample goes to the leaf it reaches (the builder's partition rule), the
    // samples are sorted by leaf (depth-first order), and the leaves' sample
    // statistics come from one classification launch, each leaf in its
    // parent's quantisation frame as the level-by-level pass would give them
    // (integer sums: the order does not matter).  The leaves then form the
    // first front; only the leaves that split go on level by level.
    struct Leaf {
      uint32_t node, depth;
      float b[6], pb[6];
    };
    std::vector<Leaf> leaves;
    std::vector<Leaf> stack;
    Leaf r0{0, 1, {}, {}};
    std::memcpy(r0.b, kdBounds, 24);
    std::memcpy(r0.pb, kdBounds, 24);
    stack.push_back(r0);
    while (!stack.empty()) {  // depth-first, left first
      const Leaf t = stack.back();
      stack.pop_back();
      const KDNode &nd = nodes[t.node];
      if (is_leaf(nd)) {
        leaves.push_back(t);
        continue;
      }
      const uint32_t dim = nd.bits >> 30, c = child_of(nd);
      Leaf l{c, t.depth + 1, {}, {}}, r{c + 1, t.depth + 1, {}, {}};
      std::memcpy(l.b, t.b, 24);
      std::memcpy(r.b, t.b, 24);
      std::memcpy(l.pb, t.b, 24);
      std::memcpy(r.pb, t.b, 24);
      l.b[3 + dim] = nd.split;
      r.b[dim] = nd.split;
      stack.push_back(r);
      stack.push_back(l);
    }
    const uint32_t L = uint32_t(leaves.size());
    // page-locked staging: tree, node -> slot, slot -> node, per-leaf jobs, statistics back
    const size_t treeBytes = (nodes.size() * sizeof(KDNode) + 15) & ~size_t(15);
    const size_t mapBytes = (nodes.size() * 4 + 15) & ~size_t(15);
    const size_t slotBytes = (size_t(L) * 4 + 15) & ~size_t(15);
    const size_t jobBytes = (size_t(L) * sizeof(KdJob) + 15) & ~size_t(15);
    const size_t accBytes = 2 * size_t(L) * sizeof(IStatsAcc);
    kdStage_.reserve(treeBytes + mapBytes + slotBytes + jobBytes + accBytes);
    unsigned char *base = kdStage_.p;
    KDNode *hTree = reinterpret_cast<KDNode *>(base);
    uint32_t *hSlot = reinterpret_cast<uint32_t *>(base + treeBytes);
    uint32_t *hNode = reinterpret_cast<uint32_t *>(base + treeBytes + mapBytes);
    KdJob *hJobs = reinterpret_cast<KdJob *>(base + treeBytes + mapBytes + slotBytes);
    IStatsAcc *hAcc = reinterpret_cast<IStatsAcc *>(base + treeBytes + mapBytes + slotBytes + jobBytes);
    std::copy(nodes.begin(), nodes.end(), hTree);
    std::fill(hSlot, hSlot + nodes.size(), ~0u);
    for (uint32_t k = 0; k < L; ++k) {
      hSlot[leaves[k].node] = k;
      hNode[k] = leaves[k].node;
      KdJob j{};
      j.dim = 0;
      j.pos = INFINITY;  // every sample on the "left": one accumulator per leaf
      j.needStats = 1u;
      quant_frame(leaves[k].pb, j.c, j.inv);
      hJobs[k] = j;
    }
    routeNodes_.reserve(nodes.size());
    nodeToJob_.reserve(nodes.size());
    leafSeg_.reserve(L);
    jobs_.reserve(L);
    acc_.reserve(2 * size_t(L));
    keys_.reserve(n);
    vals_.reserve(n);
    keysB_.reserve(n);
    valsB_.reserve(n);
    check(cudaMemcpyAsync(routeNodes_.p, hTree, nodes.size() * sizeof(KDNode), cudaMemcpyHostToDevice, stream()),
          "tree");
    check(cudaMemcpyAsync(nodeToJob_.p, hSlot, nodes.size() * 4, cudaMemcpyHostToDevice, stream()), "node slots");
    check(cudaMemcpyAsync(leafSeg_.p, hNode, size_t(L) * 4, cudaMemcpyHostToDevice, stream()), "slot nodes");
    check(cudaMemcpyAsync(jobs_.p, hJobs, size_t(L) * sizeof(KdJob), cudaMemcpyHostToDevice, stream()), "leaf jobs");
    check(kd_route(posA_.p, n, routeNodes_.p, nodeToJob_.p, L, leafSeg_.p, keys_.p, vals_.p, keysB_.p, valsB_.p,
                   posB_.p, node_.p, scratch_, stream()),
          "route");
    std::swap(posA_.p, posB_.p);
    std::swap(posA_.cap, posB_.cap);
    check(kd_job_of(node_.p, n, nodeToJob_.p, jobOf_.p, acc_.p, 2 * L, stream()), "leaf of");
    check(kd_classify(posA_.p, jobOf_.p, n, jobs_.p, isLeft_.p, acc_.p, stream()), "leaf statistics");
    check(cudaMemcpyAsync(hAcc, acc_.p, accBytes, cudaMemcpyDeviceToHost, stream()), "D2H leaf statistics");
    check(cudaStreamSynchronize(stream()), "sync");
    uint32_t begin = 0;
    for (uint32_t k = 0; k < L; ++k) {
      IStatsAcc a = hAcc[2 * k];
      const IStatsAcc &b = hAcc[2 * k + 1];  // samples with a NaN coordinate
      for (int d = 0; d < 3; ++d) {
        a.m[d] += b.m[d];
        a.v[d] += b.v[d];
        a.lo[d] = std::min(a.lo[d], b.lo[d]);
        a.hi[d] = std::max(a.hi[d], b.hi[d]);
      }
      a.n += b.n;
      Front f{leaves[k].node, leaves[k].depth, {}, begin, begin + uint32_t(a.n), stats_from_acc(a, leaves[k].pb)};
      std::memcpy(f.b, leaves[k].b, 24);
      front.push_back(f);
      begin += uint32_t(a.n);
    }
    if (begin != n) throw std::runtime_error("kd descent lost samples");
  } else {
    Front root{0, 1, {}, 0, n, rootStats};
    std::memcpy(root.b, kdBounds, 24);
    front.push_back(root);
    check(cudaMemsetAsync(node_.p, 0, size_t(n) * 4, stream()), "node ids");
  }

  std::vector<KdJob> jobs;
  std::vector<const Front *> jobFront;
  std::vector<IStatsAcc> acc;
  const uint32_t oldRegions = uint32_t(regions.size());
  while (!front.empty()) {
    jobs.clear();
    jobFront.clear();
    for (Front &f : front) {
      if (f.end == f.begin) continue;
      if (is_leaf(nodes[f.node])) {
        uint32_t r = child_of(nodes[f.node]);
        if (f.depth < cfg.maxDepth && regions[r].stats.n + float(f.end - f.begin) > float(cfg.maxSamples)) {
          // split (KDTreeBuilder.h:252-284)
          Stats merged = regions[r].stats;
          stats_merge(merged, f.st);
          float v[3] = {merged.var[0] / merged.n, merged.var[1] / merged.n, merged.var[2] / merged.n};
          int i = v[1] > v[0] ? 1 : 0;
          int dim = v[i] > v[2] ? i : 2;
          float pos = merged.mean[dim];
          RegionHost right = regions[r];
          stats_split(regions[r].stats, dim, pos, 0.25f, false);
          stats_split(right.stats, dim, pos, 0.25f, true);
          regions[r].splitFlag = true;
          right.splitFlag = true;
          regions[r].bounds[3 + dim] = pos;
          right.bounds[dim] = pos;
          regions.push_back(right);
          uint32_t rightIdx = uint32_t(regions.size() - 1);
          regionOrigin_.push_back(r < oldRegions ? r : regionOrigin_[r - oldRegions]);
          uint32_t lr0 = uint32_t(nodes.size());
          nodes.push_back(KDNode{0.0f, (3u << 30) | r});
          nodes.push_back(KDNode{0.0f, (3u << 30) | rightIdx});
          nodes[f.node].split = pos;
          nodes[f.node].bits = (uint32_t(dim) << 30) | lr0;
          splitNodes_.push_back(f.node);
        } else {
          stats_merge(regions[r].stats, f.st);
          regions[r].rb = f.begin;
          regions[r].re = f.end;
          continue;
        }
      }
      const KDNode &nd = nodes[f.node];
      KdJob j{};
      j.begin = f.begin;
      j.end = f.end;
      j.dim = nd.bits >> 30;
      j.left = child_of(nd);
      j.pos = nd.split;
      j.needStats = (is_leaf(nodes[j.left]) || is_leaf(nodes[j.left + 1])) ? 1u : 0u;
      quant_frame(f.b, j.c, j.inv);
      jobs.push_back(j);
      jobFront.push_back(&f);
    }
    if (jobs.empty()) break;
    // the level's jobs, node map and (coming back) child statistics share one
    // page-locked block: the copies run asynchronously; the previous level's
    // copies are done (its statistics were read after a synchronisation)
    const size_t jobBytes = (jobs.size() * sizeof(KdJob) + 15) & ~size_t(15);
    const size_t mapBytes = (nodes.size() * 4 + 15) & ~size_t(15);
    const size_t accBytes = 2 * jobs.size() * sizeof(IStatsAcc);
    kdStage_.reserve(jobBytes + mapBytes + accBytes);
    KdJob *hJobs = reinterpret_cast<KdJob *>(kdStage_.p);
    uint32_t *hMap = reinterpret_cast<uint32_t *>(kdStage_.p + jobBytes);
    IStatsAcc *hAcc = reinterpret_cast<IStatsAcc *>(kdStage_.p + jobBytes + mapBytes);
    std::copy(jobs.begin(), jobs.end(), hJobs);
    std::fill(hMap, hMap + nodes.size(), ~0u);
    for (size_t k = 0; k < jobs.size(); ++k) hMap[jobFront[k]->node] = uint32_t(k);
    jobs_.reserve(jobs.size());
    nodeToJob_.reserve(nodes.size());
    acc_.reserve(2 * jobs.size());
    check(cudaMemcpyAsync(jobs_.p, hJobs, jobs.size() * sizeof(KdJob), cudaMemcpyHostToDevice, stream()), "jobs");
    check(cudaMemcpyAsync(nodeToJob_.p, hMap, nodes.size() * 4, cudaMemcpyHostToDevice, stream()), "node map");
    check(kd_job_of(node_.p, n, nodeToJob_.p, jobOf_.p, acc_.p, uint32_t(2 * jobs.size()), stream()), "job of");
    check(kd_level(posA_.p, jobOf_.p, n, jobs_.p, isLeft_.p, scanLeft_.p, acc_.p, posB_.p, nodeB_.p, scratch_,
                   stream()),
          "kd level");
    std::swap(posA_.p, posB_.p);
    std::swap(posA_.cap, posB_.cap);
    std::swap(node_.p, nodeB_.p);
    std::swap(node_.cap, nodeB_.cap);
    check(cudaMemcpyAsync(hAcc, acc_.p, accBytes, cudaMemcpyDeviceToHost, stream()), "D2H acc");
    check(cudaStreamSynchronize(stream()), "sync");
    acc.assign(hAcc, hAcc + 2 * jobs.size());
    std::vector<Front> next;
    next.reserve(2 * jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k) {
      const KdJob &j = jobs[k];
      const Front &f = *jobFront[k];
      uint32_t nL = uint32_t(acc[2 * k].n), nR = uint32_t(acc[2 * k + 1].n);
      Front L{j.left, f.depth + 1, {}, j.begin, j.begin + nL, Stats()};
      Front R{j.left + 1, f.depth + 1, {}, j.begin + nL, j.begin + nL + nR, Stats()};
      std::memcpy(L.b, f.b, 24);
      std::memcpy(R.b, f.b, 24);
      L.b[3 + j.dim] = j.pos;
      R.b[j.dim] = j.pos;
      if (j.needStats) {
        L.st = stats_from_acc(acc[2 * k], f.b);
        R.st = stats_from_acc(acc[2 * k + 1], f.b);
      }
      next.push_back(L);
      next.push_back(R);
    }
    front.swap(next);
  }
}

// Region and node numbering of the reference's depth-first build: the pair of
// children of a split node is appended when the node is split, and splits
// happen in depth-first, left-first order (KDTreeBuilder.h:271-280,346-349).
void SubField::renumber(uint32_t oldNodes, uint32_t oldRegions) {
  const uint32_t numSplits = uint32_t(splitNodes_.size());
  if (numSplits == 0) return;
  std::vector<uint32_t> splitIdx(nodes.size(), ~0u);
  for (uint32_t k = 0; k < numSplits; ++k) splitIdx[splitNodes_[k]] = k;
  std::vector<uint32_t> ord(numSplits, ~0u);
  uint32_t next = 0;
  std::vector<uint32_t> stack{0};
  while (!stack.empty()) {
    uint32_t i = stack.back();
    stack.pop_back();
    if (splitIdx[i] != ~0u) ord[splitIdx[i]] = next++;
    if (!is_leaf(nodes[i])) {
      stack.push_back(child_of(nodes[i]) + 1);
      stack.push_back(child_of(nodes[i]));
    }
  }
  auto mapNode = [&](uint32_t i) -> uint32_t {
    if (i < oldNodes) return i;
    uint32_t k = (i - oldNodes) / 2, c = (i - oldNodes) % 2;
    return oldNodes + 2 * ord[k] + c;
  };
  auto mapRegion = [&](uint32_t r) -> uint32_t { return r < oldRegions ? r : oldRegions + ord[r - oldRegions]; };
  std::vector<KDNode> nn(nodes.size());
  for (uint32_t i = 0; i < nodes.size(); ++i) {
    KDNode d = nodes[i];
    if (is_leaf(d))
      d.bits = (3u << 30) | mapRegion(child_of(d));
    else
      d.bits = (d.bits & 0xC0000000u) | mapNode(child_of(d));
    nn[mapNode(i)] = d;
  }
  nodes.swap(nn);
  std::vector<RegionHost> nr(regions.size());
  std::vector<uint32_t> no(regionOrigin_.size());
  for (uint32_t r = 0; r < regions.size(); ++r) nr[mapRegion(r)] = regions[r];
  for (uint32_t k = 0; k < regionOrigin_.size(); ++k) no[ord[k]] = regionOrigin_[k];
  regions.swap(nr);
  regionOrigin_.swap(no);
}

bool SubField::prepare(SampleSide &in) {
  const uint32_t n = uint32_t(in.n);
  pending.clear();
  if (n == 0) {
    timings = UpdateTimings{};
    lastReports.clear();
    lastProfiles.clear();
    lastReportRegion.clear();
    return false;
  }
  cudaEvent_t *ev = events;
  for (int k = 0; k < 4; ++k)
    if (!ev[k]) check(cudaEventCreate(&ev[k]), "event");
  check(cudaEventRecord(ev[0], stream()), "event");
  const bool first = !initialized;
  if (first) {
    iteration = 0;
    totalSPP = 0;
  }
  for (DevArray<float4> *a : {&posA_, &posB_, &sP_, &sD_, &tmpP_, &tmpD_}) a->reserve(n);
  for (DevArray<float> *a : {&sPdf_, &tmpPdf_, &dist_}) a->reserve(n);
  for (DevArray<uint32_t> *a : {&node_, &nodeB_, &jobOf_, &isLeft_, &scanLeft_}) a->reserve(n);
  keys_.reserve(2 * size_t(n));
  vals_.reserve(2 * size_t(n));
  keys64_.reserve(2 * size_t(n));
  check(init_posidx(in.P.p, n, posA_.p, stream()), "copy samples");
  check(cudaEventRecord(ev[1], stream()), "event");

  if (first) {
    if (!boundsSet) {  // Field.h:326-344
      bounds6_.reserve(6);
      check(scene_bounds(in.P.p, n - 1, bounds6_.p, stream()), "bounds");
      uint32_t o[6];
      check(cudaMemcpyAsync(o, bounds6_.p, sizeof(o), cudaMemcpyDeviceToHost, stream()), "D2H");
      check(cudaStreamSynchronize(stream()), "sync");
      float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
      if (n > 1)
        for (int d = 0; d < 3; ++d) {
          uint32_t a = o[d], b = o[3 + d];
          uint32_t ua = (a & 0x80000000u) ? (a & 0x7FFFFFFFu) : ~a;
          uint32_t ub = (b & 0x80000000u) ? (b & 0x7FFFFFFFu) : ~b;
          float fa, fb;
          std::memcpy(&fa, &ua, 4);
          std::memcpy(&fb, &ub, 4);
          lo[d] = emin(FLT_MAX, fa);
          hi[d] = emax(FLT_MIN, fb);
        }
      for (int d = 0; d < 3; ++d) {
        float ctr = (lo[d] + hi[d]) / 2.0f;
        sceneBounds[d] = ctr + 3.0f * (lo[d] - ctr);
        sceneBounds[3 + d] = ctr + 3.0f * (hi[d] - ctr);
      }
      boundsSet = true;
    }
    std::memcpy(kdBounds, sceneBounds, 24);
    kdInit = true;
    nodes.assign(1, KDNode{0.0f, (3u << 30) | 0u});
    regions.assign(1, RegionHost());
    std::memcpy(regions[0].bounds, sceneBounds, 24);
    dRegions.reserve(1);
    check(cudaMemsetAsync(dRegions.p, 0, sizeof(RegionDir), stream()), "region 0");
    if (cfg.dqt) {
      dqtReserve(1);
      check(launch_dqt_init(dDqtHeads.p, dDqtStats.p, dDqtNodes.p, dqtStride, 0, 1, stream()), "quadtree 0");
    }
  }
  const uint32_t oldNodes = uint32_t(nodes.size()), oldRegions = uint32_t(regions.size());
  splitNodes_.clear();
  regionOrigin_.clear();
  buildTree(n, in.P.p);
  renumber(oldNodes, oldRegions);
  const uint32_t R = uint32_t(regions.size());
  dRegions.reserve(R, true);
  if (R > oldRegions) {  // new regions start as copies of the region they split from
    std::vector<uint32_t> idx(2 * (R - oldRegions));
    for (uint32_t k = 0; k < R - oldRegions; ++k) {
      idx[k] = oldRegions + k;
      idx[(R - oldRegions) + k] = regionOrigin_[k];
    }
    copyIdx_.reserve(idx.size());
    check(cudaMemcpyAsync(copyIdx_.p, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, stream()), "copy idx");
    check(copy_regions(dRegions.p, copyIdx_.p, copyIdx_.p + (R - oldRegions), R - oldRegions, stream()), "copy");
    if (cfg.dqt) {
      dqtReserve(R);
      check(launch_dqt_copy(dDqtHeads.p, dDqtStats.p, dDqtNodes.p, dqtStride, copyIdx_.p, copyIdx_.p + (R - oldRegions),
                            R - oldRegions, stream()),
            "copy quadtrees");
    }
  }
  if (cfg.knn) {  // Field.h:362-387 -> KNN.h:189-266
    std::vector<float4> m(R);
    for (uint32_t r = 0; r < R; ++r) m[r] = make_float4(regions[r].stats.mean[0], regions[r].stats.mean[1],
                                                        regions[r].stats.mean[2], 0.0f);
    means_.reserve(R);
    dNbrs.reserve(R);
    check(cudaMemcpyAsync(means_.p, m.data(), R * sizeof(float4), cudaMemcpyHostToDevice, stream()), "means");
    check(build_knn(means_.p, R, dNbrs.p, stream()), "knn");
  }
  dNodes.reserve(nodes.size());
  check(cudaMemcpyAsync(dNodes.p, nodes.data(), nodes.size() * sizeof(KDNode), cudaMemcpyHostToDevice, stream()),
        "nodes");
  check(cudaEventRecord(ev[2], stream()), "event");

  // leaves in sample order, then the per-leaf deterministic order
  std::vector<uint32_t> leafRegions;
  for (uint32_t r = 0; r < R; ++r)
    if (regions[r].re > regions[r].rb) leafRegions.push_back(r);
  std::sort(leafRegions.begin(), leafRegions.end(),
            [&](uint32_t a, uint32_t b) { return regions[a].rb < regions[b].rb; });
  const uint32_t L = uint32_t(leafRegions.size());
  std::vector<uint32_t> seg(3 * size_t(L));
  for (uint32_t k = 0; k < L; ++k) {
    seg[k] = uint32_t(regions[leafRegions[k]].rb);
    seg[L + k] = uint32_t(regions[leafRegions[k]].re);
    seg[2 * L + k] = uint32_t(regions[leafRegions[k]].re - regions[leafRegions[k]].rb);
  }
  leafSeg_.reserve(seg.size());
  check(cudaMemcpyAsync(leafSeg_.p, seg.data(), seg.size() * 4, cudaMemcpyHostToDevice, stream()), "segments");
  check(gather_and_order(posA_.p, n, in.P.p, in.D.p, in.pdf.p, leafSeg_.p, leafSeg_.p + 2 * L, L, cfg.deterministic,
                         tmpP_.p, tmpD_.p, tmpPdf_.p, keys_.p, vals_.p, keys64_.p, sP_.p, sD_.p, sPdf_.p, scratch_,
                         stream()),
        "gather");

  // directional fit / update of every region (Field.h:389-511)
  std::vector<LeafTask> tasks(R);
  for (uint32_t r = 0; r < R; ++r) {
    LeafTask &t = tasks[r];
    const RegionHost &h = regions[r];
    t.region = r;
    t.begin = uint32_t(h.rb);
    t.count = uint32_t(h.re - h.rb);
    t.flags = (first ? kTaskFit : 0u) | (h.splitFlag ? kTaskDecay : 0u);
    for (int d = 0; d < 3; ++d) {
      t.mean[d] = h.stats.mean[d];
      t.varOverN[d] = h.stats.var[d] / h.stats.n;
    }
  }
  pending = std::move(tasks);
  ensureUniformDirs();
  check(cudaEventRecord(ev[3], stream()), "event");
  pendingSamples_ = n;
  return true;
}

EmSide SubField::emSide() { return EmSide{dRegions.p, sP_.p, sD_.p, sPdf_.p, dist_.p, dUniformDirs.p, cfg}; }

void SubField::finish(std::vector<LeafReport> reports, std::vector<LeafProfile> profiles,
                      std::vector<uint32_t> regionOf, cudaEvent_t emStart, cudaEvent_t emEnd) {
  const uint32_t R = uint32_t(regions.size());
  lastReports = std::move(reports);
  lastProfiles = std::move(profiles);
  lastReportRegion = std::move(regionOf);
  for (size_t k = 0; k < lastProfiles.size(); ++k)
    if (lastReportRegion[k] < R) regions[lastReportRegion[k]].lastCost = lastProfiles[k].cycTotal;
  float ms[6];
  check(cudaEventElapsedTime(&ms[0], events[0], emEnd), "timing");
  check(cudaEventElapsedTime(&ms[1], events[0], events[1]), "timing");
  check(cudaEventElapsedTime(&ms[2], events[1], events[2]), "timing");
  check(cudaEventElapsedTime(&ms[3], events[2], emEnd), "timing");
  check(cudaEventElapsedTime(&ms[4], events[2], events[3]), "timing");
  check(cudaEventElapsedTime(&ms[5], emStart, emEnd), "timing");
  timings = UpdateTimings{ms[0], ms[1], ms[2], ms[3], ms[4], ms[5], uint64_t(pendingSamples_), R};
  for (RegionHost &h : regions) {
    h.splitFlag = false;
    h.rb = h.re = 0;
  }
  pending.clear();
  initialized = true;
  iteration++;
}

void SubField::reset() {  // Field.h:222-233
  iteration = 0;
  totalSPP = 0;
  boundsSet = false;
  initialized = false;
  kdInit = false;
  nodes.clear();
  regions.clear();
}

FieldView SubField::view() const {
  FieldView v{};
  v.nodes = dNodes.p;
  v.regions = dRegions.p;
  v.nbrs = dNbrs.p;
  std::memcpy(v.bounds, kdBounds, 24);
  v.iteration = (initialized && !nodes.empty()) ? uint32_t(iteration) : 0u;
  v.knn = cfg.knn;
  v.numNodes = uint32_t(nodes.size());
  v.parallax = cfg.parallax;
  v.dqt = cfg.dqt;
  v.dqtHeads = dDqtHeads.p;
  v.dqtNodes = dDqtNodes.p;
  v.dqtStride = dqtStride;
  return v;
}

// Node slots per region for the factory's arguments (at most the tree the
// arguments allow); growing the region count keeps the existing quadtrees.
void SubField::dqtReserve(uint32_t R) {
  const uint64_t bound = dqt_max_nodes(cfg.dqtArgs);
  if (bound > (uint64_t(1) << 18))
    throw std::runtime_error("quadtree factory arguments allow trees of more than 262144 nodes");
  const uint32_t stride = uint32_t(bound);
  if (dqtStride != 0 && dqtStride != stride) throw std::runtime_error("quadtree node stride changed");
  dqtStride = stride;
  dDqtHeads.reserve(R, true);
  dDqtStats.reserve(size_t(R) * stride, true);
  dDqtNodes.reserve(size_t(R) * stride, true);
}
DqtSide SubField::dqtSide() {
  return DqtSide{dDqtHeads.p, dDqtStats.p, dDqtNodes.p, dqtStride, sD_.p, sPdf_.p, cfg.dqtArgs, cfg.decayOnSpatialSplit};
}

std::vector<RegionDir> SubField::downloadRegions() const {
  std::vector<RegionDir> r(regions.size());
  if (r.empty()) return r;
  Context &c = Context::get();
  check(cudaMemcpyAsync(r.data(), dRegions.p, r.size() * sizeof(RegionDir), cudaMemcpyDeviceToHost, c.stream), "D2H");
  check(cudaStreamSynchronize(c.stream), "sync");
  return r;
}

// Device copies of the tree and the region neighbours after a load.
void SubField::uploadTree() {
  cudaStream_t st = stream();
  dNodes.reserve(std::max<size_t>(nodes.size(), 1));
  if (!nodes.empty())
    check(cudaMemcpyAsync(dNodes.p, nodes.data(), nodes.size() * sizeof(KDNode), cudaMemcpyHostToDevice, st), "nodes");
  const uint32_t R = uint32_t(regions.size());
  if (cfg.knn && R > 0) {
    std::vector<float4> m(R);
    for (uint32_t i = 0; i < R; ++i)
      m[i] = make_float4(regions[i].stats.mean[0], regions[i].stats.mean[1], regions[i].stats.mean[2], 0.0f);
    means_.reserve(R);
    dNbrs.reserve(R);
    check(cudaMemcpyAsync(means_.p, m.data(), R * sizeof(float4), cudaMemcpyHostToDevice, st), "means");
    check(build_knn(means_.p, R, dNbrs.p, st), "knn");
  }
  check(cudaStreamSynchronize(st), "load");
}

void SubField::uploadRegions(const std::vector<RegionDir> &r) {
  if (r.empty()) return;
  dRegions.reserve(r.size());
  check(cudaMemcpy(dRegions.p, r.data(), r.size() * sizeof(RegionDir), cudaMemcpyHostToDevice), "H2D regions");
}

bool SubField::valid() const {  // Field::isValid (Field.h:307-317)
  if (cfg.dqt) {
    std::vector<DqtHead> h(regions.size());
    if (!h.empty())
      check(cudaMemcpy(h.data(), dDqtHeads.p, h.size() * sizeof(DqtHead), cudaMemcpyDeviceToHost), "D2H");
    for (const DqtHead &q : h)
      if (!q.valid) return false;
    return true;
  }
  for (const RegionDir &r : downloadRegions())
    if (!r.valid) return false;
  return true;
}

// ------------------------------------------------------------------ field
GpuField::GpuField(const FieldConfig &cfg) {
  surface.cfg = cfg;
  volume.cfg = cfg;
  surface.isSurface = true;
  volume.isSurface = false;
}

void GpuField::update(Storage &s, bool doSurface, bool doVolume) {  // SurfaceVolumeField.h:102-148
  s.flush();
  const bool surf = doSurface && s.surf.n > 0, vol = doVolume && s.vol.n > 0;
  if (doSurface && !surf) surface.prepare(s.surf);  // clears the last update's counters
  if (doVolume && !vol) volume.prepare(s.vol);
  SubField *sides[2];
  int count = 0;
  if (surf && vol) {
    // the two trees are independent: each is built on its own stream from
    // its own host thread, so their kernels overlap on the GPU
    std::exception_ptr err;
    int device = 0;
    check(cudaGetDevice(&device), "cudaGetDevice");
    std::thread t([&] {
      try {
        check(cudaSetDevice(device), "cudaSetDevice");
        volume.prepare(s.vol);
      } catch (...) {
        err = std::current_exception();
      }
    });
    try {
      surface.prepare(s.surf);
    } catch (...) {
      t.join();
      throw;
    }
    t.join();
    if (err) std::rethrow_exception(err);
    sides[count++] = &surface;
    sides[count++] = &volume;
  } else if (surf) {
    if (surface.prepare(s.surf)) sides[count++] = &surface;
  } else if (vol) {
    if (volume.prepare(s.vol)) sides[count++] = &volume;
  }
  if (count > 0) {
    if (surface.cfg.dqt) runDqt(sides, count);
    else runEm(sides, count);
  }
  iteration++;
}

// The quadtree field type's fit / update of every region of the prepared
// sub-fields (Field.h:389-511 -> DQTFactory.h:149-281), one launch for both:
// persistent blocks take regions, largest first, from a queue.
void GpuField::runDqt(SubField *const *sides, int count) {
  Context &c = Context::get();
  cudaStream_t s = c.stream;
  std::vector<std::pair<uint32_t, LeafTask>> keyed;
  DqtSides ds{};
  uint32_t stride = 0;
  for (int i = 0; i < count; ++i) {
    SubField &f = *sides[i];
    check(cudaStreamWaitEvent(s, f.events[3], 0), "wait");
    const uint32_t side = f.isSurface ? 0u : kTaskVolume;
    ds.side[f.isSurface ? 0 : 1] = f.dqtSide();
    stride = std::max(stride, f.dqtStride);
    if (!f.cfg.fitRegions) continue;
    for (LeafTask t : f.pending) {
      t.flags |= side;
      keyed.emplace_back(t.count, t);
    }
  }
  std::stable_sort(keyed.begin(), keyed.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
  std::vector<LeafTask> all;
  for (auto &k : keyed) all.push_back(k.second);
  const uint32_t T = uint32_t(all.size());
  // two blocks per SM, on the SMs the schedule leaves to the Update
  const int sms = std::max(1, c.numSMs - std::max(0, tuning.reservedSMs));
  const int blocks = int(std::min<uint32_t>(std::max<uint32_t>(T, 1), uint32_t(2 * sms)));
  cudaEvent_t emStart, emEnd;
  check(cudaEventCreate(&emStart), "event");
  check(cudaEventCreate(&emEnd), "event");
  int err = 0;
  if (T > 0) {
    tasks_.reserve(T);
    queue_.reserve(2);
    dqtRects_.reserve(size_t(blocks) * stride);
    dqtBuild_.reserve(size_t(blocks) * stride);
    dqtLeaves_.reserve(size_t(blocks) * stride);
    check(cudaMemcpyAsync(tasks_.p, all.data(), T * sizeof(LeafTask), cudaMemcpyHostToDevice, s), "tasks");
    check(cudaMemsetAsync(queue_.p, 0, 2 * sizeof(unsigned int), s), "queue");
  }
  check(cudaEventRecord(emStart, s), "event");
  if (T > 0)
    check(launch_dqt_update(tasks_.p, T, queue_.p, ds, dqtRects_.p, dqtBuild_.p, dqtLeaves_.p, stride, blocks,
                            reinterpret_cast<int *>(queue_.p + 1), s),
          "quadtree update");
  check(cudaEventRecord(emEnd, s), "event");
  if (T > 0)
    check(cudaMemcpyAsync(&err, queue_.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s), "quadtree status");
  check(cudaStreamSynchronize(s), "update");
  if (err != 0) {
    cudaEventDestroy(emStart);
    cudaEventDestroy(emEnd);
    throw std::runtime_error("quadtree update: a tree outgrew its node slots");
  }
  for (int i = 0; i < count; ++i) {
    SubField &f = *sides[i];
    std::vector<uint32_t> region;
    for (const LeafTask &t : all)
      if (((t.flags & kTaskVolume) != 0) == !f.isSurface) region.push_back(t.region);
    f.finish(std::vector<LeafReport>(region.size()), std::vector<LeafProfile>(region.size()), std::move(region),
             emStart, emEnd);
  }
  cudaEventDestroy(emStart);
  cudaEventDestroy(emEnd);
}

// Directional fit / update of every region of the prepared sub-fields
// (Field.h:389-511) in one launch: the leaves of both, largest first, share
// one queue, and blocks without a leaf help the remaining leaves' E-steps.
// The leaf tasks of the prepared sub-fields in queue order, largest first:
// by the previous Update's measured cost of the region (when asked and
// known), else by sample count.
std::vector<LeafTask> GpuField::emOrder(SubField *const *sides, int count, bool byCost) const {
  std::vector<std::pair<uint64_t, LeafTask>> keyed;
  for (int i = 0; i < count; ++i) {
    const SubField &f = *sides[i];
    if (!f.cfg.fitRegions) continue;
    for (LeafTask t : f.pending) {
      if (!f.isSurface) t.flags |= kTaskVolume;
      const uint64_t cost = f.regions[t.region].lastCost;
      keyed.emplace_back(byCost && cost > 0 ? cost : uint64_t(t.count), t);
    }
  }
  std::stable_sort(keyed.begin(), keyed.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
  std::vector<LeafTask> all;
  all.reserve(keyed.size());
  for (const auto &k : keyed) all.push_back(k.second);
  return all;
}

// Times every candidate schedule on this Update's leaves: the state an EM
// launch changes (regions, the samples' reprojected directions and
// distances) is saved, restored before each trial and after the last, so
// the Update itself then runs once more with the fastest schedule and gives
// the same field as without tuning.
void GpuField::autotuneEm(SubField *const *sides, int count, cudaStream_t s) {
  Context &c = Context::get();
  struct Piece {
    void *dev;
    size_t bytes;
  };
  std::vector<Piece> pieces;
  for (int i = 0; i < count; ++i) {
    const EmSide e = sides[i]->emSide();
    const size_t n = sides[i]->pendingSamples();
    pieces.push_back({e.regions, sides[i]->regions.size() * sizeof(RegionDir)});
    pieces.push_back({e.dirw, n * sizeof(float4)});
    pieces.push_back({e.dist, n * sizeof(float)});
  }
  size_t total = 0;
  for (const Piece &p : pieces) total += (p.bytes + 255) & ~size_t(255);
  tuneSnap_.reserve(total);
  auto copyAll = [&](bool save) {
    size_t off = 0;
    for (const Piece &p : pieces) {
      void *snap = tuneSnap_.p + off;
      check(cudaMemcpyAsync(save ? snap : p.dev, save ? p.dev : snap, p.bytes, cudaMemcpyDeviceToDevice, s),
            "tuning snapshot");
      off += (p.bytes + 255) & ~size_t(255);
    }
  };
  copyAll(true);
  bool costs = false;
  for (int i = 0; i < count; ++i)
    for (const RegionHost &h : sides[i]->regions) costs = costs || h.lastCost > 0;
  EmSides es{};
  for (int i = 0; i < count; ++i) es.side[sides[i]->isSurface ? 0 : 1] = sides[i]->emSide();
  lastTuneTrials.clear();
  cudaEvent_t e0, e1;
  check(cudaEventCreate(&e0), "event");
  check(cudaEventCreate(&e1), "event");
  float bestMs = 0.0f;
  EmTuning best = tuning;
  for (int order = 0; order <= (costs ? 1 : 0); ++order) {
    const std::vector<LeafTask> all = emOrder(sides, count, order != 0);
    const uint32_t T = uint32_t(all.size());
    if (T == 0) break;
    tasks_.reserve(T);
    reports_.reserve(T);
    profiles_.reserve(T);
    queue_.reserve(1);
    emShare_.reserve(em_share_bytes(c.numSMs));
    check(cudaMemcpyAsync(tasks_.p, all.data(), T * sizeof(LeafTask), cudaMemcpyHostToDevice, s), "tasks");
    for (int helpers : {2, 4, 8})
      for (int div : {1, 2}) {
        const EmTuning t{helpers, div, 8, order};
        copyAll(false);
        check(cudaMemsetAsync(queue_.p, 0, sizeof(unsigned int), s), "queue");
        check(cudaEventRecord(e0, s), "event");
        check(launch_em(tasks_.p, T, queue_.p, es, reports_.p, profiles_.p, emShare_.p, c.numSMs, t, s), "em");
        check(cudaEventRecord(e1, s), "event");
        int emError = 0;
        check(cudaMemcpyAsync(&emError, emShare_.p + em_share_error_offset(c.numSMs), sizeof(int),
                              cudaMemcpyDeviceToHost, s),
              "EM status");
        check(cudaStreamSynchronize(s), "tuning trial");
        if (emError != 0) throw std::runtime_error("directional fit failed in a tuning trial (code " +
                                                   std::to_string(emError) + ")");
        float ms = 0.0f;
        check(cudaEventElapsedTime(&ms, e0, e1), "timing");
        lastTuneTrials.push_back({t, ms});
        if (lastTuneTrials.size() == 1 || ms < bestMs) {
          bestMs = ms;
          best = t;
        }
      }
  }
  copyAll(false);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  tuning = best;
}

void GpuField::runEm(SubField *const *sides, int count) {
  Context &c = Context::get();
  cudaStream_t s = sides[0]->stream();
  EmSides es{};
  for (int i = 0; i < count; ++i) {
    SubField &f = *sides[i];
    es.side[f.isSurface ? 0 : 1] = f.emSide();
    if (i > 0) check(cudaStreamWaitEvent(s, f.events[3], 0), "wait for the other tree");
  }
  if (autotuneNext) {
    autotuneNext = false;
    autotuneEm(sides, count, s);
  }
  const std::vector<LeafTask> all = emOrder(sides, count, tuning.orderByCost != 0);
  const uint32_t T = uint32_t(all.size());
  cudaEvent_t emStart, emEnd;
  check(cudaEventCreate(&emStart), "event");
  check(cudaEventCreate(&emEnd), "event");
  std::vector<LeafReport> reports(T);
  std::vector<LeafProfile> profiles(T);
  int emError = 0;
  // the plain form: the surface regions, then the volume regions, each side
  // one launch with one block per region
  const bool plain = tuning.plainLaunches != 0;
  uint32_t sideCount[2] = {0, 0};
  for (const LeafTask &t : all) ++sideCount[(t.flags & kTaskVolume) ? 1 : 0];
  const uint32_t plainMax = std::max(sideCount[0], sideCount[1]);
  int emErrors[2] = {0, 0};
  if (T > 0) {
    tasks_.reserve(T);
    reports_.reserve(T);
    profiles_.reserve(T);
    queue_.reserve(1);
    emShare_.reserve(plain ? 2 * em_share_bytes_plain(int(plainMax)) : em_share_bytes(c.numSMs));
    check(cudaMemcpyAsync(tasks_.p, all.data(), T * sizeof(LeafTask), cudaMemcpyHostToDevice, s), "tasks");
    check(cudaMemsetAsync(queue_.p, 0, sizeof(unsigned int), s), "queue");
  }
  check(cudaEventRecord(emStart, s), "event");
  // the batched form: one persistent launch for every region of both
  // sub-fields (blocks take regions from a queue and, once out of regions,
  // help the others' E-step passes)
  const int blocks = std::max(1, c.numSMs - std::max(0, tuning.reservedSMs));
  if (T > 0 && !plain)
    check(launch_em(tasks_.p, T, queue_.p, es, reports_.p, profiles_.p, emShare_.p, blocks, tuning, s), "em");
  std::vector<uint32_t> plainOrder;  // task index of launch position k (plain form)
  if (T > 0 && plain) {
    std::vector<LeafTask> bySide;
    for (int side = 0; side < 2; ++side)
      for (uint32_t k = 0; k < T; ++k)
        if (((all[k].flags & kTaskVolume) ? 1 : 0) == side) {
          bySide.push_back(all[k]);
          plainOrder.push_back(k);
        }
    check(cudaMemcpyAsync(tasks_.p, bySide.data(), T * sizeof(LeafTask), cudaMemcpyHostToDevice, s), "tasks");
    uint32_t first = 0;
    for (int side = 0; side < 2; ++side) {
      const uint32_t n = sideCount[side];
      if (n == 0) continue;
      unsigned char *share = emShare_.p + size_t(side) * em_share_bytes_plain(int(plainMax));
      check(launch_em(tasks_.p + first, n, queue_.p, es, reports_.p + first, profiles_.p + first, share, int(n),
                      tuning, s),
            "em (plain)");
      check(cudaMemcpyAsync(&emErrors[side], share + em_share_error_offset(int(n)), sizeof(int),
                            cudaMemcpyDeviceToHost, s),
            "EM status");
      first += n;
    }
  }
  check(cudaEventRecord(emEnd, s), "event");
  if (T > 0) {
    check(cudaMemcpyAsync(profiles.data(), profiles_.p, T * sizeof(LeafProfile), cudaMemcpyDeviceToHost, s),
          "profiles");
    check(cudaMemcpyAsync(reports.data(), reports_.p, T * sizeof(LeafReport), cudaMemcpyDeviceToHost, s), "reports");
    if (!plain)
      check(cudaMemcpyAsync(&emError, emShare_.p + em_share_error_offset(blocks), sizeof(int),
                            cudaMemcpyDeviceToHost, s),
            "EM status");
  }
  check(cudaStreamSynchronize(s), "update");
  if (plain) {
    emError = emErrors[0] != 0 ? emErrors[0] : emErrors[1];
    // back to the order of `all`
    std::vector<LeafReport> r(T);
    std::vector<LeafProfile> p(T);
    for (uint32_t k = 0; k < T; ++k) {
      r[plainOrder[k]] = reports[k];
      p[plainOrder[k]] = profiles[k];
    }
    reports.swap(r);
    profiles.swap(p);
  }
  if (emError != 0) {
    cudaEventDestroy(emStart);
    cudaEventDestroy(emEnd);
    throw std::runtime_error("directional fit failed: a wait between EM blocks ran out (code " +
                             std::to_string(emError) + ")");
  }
  for (int i = 0; i < count; ++i) {
    SubField &f = *sides[i];
    const uint32_t side = f.isSurface ? 0u : kTaskVolume;
    std::vector<LeafReport> r;
    std::vector<LeafProfile> p;
    std::vector<uint32_t> region;
    for (uint32_t k = 0; k < T; ++k)
      if ((all[k].flags & kTaskVolume) == side) {
        r.push_back(reports[k]);
        p.push_back(profiles[k]);
        region.push_back(all[k].region);
      }
    f.finish(std::move(r), std::move(p), std::move(region), emStart, emEnd);
  }
  cudaEventDestroy(emStart);
  cudaEventDestroy(emEnd);
}

size_t SubField::workBytes() const {
  return posA_.bytes() + posB_.bytes() + sP_.bytes() + sD_.bytes() + tmpP_.bytes() + tmpD_.bytes() + sPdf_.bytes() +
         tmpPdf_.bytes() + dist_.bytes() + node_.bytes() + nodeB_.bytes() + jobOf_.bytes() + isLeft_.bytes() +
         scanLeft_.bytes() + keys_.bytes() + vals_.bytes() + nodeToJob_.bytes() + leafSeg_.bytes() + copyIdx_.bytes() +
         keysB_.bytes() + valsB_.bytes() + routeNodes_.bytes() + keys64_.bytes() + jobs_.bytes() + acc_.bytes() +
         means_.bytes() + bounds6_.bytes() + scratch_.bytes;
}
size_t GpuField::deviceBytes() const {
  return surface.stateBytes() + surface.workBytes() + volume.stateBytes() + volume.workBytes() + tuneSnap_.bytes() +
         tasks_.bytes() + reports_.bytes() + profiles_.bytes() + queue_.bytes() + emShare_.bytes() +
         dqtRects_.bytes() + dqtBuild_.bytes() + dqtLeaves_.bytes();
}

void GpuField::setSceneBounds(const float b[6]) {  // SurfaceVolumeField.h:87-93
  float e[6];
  for (int d = 0; d < 3; ++d) {
    e[d] = b[d] - 1.01f * std::fabs(b[d]);
    e[3 + d] = b[3 + d] + 1.01f * std::fabs(b[3 + d]);
  }
  for (SubField *f : {&surface, &volume}) {
    std::memcpy(f->sceneBounds, e, 24);
    f->boundsSet = true;
  }
}

void GpuField::sceneBounds(float out[6]) const {
  for (int d = 0; d < 3; ++d) {
    out[d] = emin(surface.sceneBounds[d], volume.sceneBounds[d]);
    out[3 + d] = emax(surface.sceneBounds[3 + d], volume.sceneBounds[3 + d]);
  }
}

void GpuField::reset() {
  iteration = 0;
  totalSPP = 0;
  surface.reset();
  volume.reset();
}

// ------------------------------------------------------------------ serialisation
namespace {
struct Writer {
  std::string b;
  void raw(const void *p, size_t n) { b.append(reinterpret_cast<const char *>(p), n); }
  template <typename T>
  void put(const T &v) { raw(&v, sizeof(T)); }
  void lanes(const float *a, int v) { raw(a + v * kLanes, sizeof(float) * kLanes); }
};
void write_region_tail(Writer &w, const RegionHost &h) {  // sample statistics and range (Region.h:63-71)
  w.raw(h.stats.mean, 12);
  w.raw(h.stats.var, 12);
  w.put<float>(h.stats.n);
  w.raw(h.stats.lo, 12);
  w.raw(h.stats.hi, 12);
  w.put<uint8_t>(h.splitFlag);
  w.put<uint64_t>(h.rb);
  w.put<uint64_t>(h.re);
}
void write_knn(Writer &w, const SubField &f) {  // KNN.h:320-331
  w.put<uint8_t>(f.cfg.knn != 0);
  bool built = f.cfg.knn && !f.regions.empty() && f.initialized;
  w.put<uint8_t>(built);
  if (built) {
    w.put<uint32_t>(uint32_t(f.regions.size()));
    for (const RegionHost &h : f.regions) {
      float p[4] = {h.stats.mean[0], h.stats.mean[1], h.stats.mean[2], 0.0f};
      w.raw(p, 16);
    }
  }
}
// The quadtree field type after the common head: the factory's arguments
// (DQTFactory.h:59-61), the kd-tree, per region its validity, quadtree
// (DQT.h:88-93), bounds, training statistics (DQTFactory.h:118-123) and
// sample statistics, then the neighbour points.
void write_sub_dqt(Writer &w, const SubField &f) {
  const FieldConfig &c = f.cfg;
  w.put<DqtArgs>(c.dqtArgs);
  w.put<uint64_t>(c.minSamples);
  w.put<uint64_t>(c.maxSamples);
  w.put<uint64_t>(c.maxDepth);
  w.put<uint8_t>(f.kdInit);
  w.raw(f.kdBounds, 24);
  w.put<uint64_t>(f.nodes.size());
  for (const KDNode &n : f.nodes) {
    w.put<float>(n.split);
    w.put<uint32_t>(n.bits);
  }
  const size_t R = f.regions.size();
  w.put<uint64_t>(R);
  std::vector<DqtHead> heads(R);
  std::vector<DqtStatsNode> stats(R * size_t(f.dqtStride));
  std::vector<DqtNode> nodes(R * size_t(f.dqtStride));
  if (R > 0) {
    Context &cx = Context::get();
    check(cudaMemcpyAsync(heads.data(), f.dDqtHeads.p, R * sizeof(DqtHead), cudaMemcpyDeviceToHost, cx.stream), "D2H");
    check(cudaMemcpyAsync(stats.data(), f.dDqtStats.p, stats.size() * sizeof(DqtStatsNode), cudaMemcpyDeviceToHost,
                          cx.stream),
          "D2H");
    check(cudaMemcpyAsync(nodes.data(), f.dDqtNodes.p, nodes.size() * sizeof(DqtNode), cudaMemcpyDeviceToHost,
                          cx.stream),
          "D2H");
    check(cudaStreamSynchronize(cx.stream), "sync");
  }
  for (size_t i = 0; i < R; ++i) {
    const DqtHead &q = heads[i];
    const size_t o = i * f.dqtStride;
    w.put<uint8_t>(q.valid != 0);
    w.raw(q.pivot, 12);
    w.put<uint64_t>(q.numNodes);
    w.raw(nodes.data() + o, q.numNodes * sizeof(DqtNode));
    w.raw(f.regions[i].bounds, 24);
    w.put<float>(q.numSamples);
    w.put<uint64_t>(q.numNodes);
    w.raw(stats.data() + o, q.numNodes * sizeof(DqtStatsNode));
    write_region_tail(w, f.regions[i]);
  }
  write_knn(w, f);
}
void write_sub(Writer &w, const SubField &f) {  // Field::serialize (Field.h:240-267), CPU_8 lane layout
  const FieldConfig &c = f.cfg;
  w.put<uint8_t>(f.isSurface);
  w.put<float>(c.decayOnSpatialSplit);
  w.put<uint64_t>(f.iteration);
  w.put<uint64_t>(f.totalSPP);
  w.put<uint8_t>(c.deterministic != 0);
  w.put<uint8_t>(c.fitRegions != 0);
  w.put<uint8_t>(f.boundsSet);
  w.raw(f.sceneBounds, 24);
  w.put<uint8_t>(f.initialized);
  float t[4] = {0, 0, 0, 0};
  w.raw(t, 16);
  if (c.dqt) return write_sub_dqt(w, f);
  w.put<uint64_t>(c.initK);
  w.put<float>(c.initKappa);
  w.put<uint64_t>(c.maxK);
  w.put<uint64_t>(c.maxIter);
  w.put<float>(c.maxKappa);
  w.put<float>(c.maxMeanCosine);
  w.put<float>(c.convergence);
  w.put<float>(c.weightPrior);
  w.put<float>(c.mcPriorStrength);
  w.put<float>(c.mcPrior);
  w.put<float>(c.splitThreshold);
  w.put<float>(c.mergeThreshold);
  w.put<uint8_t>(c.partialReFit != 0);
  w.put<int32_t>(c.maxSplitItr);
  w.put<int32_t>(c.minSplit);
  w.put<int32_t>(c.minMerge);
  w.put<int32_t>(c.minRefit);
  w.put<uint64_t>(c.minSamples);
  w.put<uint64_t>(c.maxSamples);
  w.put<uint64_t>(c.maxDepth);
  w.put<uint8_t>(f.kdInit);
  w.raw(f.kdBounds, 24);
  w.put<uint64_t>(f.nodes.size());
  for (const KDNode &n : f.nodes) {
    w.put<float>(n.split);
    w.put<uint32_t>(n.bits);
  }
  std::vector<RegionDir> dir = f.downloadRegions();
  w.put<uint64_t>(f.regions.size());
  for (size_t i = 0; i < f.regions.size(); ++i) {
    const RegionDir &r = dir[i];
    const RegionHost &h = f.regions[i];
    w.put<uint8_t>(r.valid != 0);
    for (int v = 0; v < kMaxK / kLanes; ++v) {
      w.lanes(r.vmm.w, v);
      w.lanes(r.vmm.kappa, v);
      w.lanes(r.vmm.mx, v);
      w.lanes(r.vmm.my, v);
      w.lanes(r.vmm.mz, v);
      w.lanes(r.vmm.norm, v);
      w.lanes(r.vmm.e2k, v);
      w.lanes(r.vmm.mc, v);
      w.lanes(r.vmm.dist, v);
    }
    w.put<uint64_t>(r.vmm.K);
    w.raw(r.vmm.pivot, 12);
    w.raw(h.bounds, 24);
    for (int v = 0; v < kMaxK / kLanes; ++v) {
      w.lanes(r.suff.dx, v);
      w.lanes(r.suff.dy, v);
      w.lanes(r.suff.dz, v);
      w.lanes(r.suff.w, v);
      w.lanes(r.suff.dw, v);
    }
    w.put<float>(r.suff.sumWeights);
    w.put<float>(r.suff.numSamples);
    w.put<float>(r.suff.overallNumSamples);
    w.put<uint64_t>(r.suff.K);
    w.put<uint8_t>(r.suff.normalized != 0);
    for (int v = 0; v < kMaxK / kLanes; ++v) {
      w.lanes(r.split.chi2, v);
      w.lanes(r.split.mx, v);
      w.lanes(r.split.my, v);
      w.lanes(r.split.cx, v);
      w.lanes(r.split.cy, v);
      w.lanes(r.split.cz, v);
      w.lanes(r.split.n, v);
      w.lanes(r.split.sw, v);
      w.lanes(r.split.sa, v);
    }
    w.put<uint64_t>(r.split.K);
    w.put<uint64_t>(r.afterSplit);
    w.put<uint64_t>(r.afterMerge);
    w.raw(h.stats.mean, 12);
    w.raw(h.stats.var, 12);
    w.put<float>(h.stats.n);
    w.raw(h.stats.lo, 12);
    w.raw(h.stats.hi, 12);
    w.put<uint8_t>(h.splitFlag);
    w.put<uint64_t>(h.rb);
    w.put<uint64_t>(h.re);
  }
  w.put<uint8_t>(c.knn != 0);
  bool built = c.knn && !f.regions.empty() && f.initialized;
  w.put<uint8_t>(built);
  if (built) {
    w.put<uint32_t>(uint32_t(f.regions.size()));
    for (const RegionHost &h : f.regions) {
      float p[4] = {h.stats.mean[0], h.stats.mean[1], h.stats.mean[2], 0.0f};
      w.raw(p, 16);
    }
  }
}
// Reader of the same layout; a short or malformed file throws.
struct Reader {
  const std::string &b;
  size_t o = 0;
  explicit Reader(const std::string &buf) : b(buf) {}
  void raw(void *p, size_t n) {
    if (o + n > b.size()) throw std::runtime_error("field file is truncated");
    std::memcpy(p, b.data() + o, n);
    o += n;
  }
  template <typename T>
  T get() {
    T v;
    raw(&v, sizeof(T));
    return v;
  }
  void lanes(float *a, int v) { raw(a + v * kLanes, sizeof(float) * kLanes); }
  // a count of records of at least `minBytes` each that the rest of the file
  // can hold (checked before anything is allocated for them)
  uint64_t count(uint64_t minBytes) {
    const uint64_t n = get<uint64_t>();
    if (n > (b.size() - o) / minBytes) throw std::runtime_error("field file is truncated");
    return n;
  }
};
size_t bytes_left(const Reader &r) { return r.b.size() - r.o; }
void read_region_tail(Reader &r, RegionHost &h) {
  r.raw(h.stats.mean, 12);
  r.raw(h.stats.var, 12);
  h.stats.n = r.get<float>();
  r.raw(h.stats.lo, 12);
  r.raw(h.stats.hi, 12);
  h.splitFlag = r.get<uint8_t>() != 0;
  h.rb = r.get<uint64_t>();
  h.re = r.get<uint64_t>();
}
void read_knn(Reader &r, SubField &f) {
  f.cfg.knn = r.get<uint8_t>() != 0;
  if (r.get<uint8_t>() != 0) {  // KNN points (the region means), rebuilt on upload
    const uint32_t np = r.get<uint32_t>();
    if (np > (bytes_left(r)) / 16) throw std::runtime_error("field file is truncated");
    std::vector<float> pts(size_t(np) * 4);
    r.raw(pts.data(), pts.size() * sizeof(float));
  }
}
// The quadtree field type's layout (see write_sub_dqt).
void read_sub_dqt(Reader &r, SubField &f) {
  FieldConfig &c = f.cfg;
  c.dqtArgs = r.get<DqtArgs>();
  c.minSamples = r.get<uint64_t>();
  c.maxSamples = r.get<uint64_t>();
  c.maxDepth = r.get<uint64_t>();
  f.kdInit = r.get<uint8_t>() != 0;
  r.raw(f.kdBounds, 24);
  const uint64_t numNodes = r.count(8);
  if (numNodes > (uint64_t(1) << 30)) throw std::runtime_error("field file: bad node count");
  f.nodes.resize(numNodes);
  for (KDNode &n : f.nodes) {
    n.split = r.get<float>();
    n.bits = r.get<uint32_t>();
  }
  const uint64_t numRegions = r.count(150);  // a region record takes at least 150 bytes
  if (numRegions > (uint64_t(1) << 30)) throw std::runtime_error("field file: bad region count");
  f.regions.assign(numRegions, RegionHost());
  f.dqtStride = 0;
  f.dqtReserve(uint32_t(std::max<uint64_t>(numRegions, 1)));
  const size_t stride = f.dqtStride;
  std::vector<DqtHead> heads(numRegions);
  std::vector<DqtStatsNode> stats(numRegions * stride);
  std::vector<DqtNode> nodes(numRegions * stride);
  for (size_t i = 0; i < numRegions; ++i) {
    DqtHead &q = heads[i];
    q = DqtHead{};
    q.valid = r.get<uint8_t>() != 0;
    r.raw(q.pivot, 12);
    const uint64_t nn = r.count(8);
    if (nn == 0 || nn > stride) throw std::runtime_error("field file: quadtree larger than its arguments allow");
    r.raw(nodes.data() + i * stride, nn * sizeof(DqtNode));
    r.raw(f.regions[i].bounds, 24);
    q.numSamples = r.get<float>();
    const uint64_t ns = r.count(24);
    if (ns != nn) throw std::runtime_error("field file: quadtree and statistics differ in size");
    r.raw(stats.data() + i * stride, ns * sizeof(DqtStatsNode));
    q.numNodes = uint32_t(nn);
    for (size_t k = 0; k < nn; ++k) {
      const uint32_t ch = stats[i * stride + k].child;
      if (ch != nodes[i * stride + k].child || (ch != 0 && (ch <= k || ch + 4 > nn)))
        throw std::runtime_error("field file: bad quadtree");
    }
    read_region_tail(r, f.regions[i]);
  }
  for (const KDNode &n : f.nodes)
    if (child_of(n) >= (is_leaf(n) ? numRegions : numNodes)) throw std::runtime_error("field file: bad tree");
  read_knn(r, f);
  if (numRegions > 0) {
    check(cudaMemcpy(f.dDqtHeads.p, heads.data(), heads.size() * sizeof(DqtHead), cudaMemcpyHostToDevice), "H2D");
    check(cudaMemcpy(f.dDqtStats.p, stats.data(), stats.size() * sizeof(DqtStatsNode), cudaMemcpyHostToDevice), "H2D");
    check(cudaMemcpy(f.dDqtNodes.p, nodes.data(), nodes.size() * sizeof(DqtNode), cudaMemcpyHostToDevice), "H2D");
  }
  f.uploadRegions(std::vector<RegionDir>(numRegions));  // (mixture state unused by quadtree fields)
  f.uploadTree();
}
void read_sub(Reader &r, SubField &f) {  // Field::deserialize (Field.h:269-301), CPU_8 lane layout
  FieldConfig &c = f.cfg;
  f.isSurface = r.get<uint8_t>() != 0;
  c.decayOnSpatialSplit = r.get<float>();
  f.iteration = r.get<uint64_t>();
  f.totalSPP = r.get<uint64_t>();
  c.deterministic = r.get<uint8_t>() != 0;
  c.fitRegions = r.get<uint8_t>() != 0;
  f.boundsSet = r.get<uint8_t>() != 0;
  r.raw(f.sceneBounds, 24);
  f.initialized = r.get<uint8_t>() != 0;
  float t[4];
  r.raw(t, 16);  // timings of the last update
  if (c.dqt) return read_sub_dqt(r, f);
  c.initK = uint32_t(r.get<uint64_t>());
  c.initKappa = r.get<float>();
  c.maxK = uint32_t(r.get<uint64_t>());
  c.maxIter = uint32_t(r.get<uint64_t>());
  c.maxKappa = r.get<float>();
  c.maxMeanCosine = r.get<float>();
  c.convergence = r.get<float>();
  c.weightPrior = r.get<float>();
  c.mcPriorStrength = r.get<float>();
  c.mcPrior = r.get<float>();
  c.splitThreshold = r.get<float>();
  c.mergeThreshold = r.get<float>();
  c.partialReFit = r.get<uint8_t>() != 0;
  c.maxSplitItr = r.get<int32_t>();
  c.minSplit = r.get<int32_t>();
  c.minMerge = r.get<int32_t>();
  c.minRefit = r.get<int32_t>();
  c.minSamples = r.get<uint64_t>();
  c.maxSamples = r.get<uint64_t>();
  c.maxDepth = r.get<uint64_t>();
  f.kdInit = r.get<uint8_t>() != 0;
  r.raw(f.kdBounds, 24);
  const uint64_t numNodes = r.count(8);  // float split + u32 per node
  if (numNodes > (uint64_t(1) << 30)) throw std::runtime_error("field file: bad node count");
  f.nodes.resize(numNodes);
  for (KDNode &n : f.nodes) {
    n.split = r.get<float>();
    n.bits = r.get<uint32_t>();
  }
  // a region record (valid flag, mixture, bounds, statistics) takes well over
  // 1 KB; 512 bytes bounds it from below
  const uint64_t numRegions = r.count(512);
  if (numRegions > (uint64_t(1) << 30)) throw std::runtime_error("field file: bad region count");
  std::vector<RegionDir> dir(numRegions);
  f.regions.assign(numRegions, RegionHost());
  for (size_t i = 0; i < numRegions; ++i) {
    RegionDir &d = dir[i];
    std::memset(static_cast<void *>(&d), 0, sizeof(RegionDir));
    RegionHost &h = f.regions[i];
    d.valid = r.get<uint8_t>() != 0;
    for (int v = 0; v < kMaxK / kLanes; ++v) {
      r.lanes(d.vmm.w, v);
      r.lanes(d.vmm.kappa, v);
      r.lanes(d.vmm.mx, v);
      r.lanes(d.vmm.my, v);
      r.lanes(d.vmm.mz, v);
      r.lanes(d.vmm.norm, v);
      r.lanes(d.vmm.e2k, v);
      r.lanes(d.vmm.mc, v);
      r.lanes(d.vmm.dist, v);
    }
    d.vmm.K = uint32_t(r.get<uint64_t>());
    r.raw(d.vmm.pivot, 12);
    r.raw(h.bounds, 24);
    for (int v = 0; v < kMaxK / kLanes; ++v) {
      r.lanes(d.suff.dx, v);
      r.lanes(d.suff.dy, v);
      r.lanes(d.suff.dz, v);
      r.lanes(d.suff.w, v);
      r.lanes(d.suff.dw, v);
    }
    d.suff.sumWeights = r.get<float>();
    d.suff.numSamples = r.get<float>();
    d.suff.overallNumSamples = r.get<float>();
    d.suff.K = uint32_t(r.get<uint64_t>());
    d.suff.normalized = r.get<uint8_t>() != 0;
    for (int v = 0; v < kMaxK / kLanes; ++v) {
      r.lanes(d.split.chi2, v);
      r.lanes(d.split.mx, v);
      r.lanes(d.split.my, v);
      r.lanes(d.split.cx, v);
      r.lanes(d.split.cy, v);
      r.lanes(d.split.cz, v);
      r.lanes(d.split.n, v);
      r.lanes(d.split.sw, v);
      r.lanes(d.split.sa, v);
    }
    d.split.K = uint32_t(r.get<uint64_t>());
    d.afterSplit = r.get<uint64_t>();
    d.afterMerge = r.get<uint64_t>();
    r.raw(h.stats.mean, 12);
    r.raw(h.stats.var, 12);
    h.stats.n = r.get<float>();
    r.raw(h.stats.lo, 12);
    r.raw(h.stats.hi, 12);
    h.splitFlag = r.get<uint8_t>() != 0;
    h.rb = r.get<uint64_t>();
    h.re = r.get<uint64_t>();
    if (d.vmm.K > uint32_t(kMaxK) || d.suff.K > uint32_t(kMaxK) || d.split.K > uint32_t(kMaxK))
      throw std::runtime_error("field file: more than 32 lobes");
  }
  for (const KDNode &n : f.nodes)
    if (child_of(n) >= (is_leaf(n) ? numRegions : numNodes)) throw std::runtime_error("field file: bad tree");
  c.knn = r.get<uint8_t>() != 0;
  if (r.get<uint8_t>() != 0) {  // KNN points (the region means), rebuilt below
    const uint32_t np = r.get<uint32_t>();
    if (np > (bytes_left(r)) / 16) throw std::runtime_error("field file is truncated");
    std::vector<float> pts(size_t(np) * 4);
    r.raw(pts.data(), pts.size() * sizeof(float));
  }
  f.uploadRegions(dir);
  f.uploadTree();
}
}  // namespace

// PGL_SPATIAL_STRUCTURE_TYPE / PGL_DIRECTIONAL_DISTRIBUTION_TYPE values (types.h)
constexpr int32_t kSpatialKdTree = 0, kDirParallaxVmm = 0, kDirDqt = 1, kDirVmm = 2;

std::string GpuField::serialize() const {  // SurfaceVolumeField::storeToFile (SurfaceVolumeField.h:171-214)
  Writer w;
  const char hdr[] = "OPENPGL_0.6.0_FIELD";
  w.raw(hdr, sizeof(hdr));
  w.put<int32_t>(kSpatialKdTree);
  w.put<int32_t>(surface.cfg.dqt ? kDirDqt : surface.cfg.parallax ? kDirParallaxVmm : kDirVmm);
  w.put<uint64_t>(iteration);
  w.put<uint64_t>(totalSPP);
  write_sub(w, surface);
  write_sub(w, volume);
  return w.b;
}

void GpuField::deserialize(const std::string &bytes) {  // Device::newFieldFromFile (Device.h:217-260)
  Reader r(bytes);
  char hdr[sizeof("OPENPGL_0.6.0_FIELD")];
  r.raw(hdr, sizeof(hdr));
  if (std::memcmp(hdr, "OPENPGL_0.6.0_FIELD", sizeof(hdr)) != 0) throw std::runtime_error("not an Open PGL 0.6.0 field file");
  const int32_t spatial = r.get<int32_t>(), directional = r.get<int32_t>();
  if (spatial != kSpatialKdTree || (directional != kDirParallaxVmm && directional != kDirVmm && directional != kDirDqt))
    throw std::runtime_error("field file: only kd-tree fields (parallax-aware VMM, VMM, quadtree) are supported");
  const uint32_t parallax = directional == kDirParallaxVmm ? 1u : 0u;
  surface.cfg.dqt = volume.cfg.dqt = directional == kDirDqt ? 1u : 0u;
  iteration = r.get<uint64_t>();
  totalSPP = r.get<uint64_t>();
  read_sub(r, surface);
  read_sub(r, volume);
  if (r.o != bytes.size()) throw std::runtime_error("field file has trailing bytes");
  surface.cfg.parallax = volume.cfg.parallax = parallax;
}

// Field::operator== (Field.h:552-601): exact comparison after the canonical
// depth-first relabelling of the trees (KDTree.h:256-283); timings are not
// compared, as in the reference.
namespace {
void canonical(const std::vector<KDNode> &nodes, std::vector<KDNode> &out, std::vector<uint32_t> &leafData) {
  out.clear();
  leafData.clear();
  if (nodes.empty()) return;
  struct Item {
    uint32_t src, dst;
  };
  out.push_back(nodes[0]);
  std::vector<Item> stack{{0, 0}};
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    const KDNode &n = nodes[it.src];
    if (!is_leaf(n)) {
      uint32_t l = child_of(n);
      uint32_t nl = uint32_t(out.size());
      out[it.dst].bits = (out[it.dst].bits & 0xC0000000u) | nl;
      out.push_back(nodes[l]);
      out.push_back(nodes[l + 1]);
      stack.push_back({l + 1, nl + 1});
      stack.push_back({l, nl});
    } else {
      out[it.dst].bits = (3u << 30) | uint32_t(leafData.size());
      leafData.push_back(child_of(n));
    }
  }
}
// Member-wise (FieldConfig has tail padding, so no memcmp).
bool config_equal(const FieldConfig &a, const FieldConfig &b) {
  return a.maxSamples == b.maxSamples && a.maxDepth == b.maxDepth && a.minSamples == b.minSamples &&
         a.deterministic == b.deterministic && a.knn == b.knn && a.fitRegions == b.fitRegions &&
         a.decayOnSpatialSplit == b.decayOnSpatialSplit && a.initK == b.initK && a.initKappa == b.initKappa &&
         a.maxK == b.maxK && a.maxIter == b.maxIter && a.maxKappa == b.maxKappa &&
         a.maxMeanCosine == b.maxMeanCosine && a.convergence == b.convergence && a.weightPrior == b.weightPrior &&
         a.mcPriorStrength == b.mcPriorStrength && a.mcPrior == b.mcPrior && a.splitThreshold == b.splitThreshold &&
         a.mergeThreshold == b.mergeThreshold && a.useSplitMerge == b.useSplitMerge &&
         a.partialReFit == b.partialReFit && a.maxSplitItr == b.maxSplitItr && a.minSplit == b.minSplit &&
         a.minRefit == b.minRefit && a.minMerge == b.minMerge && a.dqt == b.dqt &&
         (!a.dqt || std::memcmp(&a.dqtArgs, &b.dqtArgs, sizeof(DqtArgs)) == 0);
}
// A sub-field's quadtrees in host memory (heads; nodes and statistics at the
// head's stride).
struct DqtHostState {
  std::vector<DqtHead> heads;
  std::vector<DqtStatsNode> stats;
  std::vector<DqtNode> nodes;
};
DqtHostState download_dqt(const SubField &f) {
  DqtHostState d;
  const size_t R = f.regions.size();
  d.heads.resize(R);
  d.stats.resize(R * size_t(f.dqtStride));
  d.nodes.resize(R * size_t(f.dqtStride));
  if (R == 0) return d;
  check(cudaMemcpy(d.heads.data(), f.dDqtHeads.p, R * sizeof(DqtHead), cudaMemcpyDeviceToHost), "D2H");
  check(cudaMemcpy(d.stats.data(), f.dDqtStats.p, d.stats.size() * sizeof(DqtStatsNode), cudaMemcpyDeviceToHost),
        "D2H");
  check(cudaMemcpy(d.nodes.data(), f.dDqtNodes.p, d.nodes.size() * sizeof(DqtNode), cudaMemcpyDeviceToHost), "D2H");
  return d;
}
bool sub_equal(const SubField &a, const SubField &b) {
  if (!a.initialized && !b.initialized) return true;
  bool eq = a.isSurface == b.isSurface && a.iteration == b.iteration && a.totalSPP == b.totalSPP &&
            a.boundsSet == b.boundsSet && a.initialized == b.initialized &&
            std::memcmp(a.sceneBounds, b.sceneBounds, 24) == 0 &&
            config_equal(a.cfg, b.cfg);
  std::vector<KDNode> na, nb;
  std::vector<uint32_t> da, db;
  canonical(a.nodes, na, da);
  canonical(b.nodes, nb, db);
  if (na.size() != nb.size() || da.size() != db.size() || a.regions.size() != b.regions.size()) return false;
  for (size_t i = 0; i < na.size(); ++i)
    if (na[i].split != nb[i].split || na[i].bits != nb[i].bits) eq = false;
  if (a.cfg.dqt) {  // quadtrees and their statistics (Field.h:552-601)
    const DqtHostState qa = download_dqt(a), qb = download_dqt(b);
    for (size_t i = 0; i < da.size(); ++i) {
      const DqtHead &x = qa.heads[da[i]], &y = qb.heads[db[i]];
      const RegionHost &hx = a.regions[da[i]], &hy = b.regions[db[i]];
      if (std::memcmp(&x, &y, sizeof(DqtHead)) != 0) {
        eq = false;
        continue;
      }
      const size_t oa = size_t(da[i]) * a.dqtStride, ob = size_t(db[i]) * b.dqtStride;
      if (std::memcmp(&qa.stats[oa], &qb.stats[ob], x.numNodes * sizeof(DqtStatsNode)) != 0) eq = false;
      if (std::memcmp(&qa.nodes[oa], &qb.nodes[ob], x.numNodes * sizeof(DqtNode)) != 0) eq = false;
      if (std::memcmp(&hx.stats, &hy.stats, sizeof(Stats)) != 0 || hx.splitFlag != hy.splitFlag) eq = false;
      if (std::memcmp(hx.bounds, hy.bounds, 24) != 0 || hx.rb != hy.rb || hx.re != hy.re) eq = false;
    }
    return eq;
  }
  std::vector<RegionDir> ra = a.downloadRegions(), rb = b.downloadRegions();
  for (size_t i = 0; i < da.size(); ++i) {
    const RegionDir &x = ra[da[i]], &y = rb[db[i]];
    const RegionHost &hx = a.regions[da[i]], &hy = b.regions[db[i]];
    if (std::memcmp(&x.vmm, &y.vmm, sizeof(VMMState)) != 0) eq = false;
    if (std::memcmp(&x.suff, &y.suff, sizeof(SuffState)) != 0) eq = false;
    if (std::memcmp(&x.split, &y.split, sizeof(SplitState)) != 0) eq = false;
    if (x.afterSplit != y.afterSplit || x.afterMerge != y.afterMerge) eq = false;
    if (std::memcmp(&hx.stats, &hy.stats, sizeof(Stats)) != 0 || hx.splitFlag != hy.splitFlag) eq = false;
    if (std::memcmp(hx.bounds, hy.bounds, 24) != 0 || hx.rb != hy.rb || hx.re != hy.re) eq = false;
  }
  return eq;
}
}  // namespace

bool GpuField::equals(const GpuField &o) const {
  return iteration == o.iteration && totalSPP == o.totalSPP && sub_equal(surface, o.surface) &&
         sub_equal(volume, o.volume);
}

// ------------------------------------------------------------------ sampling distributions
GpuSamplingDistribution::GpuSamplingDistribution(GpuField *f, bool vol) : field(f), volume(vol) {
  check(cudaMalloc(&dState, sizeof(SSDState)), "ssd state");
  check(cudaMallocHost(&hRes, sizeof(SSDResult)), "ssd result");
  std::memset(hRes, 0, sizeof(SSDResult));
}
GpuSamplingDistribution::~GpuSamplingDistribution() {
  if (dState) cudaFree(dState);
  if (hRes) cudaFreeHost(hRes);
}

}  // namespace pgl
