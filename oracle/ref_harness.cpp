// Drives the UNMODIFIED reference library (oracle/_ref/libopenpgl_ref.so)
// through its own public C++ wrapper only, the way a renderer would.  Used to
// produce golden outputs (tests/golden/) and to time the reference CPU path.
// Test infrastructure; never part of the product.
//
// usage: ref_harness <frames.bin> <out_prefix> <device 4|8> <threads>
//                    <maxSamplesPerLeaf> <deterministic 0|1> [queries.bin]
// frames.bin : u64 numFrames, then per frame u64 n + n * PGLSampleData (40 B)
// queries.bin: u64 n, then n * {pos f3, normal f3, sample1D f, u f2} (36 B)
// outputs    : <out_prefix>.field      (reference field file after the last frame)
//              <out_prefix>.times      (per-frame Update wall time in ms, text)
//              <out_prefix>.surfq.bin  n * {ok u32, id u32, s1d f, dir f3, pdf f,
//                                           pdfLi f} (surface queries)
//              <out_prefix>.volq.bin   same for the volume field
//              <out_prefix>.volhgq.bin same, volume field with the Henyey-Greenstein
//                                      product: direction = the query's normal,
//                                      mean cosine of query i = hg_mean_cosine(i)
//              <out_prefix>.storage    with PGL_REF_STORE_SAMPLES=1: the sample
//                                      storage holding the last frame, stored by
//                                      SampleStorage::Store before that frame's
//                                      Update, then read back by the
//                                      SampleStorage(file) constructor and compared
//                                      with operator== (result in .storage_cmp)
#include <openpgl/cpp/OpenPGL.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {
struct Query {
  float pos[3], normal[3], s1d, u[2];
};
struct QueryOut {
  uint32_t ok, id;
  float s1d, dir[3], pdf, pdfLi;
};

// Mean cosine of the phase function for query i: -0.99 .. 0.99 in steps of 0.01
// (float arithmetic; the tests compute the same values).
float hg_mean_cosine(uint64_t i) { return float(int(i % 199u)) * 0.01f - 0.99f; }

bool readAll(const char *path, std::vector<char> &buf) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  buf.resize(size_t(sz));
  size_t got = std::fread(buf.data(), 1, buf.size(), f);
  std::fclose(f);
  return got == buf.size();
}
}  // namespace

int main(int argc, char **argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: %s frames.bin out_prefix device threads maxSamplesPerLeaf deterministic [queries.bin]\n", argv[0]);
    return 2;
  }
  const std::string prefix = argv[2];
  const int dev = std::atoi(argv[3]);
  const int threads = std::atoi(argv[4]);
  const size_t maxLeaf = std::strtoull(argv[5], nullptr, 10);
  const bool deterministic = std::atoi(argv[6]) != 0;

  std::vector<char> frames;
  if (!readAll(argv[1], frames)) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 1;
  }

  openpgl::cpp::Device device(dev == 4 ? PGL_DEVICE_TYPE_CPU_4 : PGL_DEVICE_TYPE_CPU_8, size_t(threads));
  // PGL_REF_PLAIN_VMM=1 selects the plain VMM field type instead of the
  // parallax-aware one, PGL_REF_DQT=1 the directional quadtree
  const char *plain = std::getenv("PGL_REF_PLAIN_VMM");
  const char *dqt = std::getenv("PGL_REF_DQT");
  const bool parallax = !(plain && std::atoi(plain) != 0);
  PGL_DIRECTIONAL_DISTRIBUTION_TYPE kind =
      parallax ? PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM : PGL_DIRECTIONAL_DISTRIBUTION_VMM;
  if (dqt && std::atoi(dqt) != 0) kind = PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE;
  openpgl::cpp::FieldConfig cfg;
  cfg.Init(PGL_SPATIAL_STRUCTURE_KDTREE, kind, deterministic, maxLeaf);
  // PGL_REF_DQT_ARGS="leafEstimator,splitMetric,splitThreshold,footprintFactor,maxLevels"
  // overrides the quadtree factory's defaults.  FieldConfig's only member is
  // its PGLFieldArguments (cpp/FieldConfig.h:57-60), which the C++ API keeps
  // private, so the harness reaches it through the object's address.
  const char *dqtArgs = std::getenv("PGL_REF_DQT_ARGS");
  if (kind == PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE && dqtArgs && *dqtArgs) {
    static_assert(sizeof(openpgl::cpp::FieldConfig) == sizeof(PGLFieldArguments), "FieldConfig layout");
    PGLFieldArguments *args = reinterpret_cast<PGLFieldArguments *>(&cfg);
    PGLDQTFactoryArguments *d = static_cast<PGLDQTFactoryArguments *>(args->directionalDistributionArguments);
    int le = 0, sm = 0;
    unsigned levels = 12;
    float thr = 0.01f, ff = 1.0f;
    if (std::sscanf(dqtArgs, "%d,%d,%f,%f,%u", &le, &sm, &thr, &ff, &levels) != 5) {
      std::fprintf(stderr, "bad PGL_REF_DQT_ARGS\n");
      return 1;
    }
    d->leafEstimator = PGLDQTLeafEstimator(le);
    d->splitMetric = PGLDQTSplitMetric(sm);
    d->splitThreshold = thr;
    d->footprintFactor = ff;
    d->maxLevels = levels;
  }
  openpgl::cpp::Field field(&device, cfg);
  openpgl::cpp::SampleStorage storage;

  const char *p = frames.data();
  uint64_t numFrames;
  std::memcpy(&numFrames, p, 8);
  p += 8;
  FILE *times = std::fopen((prefix + ".times").c_str(), "w");
  for (uint64_t f = 0; f < numFrames; ++f) {
    uint64_t n;
    std::memcpy(&n, p, 8);
    p += 8;
    storage.AddSamples(reinterpret_cast<const PGLSampleData *>(p), size_t(n));
    p += n * sizeof(PGLSampleData);
    const char *storeSamples = std::getenv("PGL_REF_STORE_SAMPLES");
    if (f + 1 == numFrames && storeSamples && std::atoi(storeSamples) != 0) {
      storage.Store(prefix + ".storage");
      openpgl::cpp::SampleStorage back(prefix + ".storage");
      FILE *c = std::fopen((prefix + ".storage_cmp").c_str(), "w");
      std::fprintf(c, "%d %zu %zu\n", (back == storage) ? 1 : 0, back.GetSizeSurface(), back.GetSizeVolume());
      std::fclose(c);
    }
    auto t0 = std::chrono::steady_clock::now();
    field.Update(storage);
    auto t1 = std::chrono::steady_clock::now();
    storage.Clear();
    std::fprintf(times, "%.6f\n", std::chrono::duration<double, std::milli>(t1 - t0).count());
  }
  std::fclose(times);
  field.Store(prefix + ".field");

  if (argc > 7) {
    std::vector<char> qbuf;
    if (!readAll(argv[7], qbuf)) return 1;
    uint64_t nq;
    std::memcpy(&nq, qbuf.data(), 8);
    const Query *q = reinterpret_cast<const Query *>(qbuf.data() + 8);
    std::vector<QueryOut> surf(nq), vol(nq), volhg(nq);
    openpgl::cpp::SurfaceSamplingDistribution ssd(&field);
    openpgl::cpp::VolumeSamplingDistribution vsd(&field);
    for (uint64_t i = 0; i < nq; ++i) {
      pgl_point3f pos = {q[i].pos[0], q[i].pos[1], q[i].pos[2]};
      pgl_vec3f nrm = {q[i].normal[0], q[i].normal[1], q[i].normal[2]};
      pgl_point2f u = {q[i].u[0], q[i].u[1]};
      QueryOut &o = surf[i];
      std::memset(&o, 0, sizeof(o));
      float s1d = q[i].s1d;
      o.ok = ssd.Init(&field, pos, s1d) ? 1u : 0u;
      o.s1d = s1d;
      if (o.ok) {
        ssd.ApplyCosineProduct(nrm);
        pgl_vec3f d;
        o.pdf = ssd.SamplePDF(u, d);
        o.dir[0] = d.x; o.dir[1] = d.y; o.dir[2] = d.z;
        o.pdfLi = ssd.IncomingRadiancePDF(d);
        o.id = ssd.GetId();
      }
      QueryOut &v = vol[i];
      std::memset(&v, 0, sizeof(v));
      float s1dv = q[i].s1d;
      v.ok = vsd.Init(&field, pos, s1dv) ? 1u : 0u;
      v.s1d = s1dv;
      if (v.ok) {
        pgl_vec3f d;
        v.pdf = vsd.SamplePDF(u, d);
        v.dir[0] = d.x; v.dir[1] = d.y; v.dir[2] = d.z;
        v.pdfLi = vsd.IncomingRadiancePDF(d);
        v.id = vsd.GetId();
      }
      QueryOut &h = volhg[i];
      std::memset(&h, 0, sizeof(h));
      float s1dh = q[i].s1d;
      h.ok = vsd.Init(&field, pos, s1dh) ? 1u : 0u;
      h.s1d = s1dh;
      if (h.ok) {
        vsd.ApplySingleLobeHenyeyGreensteinProduct(nrm, hg_mean_cosine(i));
        pgl_vec3f d;
        h.pdf = vsd.SamplePDF(u, d);
        h.dir[0] = d.x; h.dir[1] = d.y; h.dir[2] = d.z;
        h.pdfLi = vsd.IncomingRadiancePDF(d);
        h.id = vsd.GetId();
      }
    }
    FILE *fs = std::fopen((prefix + ".surfq.bin").c_str(), "wb");
    std::fwrite(surf.data(), sizeof(QueryOut), surf.size(), fs);
    std::fclose(fs);
    FILE *fv = std::fopen((prefix + ".volq.bin").c_str(), "wb");
    std::fwrite(vol.data(), sizeof(QueryOut), vol.size(), fv);
    std::fclose(fv);
    FILE *fh = std::fopen((prefix + ".volhgq.bin").c_str(), "wb");
    std::fwrite(volhg.data(), sizeof(QueryOut), volhg.size(), fh);
    std::fclose(fh);
  }
  return 0;
}
