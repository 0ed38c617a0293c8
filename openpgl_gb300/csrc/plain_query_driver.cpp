// The plain drop-in form of guided queries, driven the way a renderer drives
// the reference: host threads, each owning a SurfaceSamplingDistribution,
// call the per-object C API for one path vertex at a time (Init, cosine
// product, then SamplePDF per 2D random number), as openpgl_bench's lookup
// loop does (openpgl_bench.cpp:343-362).  Each call is one launch chain on
// the GPU library.  Used by the benchmark beside the batched and served forms.
//
// usage: plain_query_driver <field file> <vertices file> <threads> <seconds>
// vertices file: u64 n, then n PGLGuidedVertex records (76 bytes each)
// prints: vertices done, seconds, vertices/s, per-vertex latency p50 p99 p99.9 (us)
#include <openpgl/openpgl.h>
#include <openpgl_gb300.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

int main(int argc, char **argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s field vertices threads seconds\n", argv[0]);
    return 2;
  }
  const int threads = std::max(1, std::atoi(argv[3]));
  const double seconds = std::atof(argv[4]);
  FILE *f = std::fopen(argv[2], "rb");
  if (!f) return 1;
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) return 1;
  std::vector<PGLGuidedVertex> v(n);
  if (std::fread(v.data(), sizeof(PGLGuidedVertex), n, f) != n) return 1;
  std::fclose(f);

  PGLDevice device = pglNewDevice(PGL_DEVICE_TYPE_CPU_8, 0);
  PGLField field = pglDeviceNewFieldFromFile(device, argv[1]);
  if (!field) return 1;
  std::atomic<uint64_t> next{0};
  std::vector<std::vector<float>> lat(static_cast<size_t>(threads));
  const auto t0 = std::chrono::steady_clock::now();
  const auto stop = t0 + std::chrono::duration<double>(seconds);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&, t] {
      PGLSurfaceSamplingDistribution d = pglFieldNewSurfaceSamplingDistribution(field);
      while (std::chrono::steady_clock::now() < stop) {
        const PGLGuidedVertex &q = v[next.fetch_add(1) % n];
        const auto a = std::chrono::steady_clock::now();
        float s1d = q.sample1D;
        if (pglFieldInitSurfaceSamplingDistribution(field, d, q.position, &s1d)) {
          pglSurfaceSamplingDistributionApplyCosineProduct(d, q.normal);
          for (int k = 0; k < 4; ++k) {
            pgl_vec3f dir;
            (void)pglSurfaceSamplingDistributionSamplePDF(d, q.sample2D[k], dir);
          }
        }
        lat[size_t(t)].push_back(
            float(std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - a).count()));
      }
      pglReleaseSurfaceSamplingDistribution(d);
    });
  for (auto &th : pool) th.join();
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::vector<float> all;
  for (auto &l : lat) all.insert(all.end(), l.begin(), l.end());
  std::sort(all.begin(), all.end());
  auto q = [&](double p) { return all.empty() ? 0.0 : double(all[std::min(all.size() - 1, size_t(p * all.size()))]); };
  std::printf("%zu %.6f %.1f %.2f %.2f %.2f\n", all.size(), wall, double(all.size()) / wall, q(0.5), q(0.99), q(0.999));
  pglReleaseField(field);
  pglReleaseDevice(device);
  return 0;
}
