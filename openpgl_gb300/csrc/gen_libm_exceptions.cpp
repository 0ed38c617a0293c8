// Writes the inputs at which the host C library's single-precision expf,
// cosf and sinf differ from the double-precision function rounded once to float, the
// form the device evaluates (libm_exceptions.bin, read by the library when
// its CUDA context is set up).  The reference calls std::exp(float) and
// std::cos(float) on a few sites of the directional fit (merged and split
// lobes, merge costs); glibc's float functions are not correctly rounded on
// about 0.07 % (expf) and 0.2 % (cosf) of inputs, and a single such lobe can
// steer a region's later EM iterations.  The table makes the device return
// the host library's bits everywhere: an input is listed when the two
// results differ, or when the double result lies within a few double ulps
// of a float rounding boundary (there the device's double function, a
// different implementation, could round the other way).
//
// Ranges: expf over every float in [-104, 89] (outside it both give 0 or
// infinity), cosf and sinf over every float in [0, 4] (their call sites take
// the length of a 2D vector of unit-vector components, at most about 1.5,
// and the azimuth of a quadtree point, within [-pi, pi]; the C library's
// cosf is even and its sinf odd, so callers look up |x|).
//
// usage: gen_libm_exceptions <out.bin> [threads]
// file : "PGLLIBM2", u32 nExp, u32 nCos, u32 nSin, then the three lists of
//        pairs {float x, float hostResult}, each sorted by x.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct Pair {
  float x, y;
};

uint32_t bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
float from_bits(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// true when the double value d lies within `ulps` double ulps of the midpoint
// between float(d) and its neighbour towards d (float rounding could differ)
bool near_boundary(double d, int ulps) {
  if (!std::isfinite(d) || d == 0.0) return false;
  const float f = float(d);
  if (!std::isfinite(f)) return false;
  const float g = std::nextafter(f, d > double(f) ? INFINITY : -INFINITY);
  if (!std::isfinite(g)) return false;
  const double mid = 0.5 * (double(f) + double(g));
  const double ulp = std::fabs(std::nextafter(d, INFINITY) - d);
  return std::fabs(d - mid) <= ulps * ulp;
}

template <typename F, typename D>
std::vector<Pair> scan(uint32_t lo, uint32_t hi, F hostf, D hostd, int threads) {
  std::vector<std::vector<Pair>> parts(static_cast<size_t>(threads));
  std::vector<std::thread> pool;
  const uint64_t n = uint64_t(hi) - lo + 1;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&, t] {
      const uint64_t b = lo + n * uint64_t(t) / uint64_t(threads), e = lo + n * uint64_t(t + 1) / uint64_t(threads);
      for (uint64_t u = b; u < e; ++u) {
        const float x = from_bits(uint32_t(u));
        const float y = hostf(x);
        const double d = hostd(double(x));
        if (bits(y) != bits(float(d)) || near_boundary(d, 8)) parts[size_t(t)].push_back(Pair{x, y});
      }
    });
  for (auto &th : pool) th.join();
  std::vector<Pair> out;
  for (auto &p : parts) out.insert(out.end(), p.begin(), p.end());
  return out;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s out.bin [threads]\n", argv[0]);
    return 2;
  }
  int threads = argc > 2 ? std::atoi(argv[2]) : int(std::thread::hardware_concurrency());
  if (threads < 1) threads = 1;
  auto expf_ = [](float x) { return std::exp(x); };
  auto exp_ = [](double x) { return std::exp(x); };
  auto cosf_ = [](float x) { return std::cos(x); };
  auto cos_ = [](double x) { return std::cos(x); };
  // non-negative floats in [0, 89] and negative ones in [-104, -0]
  std::vector<Pair> ex = scan(0u, bits(89.0f), expf_, exp_, threads);
  std::vector<Pair> exn = scan(0x80000000u, bits(-104.0f), expf_, exp_, threads);
  ex.insert(ex.end(), exn.begin(), exn.end());
  std::vector<Pair> co = scan(0u, bits(4.0f), cosf_, cos_, threads);
  auto sinf_ = [](float x) { return std::sin(x); };
  auto sin_ = [](double x) { return std::sin(x); };
  std::vector<Pair> si = scan(0u, bits(4.0f), sinf_, sin_, threads);
  auto byX = [](const Pair &a, const Pair &b) { return a.x < b.x; };
  std::sort(ex.begin(), ex.end(), byX);
  std::sort(co.begin(), co.end(), byX);
  std::sort(si.begin(), si.end(), byX);
  FILE *f = std::fopen(argv[1], "wb");
  if (!f) {
    std::perror(argv[1]);
    return 1;
  }
  const uint32_t ne = uint32_t(ex.size()), nc = uint32_t(co.size()), ns = uint32_t(si.size());
  bool ok = std::fwrite("PGLLIBM2", 1, 8, f) == 8 && std::fwrite(&ne, 4, 1, f) == 1 && std::fwrite(&nc, 4, 1, f) == 1 &&
            std::fwrite(&ns, 4, 1, f) == 1 && std::fwrite(ex.data(), sizeof(Pair), ex.size(), f) == ex.size() &&
            std::fwrite(co.data(), sizeof(Pair), co.size(), f) == co.size() &&
            std::fwrite(si.data(), sizeof(Pair), si.size(), f) == si.size();
  ok = (std::fclose(f) == 0) && ok;
  std::printf("expf: %u inputs, cosf: %u inputs, sinf: %u inputs\n", ne, nc, ns);
  return ok ? 0 : 1;
}
