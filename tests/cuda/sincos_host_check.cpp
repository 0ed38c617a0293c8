// Host build of sincos_df (pgl_math.cuh) against long-double sinl/cosl over
// float inputs [begin, end) by bit pattern (every `stride`-th): the largest
// relative error of the double-float values before rounding, how often the
// rounding test gives up, and every decided result that is not the exact
// value rounded to nearest.  Compiled with contraction off, as the library.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "pgl_math.cuh"

using namespace pgl;

namespace {
struct Tally {
  uint64_t n = 0, undecided = 0, wrong = 0;
  double maxErrSin = 0, maxErrCos = 0;
  float firstWrong = -1.0f;
};
double rel_err(DFloat v, long double exact) {
  const long double got = (long double)v.h + (long double)v.l;
  return double(fabsl(got - exact) / fabsl(exact));
}
void run(uint32_t begin, uint32_t end, uint32_t stride, Tally &t) {
  for (uint64_t u = begin; u < end; u += stride) {
    const float x = u2f(uint32_t(u));
    DFloat ds, dc;
    sincos_df_parts(x, &ds, &dc);
    const long double es = sinl((long double)x), ec = cosl((long double)x);
    ++t.n;
    if (es != 0.0L) t.maxErrSin = std::fmax(t.maxErrSin, rel_err(ds, es));
    t.maxErrCos = std::fmax(t.maxErrCos, rel_err(dc, ec));
    float s, c;
    if (!sincos_df(x, &s, &c)) {
      ++t.undecided;
      continue;
    }
    if (f2u(s) != f2u(float(es)) || f2u(c) != f2u(float(ec))) {
      if (t.wrong++ == 0) t.firstWrong = x;
    }
  }
}
}  // namespace

// out: n, undecided, wrong; err: max relative error of sin and cos; *firstWrong
extern "C" int sincos_host_check(uint32_t begin, uint32_t end, uint32_t stride, int threads, uint64_t *out,
                                 double *err, float *firstWrong) {
  if (threads < 1 || stride < 1) return 1;
  std::vector<Tally> t(static_cast<size_t>(threads));
  std::vector<std::thread> pool;
  const uint64_t span = (uint64_t(end) - begin + threads - 1) / threads;
  for (int i = 0; i < threads; ++i) {
    uint64_t b = begin + span * uint64_t(i), e = std::min<uint64_t>(end, b + span);
    b += (stride - (b - begin) % stride) % stride;  // keep the global stride grid
    if (b >= e) continue;
    pool.emplace_back(run, uint32_t(b), uint32_t(e), stride, std::ref(t[static_cast<size_t>(i)]));
  }
  for (auto &th : pool) th.join();
  Tally all;
  for (const Tally &x : t) {
    all.n += x.n;
    all.undecided += x.undecided;
    if (x.wrong && all.wrong == 0) all.firstWrong = x.firstWrong;
    all.wrong += x.wrong;
    all.maxErrSin = std::fmax(all.maxErrSin, x.maxErrSin);
    all.maxErrCos = std::fmax(all.maxErrCos, x.maxErrCos);
  }
  out[0] = all.n;
  out[1] = all.undecided;
  out[2] = all.wrong;
  err[0] = all.maxErrSin;
  err[1] = all.maxErrCos;
  *firstWrong = all.firstWrong;
  return 0;
}

// The double-float values (sin h, sin l, cos h, cos l) and the decided results
// (sin, cos, 1 if decided else 0) of n inputs.
extern "C" void sincos_host_values(const float *x, int n, float *parts, float *results) {
  for (int i = 0; i < n; ++i) {
    DFloat ds = {0.0f, 0.0f}, dc = {0.0f, 0.0f};
    if (f2u(x[i]) < 0x41000000u) sincos_df_parts(x[i], &ds, &dc);  // its range: +0 <= x < 8
    parts[4 * i] = ds.h;
    parts[4 * i + 1] = ds.l;
    parts[4 * i + 2] = dc.h;
    parts[4 * i + 3] = dc.l;
    float s = 0.0f, c = 0.0f;
    const bool ok = sincos_df(x[i], &s, &c);
    results[3 * i] = s;
    results[3 * i + 1] = c;
    results[3 * i + 2] = ok ? 1.0f : 0.0f;
  }
}
