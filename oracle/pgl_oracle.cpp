// ORACLE (test infrastructure only).  A CPU restatement of Open PGL v0.6.0's
// field-training and guided-query path (kd-tree field,
// FieldConfig::Init(KDTREE, PARALLAX_AWARE_VMM | VMM | QUADTREE,
// deterministic, maxLeaf), device type CPU_8), written to reproduce the
// reference's arithmetic in the reference's order:
//  * 8-lane SIMD vectors are emulated lane by lane; horizontal sums follow the
//    vfloat8 reduce tree ((0+1)+(2+3))+((4+5)+(6+7))
//    (third-party/embreeSrc/common/simd/vfloat8_avx.h:677-683);
//  * FMAs appear exactly where embree's madd/msub/fnmadd do (dot, cross, xfm,
//    rcp/rsqrt refinement; math/vec3.h:204-209, math/emath.h:312-317);
//  * RCPSS/RSQRTSS come from tables measured on x86 (gen_x86_tables.c);
//  * fastapprox exp/log/sin/acos restate the published ispc/syrah polynomials
//    (math/transcendental.h:333-472);
//  * float expressions that C++ promotes to double (M_PI literals) are
//    evaluated in double, as the reference's compiler does;
//  * the quadtree's sphere-to-square map calls the C library's atan2f, cosf
//    and sinf, as the reference does (directional/dqt/SphereToSquare.h).
// It is compiled with -ffp-contract=off, like oracle/_ref.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU baseline use it.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#include "../openpgl_gb300/csrc/x86_approx_tables.h"  // the one copy of the measured tables
#include "../openpgl_gb300/csrc/hg_table.h"

namespace orc {

static const int W = 8;       // SIMD lanes (PGL_DEVICE_TYPE_CPU_8)
static const int KMAX = 32;   // PGL_VMM_MAX_COMPONENTS
static const int NV = KMAX / W;
static const float INV4PI = (float)0.07957747154594767;  // ONE_OVER_FOUR_PI

// ------------------------------------------------------------------ numerics
static inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// x86 RCPSS (emath.h:61-85 starts from it)
static float rcpss(float x) {
  uint32_t u = fbits(x), s = u & 0x80000000u, e = (u >> 23) & 0xFF, m = u & 0x7FFFFF;
  if (e == 0) return bitsf(s | 0x7F800000u);
  if (e == 255) return m ? x : bitsf(s);
  uint32_t t = pgl_x86_rcp_table[m >> 12];
  int re = int((t >> 23) & 0xFF) - (int(e) - 127);
  if (re <= 0) return bitsf(s);
  if (re >= 255) return bitsf(s | 0x7F800000u);
  return bitsf(s | (uint32_t(re) << 23) | (t & 0x7FFFFF));
}
// x86 RSQRTSS (emath.h:129-145 starts from it)
static float rsqrtss(float x) {
  uint32_t u = fbits(x), e = (u >> 23) & 0xFF, m = u & 0x7FFFFF;
  if (u & 0x80000000u) return (e == 0 && m == 0) ? -INFINITY : NAN;
  if (e == 0) return INFINITY;
  if (e == 255) return m ? x : 0.0f;
  int ue = int(e) - 127, p = ue & 1, q = ue >> 1;
  uint32_t t = pgl_x86_rsqrt_table[p * 1024 + (m >> 13)];
  int re = int((t >> 23) & 0xFF) - q;
  return bitsf((uint32_t(re) << 23) | (t & 0x7FFFFF));
}
// embree::rcp(float), AVX2 form: r * (2 - r*a) with a fused inner step
static float rcp1(float a) { float r = rcpss(a); return r * std::fmaf(-r, a, 2.0f); }
// embree::rcp(float), SSE form r * (2 - r*a) without FMA.  The kd-tree's
// IntegerSampleStatistics and SampleStatistics members are inline functions
// emitted both by deviceCPU4.cpp (SSE) and deviceCPU8.cpp (AVX2); the linker
// keeps the first copy (deviceCPU4.cpp precedes deviceCPU8.cpp in
// openpgl/CMakeLists.txt:6-13,17-19), so every device quantises with this form.
static float rcp1sse(float a) { float r = rcpss(a); return r * (2.0f - r * a); }
// embree::rcp(vfloat8), AVX2 form: r + r*(1 - a*r) as two FMAs
static float rcp8(float a) { float r = rcpss(a); float h = std::fmaf(-a, r, 1.0f); return std::fmaf(r, h, r); }
// embree::rsqrt(float): 1.5*r + ((a*-0.5)*r)*(r*r), no FMA
static float rsqrt1(float a) {
  float r = rsqrtss(a);
  return (1.5f * r) + (((a * -0.5f) * r) * (r * r));
}
// embree::rsqrt(vfloat8), AVX2 form: fma(1.5, r, ((a*-0.5)*r)*(r*r))
static float rsqrt8(float a) {
  float r = rsqrtss(a);
  return std::fmaf(1.5f, r, ((a * -0.5f) * r) * (r * r));
}

static inline float emin(float a, float b) { return a < b ? a : b; }  // minps / embree::min
static inline float emax(float a, float b) { return a < b ? b : a; }  // embree::max
static inline float smin(float a, float b) { return (b < a) ? b : a; } // std::min
static inline float smax(float a, float b) { return (a < b) ? b : a; } // std::max
static inline bool isvalidf(float v) { return (v > -1.844E18f) & (v < 1.844E18f); }

// fastapprox::exp (transcendental.h:333-384)
static float fexp(float v) {
  const float ln2Part1 = (float)0.6931457519, ln2Part2 = (float)1.4286067653e-6;
  const float oneOverLn2 = 1.44269502162933349609375f;
  float scaled = v * oneOverLn2;
  float kReal = std::floor(scaled);
  int k = int(kReal);
  float x = v - kReal * ln2Part1;
  x -= kReal * ln2Part2;
  const float c2 = 0.4999999105930328369140625f, c3 = 0.166668415069580078125f,
              c4 = 4.16539050638675689697265625e-2f, c5 = 8.378830738365650177001953125e-3f,
              c6 = 1.304379315115511417388916015625e-3f, c7 = 2.7555381529964506626129150390625e-4f;
  float r = x * c7 + c6;
  r = x * r + c5;
  r = x * r + c4;
  r = x * r + c3;
  r = x * r + c2;
  r = x * r + 1.0f;
  r = x * r + 1.0f;
  int biasedN = (k + 127) << 23;
  r *= bitsf(uint32_t(biasedN));
  if (kReal > 127) r = INFINITY;
  if (kReal <= -127) r = 0.0f;
  return r;
}
// fastapprox::log (transcendental.h:424-472)
static float flog(float v) {
  bool useNan = v < 0.0f, useInf = v == 0.0f;
  float patched = (useNan || useInf) ? 1.0f : v;
  int32_t iv;
  std::memcpy(&iv, &patched, 4);
  int exponent = ((iv >> 23) + 1) - 127;
  int32_t blended = (iv & int32_t(0x807FFFFF)) | (126 << 23);
  float reduced;
  std::memcpy(&reduced, &blended, 4);
  const float ln2 = 0.693147182464599609375f;
  float x1 = 1.0f - reduced;
  const float c1 = 0.50000095367431640625f, c2 = 0.33326041698455810546875f, c3 = 0.2519190013408660888671875f,
              c4 = 0.17541764676570892333984375f, c5 = 0.3424419462680816650390625f, c6 = -0.599632322788238525390625f,
              c7 = 1.98442304134368896484375f, c8 = -2.4899270534515380859375f, c9 = 1.7491014003753662109375f;
  float r = x1 * c9 + c8;
  r = x1 * r + c7;
  r = x1 * r + c6;
  r = x1 * r + c5;
  r = x1 * r + c4;
  r = x1 * r + c3;
  r = x1 * r + c2;
  r = x1 * r + c1;
  r = x1 * r + 1.0f;
  r *= -x1;
  r += float(exponent) * ln2;
  if (useNan) return NAN;
  if (useInf) return -INFINITY;
  return r;
}
// fastapprox::sin (transcendental.h:18-63)
static float fsin(float v) {
  const float piOverTwo = 1.57079637050628662109375f, twoOverPi = 0.636619746685028076171875f;
  float scaled = v * twoOverPi;
  float kReal = std::floor(scaled);
  int k = int(kReal);
  float x = v - kReal * piOverTwo;
  int kMod4 = k & 3;
  bool useCos = (kMod4 == 1) | (kMod4 == 3);
  bool flip = kMod4 > 1;
  float outside = useCos ? 1.0f : x;
  float c2 = useCos ? -0.5f : -0.16666667163372039794921875f;
  float c4 = useCos ? 4.166664183139801025390625e-2f : 8.333347737789154052734375e-3f;
  float c6 = useCos ? -1.388833043165504932403564453125e-3f : -1.9842604524455964565277099609375e-4f;
  float c8 = useCos ? 2.47562347794882953166961669921875e-5f : 2.760012648650445044040679931640625e-6f;
  float c10 = useCos ? -2.59630184018533327616751194000244140625e-7f : -2.50293279435709337121807038784027099609375e-8f;
  float x2 = x * x;
  float f = x2 * c10 + c8;
  f = x2 * f + c6;
  f = x2 * f + c4;
  f = x2 * f + c2;
  f = x2 * f + 1.0f;
  f *= outside;
  return flip ? -f : f;
}
// fastapprox::acos via asin (transcendental.h:240-270)
static float facos(float x0) {
  bool isneg = x0 < 0.0f;
  float x = std::fabs(x0);
  bool isnan_ = x > 1.0f;
  float v = 1.57079517841339111328125f +
            x * (-0.21450997889041900634765625f +
                 x * (8.78556668758392333984375e-2f +
                      x * (-4.489909112453460693359375e-2f +
                           x * (1.928029954433441162109375e-2f + x * (-4.3095736764371395111083984375e-3f)))));
  v *= -std::sqrt(1.0f - x);
  v = v + 1.57079637050628662109375f;
  v = (v < 0.0f) ? 0.0f : v;
  v = isneg ? -v : v;
  v = isnan_ ? NAN : v;
  return 1.57079637050628662109375f - v;
}

struct V3 {
  float x, y, z;
};
static inline V3 v3(float x, float y, float z) { return {x, y, z}; }
static inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 mulv(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 divs(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
// embree::dot: madd(a.x,b.x, madd(a.y,b.y, a.z*b.z)), fused under AVX2
static inline float dotf(V3 a, V3 b) { return std::fmaf(a.x, b.x, std::fmaf(a.y, b.y, a.z * b.z)); }
static inline V3 crossf(V3 a, V3 b) {
  return {std::fmaf(a.y, b.z, -(a.z * b.y)), std::fmaf(a.z, b.x, -(a.x * b.z)), std::fmaf(a.x, b.y, -(a.y * b.x))};
}
static inline float lengthf(V3 a) { return std::sqrt(dotf(a, a)); }

struct Frame {
  V3 vx, vy, vz;
};
// embree::frame(N) (linearspace3.h:117-124); lane8 selects the vfloat8 rsqrt
static Frame frameOf(V3 N, bool lane8) {
  V3 dx0 = v3(0.0f, N.z, -N.y), dx1 = v3(-N.z, 0.0f, N.x);
  V3 d = dotf(dx0, dx0) > dotf(dx1, dx1) ? dx0 : dx1;
  float r = lane8 ? rsqrt8(dotf(d, d)) : rsqrt1(dotf(d, d));
  V3 dx = mul(d, r);
  V3 c = crossf(N, dx);
  float r2 = lane8 ? rsqrt8(dotf(c, c)) : rsqrt1(dotf(c, c));
  V3 dy = mul(c, r2);
  return {dx, dy, N};
}
// LinearSpace3 * Vec3 (linearspace3.h:150)
static inline V3 xfm(const Frame &f, V3 b) {
  return {std::fmaf(b.x, f.vx.x, std::fmaf(b.y, f.vy.x, b.z * f.vz.x)),
          std::fmaf(b.x, f.vx.y, std::fmaf(b.y, f.vy.y, b.z * f.vz.y)),
          std::fmaf(b.x, f.vx.z, std::fmaf(b.y, f.vy.z, b.z * f.vz.z))};
}
// LinearSpace3::inverse() = adjoint()/det() (linearspace3.h:45-54)
static Frame inverseOf(const Frame &a) {
  V3 c0 = crossf(a.vy, a.vz), c1 = crossf(a.vz, a.vx), c2 = crossf(a.vx, a.vy);
  float det = dotf(a.vx, c0);
  Frame t{v3(c0.x, c1.x, c2.x), v3(c0.y, c1.y, c2.y), v3(c0.z, c1.z, c2.z)};
  return {divs(t.vx, det), divs(t.vy, det), divs(t.vz, det)};
}

// vfloat8 horizontal add over lanes [v*W, v*W+8)
static inline float reduce8(const float *l) {
  float a0 = l[0] + l[1], a2 = l[2] + l[3], a4 = l[4] + l[5], a6 = l[6] + l[7];
  float b0 = a0 + a2, b4 = a4 + a6;
  return b0 + b4;
}
static inline int vecs(size_t K) { return int((K + W - 1) / W); }

static inline float MeanCosineToKappa(float mc) {
  float mc2 = mc * mc;
  return (mc * 3.0f - mc * mc2) / (1.0f - mc2);
}
static inline float KappaToMeanCosine(float k) {
  float m = 1.0f / std::tanh(k) - 1.0f / k;
  return k > 0.0f ? m : 0.0f;
}

// ------------------------------------------------------------------ data
struct Sample {
  float pos[3], dir[3], weight, pdf, distance;
  uint32_t flags;
};
static_assert(sizeof(Sample) == 40, "PGLSampleData is 40 bytes");

struct Stats {  // SampleStatistics (SampleStatistics.h:12-193)
  float mean[3] = {0, 0, 0}, var[3] = {0, 0, 0}, n = 0;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
};

struct VMM {  // ParallaxAwareVonMisesFisherMixture<8,32,true> (PAVMM.h:60-72)
  float w[KMAX], kappa[KMAX], mx[KMAX], my[KMAX], mz[KMAX], norm[KMAX], e2k[KMAX], mc[KMAX], dist[KMAX];
  uint64_t K;
  float pivot[3];
};
struct Suff {  // WEM SufficientStatistics (WEMFactory.h:93-168)
  float dx[KMAX], dy[KMAX], dz[KMAX], w[KMAX], dw[KMAX];
  float sumWeights, numSamples, overallNumSamples;
  uint64_t K;
  bool normalized;
};
struct Split {  // ComponentSplitStatistics (Splitter.h:66-118)
  float chi2[KMAX], mx[KMAX], my[KMAX], cx[KMAX], cy[KMAX], cz[KMAX], n[KMAX], sw[KMAX], sa[KMAX];
  uint64_t K;
};
struct Region {  // Region<VMM, ASMF::Statistics> + Range (Region.h, Range.h)
  bool valid;
  VMM vmm;
  float bounds[6];
  Suff suff;
  Split split;
  uint64_t afterSplit, afterMerge;
  Stats stats;
  bool splitFlag;
  uint64_t rb, re;
};
struct Node {
  float split;
  uint32_t bits;
  bool leaf() const { return (bits >> 30) == 3; }
  uint32_t dim() const { return bits >> 30; }
  uint32_t child() const { return bits & 0x3FFFFFFFu; }
};

struct Config {  // effective values of FieldConfig::Init (api.cpp:755-787, Device.h:99-136)
  uint64_t maxSamples = 32000, maxDepth = 32, minSamples = 100;
  bool deterministic = true, knn = true;
  uint64_t initK = 16;
  float initKappa = 0.5f;
  uint64_t maxK = 32, maxIter = 100;
  float maxKappa = 320000.f, maxMeanCosine = 0, convergence = 0.005f, weightPrior = 0.01f;
  float mcPriorStrength = 0.2f, mcPrior = 0.0f;
  float splitThreshold = 0.5f, mergeThreshold = 0.025f;
  bool useSplitMerge = true, partialReFit = true;
  int maxSplitItr = 1, minSplit = 4000, minRefit = 4000, minMerge = 8000;
  bool parallax = true;  // PARALLAX_AWARE_VMM; false: VMM (Device.h:139-178)
  bool dqt = false;      // PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE (Device.h:185-210)
};

// ------------------------------------------------------------------ VMM ops
static void vmmCalcNorm(VMM &v) {  // PAVMM.h:852-863
  int c = vecs(v.K);
  for (int k = 0; k < c * W; ++k) {
    v.e2k[k] = fexp(-2.0f * v.kappa[k]);
    float nrm = v.kappa[k] / (6.2831855f * (1.0f - v.e2k[k]));
    v.norm[k] = v.kappa[k] > 0.0f ? nrm : INV4PI;
  }
}
static void vmmCalcMeanCosines(VMM &v) {  // PAVMM.h:866-877
  int c = vecs(v.K);
  for (int k = 0; k < c * W; ++k) {
    float th = 1.0f - 2.0f / (fexp(2.0f * v.kappa[k]) - 1.0f);
    float m = 1.0f / th - 1.0f / v.kappa[k];
    v.mc[k] = v.kappa[k] > 0.0f ? m : 0.0f;
  }
}

static float g_uniformDirs[KMAX][KMAX][3];  // WEMFactory.h:668-700
static void initUniformDirections() {
  const float gr = 1.618033988749895f;
  for (uint32_t l = 0; l < KMAX; ++l)
    for (uint32_t n = 0; n < KMAX; ++n) {
      if (n < l + 1) {
        float phi = float(2.0 * M_PI * double(float(n) / gr));
        float z = 1.0f - ((2.0f * float(n) + 1.0f) / float(l + 1));
        float theta = std::acos(z);
        float ct = std::cos(theta), st = std::sin(theta), cp = std::cos(phi), sp = std::sin(phi);
        g_uniformDirs[l][n][0] = st * cp;
        g_uniformDirs[l][n][1] = st * sp;
        g_uniformDirs[l][n][2] = ct;
      } else {
        g_uniformDirs[l][n][0] = 0.0f;
        g_uniformDirs[l][n][1] = 0.0f;
        g_uniformDirs[l][n][2] = 1.0f;
      }
    }
}

static void vmmInitUniform(VMM &v, int K, float kappa) {  // WEMFactory.h:633-664
  v.K = uint64_t(K);
  float weight = 1.0f / float(K);
  for (int n = 0; n < KMAX; ++n) {
    v.mx[n] = g_uniformDirs[K - 1][n][0];
    v.my[n] = g_uniformDirs[K - 1][n][1];
    v.mz[n] = g_uniformDirs[K - 1][n][2];
    if (n < K) {
      v.kappa[n] = kappa;
      v.w[n] = weight;
    } else {
      v.kappa[n] = 0.0f;
      v.w[n] = 0.0f;
      v.norm[n] = INV4PI;
      v.e2k[n] = 1.0f;
      v.mc[n] = 0.0f;
    }
  }
  vmmCalcNorm(v);
  vmmCalcMeanCosines(v);
}

// softAssignment (PAVMM.h:697-733); a[] gets the normalised responsibilities
static bool softAssign(const VMM &v, V3 d, float *a, float &pdf) {
  int c = vecs(v.K);
  float pv[W] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < c * W; ++k) {
    float ct = dotf(d, v3(v.mx[k], v.my[k], v.mz[k]));
    float cm1 = emin(ct - 1.0f, 0.0f);
    float ev = v.norm[k] * fexp(v.kappa[k] * cm1);
    a[k] = v.w[k] * ev;
    pv[k % W] += a[k];
  }
  pdf = reduce8(pv);
  if (pdf <= 1e-16f) return false;
  float inv = rcp1(pdf);
  for (int k = 0; k < c * W; ++k) a[k] *= inv;
  return true;
}
static float vmmPdf(const VMM &v, V3 d) {  // PAVMM.h:676-694
  int c = vecs(v.K);
  float pv[W] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < c * W; ++k) {
    float ct = dotf(d, v3(v.mx[k], v.my[k], v.mz[k]));
    float cm1 = emin(ct - 1.0f, 0.0f);
    float ev = v.norm[k] * fexp(v.kappa[k] * cm1);
    pv[k % W] += v.w[k] * ev;
  }
  return reduce8(pv);
}

static void vmmSwap(VMM &v, int i, int j) {
  if (i == j) return;
  std::swap(v.w[i], v.w[j]);
  std::swap(v.kappa[i], v.kappa[j]);
  std::swap(v.e2k[i], v.e2k[j]);
  std::swap(v.mc[i], v.mc[j]);
  std::swap(v.norm[i], v.norm[j]);
  std::swap(v.mx[i], v.mx[j]);
  std::swap(v.my[i], v.my[j]);
  std::swap(v.mz[i], v.mz[j]);
  std::swap(v.dist[i], v.dist[j]);
}
static void vmmClear(VMM &v, int i) {
  v.w[i] = 0.0f;
  v.kappa[i] = 0.0f;
  v.e2k[i] = 1.0f;
  v.mc[i] = 0.0f;
  v.norm[i] = INV4PI;
  v.mx[i] = 0.0f;
  v.my[i] = 0.0f;
  v.mz[i] = 1.0f;
  v.dist[i] = 0.0f;
}
static void vmmMerge(VMM &v, int i0, int i1) {  // PAVMM.h:259-343
  if (i0 == i1) return;
  float w0 = v.w[i0], w1 = v.w[i1], mc0 = v.mc[i0], mc1 = v.mc[i1];
  float kappa = 0.0f, nrm = INV4PI, e2k = 1.0f;
  float w = w0 + w1;
  float mx = (w0 * mc0) * v.mx[i0] + (w1 * mc1) * v.mx[i1];
  float my = (w0 * mc0) * v.my[i0] + (w1 * mc1) * v.my[i1];
  float mz = (w0 * mc0) * v.mz[i0] + (w1 * mc1) * v.mz[i1];
  mx /= w;
  my /= w;
  mz /= w;
  float mc = mx * mx + my * my + mz * mz;
  if (mc > 0.0f) {
    mc = std::sqrt(mc);
    kappa = MeanCosineToKappa(mc);
    kappa = kappa < 1e-3f ? 0.f : kappa;
    e2k = std::exp(-2.0f * kappa);
    nrm = float(double(kappa) / (2.0 * M_PI * double(1.0f - e2k)));
    mx /= mc;
    my /= mc;
    mz /= mc;
  } else {
    mx = v.mx[i0];
    my = v.my[i0];
    mz = v.mz[i0];
  }
  v.w[i0] = w;
  v.kappa[i0] = kappa;
  v.mc[i0] = mc;
  v.norm[i0] = nrm;
  v.e2k[i0] = e2k;
  v.mx[i0] = mx;
  v.my[i0] = my;
  v.mz[i0] = mz;
  float d0 = v.dist[i0], d1 = v.dist[i1];
  float nd = w0 * d0 + w1 * d1;
  nd /= (w0 + w1);
  v.dist[i0] = nd;
  vmmSwap(v, i1, int(v.K) - 1);
  vmmClear(v, int(v.K) - 1);
  v.K -= 1;
}
static void vmmSplit(VMM &v, int i0, int i1, float w0, float w1, V3 m0, V3 m1, float mc0, float mc1) {  // PAVMM.h:225-255
  v.dist[i1] = v.dist[i0];
  v.w[i0] = w0;
  v.mc[i0] = mc0;
  v.kappa[i0] = MeanCosineToKappa(mc0);
  v.mx[i0] = m0.x;
  v.my[i0] = m0.y;
  v.mz[i0] = m0.z;
  v.w[i1] = w1;
  v.mc[i1] = mc1;
  v.kappa[i1] = MeanCosineToKappa(mc1);
  v.mx[i1] = m1.x;
  v.my[i1] = m1.y;
  v.mz[i1] = m1.z;
  if (uint64_t(i1) == v.K) v.K++;
  vmmCalcNorm(v);
}
static void vmmParallaxShift(VMM &v, V3 s) {  // PAVMM.h:809-831
  int c = vecs(v.K);
  for (int k = 0; k < c * W; ++k) {
    V3 p = add(mul(v3(v.mx[k], v.my[k], v.mz[k]), v.dist[k]), s);
    float len = lengthf(p);
    p = divs(p, len);
    bool cond = (v.dist[k] > 0.0f) && (v.dist[k] >= -FLT_MAX) && (v.dist[k] <= FLT_MAX);
    if (cond) {
      v.mx[k] = p.x;
      v.my[k] = p.y;
      v.mz[k] = p.z;
    }
    v.dist[k] = v.dist[k] > 0.0f ? len : 0.0f;
  }
  v.pivot[0] -= s.x;
  v.pivot[1] -= s.y;
  v.pivot[2] -= s.z;
}
static float vmmProduct(VMM &v, float weight, V3 n, float kappa, float normalization) {  // PAVMM.h:609-671
  int c = vecs(v.K);
  float piv[W] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < c * W; ++k) {
    V3 mu = v3(v.mx[k], v.my[k], v.mz[k]);
    V3 nm = add(mul(mu, v.kappa[k]), mul(n, kappa));
    float nk = std::sqrt(dotf(nm, nm));
    bool chk = nk > 1e-3f;
    nk = chk ? nk : 0.0f;
    nm = chk ? divs(nm, nk) : mu;
    float ne = fexp(-2.0f * nk);
    float nn = nk / (6.2831855f * (1.0f - ne));
    nn = chk ? nn : INV4PI;
    float scale = (v.norm[k] * normalization) / nn;
    float c0 = dotf(mu, nm), c1 = dotf(n, nm);
    float ev = fexp(v.kappa[k] * (c0 - 1.0f) + kappa * (c1 - 1.0f));
    scale *= ev;
    scale *= v.w[k] * weight;
    v.w[k] = scale;
    v.kappa[k] = nk;
    v.mx[k] = nm.x;
    v.my[k] = nm.y;
    v.mz[k] = nm.z;
    v.norm[k] = nn;
    v.e2k[k] = ne;
    piv[k % W] += v.w[k];
  }
  float integral = reduce8(piv);
  for (int k = 0; k < c * W; ++k) v.w[k] /= integral;
  return integral;
}
static V3 squareToUniformSphere(float sx, float sy) {
  float z = 1.0f - 2.0f * sy;
  float r = std::sqrt(smax(0.f, (1.0f - z * z)));
  float sp, cp;
  sincosf(float(2.0 * M_PI * double(sx)), &sp, &cp);
  return v3(r * cp, r * sp, z);
}
static V3 vmmSample(const VMM &v, float ux, float uy) {  // PAVMM.h:737-806
  uint32_t sv = 0, sc = 0;
  float searched = uy, sumW = 0.0f, cdf = 0.0f;
  uint32_t quot = uint32_t((v.K - 1) / W), rem = uint32_t((v.K - 1) % W);
  for (;;) {
    cdf = reduce8(&v.w[sv * W]);
    if (sumW + cdf >= searched || sv + 1 >= quot + 1) break;
    sumW += cdf;
    sv++;
  }
  uint32_t maxSel = (sv == quot) ? rem + 1 : W;
  for (;;) {
    cdf = v.w[sv * W + sc];
    if (sumW + cdf >= searched || sc + 1 >= maxSel) break;
    sumW += cdf;
    sc++;
  }
  float u1 = smin(1.0f - FLT_EPSILON, (searched - sumW) / cdf);
  int s = int(sv * W + sc);
  float k = v.kappa[s], e2k = v.e2k[s];
  V3 mu = v3(v.mx[s], v.my[s], v.mz[s]);
  V3 d;
  if (k == 0.0f) {
    d = squareToUniformSphere(ux, u1);
  } else {
    float ct = 1.f + (flog(1.0f + ((e2k - 1.f) * ux))) / k;
    ct = smin(1.0f, smax(ct, -1.f));
    float st = std::sqrt(1.f - ct * ct);
    float phi = float(2.0 * M_PI * double(u1));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    d = v3(st * cp, st * sp, ct);
  }
  return xfm(frameOf(mu, false), d);
}
static bool vmmIsValid(const VMM &v) {  // PAVMM.h:422-513
  bool ok = true;
  for (uint64_t k = 0; k < v.K; ++k) {
    ok = ok && isvalidf(v.w[k]) && v.w[k] >= 0.0f && v.w[k] <= 1.0f + 1e-6f;
    ok = ok && isvalidf(v.kappa[k]) && v.kappa[k] >= 0.0f;
    ok = ok && isvalidf(v.mc[k]) && v.mc[k] >= 0.0f && v.mc[k] <= 1.0f;
    ok = ok && isvalidf(v.mx[k]) && v.mx[k] >= -1.0f && v.mx[k] <= 1.0f;
    ok = ok && isvalidf(v.my[k]) && v.my[k] >= -1.0f && v.my[k] <= 1.0f;
    ok = ok && isvalidf(v.mz[k]) && v.mz[k] >= -1.0f && v.mz[k] <= 1.0f;
    ok = ok && isvalidf(v.norm[k]) && v.norm[k] >= 0.0f;
    ok = ok && isvalidf(v.e2k[k]);
    ok = ok && isvalidf(v.dist[k]) && v.dist[k] >= 0.0f;
  }
  for (uint64_t k = v.K; k < KMAX; ++k) {
    ok = ok && v.w[k] == 0.0f && v.kappa[k] == 0.0f && v.mx[k] == 0.0f && v.my[k] == 0.0f && v.mz[k] == 1.0f;
    ok = ok && v.mc[k] == 0.0f && std::fabs(v.norm[k] - INV4PI) < 1e-6f && v.e2k[k] == 1.0f && v.dist[k] == 0.0f;
  }
  return ok;
}

// ------------------------------------------------------------------ stats ops
static void suffClear(Suff &s, uint64_t K) {
  s.K = K;
  int c = vecs(K);
  for (int k = 0; k < c * W; ++k) s.dx[k] = s.dy[k] = s.dz[k] = s.w[k] = s.dw[k] = 0.0f;
  s.sumWeights = 0.0f;
  s.numSamples = 0.0f;
  s.normalized = false;
}
static void suffNormalize(Suff &s, float n) {  // WEMFactory.h:553-572
  int c = vecs(s.K);
  s.numSamples = n;
  float sv[W] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < c * W; ++k) sv[k % W] += s.w[k];
  s.sumWeights = reduce8(sv);
  float nrm = n / s.sumWeights;
  for (int k = 0; k < c * W; ++k) {
    s.dx[k] *= nrm;
    s.dy[k] *= nrm;
    s.dz[k] *= nrm;
    s.w[k] *= nrm;
  }
  s.normalized = true;
}
static void suffAdd(Suff &a, const Suff &b) {  // operator+= (WEMFactory.h:575-593)
  int c = vecs(a.K);
  a.sumWeights += b.sumWeights;
  a.numSamples += b.numSamples;
  a.overallNumSamples += b.numSamples;
  for (int k = 0; k < c * W; ++k) {
    a.dx[k] += b.dx[k];
    a.dy[k] += b.dy[k];
    a.dz[k] += b.dz[k];
    a.w[k] += b.w[k];
    a.dw[k] += b.dw[k];
  }
}
static void suffMaskedReplace(Suff &a, const bool *mask, const Suff &b) {  // WEMFactory.h:448-468
  float sv[W] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < KMAX; ++k) {
    if (mask[k]) {
      a.dx[k] = b.dx[k];
      a.dy[k] = b.dy[k];
      a.dz[k] = b.dz[k];
      a.w[k] = b.w[k];
      a.dw[k] = b.dw[k];
    }
    sv[k % W] += a.w[k];
  }
  if (a.normalized)
    a.numSamples = reduce8(sv);
  else
    a.sumWeights = reduce8(sv);
}
static void suffDecay(Suff &s, float a) {
  for (int k = 0; k < KMAX; ++k) {
    s.dx[k] *= a;
    s.dy[k] *= a;
    s.dz[k] *= a;
    s.w[k] *= a;
    s.dw[k] *= a;
  }
  s.numSamples *= a;
  s.sumWeights *= a;
}
static void suffParallaxShift(Suff &s, const VMM &v, V3 shift) {  // WEMFactory.h:265-283
  int c = vecs(v.K);
  for (int k = 0; k < c * W; ++k) {
    V3 d0 = v3(s.dx[k], s.dy[k], s.dz[k]);
    V3 d = d0;
    float smc = lengthf(d);
    d = divs(d, smc);
    d = mul(d, v.dist[k]);
    d = add(d, shift);
    d = divs(d, lengthf(d));
    d = mul(d, smc);
    d = smc > 0.0f ? d : d0;
    if (v.dist[k] > 0.0f) {
      s.dx[k] = d.x;
      s.dy[k] = d.y;
      s.dz[k] = d.z;
    }
  }
}
static void suffSplit(Suff &s, int i, int j, V3 m0, V3 m1, float mc0, float mc1) {  // WEMFactory.h:516-550
  float sw = s.w[i];
  sw /= 2.0f;
  s.w[i] = sw;
  s.dx[i] = (m0.x * mc0) * sw;
  s.dy[i] = (m0.y * mc0) * sw;
  s.dz[i] = (m0.z * mc0) * sw;
  s.w[j] = sw;
  s.dx[j] = (m1.x * mc1) * sw;
  s.dy[j] = (m1.y * mc1) * sw;
  s.dz[j] = (m1.z * mc1) * sw;
  float t = s.dw[i] * 0.5f;
  s.dw[i] = t;
  s.dw[j] = t;
  s.K += 1;
}
static void suffMerge(Suff &s, int i0, int i1) {  // WEMFactory.h:485-513
  int L = int(s.K) - 1;
  s.dx[i0] += s.dx[i1];
  s.dy[i0] += s.dy[i1];
  s.dz[i0] += s.dz[i1];
  s.w[i0] += s.w[i1];
  s.dw[i0] += s.dw[i1];
  s.dx[i1] = s.dx[L];
  s.dy[i1] = s.dy[L];
  s.dz[i1] = s.dz[L];
  s.w[i1] = s.w[L];
  s.dw[i1] = s.dw[L];
  s.dx[L] = s.dy[L] = s.dz[L] = s.w[L] = s.dw[L] = 0.0f;
  s.K--;
}
static bool suffIsValid(const Suff &s) {
  bool ok = true;
  for (uint64_t k = 0; k < s.K && k < KMAX; ++k)
    ok = ok && isvalidf(s.dx[k]) && isvalidf(s.dy[k]) && isvalidf(s.dz[k]) && isvalidf(s.w[k]) && s.w[k] >= 0.0f &&
         isvalidf(s.dw[k]) && s.dw[k] >= 0.0f;
  for (uint64_t k = s.K; k < KMAX; ++k)
    ok = ok && s.dx[k] == 0.0f && s.dy[k] == 0.0f && s.dz[k] == 0.0f && s.w[k] == 0.0f && s.dw[k] == 0.0f;
  ok = ok && isvalidf(s.numSamples) && s.numSamples >= 0.0f && isvalidf(s.sumWeights) && s.sumWeights >= 0.0f;
  return ok;
}

static void splitClear(Split &s, uint64_t K) {
  s.K = K;
  int c = vecs(K);
  for (int k = 0; k < c * W; ++k)
    s.chi2[k] = s.cx[k] = s.cy[k] = s.cz[k] = s.mx[k] = s.my[k] = s.n[k] = s.sw[k] = s.sa[k] = 0.0f;
}
static void splitZeroLane(Split &s, int i) {
  s.chi2[i] = s.sa[i] = s.n[i] = s.sw[i] = s.mx[i] = s.my[i] = s.cx[i] = s.cy[i] = s.cz[i] = 0.0f;
}
static void splitDecay(Split &s, float a) {
  int c = vecs(s.K);
  for (int k = 0; k < c * W; ++k) {
    s.cx[k] *= a;
    s.cy[k] *= a;
    s.cz[k] *= a;
    s.n[k] *= a;
    s.sw[k] *= a;
    s.sa[k] *= a;
  }
}
static bool splitIsValid(const Split &s) {
  bool lane[W];
  for (int j = 0; j < W; ++j) lane[j] = true;
  for (int k = 0; k < KMAX; ++k) {
    bool ok = isvalidf(s.mx[k]) && isvalidf(s.my[k]) && isvalidf(s.cx[k]) && isvalidf(s.cy[k]) && isvalidf(s.cz[k]) &&
              isvalidf(s.chi2[k]) && s.chi2[k] >= 0.0f && isvalidf(s.sw[k]) && s.sw[k] >= 0.0f && isvalidf(s.sa[k]) &&
              s.sa[k] >= 0.0f && isvalidf(s.n[k]) && s.n[k] >= 0.0f;
    lane[k % W] = lane[k % W] && ok;
  }
  bool any = false;
  for (int j = 0; j < W; ++j) any = any || lane[j];
  return any && s.K > 0 && s.K <= KMAX;
}

// ------------------------------------------------------------------ WEM
struct Unassigned {
  float sw = 0.0f;
  V3 d = {0, 0, 0};
};

static float eStep(VMM &v, Suff &st, Unassigned &un, const Sample *S, size_t n) {  // WEMFactory.h:847-892
  un = Unassigned();
  suffClear(st, v.K);
  st.K = v.K;
  st.numSamples = float(n);
  int c = vecs(st.K);
  float ll = 0.0f;
  float a[KMAX];
  for (size_t i = 0; i < n; ++i) {
    const Sample &s = S[i];
    V3 d = v3(s.dir[0], s.dir[1], s.dir[2]);
    float pdf;
    if (!softAssign(v, d, a, pdf)) {
      un.sw += s.weight;
      un.d = add(un.d, mul(d, s.weight));
      continue;
    }
    ll += s.weight * std::log(pdf);
    for (int k = 0; k < c * W; ++k) {
      st.dx[k] += (d.x * a[k]) * s.weight;
      st.dy[k] += (d.y * a[k]) * s.weight;
      st.dz[k] += (d.z * a[k]) * s.weight;
      st.w[k] += a[k] * s.weight;
    }
  }
  return ll;
}
static void handleUnassigned(const Unassigned &un, VMM &v, Suff &cur, Suff &prev) {  // WEMFactory.h:731-748
  int t = int(cur.K);
  cur.K++;
  cur.w[t] = un.sw;
  cur.dx[t] = un.d.x;
  cur.dy[t] = un.d.y;
  cur.dz[t] = un.d.z;
  prev.K++;
  prev.w[t] = 0.0f;
  prev.dx[t] = prev.dy[t] = prev.dz[t] = 0.0f;
  v.K++;
}
static void mapWeights(VMM &v, const Suff &cur, const Suff &prev, float prior) {  // WEMFactory.h:895-927
  int c = vecs(v.K);
  float K = float(v.K);
  float N = cur.numSamples + prev.numSamples;
  for (int k = 0; k < c * W; ++k) {
    float w = cur.w[k] + prev.w[k];
    v.w[k] = (prior + w) / ((prior * K) + N);
  }
  int rem = int(v.K % W);
  if (rem > 0)
    for (int i = rem; i < W; ++i) v.w[(c - 1) * W + i] = 0.0f;
}
static void mapMeanDirKappa(VMM &v, const Suff &cur, const Suff &prev, const Config &cfg, const bool *mask) {
  // WEMFactory.h:930-999 (mask == nullptr) and :1081-1148 (partial)
  float curN = cur.numSamples, prevN = prev.numSamples, N = curN + prevN;
  float overallN = cur.numSamples + prev.overallNumSamples;
  float curW = curN / N, prevW = 1.0f - curW;
  int c = vecs(v.K), rem = int(v.K % W);
  for (int k = 0; k < c * W; ++k) {
    float partialN = v.w[k] * overallN;
    V3 cm = cur.w[k] > 0.0f ? v3(cur.dx[k] / cur.w[k], cur.dy[k] / cur.w[k], cur.dz[k] / cur.w[k]) : v3(0, 0, 0);
    V3 pm = prev.w[k] > 0.0f ? v3(prev.dx[k] / prev.w[k], prev.dy[k] / prev.w[k], prev.dz[k] / prev.w[k]) : v3(0, 0, 0);
    V3 md = add(mul(cm, curW), mul(pm, prevW));
    float mc = lengthf(md);
    bool upd = mask ? mask[k] : true;
    if (upd && mc > 0.0f) {
      v.mx[k] = md.x / mc;
      v.my[k] = md.y / mc;
      v.mz[k] = md.z / mc;
    }
    mc = (cfg.mcPrior * cfg.mcPriorStrength + mc * partialN) / (cfg.mcPriorStrength + partialN);
    mc = emin(cfg.maxMeanCosine, mc);
    if (upd) {
      v.mc[k] = mc;
      v.kappa[k] = MeanCosineToKappa(mc);
    }
  }
  if (rem > 0)
    for (int i = rem; i < W; ++i) {
      int k = (c - 1) * W + i;
      v.mx[k] = 0.0f;
      v.my[k] = 0.0f;
      v.mz[k] = 1.0f;
      v.mc[k] = 0.0f;
      v.kappa[k] = 0.0f;
      if (!mask) {
        v.norm[k] = INV4PI;
        v.e2k[k] = 1.0f;
      }
    }
  vmmCalcNorm(v);
}
static void mapPartialWeights(VMM &v, const bool *mask, const Suff &cur, const Suff &prev, float prior) {  // :1030-1078
  int c = vecs(v.K);
  float K = float(v.K);
  float N = cur.numSamples + prev.numSamples;
  float sw[W] = {0, 0, 0, 0, 0, 0, 0, 0}, sp[W] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < c * W; ++k) {
    float w = cur.w[k] + prev.w[k];
    w = (prior + w) / ((prior * K) + N);
    sp[k % W] += mask[k] ? w : 0.0f;
    sw[k % W] += mask[k] ? 0.0f : v.w[k];
    v.w[k] = mask[k] ? w : v.w[k];
  }
  float inv = 1.0f / reduce8(sp);
  inv *= 1.0f - reduce8(sw);
  for (int k = 0; k < c * W; ++k) v.w[k] = mask[k] ? v.w[k] * inv : v.w[k];
  int rem = int(v.K % W);
  if (rem > 0)
    for (int i = rem; i < W; ++i) v.w[(c - 1) * W + i] = 0.0f;
}

static int emLoop(VMM &v, Suff &prev, const Sample *S, size_t n, const Config &cfg, bool *mask) {
  // updateMixture (WEMFactory.h:751-795) / partialUpdateMixture (:798-844)
  Suff cur;
  std::memset(&cur, 0, sizeof(cur));
  suffClear(cur, KMAX);
  int it = 0;
  bool converged = false;
  float prevLL = 0.0f, invPrevLL = 1.0f;
  Unassigned un;
  while (!converged && uint64_t(it) < cfg.maxIter) {
    float ll = eStep(v, cur, un, S, n);
    if (un.sw > 0.0f && cur.K < KMAX) {
      handleUnassigned(un, v, cur, prev);
      if (mask) mask[v.K - 1] = true;
    }
    suffNormalize(cur, cur.numSamples);
    if (mask) {
      mapPartialWeights(v, mask, cur, prev, cfg.weightPrior);
      mapMeanDirKappa(v, cur, prev, cfg, mask);
    } else {
      mapWeights(v, cur, prev, cfg.weightPrior);
      mapMeanDirKappa(v, cur, prev, cfg, nullptr);
    }
    it++;
    if (it > 1) {
      float rel = std::fabs(ll - prevLL) * invPrevLL;
      if (rel < cfg.convergence) converged = true;
      prevLL = ll;
      invPrevLL = 1.0f / std::fabs(ll);
    }
  }
  suffAdd(prev, cur);
  return it;
}

static void componentDistances(VMM &v, Suff &s, const Sample *S, size_t n, bool init) {  // WEMFactory.h:1199-1326
  int c = vecs(v.K), rem = int(v.K % W);
  float bd[KMAX], bw[KMAX], a[KMAX];
  for (int k = 0; k < c * W; ++k) bd[k] = bw[k] = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    float sd = rcp1(S[i].distance);
    float pdf;
    if (softAssign(v, v3(S[i].dir[0], S[i].dir[1], S[i].dir[2]), a, pdf)) {
      for (int k = 0; k < c * W; ++k) {
        float w = (S[i].weight * a[k]) * ((a[k] * pdf) / v.w[k]);
        bd[k] += w * sd;
        bw[k] += w;
      }
    }
  }
  for (int k = 0; k < c * W; ++k) {
    if (init) {
      s.dw[k] = bw[k];
      v.dist[k] = s.dw[k] / bd[k];
    } else {
      float inv = bd[k];
      inv += v.dist[k] > 0.0f ? (s.dw[k] / v.dist[k]) : 0.0f;
      s.dw[k] += bw[k];
      v.dist[k] = s.dw[k] / inv;
    }
  }
  if (rem > 0)
    for (int i = rem; i < W; ++i) {
      v.dist[(c - 1) * W + i] = 0.0f;
      s.dw[(c - 1) * W + i] = 0.0f;
    }
}

// ------------------------------------------------------------------ split / merge
static void updateSplitStats(const VMM &v, Split &sp, float mcEst, const Sample *S, size_t n) {  // Splitter.h:439-523
  int c = vecs(sp.K);
  float a[KMAX];
  Frame inv[KMAX];
  for (int k = 0; k < c * W; ++k) inv[k] = inverseOf(frameOf(v3(v.mx[k], v.my[k], v.mz[k]), true));
  for (size_t i = 0; i < n; ++i) {
    const Sample &s = S[i];
    V3 d = v3(s.dir[0], s.dir[1], s.dir[2]);
    float pdf;
    if (!softAssign(v, d, a, pdf)) continue;
    float value = s.weight * s.pdf;
    for (int k = 0; k < c * W; ++k) {
      float vmf = a[k] * pdf;
      float pvp = vmf * value;
      pvp /= (mcEst * pdf);
      float chi = (value * value) * vmf;
      chi /= ((mcEst * mcEst) * pdf) * pdf;
      chi -= 2.0f * pvp;
      chi += vmf;
      chi /= s.pdf;
      chi = a[k] > 0.0f ? chi : 0.0f;
      sp.sa[k] += a[k];
      sp.n[k] += 1.0f;
      sp.chi2[k] += (chi - sp.chi2[k]) / sp.n[k];
      V3 ld = xfm(inv[k], d);
      float aw = a[k] * s.weight;
      sp.sw[k] += aw;
      sp.mx[k] += 0.0f;
      sp.my[k] += 0.0f;
      sp.cx[k] += aw * (ld.x * ld.x);
      sp.cy[k] += aw * (ld.y * ld.y);
      sp.cz[k] += aw * (ld.x * ld.y);
    }
  }
}
static void map3Dto2D(V3 d, float &x, float &y) {  // Splitter.h:161-171
  float alpha = facos(d.z);
  float inv_sinc = alpha / fsin(alpha);
  x = alpha > 0.0f ? d.x * inv_sinc : 0.0f;
  y = alpha > 0.0f ? d.y * inv_sinc : 0.0f;
}
static V3 map2Dto3D(float x, float y) {  // Splitter.h:174-186
  float len = std::sqrt(x * x + y * y);
  float sinc = fsin(len) / len;
  V3 r;
  r.x = len > 0.0f ? x * sinc : 0.0f;
  r.y = len > 0.0f ? y * sinc : 0.0f;
  r.z = std::cos(len);
  return r;
}
static bool splitComponent(VMM &v, Split &sp, Suff &suff, int idx) {  // Splitter.h:527-665
  float numAssigned = sp.sa[idx];
  float invSW = rcp1(sp.sw[idx]);
  float meanx = sp.mx[idx], meany = sp.my[idx];
  float cx = sp.cx[idx] * invSW, cy = sp.cy[idx] * invSW, cz = sp.cz[idx] * invSW;
  float D = std::sqrt((cx - cy) * (cx - cy) + ((cz * cz) * 4.0f)) * 0.5f;
  float ev0 = float(double(cx + cy) * 0.5);
  ev0 += D;
  float e0x = -cz, e0y = cx - ev0;
  float l0 = std::sqrt(e0x * e0x + e0y * e0y);
  e0x /= l0;
  e0y /= l0;
  float w = v.w[idx], mc = v.mc[idx], kappa = v.kappa[idx];
  if (double(kappa) >= 32000.0 * 0.9) return false;
  V3 mu = v3(v.mx[idx], v.my[idx], v.mz[idx]);
  float nw0 = w * 0.5f, nw1 = nw0;
  V3 m0 = mu, m1 = mu;
  float nmc0 = mc, nmc1 = mc * mc;
  if (D > 1e-8f) {
    float ax = (e0x * ev0) * 0.5f, ay = (e0y * ev0) * 0.5f;
    Frame fr = frameOf(mu, false);
    m0 = xfm(fr, map2Dto3D(meanx + ax, meany + ay));
    nmc0 = mc / std::fabs(dotf(mu, m0));
    nmc0 = smin(nmc0, KappaToMeanCosine(32000.0f));
    nmc1 = nmc0;
    m1 = xfm(fr, map2Dto3D(meanx - ax, meany - ay));
  } else {
    if (numAssigned < 2.0f) return false;
  }
  int K = int(v.K);
  vmmSplit(v, idx, K, nw0, nw1, m0, m1, nmc0, nmc1);
  suffSplit(suff, idx, K, m0, m1, nmc0, nmc1);
  splitZeroLane(sp, idx);
  splitZeroLane(sp, K);
  sp.K = uint64_t(K + 1);
  return true;
}
struct Cand {
  size_t idx;
  float chi;
};
static std::vector<Cand> splitCandidates(const Split &sp) {  // Splitter.h:1103-1117
  std::vector<Cand> c;
  for (size_t k = 0; k < sp.K; ++k) c.push_back({k, sp.chi2[k]});
  std::sort(c.begin(), c.end(), [](Cand a, Cand b) { return a.chi > b.chi; });
  return c;
}

static float productScale(V3 m0, float k0, float n0, V3 m1, float k1, float n1, V3 &pm, float &pk, float &pn) {
  // Merger.h:368-396 (_Product)
  pm = add(mul(m0, k0), mul(m1, k1));
  pk = std::sqrt(dotf(pm, pm));
  pn = float(1.0 / (4.0 * M_PI));
  if (pk > 1e-3f) {
    float pe = std::exp(-2.0f * pk);
    pn = float(double(pk) / (2.0 * M_PI * double(1.0f - pe)));
    pm = divs(pm, pk);
  } else {
    pk = 0.0f;
    pm = m0;
  }
  float scale = (n0 * n1) / pn;
  float c0 = dotf(m0, pm), c1 = dotf(m1, pm);
  scale *= std::exp(k0 * (c0 - 1.0f) + k1 * (c1 - 1.0f));
  return scale;
}
static float integratedDivision(V3 m0, float k0, float n0, V3 m1, float k1, float n1, float e2k1) {  // Merger.h:337-365
  V3 pm = add(mul(m0, k0), mul(m1, k1));
  float pk = std::sqrt(dotf(pm, pm));
  float pn = float(1.0 / (4.0 * M_PI));
  if (pk > 1e-3f) {
    float pe = std::exp(-2.0f * pk);
    pn = float(double(pk) / (2.0 * M_PI * double(1.0f - pe)));
    pm = divs(pm, pk);
  } else {
    pk = 0.0f;
    pm = m0;
  }
  float scale = (n0 * n1) / pn;
  float c0 = dotf(m0, pm), c1 = dotf(m1, pm);
  scale = float(double(scale) * ((4.0 * M_PI * M_PI * double(1.0f - e2k1)) / double(k1 * k1)));
  scale *= std::exp((k0 * (c0 - 1.0f) + k1 * (c1 - 1.0f)) + (2.0f * k1));
  return scale;
}
static float mergeCost(const VMM &v, int i0, int i1) {  // Merger.h:92-177
  float w0 = v.w[i0], k0 = v.kappa[i0], mc0 = v.mc[i0], n0 = v.norm[i0];
  float w1 = v.w[i1], k1 = v.kappa[i1], mc1 = v.mc[i1], n1 = v.norm[i1];
  V3 m0 = v3(v.mx[i0], v.my[i0], v.mz[i0]), m1 = v3(v.mx[i1], v.my[i1], v.mz[i1]);
  if (i0 == i1) {
    w0 /= 2.0f;
    w1 /= 2.0f;
  }
  float w = w0 + w1, kappa = 0.0f, mc = 0.0f, nrm = INV4PI, e2k = 1.0f;
  V3 m = add(mul(m0, w0 * mc0), mul(m1, w1 * mc1));
  m = divs(m, w);
  mc = m.x * m.x + m.y * m.y + m.z * m.z;
  if (mc > 0.f) {
    mc = std::sqrt(mc);
    kappa = MeanCosineToKappa(mc);
    kappa = kappa < 1e-3f ? 0.f : kappa;
    e2k = std::exp(-2.0f * kappa);
    nrm = float(double(kappa) / (2.0 * M_PI * double(1.0f - e2k)));
    m = divs(m, mc);
  } else {
    m = m0;
  }
  V3 nm = v3(-m.x, -m.y, -m.z);
  V3 m00, m11, m01;
  float k00, k11, k01, n00, n11, n01;
  float s00 = productScale(m0, k0, n0, m0, k0, n0, m00, k00, n00);
  float s11 = productScale(m1, k1, n1, m1, k1, n1, m11, k11, n11);
  float s01 = productScale(m0, k0, n0, m1, k1, n1, m01, k01, n01);
  float w00 = w0 * w0, w11 = w1 * w1, w01 = w0 * w1;
  float chi = 0.0f;
  chi += (w00 / w) * (s00 * integratedDivision(m00, k00, n00, nm, kappa, nrm, e2k));
  chi += (w11 / w) * (s11 * integratedDivision(m11, k11, n11, nm, kappa, nrm, e2k));
  chi += 2.0f * (w01 / w) * (s01 * integratedDivision(m01, k01, n01, nm, kappa, nrm, e2k));
  chi -= w;
  return chi;
}
static void splitMergeStats(Split &s, int I, int J, float wI, V3 muI, float wJ, V3 muJ, float wK, V3 muK) {
  // Splitter.h:994-1100 (OPENPGL_ZERO_MEAN)
  int L = int(s.K) - 1;
  Frame invK = inverseOf(frameOf(muK, false));
  float ix, iy, jx, jy;
  map3Dto2D(xfm(invK, muI), ix, iy);
  map3Dto2D(xfm(invK, muJ), jx, jy);
  float invWK = (wK > 0.f) ? rcp1(wK) : 1.f;
  float swI = s.sw[I], swJ = s.sw[J], swK = swI + swJ;
  V3 cI = (swI > 0.f) ? mul(v3(s.cx[I], s.cy[I], s.cz[I]), rcp1(swI)) : v3(0, 0, 0);
  V3 cJ = (swJ > 0.f) ? mul(v3(s.cx[J], s.cy[J], s.cz[J]), rcp1(swJ)) : v3(0, 0, 0);
  V3 mII = v3(ix * ix, iy * iy, ix * iy), mJJ = v3(jx * jx, jy * jy, jx * jy);
  V3 cK = add(add(add(mul(cI, wI), mul(mII, wI)), mul(cJ, wJ)), mul(mJJ, wJ));
  cK = mul(cK, invWK);
  V3 scK = mul(cK, swK);
  float saK = s.sa[I] + s.sa[J];
  float nK = invWK * (wI * s.n[I] + wJ * s.n[J]);
  float chiK = s.chi2[I] + s.chi2[J];
  s.mx[I] = 0.0f;
  s.my[I] = 0.0f;
  s.cx[I] = scK.x;
  s.cy[I] = scK.y;
  s.cz[I] = scK.z;
  s.sw[I] = swK;
  s.n[I] = nK;
  s.sa[I] = saK;
  s.chi2[I] = chiK;
  s.mx[J] = s.mx[L];
  s.my[J] = s.my[L];
  s.cx[J] = s.cx[L];
  s.cy[J] = s.cy[L];
  s.cz[J] = s.cz[L];
  s.sw[J] = s.sw[L];
  s.n[J] = s.n[L];
  s.sa[J] = s.sa[L];
  s.chi2[J] = s.chi2[L];
  splitZeroLane(s, L);
  s.K--;
}
static int performMerging(VMM &v, float thr, Suff &suff, Split &sp) {  // Merger.h:67-89, :218-279
  int total = 0;
  for (;;) {
    if (!(v.K > uint64_t(W))) break;
    int K = int(v.K), ci = 0, cj = 0;
    float minCost = FLT_MAX;
    bool found = false;
    for (int i = 0; i < K - 1; ++i)
      for (int j = i + 1; j < K; ++j) {
        float cost = mergeCost(v, i, j);
        if (cost < thr && cost < minCost && sp.n[i] > 0.0f && sp.n[j] > 0.0f) {
          ci = i;
          cj = j;
          minCost = cost;
          found = true;
        }
      }
    if (!found) break;
    V3 muI = v3(v.mx[ci], v.my[ci], v.mz[ci]), muJ = v3(v.mx[cj], v.my[cj], v.mz[cj]);
    float wI = v.w[ci], wJ = v.w[cj];
    vmmMerge(v, ci, cj);
    V3 muK = v3(v.mx[ci], v.my[ci], v.mz[ci]);
    float wK = v.w[ci];
    splitMergeStats(sp, ci, cj, wI, muI, wJ, muJ, wK, muK);
    suffMerge(suff, ci, cj);
    total++;
  }
  return total;
}
static void recursiveSplitting(VMM &v, Suff &suff, float thr, float mcEst, const Sample *S, size_t n, const Config &cfg) {
  // Splitter.h:293-356
  bool mask[KMAX];
  Split sp;
  std::memset(&sp, 0, sizeof(sp));
  Suff temp = suff;
  int numSplits = -1;
  while (v.K < KMAX && numSplits != 0) {
    numSplits = 0;
    splitClear(sp, KMAX);
    splitClear(sp, v.K);
    updateSplitStats(v, sp, mcEst, S, n);
    std::vector<Cand> cands = splitCandidates(sp);
    for (int k = 0; k < KMAX; ++k) mask[k] = false;
    size_t numComp = v.K;
    for (size_t k = 0; k < numComp; ++k) {
      if (cands[k].chi > thr && v.K < KMAX) {
        bool ok = splitComponent(v, sp, temp, int(cands[k].idx));
        mask[cands[k].idx] = true;
        mask[v.K - 1] = true;
        if (ok) numSplits++;
      }
    }
    if (numSplits > 0) {
      suffClear(temp, v.K);
      emLoop(v, temp, S, n, cfg, mask);
      suff.K = v.K;
      suffMaskedReplace(suff, mask, temp);
    }
  }
}

static void asmFit(Region &r, const Sample *S, size_t n, const Config &cfg) {  // ASMF.h:303-347
  VMM &v = r.vmm;
  suffClear(r.suff, cfg.initK);
  splitClear(r.split, cfg.initK);
  r.afterSplit = r.afterMerge = 0;
  vmmInitUniform(v, int(cfg.initK), cfg.initKappa);
  suffClear(r.suff, cfg.initK);
  r.suff.normalized = true;
  emLoop(v, r.suff, S, n, cfg, nullptr);
  componentDistances(v, r.suff, S, n, true);
  if (cfg.useSplitMerge) {
    float mcEst = r.suff.sumWeights / r.suff.numSamples;
    recursiveSplitting(v, r.suff, cfg.splitThreshold, mcEst, S, n, cfg);
    splitClear(r.split, v.K);
    updateSplitStats(v, r.split, mcEst, S, n);
    performMerging(v, cfg.mergeThreshold, r.suff, r.split);
  }
  r.afterSplit = 0;
  r.afterMerge = 0;
  componentDistances(v, r.suff, S, n, true);
}
static void asmUpdate(Region &r, const Sample *S, size_t n, const Config &cfg) {  // ASMF.h:352-462
  VMM &v = r.vmm;
  uint64_t prevK = v.K;
  emLoop(v, r.suff, S, n, cfg, nullptr);
  if (prevK < v.K) r.split.K = v.K;
  if (cfg.useSplitMerge) {
    float mcEst = r.suff.sumWeights / r.suff.numSamples;
    r.afterSplit += n;
    r.afterMerge += n;
    updateSplitStats(v, r.split, mcEst, S, n);
    if (r.afterSplit >= uint64_t(int64_t(cfg.minSplit))) {
      bool mask[KMAX];
      for (int k = 0; k < KMAX; ++k) mask[k] = false;
      std::vector<Cand> cands = splitCandidates(r.split);
      int total = 0;
      for (size_t k = 0; k < cands.size(); ++k) {
        if (cands[k].chi > cfg.splitThreshold && v.K < KMAX) {
          splitComponent(v, r.split, r.suff, int(cands[k].idx));
          mask[cands[k].idx] = true;
          mask[v.K - 1] = true;
          total++;
        }
      }
      if (total > 0 && cfg.partialReFit && n >= uint64_t(int64_t(cfg.minRefit))) {
        Suff temp = r.suff;
        suffClear(temp, v.K);
        emLoop(v, temp, S, n, cfg, mask);
        r.suff.K = v.K;
        suffMaskedReplace(r.suff, mask, temp);
        r.split.K = v.K;
      }
      r.afterSplit = 0;
    }
    if (r.afterMerge >= uint64_t(int64_t(cfg.minMerge))) {
      performMerging(v, cfg.mergeThreshold, r.suff, r.split);
      r.afterMerge = 0;
    }
  }
  componentDistances(v, r.suff, S, n, false);
}

// ------------------------------------------------------------------ spatial
struct IStats {  // IntegerSampleStatistics, INTERGER_V2 (SampleStatistics.h:195-342)
  int64_t m[3] = {0, 0, 0}, v[3] = {0, 0, 0};
  uint32_t n = 0;
  int64_t lo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, hi[3] = {-INT32_MAX, -INT32_MAX, -INT32_MAX};
  float center[3], half[3], inv[3];
  explicit IStats(const float *b) {
    for (int d = 0; d < 3; ++d) {
      float ext = b[3 + d] - b[d];
      half[d] = ext * 0.5f;
      inv[d] = rcp1sse(half[d]);
      center[d] = b[d] + half[d];
    }
  }
  void add(const float *p) {
    n++;
    for (int d = 0; d < 3; ++d) {
      float t = (p[d] - center[d]) * inv[d];
      float tv = (t * t) * 4096.f;
      t *= 4096.f;
      int64_t it = int64_t(t);
      m[d] += it;
      v[d] += int64_t(tv);
      lo[d] = std::min(lo[d], it);
      hi[d] = std::max(hi[d], it);
    }
  }
  Stats toStats() const {
    Stats s;
    if (n > 0) {
      float invN = 1.f / float(n);
      float mean[3], var[3];
      for (int d = 0; d < 3; ++d) {
        mean[d] = (float(m[d]) / 4096.f) * invN;
        var[d] = (float(v[d]) / 4096.f) * invN;
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
        float lw = ((float(lo[d]) - 0.0f) / 4096.f) * half[d] + center[d];
        float up = ((float(hi[d]) + 0.0f) / 4096.f) * half[d] + center[d];
        s.lo[d] = lw;
        s.hi[d] = up;
      }
      s.n = float(n);
    }
    return s;
  }
};
static void statsMerge(Stats &a, const Stats &b) {  // SampleStatistics.h:101-118
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
static void statsSplit(Stats &s, int dim, float pos, float decay, bool lower) {  // SampleStatistics.h:68-99
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

struct Neighbours {
  uint32_t ids[8];
  float px[8], py[8], pz[8];
  uint32_t size;
};

// ------------------------------------------------------------------ directional quadtree
// DirectionalQuadtree<SphereToSquareCylindrical> and DirectionalQuadtreeFactory
// (dqt/DQT.h, DQTFactory.h, Traversal.h, Rect.h, SphereToSquare.h) at the
// defaults of PGLDQTFactoryArguments (include/openpgl/config.h:95-102):
// REJECTION_SAMPLING leaf estimator, MEAN split metric, split threshold 0.01,
// footprint factor 1, 12 levels; the PER_LEAF estimator, the SECOND_MOMENT
// metric and a zero footprint are the factory's other branches
// (DQTFactory.h:168-186).
struct DqtConfig {  // DQTFactory.h:33-70, stored as the raw 20-byte struct
  int32_t leafEstimator = 0, splitMetric = 0;
  float splitThreshold = 0.01f, footprintFactor = 1.0f;
  uint32_t maxLevels = 12;
};
static_assert(sizeof(DqtConfig) == 20, "DirectionalQuadtreeFactory::Configuration is 20 bytes");
struct DqtNode {  // DirectionalQuadtreeNode (DQT.h:12-23)
  uint32_t child = 0;
  float weight = 0.0f;
};
struct DqtStatsNode {  // DirectionalQuadtreeFactory::StatsNode (DQTFactory.h:72-81)
  uint32_t child = 0;
  float sampleWeight = 0.0f, splitWeight = 0.0f, numSamples = 0.0f, first = 0.0f, second = 0.0f;
};
static_assert(sizeof(DqtStatsNode) == 24, "StatsNode is 24 bytes");
struct DqtRegion {  // the quadtree of a region and its training statistics
  float pivot[3] = {0.0f, 0.0f, 0.0f};
  std::vector<DqtNode> nodes = {DqtNode()};
  float numSamples = 0.0f;
  std::vector<DqtStatsNode> stats = {DqtStatsNode()};
};
struct Box2 {  // Rect<float> (Rect.h:8-40)
  float x0, y0, x1, y1;
  float area() const { return (x1 - x0) * (y1 - y0); }
  Box2 child(uint32_t c) const {
    const float mx = (x0 + x1) / 2.0f, my = (y0 + y1) / 2.0f;
    return {(c & 1) ? mx : x0, (c & 2) ? my : y0, (c & 1) ? x1 : mx, (c & 2) ? y1 : my};
  }
  Box2 intersect(const Box2 &o) const {
    Box2 r{smax(x0, o.x0), smax(y0, o.y0), smin(x1, o.x1), smin(y1, o.y1)};
    r.x1 = smax(r.x0, r.x1);
    r.y1 = smax(r.y0, r.y1);
    return r;
  }
};
static inline float clampf(float v, float lo, float hi) { return emax(lo, emin(v, hi)); }  // embree::clamp

// SphereToSquareCylindrical (SphereToSquare.h:34-61): x = (cos theta + 1) / 2,
// y = phi / 2pi + 1/2 (phi from libm's atan2f, the division in double).
static void dqtDirToPoint(V3 d, float &px, float &py) {
  const float dx = clampf(d.x, -1.f, 1.f), dy = clampf(d.y, -1.f, 1.f), dz = clampf(d.z, -1.f, 1.f);
  const float phi = std::atan2(dy, dx);
  px = clampf((dz + 1.0f) / 2.0f, 0.f, 1.f);
  py = clampf(float(double(phi) / (2.0 * M_PI) + 0.5), 0.f, 1.f);
}
static V3 dqtPointToDir(float px, float py) {
  px = clampf(px, 0.f, 1.f);
  py = clampf(py, 0.f, 1.f);
  const float cosTheta = 2.0f * px - 1.0f;
  const float sinTheta = std::sqrt(1.0f - cosTheta * cosTheta);
  const float phi = float((double(py) - 0.5) * 2.0 * M_PI);
  return v3(clampf(sinTheta * std::cos(phi), -1.f, 1.f), clampf(sinTheta * std::sin(phi), -1.f, 1.f),
            clampf(cosTheta, -1.f, 1.f));
}
static const float kDqtJacobian = 4.0f * float(M_PI);

// queryNode (Traversal.h:37-49): the leaf a point of the unit square falls in
template <typename N>
static uint32_t dqtQuery(const N *nodes, float px, float py, Box2 &rect) {
  rect = {0.f, 0.f, 1.f, 1.f};
  uint32_t idx = 0;
  while (nodes[idx].child > 0) {
    uint32_t c = 0;
    if (px >= 0.5f) { px -= 0.5f; c += 1; }
    if (py >= 0.5f) { py -= 0.5f; c += 2; }
    px *= 2.0f;
    py *= 2.0f;
    rect = rect.child(c);
    idx = nodes[idx].child + c;
  }
  return idx;
}

// Footprint splat (Traversal.h:61-90): a box of footprintFactor times the size
// of the leaf the point falls in, centred on the point and clipped to the unit
// square; every leaf it overlaps receives the overlap's share of the box area.
// Leaves are visited depth first, children in order 0..3.
template <typename F>
static void dqtSplatVisit(std::vector<DqtStatsNode> &nodes, const Box2 &filter, float filterArea, uint32_t i,
                          Box2 rect, F &apply) {
  const float a = filter.intersect(rect).area();
  if (a == 0.0f) return;
  if (nodes[i].child == 0) {
    apply(nodes[i], a / filterArea);
    return;
  }
  for (uint32_t c = 0; c < 4; ++c) dqtSplatVisit(nodes, filter, filterArea, nodes[i].child + c, rect.child(c), apply);
}

static void dqtBuildSplit(std::vector<DqtStatsNode> &nodes, uint32_t p, uint32_t i) {  // DQTFactory.h:313-324
  DqtStatsNode &n = nodes[i];
  const DqtStatsNode &par = nodes[p];
  n.child = 0;
  n.numSamples = par.numSamples / 4;
  n.first = par.first / 4;
  n.second = par.second / 4;
  n.sampleWeight = par.sampleWeight / 4;
  n.splitWeight = par.splitWeight / 4;
}

// buildRecursive (DQTFactory.h:283-311): the new tree in depth-first order,
// the four children of a node allocated together when it is reached.
static void dqtBuild(std::vector<DqtStatsNode> &out, const std::vector<DqtStatsNode> &old, const DqtConfig &cfg,
                     uint32_t i, uint32_t j, uint32_t level) {
  const DqtStatsNode on = old[i];
  out[j] = on;
  if (level < cfg.maxLevels && on.splitWeight > cfg.splitThreshold * old[0].splitWeight) {
    const uint32_t c0 = uint32_t(out.size());
    out[j].child = c0;
    out.resize(out.size() + 4);
    if (on.child > 0) {
      for (uint32_t c = 0; c < 4; ++c) dqtBuild(out, old, cfg, on.child + c, c0 + c, level + 1);
    } else {
      for (uint32_t c = 0; c < 4; ++c) dqtBuildSplit(out, j, c0 + c);
    }
  } else {
    out[j].child = 0;
  }
}

// SphereToSquareCylindrical::area (SphereToSquare.h:57-59)
static inline float dqtArea(const Box2 &r) { return 4.0f * float(M_PI) * (r.x1 - r.x0) * (r.y1 - r.y0); }

// sample and split weights bottom-up (DQTFactory.h:232-263): a leaf's sample
// weight is its first moment times 1 / (decayed sample count) (rejection
// sampling) or times its solid angle / its own sample count (per leaf); its
// split weight is the same (mean) or sqrt(solid angle * second moment); an
// inner node's are the sums of its children's in order
static void dqtWeights(std::vector<DqtStatsNode> &nodes, uint32_t i, Box2 rect, const DqtConfig &cfg, float numSamples) {
  DqtStatsNode &n = nodes[i];
  if (n.child > 0) {
    for (uint32_t c = 0; c < 4; ++c) dqtWeights(nodes, nodes[i].child + c, rect.child(c), cfg, numSamples);
    DqtStatsNode &m = nodes[i];
    m.sampleWeight = 0.0f;
    m.splitWeight = 0.0f;
    for (uint32_t c = 0; c < 4; ++c) {
      m.sampleWeight += nodes[m.child + c].sampleWeight;
      m.splitWeight += nodes[m.child + c].splitWeight;
    }
  } else {
    const float k = cfg.leafEstimator == 0 ? 1.0f / numSamples : dqtArea(rect) / n.numSamples;
    const float first = n.first * k, second = n.second * k;
    n.sampleWeight = first;
    n.splitWeight = cfg.splitMetric == 0 ? first : std::sqrt(dqtArea(rect) * second);
  }
}

static void dqtUpdate(DqtRegion &r, const Sample *S, size_t n, const DqtConfig &cfg) {  // DQTFactory.h:199-281
  // the dispatch of DQTFactory.h:168-185 runs no branch for other values
  if (!(cfg.footprintFactor >= 0.0f) || (cfg.leafEstimator != 0 && cfg.leafEstimator != 1) ||
      (cfg.splitMetric != 0 && cfg.splitMetric != 1))
    return;
  r.numSamples += float(n);
  const float ff = cfg.footprintFactor;
  for (size_t i = 0; i < n; ++i) {
    const Sample &s = S[i];
    float first, second;
    if (cfg.leafEstimator == 0) {  // REJECTION_SAMPLING
      first = s.weight;
      second = s.weight * s.weight * s.pdf;
    } else {  // PER_LEAF
      first = s.weight * s.pdf;
      second = first * first;
    }
    float px, py;
    dqtDirToPoint(v3(s.dir[0], s.dir[1], s.dir[2]), px, py);
    auto apply = [&](DqtStatsNode &node, float w) {
      node.numSamples += w;
      node.first += w * first;
      node.second += w * second;
    };
    Box2 leaf;
    const uint32_t li = dqtQuery(r.stats.data(), px, py, leaf);
    if (ff > 0.0f) {
      const float hx = ff * (leaf.x1 - leaf.x0) / 2.0f, hy = ff * (leaf.y1 - leaf.y0) / 2.0f;
      const Box2 filter = Box2{px - hx, py - hy, px + hx, py + hy}.intersect(Box2{0.f, 0.f, 1.f, 1.f});
      dqtSplatVisit(r.stats, filter, filter.area(), 0, Box2{0.f, 0.f, 1.f, 1.f}, apply);
    } else {
      apply(r.stats[li], 1.0f);
    }
  }
  dqtWeights(r.stats, 0, Box2{0.f, 0.f, 1.f, 1.f}, cfg, r.numSamples);
  std::vector<DqtStatsNode> old;
  old.swap(r.stats);
  r.stats.resize(1);
  dqtBuild(r.stats, old, cfg, 0, 0, 0);
  r.nodes.resize(r.stats.size());
  for (size_t i = 0; i < r.stats.size(); ++i) r.nodes[i] = DqtNode{r.stats[i].child, r.stats[i].sampleWeight};
}

static void dqtDecay(DqtRegion &r, float a) {  // Statistics::decay (DQTFactory.h:109-116)
  r.numSamples *= a;
  for (DqtStatsNode &n : r.stats) {
    n.numSamples *= a;
    n.first *= a;
    n.second *= a;
  }
}

static void dqtFit(DqtRegion &r, const Sample *S, size_t n, const DqtConfig &cfg) {  // DQTFactory.h:149-155
  for (int i = 0; i < 5; ++i) {
    dqtDecay(r, 0.25f);
    dqtUpdate(r, S, n, cfg);
  }
}

static bool dqtValid(const DqtRegion &r) {  // DirectionalQuadtree::isValid (DQT.h:40-42)
  return !std::isinf(r.nodes[0].weight) && r.nodes[0].weight > 0;
}
static bool dqtStatsValid(const DqtRegion &r) {  // Statistics::isValid (DQTFactory.h:95-107)
  auto ok = [](float v) { return !std::isnan(v) && !std::isinf(v) && v >= 0; };
  for (const DqtStatsNode &n : r.stats)
    if (!ok(n.sampleWeight) || !ok(n.splitWeight) || !ok(n.numSamples) || !ok(n.first) || !ok(n.second)) return false;
  return r.stats[0].sampleWeight > 0 && r.stats[0].splitWeight > 0;
}

// samplePdf (DQT.h:62-72, :115-153): a stochastic descent that picks the
// left/right half by u.x and the top/bottom half by u.y, each rescaled into
// the chosen part; pdf = leaf weight / (root weight * leaf area) / 4pi
static float dqtSamplePdf(const DqtRegion &r, float ux, float uy, V3 &dir) {
  const std::vector<DqtNode> &N = r.nodes;
  float span = 1.0f, x = 0.0f, y = 0.0f;
  auto rescale = [](float t, float &u) {
    if (u < t) {
      u /= t;
      return true;
    }
    u -= t;
    u /= 1.0f - t;
    return false;
  };
  uint32_t idx = 0;
  while (N[idx].child > 0) {
    span /= 2.0f;
    uint32_t off = 0;
    const DqtNode *c = &N[N[idx].child];
    const float wl = c[0].weight + c[2].weight, wr = c[1].weight + c[3].weight;
    if (!rescale(wl / (wl + wr), ux)) {
      off += 1;
      x += span;
    }
    const float wt = c[off].weight, wb = c[off + 2].weight;
    if (!rescale(wt / (wt + wb), uy)) {
      off += 2;
      y += span;
    }
    idx = N[idx].child + off;
  }
  float pdf = N[idx].weight / (N[0].weight * span * span);
  const float px = x + ux * span, py = y + uy * span;
  pdf /= kDqtJacobian;
  dir = dqtPointToDir(px, py);
  return pdf;
}
static float dqtPdf(const DqtRegion &r, V3 d) {  // DQT.h:53-60, :155-159
  float px, py;
  dqtDirToPoint(d, px, py);
  Box2 rect;
  const uint32_t i = dqtQuery(r.nodes.data(), px, py, rect);
  const float p = r.nodes[i].weight / (r.nodes[0].weight * rect.area()) / kDqtJacobian;
  return smin(FLT_MAX, p);
}

struct SubField {
  Config cfg;
  bool isSurface = true;
  float decay = 0.25f;
  uint64_t iteration = 0, totalSPP = 0;
  bool boundsSet = false, initialized = false;
  float sceneBounds[6] = {0, 0, 0, 0, 0, 0};
  float kdBounds[6] = {0, 0, 0, 0, 0, 0};
  bool kdInit = false;
  std::vector<Node> nodes;
  std::vector<Region> regions;
  std::vector<DqtRegion> dqts;  // the quadtree field type: region i's quadtree and statistics
  DqtConfig dqtCfg;
  std::vector<Neighbours> nbrs;
  std::vector<Sample> samples;
  int threads = 1;

  void estimateSceneBounds() {  // Field.h:326-344 (the loop stops one short of the end)
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {FLT_MIN, FLT_MIN, FLT_MIN};
    size_t n = samples.size();
    for (size_t i = 0; i + 1 < n; ++i)
      for (int d = 0; d < 3; ++d) {
        lo[d] = emin(lo[d], samples[i].pos[d]);
        hi[d] = emax(hi[d], samples[i].pos[d]);
      }
    for (int d = 0; d < 3; ++d) {
      float c = (lo[d] + hi[d]) * 0.5f;
      sceneBounds[d] = c + 3.0f * (lo[d] - c);
      sceneBounds[3 + d] = c + 3.0f * (hi[d] - c);
    }
    boundsSet = true;
  }

  Region newRegion() {
    Region r;
    std::memset(static_cast<void *>(&r), 0, sizeof(r));
    r.stats = Stats();
    return r;
  }

  static void splitDimPos(const Stats &s, uint8_t &dim, float &pos) {  // KDTreeBuilder.h:218-230
    float v[3] = {s.var[0] / s.n, s.var[1] / s.n, s.var[2] / s.n};
    int i = v[1] > v[0] ? 1 : 0;
    dim = uint8_t(v[i] > v[2] ? i : 2);
    pos = s.mean[dim];
  }

  void updateNode(uint32_t nodeIdx, uint64_t depth, const float *bounds, size_t b, size_t e, const Stats &st) {
    // KDTreeBuilder.h:233-350, serial order (left subtree first)
    if (e - b == 0) return;
    uint8_t dim = 0;
    float pos = 0.0f;
    uint32_t lr0;
    if (nodes[nodeIdx].leaf()) {
      uint32_t di = nodes[nodeIdx].child();
      Region &reg = regions[di];
      if (depth < cfg.maxDepth && reg.stats.n + float(e - b) > float(cfg.maxSamples)) {
        Stats merged = reg.stats;
        statsMerge(merged, st);
        splitDimPos(merged, dim, pos);
        Region right = reg;
        statsSplit(regions[di].stats, dim, pos, 0.25f, false);
        statsSplit(right.stats, dim, pos, 0.25f, true);
        regions[di].splitFlag = true;
        right.splitFlag = true;
        regions[di].bounds[3 + dim] = pos;
        right.bounds[dim] = pos;
        regions.push_back(right);
        if (cfg.dqt) dqts.push_back(dqts[di]);
        uint32_t rightIdx = uint32_t(regions.size() - 1);
        lr0 = uint32_t(nodes.size());
        nodes.push_back(Node{0.0f, 0});
        nodes.push_back(Node{0.0f, 0});
        nodes[nodeIdx].split = pos;
        nodes[nodeIdx].bits = (uint32_t(dim) << 30) | lr0;
        nodes[lr0].bits = (3u << 30) | di;
        nodes[lr0 + 1].bits = (3u << 30) | rightIdx;
      } else {
        statsMerge(regions[di].stats, st);
        regions[di].rb = b;
        regions[di].re = e;
        return;
      }
    } else {
      dim = uint8_t(nodes[nodeIdx].dim());
      pos = nodes[nodeIdx].split;
      lr0 = nodes[nodeIdx].child();
    }
    float cb[2][6];
    std::memcpy(cb[0], bounds, 24);
    std::memcpy(cb[1], bounds, 24);
    cb[0][3 + dim] = pos;
    cb[1][dim] = pos;
    bool needStats = nodes[lr0].leaf() || nodes[lr0 + 1].leaf();
    IStats il(bounds), ir(bounds);
    // stable partition: < pivot left (KDTreeBuilder.h:193)
    std::vector<Sample> right;
    size_t w = b;
    for (size_t i = b; i < e; ++i) {
      const Sample &s = samples[i];
      if (s.pos[dim] < pos) {
        if (needStats) il.add(s.pos);
        samples[w++] = s;
      } else {
        if (needStats) ir.add(s.pos);
        right.push_back(s);
      }
    }
    std::copy(right.begin(), right.end(), samples.begin() + w);
    Stats sl, sr;
    if (needStats) {
      sl = il.toStats();
      sr = ir.toStats();
    }
    updateNode(lr0, depth + 1, cb[0], b, w, sl);
    updateNode(lr0 + 1, depth + 1, cb[1], w, e, sr);
  }

  void updateTree() {  // KDTreeBuilder.h:76-118
    Stats st;
    size_t n = samples.size();
    if (nodes[0].leaf()) {
      IStats is(kdBounds);
      for (size_t i = 0; i < n; ++i) is.add(samples[i].pos);
      st = is.toStats();
    }
    updateNode(0, 1, kdBounds, 0, n, st);
  }

  void buildKNN() {  // KNN.h:189-266, nanoflann L2 (a-b)^2 summed in dimension order
    size_t R = regions.size();
    nbrs.assign(R, Neighbours());
    for (size_t n = 0; n < R; ++n) {
      const float *q = regions[n].stats.mean;
      std::vector<std::pair<float, uint32_t>> d(R);
      for (size_t j = 0; j < R; ++j) {
        const float *p = regions[j].stats.mean;
        float dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
        float r = 0.0f;
        r += dx * dx;
        r += dy * dy;
        r += dz * dz;
        d[j] = {r, uint32_t(j)};
      }
      size_t k = std::min<size_t>(8, R);
      std::partial_sort(d.begin(), d.begin() + k, d.end());
      Neighbours &nb = nbrs[n];
      nb.size = uint32_t(k);
      for (size_t i = 0; i < 8; ++i) {
        if (i < k) {
          uint32_t id = d[i].second;
          nb.ids[i] = id;
          nb.px[i] = regions[id].stats.mean[0];
          nb.py[i] = regions[id].stats.mean[1];
          nb.pz[i] = regions[id].stats.mean[2];
        } else {
          nb.ids[i] = ~0u;
          nb.px[i] = nb.py[i] = nb.pz[i] = 0.0f;
        }
      }
    }
  }

  template <typename F>
  void parallelRegions(F f) {
    size_t R = regions.size();
    if (threads <= 1 || R < 2) {
      for (size_t i = 0; i < R; ++i) f(i);
      return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
      pool.emplace_back([&] {
        for (;;) {
          size_t i = next.fetch_add(1);
          if (i >= R) break;
          f(i);
        }
      });
    for (auto &th : pool) th.join();
  }

  static bool sampleLess(const Sample &a, const Sample &b) {  // SampleData.h:82-93
    if (a.weight != b.weight) return a.weight < b.weight;
    if (a.pdf != b.pdf) return a.pdf < b.pdf;
    if (a.distance != b.distance) return a.distance < b.distance;
    for (int d = 0; d < 3; ++d)
      if (a.pos[d] != b.pos[d]) return a.pos[d] < b.pos[d];
    for (int d = 0; d < 3; ++d)
      if (a.dir[d] != b.dir[d]) return a.dir[d] < b.dir[d];
    return false;
  }

  void prepare(Region &r, size_t b, size_t e) {  // WEMFactory.h:1151-1196
    if (!cfg.parallax) return;  // WEMFactory.h:1186: plain VMMs keep their samples
    const Stats &st = r.stats;
    V3 var = v3(st.var[0] / st.n, st.var[1] / st.n, st.var[2] / st.n);
    float minD = lengthf(var);
    minD = 3.f * 3.f * std::sqrt(minD);
    for (size_t i = b; i < e; ++i) {
      Sample &s = samples[i];
      if (std::isinf(s.distance)) {
        std::memcpy(s.pos, st.mean, 12);
        continue;
      } else if (!(s.distance > 0.0f)) {
        continue;
      }
      float dist = std::fmax(minD, s.distance);
      V3 o = add(v3(s.pos[0], s.pos[1], s.pos[2]), mul(v3(s.dir[0], s.dir[1], s.dir[2]), dist));
      V3 nd = sub(o, v3(st.mean[0], st.mean[1], st.mean[2]));
      float nl = lengthf(nd);
      nd = divs(nd, nl);
      std::memcpy(s.pos, st.mean, 12);
      s.distance = nl;
      s.dir[0] = nd.x;
      s.dir[1] = nd.y;
      s.dir[2] = nd.z;
    }
  }

  void fitRegions() {  // Field.h:389-439
    parallelRegions([&](size_t n) {
      Region &r = regions[n];
      float mean[3];
      std::memcpy(mean, r.stats.mean, 12);
      if (r.re - r.rb > 0) {
        if (cfg.deterministic) std::sort(samples.begin() + r.rb, samples.begin() + r.re, sampleLess);
        if (cfg.dqt) {  // the quadtree factory prepares nothing (DQTFactory.h:146-147)
          DqtRegion &q = dqts[n];
          dqtFit(q, samples.data() + r.rb, r.re - r.rb, dqtCfg);
          std::memcpy(q.pivot, mean, 12);
          r.valid = dqtValid(q);
          r.splitFlag = false;
          r.rb = r.re = 0;
          return;
        }
        prepare(r, r.rb, r.re);
        asmFit(r, samples.data() + r.rb, r.re - r.rb, cfg);
        std::memcpy(r.vmm.pivot, mean, 12);
        r.valid = vmmIsValid(r.vmm);
        r.splitFlag = false;
      } else {
        r.valid = false;
        r.splitFlag = false;
      }
      r.rb = r.re = 0;
    });
    initialized = true;
  }

  void updateRegions() {  // Field.h:441-511
    parallelRegions([&](size_t n) {
      Region &r = regions[n];
      if (r.splitFlag) {
        if (cfg.dqt) {
          dqtDecay(dqts[n], decay);
        } else {
          suffDecay(r.suff, decay);
          splitDecay(r.split, decay);
        }
        r.splitFlag = false;
      }
      float mean[3];
      std::memcpy(mean, r.stats.mean, 12);
      if (r.re - r.rb > 0) {
        if (cfg.deterministic) std::sort(samples.begin() + r.rb, samples.begin() + r.re, sampleLess);
        if (cfg.dqt) {  // no parallax compensation (DQT.h:28-30), no preparation
          dqtUpdate(dqts[n], samples.data() + r.rb, r.re - r.rb, dqtCfg);
          r.valid = dqtValid(dqts[n]) && dqtStatsValid(dqts[n]);
          r.rb = r.re = 0;
          return;
        }
        if (cfg.parallax) {  // Field.h:476-482
          V3 shift = v3(r.vmm.pivot[0] - mean[0], r.vmm.pivot[1] - mean[1], r.vmm.pivot[2] - mean[2]);
          suffParallaxShift(r.suff, r.vmm, shift);
          vmmParallaxShift(r.vmm, shift);
        }
        prepare(r, r.rb, r.re);
        asmUpdate(r, samples.data() + r.rb, r.re - r.rb, cfg);
        r.valid = vmmIsValid(r.vmm) && suffIsValid(r.suff) && splitIsValid(r.split);
      }
      r.rb = r.re = 0;
    });
  }

  void build(const std::vector<Sample> &in) {  // Field.h:147-185
    iteration = 0;
    totalSPP = 0;
    if (!in.empty()) {
      samples = in;
      if (!boundsSet) estimateSceneBounds();
      std::memcpy(kdBounds, sceneBounds, 24);
      kdInit = true;
      nodes.clear();
      nodes.push_back(Node{0.0f, (3u << 30) | 0u});
      regions.clear();
      regions.push_back(newRegion());
      dqts.assign(cfg.dqt ? 1 : 0, DqtRegion());
      std::memcpy(regions[0].bounds, sceneBounds, 24);
      updateTree();
      if (cfg.knn) buildKNN();
      fitRegions();
    }
    iteration++;
  }
  void update(const std::vector<Sample> &in) {  // Field.h:187-220
    if (!in.empty()) {
      samples = in;
      updateTree();
      if (cfg.knn) buildKNN();
      updateRegions();
    }
    iteration++;
  }

  int32_t leafAt(const float *p) const {  // KDTree.h:380-395
    uint32_t i = 0;
    while (!nodes[i].leaf()) i = nodes[i].child() + (p[nodes[i].dim()] >= nodes[i].split ? 1u : 0u);
    return int32_t(nodes[i].child());
  }

  // KNN.h:22-28, :134-148
  uint32_t approximateClosest(uint32_t region, const float *p, float *s1d) const {
    const Neighbours &nb = nbrs[region];
    uint32_t size = std::min<uint32_t>(4, nb.size);
    uint32_t sel = uint32_t(*s1d * float(size));
    *s1d = (*s1d - float(sel) / float(size)) * float(size);
    sel = std::min(sel, size - 1);
    uint32_t key[8];
    for (int i = 0; i < 8; ++i) {
      V3 d = v3(nb.px[i] - p[0], nb.py[i] - p[1], nb.pz[i] - p[2]);
      float dd = dotf(d, d);
      uint32_t kb = (fbits(dd) & ~7u) | uint32_t(i);
      if (nb.ids[i] == ~0u) kb = fbits(INFINITY);
      key[i] = kb;
    }
    float fk[8];
    for (int i = 0; i < 8; ++i) fk[i] = bitsf(key[i]);
    std::sort(fk, fk + 8);
    return nb.ids[fbits(fk[sel]) & 7u];
  }
};

struct QueryIn {
  float pos[3], normal[3], s1d, u[2];
};
struct QueryOut {
  uint32_t ok, id;
  float s1d, dir[3], pdf, pdfLi;
};

struct Field {
  SubField surface, volume;
  uint64_t iteration = 0;
};

// A quadtree query (DQTSurfaceSamplingDistribution.h, DQTVolumeSamplingDistribution.h):
// neither the cosine nor the Henyey-Greenstein product is supported, so the
// surface, volume and phase-function queries all sample the region's quadtree.
static void dqtQueryOut(const DqtRegion &r, const QueryIn &q, uint32_t leaf, QueryOut &o) {
  V3 d;
  const float pdf = dqtSamplePdf(r, q.u[0], q.u[1], d);
  o.ok = 1;
  o.id = leaf;
  o.dir[0] = d.x;
  o.dir[1] = d.y;
  o.dir[2] = d.z;
  o.pdf = pdf;
  o.pdfLi = dqtPdf(r, d);
}

static void runQuery(const SubField &f, const QueryIn &q, QueryOut &o, bool cosine) {
  std::memset(&o, 0, sizeof(o));
  float s1d = q.s1d;
  o.s1d = s1d;
  if (!(f.iteration > 0)) return;
  const float *b = f.kdBounds;
  for (int d = 0; d < 3; ++d)
    if (!(q.pos[d] >= b[d] && q.pos[d] <= b[3 + d])) return;
  uint32_t leaf = uint32_t(f.leafAt(q.pos));
  uint32_t reg = leaf;
  if (f.cfg.knn && s1d >= 0.f) reg = f.approximateClosest(leaf, q.pos, &s1d);
  o.s1d = s1d;
  const Region &r = f.regions[reg];
  if (!r.valid) return;
  if (f.cfg.dqt) return dqtQueryOut(f.dqts[reg], q, leaf, o);
  VMM li = r.vmm;
  V3 shift = v3(li.pivot[0] - q.pos[0], li.pivot[1] - q.pos[1], li.pivot[2] - q.pos[2]);
  if (f.cfg.parallax) vmmParallaxShift(li, shift);  // VMMSurfaceSamplingDistribution.h:41-46
  VMM g = li;
  if (cosine) {
    const float ck = 2.18853f;
    const float cn = float(double(2.18853f) / (2.0 * M_PI * double(1.0f - std::exp(-2.0f * 2.18853f))));
    vmmProduct(g, 1.0f, v3(q.normal[0], q.normal[1], q.normal[2]), ck, cn);
  }
  V3 d = vmmSample(g, (q.u[0] - 0.0f) / 1.0f, q.u[1]);
  o.ok = 1;
  o.id = leaf;
  o.dir[0] = d.x;
  o.dir[1] = d.y;
  o.dir[2] = d.z;
  o.pdf = 0.0f + 1.0f * vmmPdf(g, d);
  o.pdfLi = vmmPdf(li, d);
}

// Volume query with the single-lobe Henyey-Greenstein product
// (VMMVolumeSamplingDistribution.h:54-128, VMMPhaseFunctions.h:45-57): the
// shifted mixture times each lobe of the phase function's three-lobe fit
// (lobes of the fit's sign facing dir, else -dir), products weighted by their
// integrals; a sample picks a product by u.x, then samples it with u.x
// rescaled; the pdf is the weighted sum of the products' pdfs.
static void runQueryHG(const SubField &f, const QueryIn &q, float meanCosine, QueryOut &o) {
  std::memset(&o, 0, sizeof(o));
  float s1d = q.s1d;
  o.s1d = s1d;
  if (!(f.iteration > 0)) return;
  const float *b = f.kdBounds;
  for (int d = 0; d < 3; ++d)
    if (!(q.pos[d] >= b[d] && q.pos[d] <= b[3 + d])) return;
  uint32_t leaf = uint32_t(f.leafAt(q.pos));
  uint32_t reg = leaf;
  if (f.cfg.knn && s1d >= 0.f) reg = f.approximateClosest(leaf, q.pos, &s1d);
  o.s1d = s1d;
  const Region &r = f.regions[reg];
  if (!r.valid) return;
  if (f.cfg.dqt) return dqtQueryOut(f.dqts[reg], q, leaf, o);
  VMM li = r.vmm;
  V3 shift = v3(li.pivot[0] - q.pos[0], li.pivot[1] - q.pos[1], li.pivot[2] - q.pos[2]);
  if (f.cfg.parallax) vmmParallaxShift(li, shift);  // VMMSurfaceSamplingDistribution.h:41-46
  const float absG = std::fabs(meanCosine);
  const float step = (pgl::kHgMaxMeanCosine - pgl::kHgMinMeanCosine) / float(pgl::kHgFits);
  int idx = int(std::floor((absG - pgl::kHgMinMeanCosine) / step));
  idx = std::min(idx, pgl::kHgFits - 1);
  const V3 dir = v3(q.normal[0], q.normal[1], q.normal[2]);
  VMM g[pgl::kHgLobes];
  float w[pgl::kHgLobes];
  float sum = 0.0f;
  for (int i = 0; i < pgl::kHgLobes; ++i) {
    const pgl::HgLobeFit &fit = pgl::kHgTable[idx][i];
    g[i] = li;
    const V3 out = meanCosine * fit.meanCosine > 0.f ? dir : v3(-dir.x, -dir.y, -dir.z);
    w[i] = vmmProduct(g[i], fit.weight, out, fit.kappa, fit.normalization);
    sum += w[i];
  }
  for (int i = 0; i < pgl::kHgLobes; ++i) w[i] /= sum;
  float acc = 0.0f;
  int i = 0;
  for (; i < pgl::kHgLobes - 1; ++i) {
    const float next = acc + w[i];
    if (next > q.u[0]) break;
    acc = next;
  }
  V3 d = vmmSample(g[i], (q.u[0] - acc) / w[i], q.u[1]);
  float pdf = 0.0f;
  for (int k = 0; k < pgl::kHgLobes; ++k) pdf += w[k] * vmmPdf(g[k], d);
  o.ok = 1;
  o.id = leaf;
  o.dir[0] = d.x;
  o.dir[1] = d.y;
  o.dir[2] = d.z;
  o.pdf = pdf;
  o.pdfLi = vmmPdf(li, d);
}

// ------------------------------------------------------------------ field file
struct Writer {
  std::string b;
  void raw(const void *p, size_t n) { b.append(reinterpret_cast<const char *>(p), n); }
  template <typename T>
  void put(const T &v) { raw(&v, sizeof(T)); }
  void lanes(const float *a, int v) { raw(a + v * W, sizeof(float) * W); }
};
static void writeKnn(Writer &w, const SubField &f) {
  w.put<uint8_t>(f.cfg.knn);
  bool built = f.cfg.knn && !f.regions.empty() && f.initialized;
  w.put<uint8_t>(built);
  if (built) {
    w.put<uint32_t>(uint32_t(f.regions.size()));
    for (const Region &r : f.regions) {
      float p[4] = {r.stats.mean[0], r.stats.mean[1], r.stats.mean[2], 0.0f};
      w.raw(p, 16);
    }
  }
}
static void writeKdHead(Writer &w, const SubField &f) {
  w.put<uint64_t>(f.cfg.minSamples);
  w.put<uint64_t>(f.cfg.maxSamples);
  w.put<uint64_t>(f.cfg.maxDepth);
  w.put<uint8_t>(f.kdInit);
  w.raw(f.kdBounds, 24);
  w.put<uint64_t>(f.nodes.size());
  for (const Node &n : f.nodes) {
    w.put<float>(n.split);
    w.put<uint32_t>(n.bits);
  }
  w.put<uint64_t>(f.regions.size());
}
static void writeRegionTail(Writer &w, const Region &r) {
  w.raw(r.stats.mean, 12);
  w.raw(r.stats.var, 12);
  w.put<float>(r.stats.n);
  w.raw(r.stats.lo, 12);
  w.raw(r.stats.hi, 12);
  w.put<uint8_t>(r.splitFlag);
  w.put<uint64_t>(r.rb);
  w.put<uint64_t>(r.re);
}
// The quadtree field after the common head: the factory configuration
// (DQTFactory.h:59-61), the kd-tree, per region the validity flag, the
// quadtree (DQT.h:88-93), the bounds, the training statistics
// (DQTFactory.h:118-123) and the sample statistics, then the neighbour points.
static void writeSubDqt(Writer &w, const SubField &f) {
  w.put<DqtConfig>(f.dqtCfg);
  writeKdHead(w, f);
  for (size_t i = 0; i < f.regions.size(); ++i) {
    const Region &r = f.regions[i];
    const DqtRegion &q = f.dqts[i];
    w.put<uint8_t>(r.valid);
    w.raw(q.pivot, 12);
    w.put<uint64_t>(q.nodes.size());
    w.raw(q.nodes.data(), q.nodes.size() * sizeof(DqtNode));
    w.raw(r.bounds, 24);
    w.put<float>(q.numSamples);
    w.put<uint64_t>(q.stats.size());
    w.raw(q.stats.data(), q.stats.size() * sizeof(DqtStatsNode));
    writeRegionTail(w, r);
  }
  writeKnn(w, f);
}

static void writeSub(Writer &w, const SubField &f) {  // same layout as Field::serialize (Field.h:240-267)
  w.put<uint8_t>(f.isSurface);
  w.put<float>(f.decay);
  w.put<uint64_t>(f.iteration);
  w.put<uint64_t>(f.totalSPP);
  w.put<uint8_t>(f.cfg.deterministic);
  w.put<uint8_t>(1);
  w.put<uint8_t>(f.boundsSet);
  w.raw(f.sceneBounds, 24);
  w.put<uint8_t>(f.initialized);
  float t[4] = {0, 0, 0, 0};
  w.raw(t, 16);
  const Config &c = f.cfg;
  if (c.dqt) return writeSubDqt(w, f);
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
  w.put<uint8_t>(c.partialReFit);
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
  for (const Node &n : f.nodes) {
    w.put<float>(n.split);
    w.put<uint32_t>(n.bits);
  }
  w.put<uint64_t>(f.regions.size());
  for (const Region &r : f.regions) {
    w.put<uint8_t>(r.valid);
    for (int v = 0; v < NV; ++v) {
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
    w.raw(r.bounds, 24);
    for (int v = 0; v < NV; ++v) {
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
    w.put<uint8_t>(r.suff.normalized);
    for (int v = 0; v < NV; ++v) {
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
    w.raw(r.stats.mean, 12);
    w.raw(r.stats.var, 12);
    w.put<float>(r.stats.n);
    w.raw(r.stats.lo, 12);
    w.raw(r.stats.hi, 12);
    w.put<uint8_t>(r.splitFlag);
    w.put<uint64_t>(r.rb);
    w.put<uint64_t>(r.re);
  }
  w.put<uint8_t>(f.cfg.knn);
  bool built = f.cfg.knn && !f.regions.empty() && f.initialized;
  w.put<uint8_t>(built);
  if (built) {
    w.put<uint32_t>(uint32_t(f.regions.size()));
    for (const Region &r : f.regions) {
      float p[4] = {r.stats.mean[0], r.stats.mean[1], r.stats.mean[2], 0.0f};
      w.raw(p, 16);
    }
  }
}

}  // namespace orc

using namespace orc;

extern "C" {

void *orc_field_new(int deterministic, uint64_t maxSamplesPerLeaf, int threads) {
  static bool once = (initUniformDirections(), true);
  (void)once;
  Field *f = new Field();
  for (SubField *s : {&f->surface, &f->volume}) {
    s->cfg.deterministic = deterministic != 0;
    s->cfg.maxSamples = maxSamplesPerLeaf;
    s->cfg.minSplit = int(maxSamplesPerLeaf / 8);
    s->cfg.minRefit = int(maxSamplesPerLeaf / 8);
    s->cfg.minMerge = int(maxSamplesPerLeaf / 4);
    s->cfg.maxMeanCosine = KappaToMeanCosine(s->cfg.maxKappa);
    s->threads = threads < 1 ? 1 : threads;
  }
  f->surface.isSurface = true;
  f->volume.isSurface = false;
  return f;
}

void orc_field_free(void *h) { delete static_cast<Field *>(h); }

void orc_field_set_scene_bounds(void *h, const float *b6) {  // SurfaceVolumeField.h:87-93
  Field *f = static_cast<Field *>(h);
  float b[6];
  for (int d = 0; d < 3; ++d) {
    b[d] = b6[d] - 1.01f * std::fabs(b6[d]);
    b[3 + d] = b6[3 + d] + 1.01f * std::fabs(b6[3 + d]);
  }
  for (SubField *s : {&f->surface, &f->volume}) {
    std::memcpy(s->sceneBounds, b, 24);
    s->boundsSet = true;
  }
}

// pglFieldUpdate with a sample storage that holds exactly these samples
// (SampleDataStorage.h:72-90 routes by the inside-volume flag).
void orc_field_update(void *h, const Sample *samples, uint64_t n) {
  Field *f = static_cast<Field *>(h);
  std::vector<Sample> surf, vol;
  for (uint64_t i = 0; i < n; ++i) (samples[i].flags & 2u ? vol : surf).push_back(samples[i]);
  if (!surf.empty()) {
    if (!f->surface.initialized)
      f->surface.build(surf);
    else
      f->surface.update(surf);
  }
  if (!vol.empty()) {
    if (!f->volume.initialized)
      f->volume.build(vol);
    else
      f->volume.update(vol);
  }
  f->iteration++;
}

uint64_t orc_field_iteration(void *h) { return static_cast<Field *>(h)->iteration; }

uint64_t orc_field_store(void *h, char *out, uint64_t cap) {
  Field *f = static_cast<Field *>(h);
  Writer w;
  const char hdr[] = "OPENPGL_0.6.0_FIELD";
  w.raw(hdr, sizeof(hdr));
  w.put<int32_t>(0);                             // kd-tree
  // PARALLAX_AWARE_VMM, QUADTREE or VMM (include/openpgl/types.h:8-13)
  w.put<int32_t>(f->surface.cfg.dqt ? 1 : f->surface.cfg.parallax ? 0 : 2);
  w.put<uint64_t>(f->iteration);
  w.put<uint64_t>(0);
  writeSub(w, f->surface);
  writeSub(w, f->volume);
  if (out && cap >= w.b.size()) std::memcpy(out, w.b.data(), w.b.size());
  return w.b.size();
}

void orc_field_query(void *h, int volume, int cosine, const QueryIn *q, QueryOut *o, uint64_t n) {
  Field *f = static_cast<Field *>(h);
  const SubField &s = volume ? f->volume : f->surface;
  for (uint64_t i = 0; i < n; ++i) runQuery(s, q[i], o[i], cosine != 0);
}

// The plain VMM field type (PGL_DIRECTIONAL_DISTRIBUTION_VMM) instead of the
// parallax-aware one; call before the first update.
void orc_field_set_parallax(void *h, int parallax) {
  Field *f = static_cast<Field *>(h);
  f->surface.cfg.parallax = f->volume.cfg.parallax = parallax != 0;
}

// The directional quadtree field type (PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE,
// default factory arguments); call before the first update.
void orc_field_set_dqt(void *h) {
  Field *f = static_cast<Field *>(h);
  f->surface.cfg.dqt = f->volume.cfg.dqt = true;
}
// PGLDQTFactoryArguments other than the defaults (config.h:95-102)
void orc_field_set_dqt_args(void *h, int leafEstimator, int splitMetric, float splitThreshold, float footprintFactor,
                            uint32_t maxLevels) {
  Field *f = static_cast<Field *>(h);
  for (SubField *s : {&f->surface, &f->volume}) {
    s->dqtCfg.leafEstimator = leafEstimator;
    s->dqtCfg.splitMetric = splitMetric;
    s->dqtCfg.splitThreshold = splitThreshold;
    s->dqtCfg.footprintFactor = footprintFactor;
    s->dqtCfg.maxLevels = maxLevels;
  }
}

// Volume queries with the Henyey-Greenstein product, query i with mean cosine g[i]
// and q[i].normal as the direction of the phase function.
void orc_field_query_hg(void *h, const QueryIn *q, const float *g, QueryOut *o, uint64_t n) {
  Field *f = static_cast<Field *>(h);
  for (uint64_t i = 0; i < n; ++i) runQueryHG(f->volume, q[i], g[i], o[i]);
}

// Region index of each position (kd traversal only) for leaf-assignment checks.
void orc_field_leaf_of(void *h, int volume, const float *pos, int32_t *out, uint64_t n) {
  Field *f = static_cast<Field *>(h);
  const SubField &s = volume ? f->volume : f->surface;
  for (uint64_t i = 0; i < n; ++i) out[i] = s.nodes.empty() ? -1 : s.leafAt(pos + 3 * i);
}

float orc_fexp(float x) { return fexp(x); }
float orc_flog(float x) { return flog(x); }
float orc_rcp(float x) { return rcp1(x); }
float orc_rsqrt(float x) { return rsqrt1(x); }
}

extern "C" {
// Integer position statistics of a sample set relative to a box, and their
// float conversion (IntegerSampleStatistics, SampleStatistics.h:195-342).
// out_i: mean[3], var[3], lo[3], hi[3], n; out_f: mean[3], var[3], n, lo[3], hi[3], inv[3], center[3]
void orc_istats(const Sample *s, uint64_t n, const float *bounds, int64_t *out_i, float *out_f) {
  IStats st(bounds);
  for (uint64_t i = 0; i < n; ++i) st.add(s[i].pos);
  for (int d = 0; d < 3; ++d) {
    out_i[d] = st.m[d];
    out_i[3 + d] = st.v[d];
    out_i[6 + d] = st.lo[d];
    out_i[9 + d] = st.hi[d];
  }
  out_i[12] = st.n;
  Stats ss = st.toStats();
  for (int d = 0; d < 3; ++d) {
    out_f[d] = ss.mean[d];
    out_f[3 + d] = ss.var[d];
    out_f[7 + d] = ss.lo[d];
    out_f[10 + d] = ss.hi[d];
    out_f[13 + d] = st.inv[d];
    out_f[16 + d] = st.center[d];
  }
  out_f[6] = ss.n;
}
}

extern "C" {
// SampleStatistics::merge on packed {mean[3], var[3], n, lo[3], hi[3]} records.
void orc_stats_merge(const float *a, const float *b, float *o) {
  Stats A, B;
  for (int d = 0; d < 3; ++d) {
    A.mean[d] = a[d]; A.var[d] = a[3 + d]; A.lo[d] = a[7 + d]; A.hi[d] = a[10 + d];
    B.mean[d] = b[d]; B.var[d] = b[3 + d]; B.lo[d] = b[7 + d]; B.hi[d] = b[10 + d];
  }
  A.n = a[6];
  B.n = b[6];
  statsMerge(A, B);
  for (int d = 0; d < 3; ++d) { o[d] = A.mean[d]; o[3 + d] = A.var[d]; o[7 + d] = A.lo[d]; o[10 + d] = A.hi[d]; }
  o[6] = A.n;
}
}
