// Scalar arithmetic of the guiding field, shared by host and device code.
//
// Open PGL's CPU_8 device (the reference) runs its math on 8-wide AVX2
// vectors.  To give the same numbers, every function here performs the same
// IEEE operations in the same order:
//  * translation units that include this file are compiled with FMA
//    contraction disabled (nvcc --fmad=false, g++ -ffp-contract=off); FMAs
//    are written out (fmaf) exactly where embree's madd/msub/fnmadd are
//    (third-party/embreeSrc/common/math/vec3.h:204-209, linearspace3.h:150);
//  * approximate reciprocals start from the x86 RCPSS/RSQRTSS values, held in
//    tables measured on x86 (x86_approx_tables.h), then take the same Newton
//    step as embree::rcp/rsqrt (math/emath.h:61-145, simd/vfloat8_avx.h:254-290);
//  * fast exp/log/sin/acos follow the published ispc/syrah polynomials that
//    the reference vendors (math/transcendental.h:18-472);
//  * horizontal sums over a group of 8 lanes use the vfloat8 reduce tree
//    ((0+1)+(2+3))+((4+5)+(6+7)) (simd/vfloat8_avx.h:677-683).
#pragma once

#include <cstdint>
#include <cmath>
#include <cfloat>

#include <vector_types.h>

#ifdef __CUDACC__
#define PGL_HD __host__ __device__ __forceinline__
#else
#define PGL_HD inline
#endif

namespace pgl {

constexpr int kLanes = 8;       // SIMD width of the CPU_8 reference
constexpr int kMaxK = 32;       // PGL_VMM_MAX_COMPONENTS
constexpr float kInv4Pi = 0.07957747154594767f;
constexpr float kTwoPiF = 6.28318530717958647692f;  // (float)(2*M_PI)
constexpr double kPiD = 3.14159265358979323846;

}  // namespace pgl
#include "x86_approx_tables.h"
namespace pgl {
// rcp/rsqrt seed tables: the host reads the static arrays of
// x86_approx_tables.h; every CUDA translation unit has its own constant-memory
// copy, filled by the upload function that PGL_DEFINE_TABLE_UPLOAD defines.
// Inputs at which the host C library's expf and cosf differ from the
// double-precision function rounded once (gen_libm_exceptions.cpp writes
// them, the library loads them into device memory when it sets up CUDA):
// sorted {x, host result} pairs.
struct LibmTables {
  const float2 *expf;
  const float2 *cosf;
  const float2 *sinf;
  uint32_t numExpf, numCosf, numSinf;
};
#ifdef __CUDACC__
static __constant__ uint32_t d_rcp_table[2048];
static __constant__ uint32_t d_rsqrt_table[2048];
static __constant__ LibmTables d_libm;
#define PGL_DEFINE_TABLE_UPLOAD(fn)                                                                  \
  cudaError_t fn(const LibmTables &libm) {                                                           \
    cudaError_t e = cudaMemcpyToSymbol(d_rcp_table, pgl_x86_rcp_table, sizeof(pgl_x86_rcp_table));     \
    if (e != cudaSuccess) return e;                                                                  \
    e = cudaMemcpyToSymbol(d_libm, &libm, sizeof(LibmTables));                                       \
    if (e != cudaSuccess) return e;                                                                  \
    return cudaMemcpyToSymbol(d_rsqrt_table, pgl_x86_rsqrt_table, sizeof(pgl_x86_rsqrt_table));       \
  }
#endif

PGL_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  __builtin_memcpy(&u, &f, 4);
  return u;
#endif
}
PGL_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
#endif
}
PGL_HD uint32_t rcp_seed(uint32_t idx) {
#ifdef __CUDA_ARCH__
  return d_rcp_table[idx];
#else
  return pgl_x86_rcp_table[idx];
#endif
}
PGL_HD uint32_t rsqrt_seed(uint32_t idx) {
#ifdef __CUDA_ARCH__
  return d_rsqrt_table[idx];
#else
  return pgl_x86_rsqrt_table[idx];
#endif
}
PGL_HD float fmaf_(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

// x86 RCPSS: 12-bit reciprocal estimate (sign/zero/inf/denormal handling of the
// instruction; the mantissa comes from the measured table).
PGL_HD float rcpss(float x) {
  uint32_t u = f2u(x), s = u & 0x80000000u, e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  if (e == 0) return u2f(s | 0x7F800000u);
  if (e == 255) return m ? x : u2f(s);
  uint32_t t = rcp_seed(m >> 12);
  int re = int((t >> 23) & 0xFFu) - (int(e) - 127);
  if (re <= 0) return u2f(s);
  if (re >= 255) return u2f(s | 0x7F800000u);
  return u2f(s | (uint32_t(re) << 23) | (t & 0x7FFFFFu));
}
// x86 RSQRTSS
PGL_HD float rsqrtss(float x) {
  uint32_t u = f2u(x), e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  if (u & 0x80000000u) return (e == 0 && m == 0) ? -INFINITY : NAN;
  if (e == 0) return INFINITY;
  if (e == 255) return m ? x : 0.0f;
  int ue = int(e) - 127, p = ue & 1, q = ue >> 1;
  uint32_t t = rsqrt_seed(uint32_t(p) * 1024u + (m >> 13));
  int re = int((t >> 23) & 0xFFu) - q;
  return u2f((uint32_t(re) << 23) | (t & 0x7FFFFFu));
}
// embree::rcp(float) in an AVX2 unit: r * fnmadd(r, a, 2)
PGL_HD float rcp_avx2(float a) {
  float r = rcpss(a);
  return r * fmaf_(-r, a, 2.0f);
}
// embree::rcp(float) in an SSE unit: r * (2 - r*a).  The kd-tree statistics
// use this form on every device: their inline members are emitted by the
// SSE translation unit first and the linker keeps that copy.
PGL_HD float rcp_sse(float a) {
  float r = rcpss(a);
  return r * (2.0f - r * a);
}
// embree::rsqrt(float) (no FMA in the scalar form)
PGL_HD float rsqrt_scalar(float a) {
  float r = rsqrtss(a);
  return (1.5f * r) + (((a * -0.5f) * r) * (r * r));
}
// embree::rsqrt(vfloat8), AVX2 form
PGL_HD float rsqrt_lane(float a) {
  float r = rsqrtss(a);
  return fmaf_(1.5f, r, ((a * -0.5f) * r) * (r * r));
}

PGL_HD float emin(float a, float b) { return a < b ? a : b; }   // embree::min, MINPS
PGL_HD float emax(float a, float b) { return a < b ? b : a; }   // embree::max
PGL_HD float smin(float a, float b) { return (b < a) ? b : a; }  // std::min
PGL_HD float smax(float a, float b) { return (a < b) ? b : a; }  // std::max
PGL_HD bool isvalidf(float v) { return (v > -1.844E18f) & (v < 1.844E18f); }

PGL_HD float floorf_(float x) {
#ifdef __CUDA_ARCH__
  return floorf(x);
#else
  return std::floor(x);
#endif
}

// Double-float arithmetic: a value h + l held as two floats, |l| <= ulp(h)/2
// (T. J. Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971), from the error-free sum (Knuth) and the
// error-free product by FMA.
struct DFloat {
  float h, l;
};
PGL_HD DFloat df_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = a + b;
  return {s, b - (s - a)};
}
PGL_HD DFloat df_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
PGL_HD DFloat df_two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf_(a, b, -p)};
}
PGL_HD DFloat df_mul(DFloat a, DFloat b) {
  const float p = a.h * b.h;
  float e = fmaf_(a.h, b.h, -p);
  e = fmaf_(a.h, b.l, e);
  e = fmaf_(a.l, b.h, e);
  return df_fast_two_sum(p, e);
}
PGL_HD DFloat df_mul_f(DFloat a, float b) {
  const float p = a.h * b;
  return df_fast_two_sum(p, fmaf_(a.l, b, fmaf_(a.h, b, -p)));
}
// a + b where the sum does not cancel (|a + b| well above |a| / 2 or |b| / 2)
PGL_HD DFloat df_add(DFloat a, DFloat b) {
  const DFloat s = df_two_sum(a.h, b.h);
  return df_fast_two_sum(s.h, s.l + (a.l + b.l));
}

// sin x and cos x of a float +0 <= x < 8 in double-float arithmetic, before
// rounding: the additive reduction of W. J. Cody and W. Waite (Software
// Manual for the Elementary Functions, 1980) by pi/2 = C1 + C2 + C3 (floats;
// k <= 5 and |x - k C1| < 1, so fma(-k, C1, x) is exact), then the Taylor
// series of sin r and cos r for |r| <= pi/4 (to r^15 and r^16), the leading
// coefficients as double-floats, the tails in float.  The constants are the
// exact values rounded to float (hi) and the remainders rounded to float (lo).
// The relative error of either result is below 2^-41 on every float of the
// range (checked against long double).
PGL_HD void sincos_df_parts(float x, DFloat *s, DFloat *c) {
  const float kf = rintf(x * 0x1.45f306p-1f);  // x * 2/pi to the nearest integer
  const float t1 = fmaf_(-kf, 0x1.921fb6p+0f, x);
  const DFloat p = df_two_prod(kf, -0x1.777a5cp-25f);
  const DFloat s0 = df_two_sum(t1, -p.h);
  const DFloat r = df_two_sum(s0.h, (s0.l - p.l) - kf * -0x1.ee59dap-50f);
  const DFloat z = df_mul(r, r);
  // sin r = r + r z (S1 + z (S2 + z (S3 + z T))), S_i = (-1)^i / (2i + 1)!
  const float t = fmaf_(fmaf_(fmaf_(-0x1.ae7f3ep-41f, z.h, 0x1.612462p-33f), z.h, -0x1.ae6456p-26f), z.h,
                        0x1.71de3ap-19f);
  DFloat a = df_add({-0x1.a01a02p-13f, 0x1.7f97fap-39f}, df_mul_f(z, t));
  a = df_add({0x1.111112p-7f, -0x1.dddddep-32f}, df_mul(z, a));
  a = df_add({-0x1.555556p-3f, 0x1.555556p-28f}, df_mul(z, a));
  const DFloat sr = df_add(r, df_mul(r, df_mul(z, a)));
  // cos r = 1 + z (-1/2 + z (C2 + z (C3 + z T'))), C_i = (-1)^i / (2i)!
  const float tc = fmaf_(fmaf_(fmaf_(fmaf_(0x1.ae7f3ep-45f, z.h, -0x1.93974ap-37f), z.h, 0x1.1eed8ep-29f), z.h,
                               -0x1.27e4fcp-22f), z.h, 0x1.a01a02p-16f);
  DFloat b = df_add({-0x1.6c16c2p-10f, 0x1.27d27ep-35f}, df_mul_f(z, tc));
  b = df_add({0x1.555556p-5f, -0x1.555556p-30f}, df_mul(z, b));
  b = df_add({-0.5f, 0.0f}, df_mul(z, b));
  const DFloat cr = df_add({1.0f, 0.0f}, df_mul(z, b));
  const DFloat nsr = {-sr.h, -sr.l}, ncr = {-cr.h, -cr.l};
  switch (int(kf) & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = nsr; break;
    case 2: *s = nsr; *c = ncr; break;
    default: *s = ncr; *c = sr; break;
  }
}
// A double-float rounded to float by A. Ziv's test ("Fast evaluation of
// elementary mathematical functions with correctly rounded last bit", ACM
// TOMS 17(3), 1991): the value, widened by 2^-38 relative on either side,
// must round to one float, which then is the exact value rounded to nearest.
PGL_HD bool df_round_checked(DFloat v, float *out) {
  const float e = fabsf(v.h) * 0x1p-38f;
  const float lo = v.h + (v.l - e), hi = v.h + (v.l + e);
  *out = lo;
  return lo == hi;
}
// sin x and cos x correctly rounded for +0 <= x < 8, in float arithmetic;
// false (outputs unspecified) where the test above cannot decide or x is
// outside that range.  Where it returns true, both equal the double-precision
// functions rounded once to float.
PGL_HD bool sincos_df(float x, float *s, float *c) {
  if (f2u(x) >= 0x41000000u) return false;  // not +0 <= x < 8 (-0 keeps its sign on the double path)
  DFloat ds, dc;
  sincos_df_parts(x, &ds, &dc);
  const bool okS = df_round_checked(ds, s);
  const bool okC = df_round_checked(dc, c);
  return okS && okC;
}

// Single-precision exp/log/cos/sin/sincos as the host C library returns them
// (std::exp(float) etc. on the reference side).  On the device each is
// evaluated in double and rounded once to float: that is the correctly rounded
// result except where the exact value lies within ~2^-29 ulp of a rounding
// boundary, and it equals the C library's float result wherever that one is
// correctly rounded.  glibc's expf and cosf are not on about 0.07 % and 0.2 %
// of inputs; lib_expf and lib_cosf take the host library's result for those
// inputs (and for those near a rounding boundary) from its exception table.
#ifdef __CUDA_ARCH__
__device__ __forceinline__ float libm_lookup(const float2 *t, uint32_t n, float x, float r) {
  if (t == nullptr || n == 0 || !(x >= t[0].x && x <= t[n - 1].x)) return r;
  uint32_t lo = 0, hi = n - 1;  // t[lo].x <= x <= t[hi].x
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (t[mid].x < x) lo = mid + 1;
    else hi = mid;
  }
  return t[lo].x == x ? t[lo].y : r;
}
#endif
PGL_HD float lib_expf(float x) {
#ifdef __CUDA_ARCH__
  return libm_lookup(d_libm.expf, d_libm.numExpf, x, float(exp(double(x))));
#else
  return std::exp(x);
#endif
}
PGL_HD float lib_cosf(float x) {
#ifdef __CUDA_ARCH__
  return libm_lookup(d_libm.cosf, d_libm.numCosf, x, float(cos(double(x))));
#else
  return std::cos(x);
#endif
}
// sinf of the host C library (odd: the table holds x >= 0)
PGL_HD float lib_sinf(float x) {
#ifdef __CUDA_ARCH__
  const float a = fabsf(x);
  const float r = libm_lookup(d_libm.sinf, d_libm.numSinf, a, float(sin(double(a))));
  return x < 0.0f ? -r : r;
#else
  return std::sin(x);
#endif
}
// cosf of the host C library for any sign (even)
PGL_HD float lib_cosf_any(float x) {
#ifdef __CUDA_ARCH__
  return lib_cosf(fabsf(x));
#else
  return std::cos(x);
#endif
}
// On the device: the float evaluation of sincos_df where it decides (all but
// about 3 in 100,000 inputs of [0, 2 pi]), which gives the same bits as the
// double path below (checked on every float of [0, 8)) at a small fraction
// of its cost: a double-precision instruction occupies a warp scheduler for
// tens of cycles on this part.
PGL_HD void lib_sincosf(float x, float *s, float *c) {
#ifdef __CUDA_ARCH__
  if (sincos_df(x, s, c)) return;
  double sd, cd;
  sincos(double(x), &sd, &cd);
  *s = float(sd);
  *c = float(cd);
#else
  *s = std::sin(x);
  *c = std::cos(x);
#endif
}

// a / b, correctly rounded, from y = RN(1/b) (Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990): with y within half an ulp of 1/b and q0 = RN(a y)
// within one ulp of a/b, the residual r = a - b q0 is exact under FMA and
// RN(q0 + r y) = RN(a / b).  The theorem assumes that nothing underflows or
// overflows, so operands and quotient outside [1e-30, 1e30] in magnitude
// (zeros, infinities and NaNs included) take the division instead.
PGL_HD float div_rcp(float a, float b, float y) {
  float q0 = a * y;
  float r = fmaf_(-q0, b, a);
  float q = fmaf_(r, y, q0);
  const float aa = a < 0.0f ? -a : a, aq = q < 0.0f ? -q : q;
  if (!(aa >= 1e-30f && aa <= 1e30f && aq >= 1e-30f && aq <= 1e30f)) q = a / b;
  return q;
}
// y = RN(1/b) for 1e-30 <= |b| <= 1e30, else 0 (div_rcp then divides).
PGL_HD float rcp_for_div(float b) {
  const float ab = b < 0.0f ? -b : b;
  return (ab >= 1e-30f && ab <= 1e30f) ? 1.0f / b : 0.0f;
}

// a / b rounded to nearest from an approximate reciprocal y (relative error
// a few 2^-24): q1 = q0 + (a - b q0) y with q0 = a y is a faithful quotient
// (one of the two floats around a/b); the remainder a - b q of a faithful q
// is exact under FMA; so RN(a/b) is whichever of q1 and its neighbour towards
// a/b has the smaller remainder (a quotient of floats is never exactly half
// way between two floats).  Valid for normal b and |a|, |a/b| in
// [1e-30, 1e30]; the caller checks the range.
PGL_HD float div_faithful_fix(float a, float b, float y) {
  const float q0 = a * y;
  const float r0 = fmaf_(-q0, b, a);
  const float q1 = fmaf_(r0, y, q0);
  const float r1 = fmaf_(-q1, b, a);
  const bool up = (r1 > 0.0f) == (b > 0.0f);  // a/b above q1
  const uint32_t u = f2u(q1);
  const float q2 = u2f(((q1 > 0.0f) == up) ? u + 1u : u - 1u);
  const float r2 = fmaf_(-q2, b, a);
  const float ar1 = r1 < 0.0f ? -r1 : r1, ar2 = r2 < 0.0f ? -r2 : r2;
  return (r1 != 0.0f && ar2 < ar1) ? q2 : q1;
}
// approximate reciprocal (the hardware's rcp.approx; about one ulp)
PGL_HD float rcp_approx(float b) {
#ifdef __CUDA_ARCH__
  float y;
  asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(b));
  return y;
#else
  return 1.0f / b;
#endif
}

// RN(1/b) for 1e-30 <= |b| <= 1e30 (div_faithful_fix from the approximate
// reciprocal).
PGL_HD float rcp_rn(float b) { return div_faithful_fix(1.0f, b, rcp_approx(b)); }
// The three FMA-unit steps of Markstein's division (div_rcp) without the
// range check: the caller checks |a| and the result against [1e-30, 1e30].
PGL_HD float markstein_q(float a, float b, float y) {
  const float q0 = a * y;
  return fmaf_(fmaf_(-q0, b, a), y, q0);
}

// fastapprox::exp
PGL_HD float fexp(float v) {
  const float ln2Part1 = float(0.6931457519), ln2Part2 = float(1.4286067653e-6);
  const float oneOverLn2 = 1.44269502162933349609375f;
  float scaled = v * oneOverLn2;
  float kReal = floorf_(scaled);
  int k = int(kReal);
  float x = v - kReal * ln2Part1;
  x -= kReal * ln2Part2;
  float r = x * 2.7555381529964506626129150390625e-4f + 1.304379315115511417388916015625e-3f;
  r = x * r + 8.378830738365650177001953125e-3f;
  r = x * r + 4.16539050638675689697265625e-2f;
  r = x * r + 0.166668415069580078125f;
  r = x * r + 0.4999999105930328369140625f;
  r = x * r + 1.0f;
  r = x * r + 1.0f;
  r *= u2f(uint32_t((k + 127) << 23));
  if (kReal > 127.0f) r = INFINITY;
  if (kReal <= -127.0f) r = 0.0f;
  return r;
}
// fastapprox::log
PGL_HD float flog(float v) {
  bool useNan = v < 0.0f, useInf = v == 0.0f;
  float patched = (useNan || useInf) ? 1.0f : v;
  int32_t iv = int32_t(f2u(patched));
  int exponent = ((iv >> 23) + 1) - 127;
  float reduced = u2f(uint32_t((iv & int32_t(0x807FFFFF)) | (126 << 23)));
  float x1 = 1.0f - reduced;
  float r = x1 * 1.7491014003753662109375f + -2.4899270534515380859375f;
  r = x1 * r + 1.98442304134368896484375f;
  r = x1 * r + -0.599632322788238525390625f;
  r = x1 * r + 0.3424419462680816650390625f;
  r = x1 * r + 0.17541764676570892333984375f;
  r = x1 * r + 0.2519190013408660888671875f;
  r = x1 * r + 0.33326041698455810546875f;
  r = x1 * r + 0.50000095367431640625f;
  r = x1 * r + 1.0f;
  r *= -x1;
  r += float(exponent) * 0.693147182464599609375f;
  if (useNan) return NAN;
  if (useInf) return -INFINITY;
  return r;
}
// fastapprox::sin
PGL_HD float fsin(float v) {
  float scaled = v * 0.636619746685028076171875f;
  float kReal = floorf_(scaled);
  int k = int(kReal);
  float x = v - kReal * 1.57079637050628662109375f;
  int m4 = k & 3;
  bool useCos = (m4 == 1) | (m4 == 3);
  bool flip = m4 > 1;
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
// fastapprox::acos (= pi/2 - asin)
PGL_HD float facos(float x0) {
  bool neg = x0 < 0.0f;
  float x = fabsf(x0);
  bool nanres = x > 1.0f;
  float v = 1.57079517841339111328125f +
            x * (-0.21450997889041900634765625f +
                 x * (8.78556668758392333984375e-2f +
                      x * (-4.489909112453460693359375e-2f +
                           x * (1.928029954433441162109375e-2f + x * (-4.3095736764371395111083984375e-3f)))));
  v *= -sqrtf(1.0f - x);
  v = v + 1.57079637050628662109375f;
  v = (v < 0.0f) ? 0.0f : v;
  v = neg ? -v : v;
  v = nanres ? NAN : v;
  return 1.57079637050628662109375f - v;
}

struct V3 {
  float x, y, z;
};
PGL_HD V3 mk(float x, float y, float z) { return V3{x, y, z}; }
PGL_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
PGL_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
PGL_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
PGL_HD V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
// embree::dot = madd(a.x,b.x, madd(a.y,b.y, a.z*b.z))
PGL_HD float dot(V3 a, V3 b) { return fmaf_(a.x, b.x, fmaf_(a.y, b.y, a.z * b.z)); }
PGL_HD V3 cross(V3 a, V3 b) {
  return V3{fmaf_(a.y, b.z, -(a.z * b.y)), fmaf_(a.z, b.x, -(a.x * b.z)), fmaf_(a.x, b.y, -(a.y * b.x))};
}
PGL_HD float length(V3 a) { return sqrtf(dot(a, a)); }

struct Frame {
  V3 vx, vy, vz;
};
// embree::frame(N); lane=true picks the vector rsqrt refinement
PGL_HD Frame frame_of(V3 N, bool lane) {
  V3 dx0 = mk(0.0f, N.z, -N.y), dx1 = mk(-N.z, 0.0f, N.x);
  V3 d = dot(dx0, dx0) > dot(dx1, dx1) ? dx0 : dx1;
  float r = lane ? rsqrt_lane(dot(d, d)) : rsqrt_scalar(dot(d, d));
  V3 dx = d * r;
  V3 c = cross(N, dx);
  float r2 = lane ? rsqrt_lane(dot(c, c)) : rsqrt_scalar(dot(c, c));
  return Frame{dx, c * r2, N};
}
PGL_HD V3 xfm(const Frame &f, V3 b) {
  return V3{fmaf_(b.x, f.vx.x, fmaf_(b.y, f.vy.x, b.z * f.vz.x)),
            fmaf_(b.x, f.vx.y, fmaf_(b.y, f.vy.y, b.z * f.vz.y)),
            fmaf_(b.x, f.vx.z, fmaf_(b.y, f.vy.z, b.z * f.vz.z))};
}
PGL_HD Frame inverse_of(const Frame &a) {
  V3 c0 = cross(a.vy, a.vz), c1 = cross(a.vz, a.vx), c2 = cross(a.vx, a.vy);
  float det = dot(a.vx, c0);
  return Frame{mk(c0.x, c1.x, c2.x) / det, mk(c0.y, c1.y, c2.y) / det, mk(c0.z, c1.z, c2.z) / det};
}

PGL_HD float reduce8(const float *l) {
  float a0 = l[0] + l[1], a2 = l[2] + l[3], a4 = l[4] + l[5], a6 = l[6] + l[7];
  return (a0 + a2) + (a4 + a6);
}
PGL_HD int vec_count(int K) { return (K + kLanes - 1) / kLanes; }

PGL_HD float mean_cosine_to_kappa(float mc) {
  float mc2 = mc * mc;
  return (mc * 3.0f - mc * mc2) / (1.0f - mc2);
}

// (float)(k / (2*pi*(1-e))) evaluated in double, as the reference's scalar
// code does where a float meets the M_PI literal.
PGL_HD float vmf_norm_double(float k, float e) { return float(double(k) / (2.0 * kPiD * double(1.0f - e))); }

}  // namespace pgl
