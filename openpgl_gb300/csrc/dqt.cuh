// Directional quadtree field type on the device: the quadtree of a region,
// its training statistics, and the arithmetic of Open PGL's
// DirectionalQuadtree<SphereToSquareCylindrical> and
// DirectionalQuadtreeFactory (directional/dqt/DQT.h, DQTFactory.h,
// Traversal.h, Rect.h, SphereToSquare.h), shared by the update kernel and the
// queries.  Every float operation is the reference's, in its order (the
// translation units are compiled without contraction), so that a region's
// quadtree carries the reference's bits.
#pragma once

#include <cstdint>

#include "pgl_math.cuh"

namespace pgl {

// DirectionalQuadtreeFactory::Configuration (DQTFactory.h:33-70), the raw
// 20-byte struct of the field file.
struct DqtArgs {
  int32_t leafEstimator = 0;  // 0: rejection sampling, 1: per leaf
  int32_t splitMetric = 0;    // 0: mean, 1: second moment
  float splitThreshold = 0.01f;
  float footprintFactor = 1.0f;
  uint32_t maxLevels = 12;
};
static_assert(sizeof(DqtArgs) == 20, "the factory configuration is 20 bytes");

// DirectionalQuadtreeNode (DQT.h:12-23)
struct DqtNode {
  uint32_t child;
  float weight;
};
// DirectionalQuadtreeFactory::StatsNode (DQTFactory.h:72-81)
struct DqtStatsNode {
  uint32_t child;
  float sampleWeight, splitWeight, numSamples, first, second;
};
static_assert(sizeof(DqtNode) == 8 && sizeof(DqtStatsNode) == 24, "node layouts");

// A region's quadtree: the head, then `stride` node slots of each kind in the
// sub-field's node arrays.
struct DqtHead {
  float pivot[3];
  float numSamples;   // the statistics' decayed sample count
  uint32_t numNodes;  // nodes of the quadtree (and of its statistics)
  uint32_t valid;
  uint32_t pad[2];
};

// Upper bound on a region's nodes for the factory arguments: a node splits
// only while its split weight exceeds threshold x the root's, and the split
// weights of one level sum to at most the root's, so fewer than
// 1 / threshold nodes split per level, each adding four.
inline uint64_t dqt_max_nodes(const DqtArgs &a) {
  if (!(a.splitThreshold > 0.0f)) return ~uint64_t(0);
  const double per = std::ceil(1.0 / double(a.splitThreshold));
  return uint64_t(1.0 + 4.0 * double(a.maxLevels) * per);
}

// Rect<float> (Rect.h:8-40)
struct Box2 {
  float x0, y0, x1, y1;
  PGL_HD float area() const { return (x1 - x0) * (y1 - y0); }
  PGL_HD Box2 child(uint32_t c) const {
    const float mx = (x0 + x1) / 2.0f, my = (y0 + y1) / 2.0f;
    return Box2{(c & 1) ? mx : x0, (c & 2) ? my : y0, (c & 1) ? x1 : mx, (c & 2) ? y1 : my};
  }
  PGL_HD Box2 intersect(const Box2 &o) const {
    Box2 r{smax(x0, o.x0), smax(y0, o.y0), smin(x1, o.x1), smin(y1, o.y1)};
    r.x1 = smax(r.x0, r.x1);
    r.y1 = smax(r.y0, r.y1);
    return r;
  }
};

PGL_HD float dqt_clamp(float v, float lo, float hi) { return emax(lo, emin(v, hi)); }  // embree::clamp

// The C library's single-precision atan2 as glibc computes it: the fdlibm
// algorithm (Sun Microsystems, 1993; argument reduction by the tangent's
// addition formula onto [0, 7/16) around atan(0.5), atan(1), atan(1.5) or
// atan(inf), then an odd polynomial of degree 23 split into two halves in
// z^2), all in single precision.  Checked against glibc 2.39 on 2e8 random
// argument pairs: equal except for 0.003 % with |y/x| above 2^24.
PGL_HD float fd_atanf(float x) {
  const float atanhi[4] = {4.6364760399e-01f, 7.8539812565e-01f, 9.8279368877e-01f, 1.5707962513e+00f};
  const float atanlo[4] = {5.0121582440e-09f, 3.7748947079e-08f, 3.4473217170e-08f, 7.5497894159e-08f};
  const float aT[11] = {3.3333334327e-01f,  -2.0000000298e-01f, 1.4285714924e-01f,  -1.1111110449e-01f,
                        9.0908870101e-02f,  -7.6918758452e-02f, 6.6610731184e-02f,  -5.8335702866e-02f,
                        4.9768779427e-02f,  -3.6531571299e-02f, 1.6285819933e-02f};
  const int32_t hx = int32_t(f2u(x)), ix = hx & 0x7fffffff;
  int id;
  if (ix >= 0x4c800000) {  // |x| >= 2^26
    if (ix > 0x7f800000) return x + x;
    return hx > 0 ? atanhi[3] + atanlo[3] : -atanhi[3] - atanlo[3];
  }
  if (ix < 0x3ee00000) {  // |x| < 7/16
    if (ix < 0x31000000) return x;
    id = -1;
  } else {
    x = fabsf(x);
    if (ix < 0x3f980000) {
      if (ix < 0x3f300000) {
        id = 0;
        x = (2.0f * x - 1.0f) / (2.0f + x);
      } else {
        id = 1;
        x = (x - 1.0f) / (x + 1.0f);
      }
    } else if (ix < 0x401c0000) {
      id = 2;
      x = (x - 1.5f) / (1.0f + 1.5f * x);
    } else {
      id = 3;
      x = -1.0f / x;
    }
  }
  const float z = x * x, w = z * z;
  const float s1 = z * (aT[0] + w * (aT[2] + w * (aT[4] + w * (aT[6] + w * (aT[8] + w * aT[10])))));
  const float s2 = w * (aT[1] + w * (aT[3] + w * (aT[5] + w * (aT[7] + w * aT[9]))));
  if (id < 0) return x - x * (s1 + s2);
  const float r = atanhi[id] - ((x * (s1 + s2) - atanlo[id]) - x);
  return hx < 0 ? -r : r;
}
PGL_HD float fd_atan2f(float y, float x) {
  const float piO4 = 7.8539818525e-01f, piO2 = 1.5707963705e+00f, pi = 3.1415927410e+00f;
  const float piLo = -8.7422776573e-08f, tiny = 1.0e-30f;
  const int32_t hx = int32_t(f2u(x)), ix = hx & 0x7fffffff, hy = int32_t(f2u(y)), iy = hy & 0x7fffffff;
  if (ix > 0x7f800000 || iy > 0x7f800000) return x + y;
  if (hx == 0x3f800000) return fd_atanf(y);
  const int m = ((hy >> 31) & 1) | ((hx >> 30) & 2);
  if (iy == 0) {
    if (m < 2) return y;
    return m == 2 ? pi + tiny : -pi - tiny;
  }
  if (ix == 0) return hy < 0 ? -piO2 - tiny : piO2 + tiny;
  if (ix == 0x7f800000) {
    if (iy == 0x7f800000) {
      const float r[4] = {piO4 + tiny, -piO4 - tiny, 3.0f * piO4 + tiny, -3.0f * piO4 - tiny};
      return r[m];
    }
    const float r[4] = {0.0f, -0.0f, pi + tiny, -pi - tiny};
    return r[m];
  }
  if (iy == 0x7f800000) return hy < 0 ? -piO2 - tiny : piO2 + tiny;
  const int32_t k = (iy - ix) >> 23;
  float z;
  if (k > 60) z = piO2 + 0.5f * piLo;
  else if (hx < 0 && k < -60) z = 0.0f;
  else z = fd_atanf(fabsf(y / x));
  switch (m) {
    case 0:
      return z;
    case 1:
      return u2f(f2u(z) ^ 0x80000000u);
    case 2:
      return pi - (z - piLo);
    default:
      return (z - piLo) - pi;
  }
}

// SphereToSquareCylindrical (SphereToSquare.h:34-61): x = (cos theta + 1) / 2,
// y = phi / 2pi + 1/2, phi = atan2(d.y, d.x), the division in double.
PGL_HD void dqt_dir_to_point(float dx, float dy, float dz, float &px, float &py) {
  dx = dqt_clamp(dx, -1.f, 1.f);
  dy = dqt_clamp(dy, -1.f, 1.f);
  dz = dqt_clamp(dz, -1.f, 1.f);
  const float phi = fd_atan2f(dy, dx);
  px = dqt_clamp((dz + 1.0f) / 2.0f, 0.f, 1.f);
  py = dqt_clamp(float(double(phi) / (2.0 * kPiD) + 0.5), 0.f, 1.f);
}
// SphereToSquareCylindrical::area (SphereToSquare.h:57-59)
PGL_HD float dqt_area(const Box2 &r) { return 4.0f * 3.14159274101257324f * (r.x1 - r.x0) * (r.y1 - r.y0); }
constexpr float kDqtJacobian = 4.0f * 3.14159274101257324f;

// queryNode (Traversal.h:37-49): the leaf that a point of the unit square
// falls in, and its rectangle.
template <typename N>
PGL_HD uint32_t dqt_query(const N *nodes, float px, float py, Box2 &rect) {
  rect = Box2{0.f, 0.f, 1.f, 1.f};
  uint32_t idx = 0;
  while (nodes[idx].child > 0) {
    uint32_t c = 0;
    if (px >= 0.5f) {
      px -= 0.5f;
      c += 1;
    }
    if (py >= 0.5f) {
      py -= 0.5f;
      c += 2;
    }
    px *= 2.0f;
    py *= 2.0f;
    rect = rect.child(c);
    idx = nodes[idx].child + c;
  }
  return idx;
}

}  // namespace pgl
