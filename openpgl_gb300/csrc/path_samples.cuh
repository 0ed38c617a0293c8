// Training samples from a path's segments and the path's pixel estimate
// (PathSegmentDataStorage.h:161-316 prepareSamples, :318-385
// calculatePixelEstimate, PathSegmentData.h:19-104 isValid), shared by the
// host storage object (the reference's per-path API) and the device batch
// kernel, so both give the same bits.  The reference instantiates this code
// in its SSE translation unit (api.cpp), where embree's dot product is
// a.x*b.x + (a.y*b.y + a.z*b.z) with separate roundings (no FMA).
#pragma once

#include <cstddef>
#include <cstdint>

#include "pgl_internal.h"

namespace pgl {

// PGLPathSegmentData (data.h), field for field: 136 bytes.
struct PathSegmentRecord {
  float px, py, pz;              // position
  float dix, diy, diz;           // directionIn
  float dox, doy, doz;           // directionOut
  float nx, ny, nz;              // normal
  uint8_t volumeScatter, pad0[3];
  float pdfDirectionIn;
  uint8_t isDelta, pad1[3];
  float sw[3];                   // scatteringWeight
  float tw[3];                   // transmittanceWeight
  float dc[3];                   // directContribution
  float miWeight;
  float sc[3];                   // scatteredContribution
  float rr;                      // russianRouletteProbability
  float eta, roughness;
  uint32_t pad2;
  uint64_t regionPtr;
};
static_assert(sizeof(PathSegmentRecord) == 136, "PGLPathSegmentData layout");

struct PathFlags {
  bool useNEEMiWeights, guideDirectLight, rrAffectsDirectContribution;
};

PGL_HD float seg_dot(float ax, float ay, float az, float bx, float by, float bz) {
  return ax * bx + (ay * by + az * bz);
}

// Appends the samples of path seg[0, n) to out (at most cap, counted from
// out's start); returns how many it would write (the count is exact even
// when cap is smaller).
PGL_HD uint32_t path_prepare_samples(const PathSegmentRecord *seg, int n, float maxDistance, PathFlags fl,
                                     PGLSampleRecord *out, uint32_t cap) {
  const float minPDF = 0.1f, maxThroughput = 10.0f;
  uint32_t made = 0;
  float lastDistance = 0.0f;
  for (int i = n - 2; i >= 0; --i) {
    const PathSegmentRecord &cur = seg[i];
    const PathSegmentRecord &nxt = seg[i + 1];
    const float ex = nxt.px - cur.px, ey = nxt.py - cur.py, ez = nxt.pz - cur.pz;
    const float currentDistance = sqrtf(seg_dot(ex, ey, ez, ex, ey, ez));
    const float distance = fminf(currentDistance + lastDistance, 2.0f * maxDistance);
    if (!cur.isDelta && cur.roughness >= 0.3f) {
      lastDistance = 0.0f;
    } else {
      lastDistance = distance;
      if (cur.eta != 1.0f) {
        const float cosThetaI = seg_dot(cur.nx, cur.ny, cur.nz, cur.dox, cur.doy, cur.doz);
        const float cosThetaO = seg_dot(cur.nx, cur.ny, cur.nz, cur.dix, cur.diy, cur.diz);
        lastDistance *= fabsf(cosThetaI / (cosThetaO * cur.eta));
      }
    }
    // samples only on non-delta vertices sampled by a non-delta technique
    if (!cur.isDelta && cur.roughness > 0.01f) {
      const float pdf = minPDF < cur.pdfDirectionIn ? cur.pdfDirectionIn : minPDF;  // std::max
      float t[3] = {1.0f, 1.0f, 1.0f}, c[3] = {0.0f, 0.0f, 0.0f};
      float previousRR = 1.0f;
      for (int j = i + 1; j < n; ++j) {
        const PathSegmentRecord &s = seg[j];
        const PathSegmentRecord &p = seg[j - 1];
        for (int k = 0; k < 3; ++k) t[k] = t[k] * p.tw[k];
        float ct[3];
        for (int k = 0; k < 3; ++k) ct[k] = t[k] < maxThroughput ? t[k] : maxThroughput;  // embree::min
        for (int k = 0; k < 3; ++k) c[k] += ct[k] * s.sc[k];
        float dc[3] = {s.dc[0], s.dc[1], s.dc[2]};
        if (!fl.rrAffectsDirectContribution)
          for (int k = 0; k < 3; ++k) dc[k] *= previousRR;
        if (j == i + 1 && !fl.useNEEMiWeights) {
          if (fl.guideDirectLight)
            for (int k = 0; k < 3; ++k) c[k] += ct[k] * dc[k];
        } else if (j > i + 1 || fl.guideDirectLight) {
          for (int k = 0; k < 3; ++k) c[k] += (ct[k] * s.miWeight) * dc[k];
        }
        for (int k = 0; k < 3; ++k) t[k] = t[k] * s.sw[k];
        if (s.rr > 0.f) {
          for (int k = 0; k < 3; ++k) t[k] /= s.rr;
        } else {
          t[0] = t[1] = t[2] = 0.0f;
        }
        previousRR = s.rr;
      }
      if ((c[0] > 0.0f || c[1] > 0.0f || c[2] > 0.0f) && distance > 0) {
        if (made < cap) {
          PGLSampleRecord r;
          r.px = cur.px;
          r.py = cur.py;
          r.pz = cur.pz;
          r.dx = cur.dix;
          r.dy = cur.diy;
          r.dz = cur.diz;
          r.weight = ((c[0] + c[1] + c[2]) / 3.0f) / pdf;
          r.pdf = pdf;
          r.distance = distance;
          r.flags = cur.volumeScatter ? 2u : 0u;  // EInsideVolume
          out[made] = r;
        }
        ++made;
      }
    }
  }
  return made;
}

// calculatePixelEstimate: the radiance the path carries to its first vertex.
PGL_HD void path_pixel_estimate(const PathSegmentRecord *seg, int n, bool rrAffectsDirectContribution, float out[3]) {
  out[0] = out[1] = out[2] = 0.0f;
  if (n == 0) return;
  float t[3] = {1.0f, 1.0f, 1.0f}, c[3] = {0.0f, 0.0f, 0.0f};
  float previousRR = 1.0f;
  for (int j = 1; j < n; ++j) {
    const PathSegmentRecord &s = seg[j];
    const PathSegmentRecord &p = seg[j - 1];
    for (int k = 0; k < 3; ++k) t[k] = t[k] * p.tw[k];
    for (int k = 0; k < 3; ++k) c[k] += t[k] * s.sc[k];
    float dc[3] = {s.dc[0], s.dc[1], s.dc[2]};
    if (!rrAffectsDirectContribution)
      for (int k = 0; k < 3; ++k) dc[k] *= previousRR;
    for (int k = 0; k < 3; ++k) c[k] += (t[k] * s.miWeight) * dc[k];
    for (int k = 0; k < 3; ++k) t[k] = t[k] * s.sw[k];
    if (s.rr > 0.f) {
      for (int k = 0; k < 3; ++k) t[k] /= s.rr;
    } else {
      t[0] = t[1] = t[2] = 0.0f;
    }
    previousRR = s.rr;
  }
  const PathSegmentRecord &f = seg[0];
  if (n == 1) {
    for (int k = 0; k < 3; ++k) out[k] = f.dc[k] + f.sc[k];
  } else {
    for (int k = 0; k < 3; ++k) out[k] = (f.dc[k] + f.sc[k]) + f.sw[k] * c[k];
  }
}

// isValid(PathSegmentData), as the reference checks it (its Russian-roulette
// test reads miWeight >= 0 for the lower bound).
PGL_HD bool seg_unit(float v) { return isvalidf(v) && v <= 1.0f && v >= -1.0f; }
PGL_HD bool seg_nonneg3(const float *v) {
  bool ok = true;
  for (int k = 0; k < 3; ++k) ok = ok && isvalidf(v[k]) && v[k] >= 0.0f;
  return ok;
}
PGL_HD bool path_segment_valid(const PathSegmentRecord &s) {
  bool v = isvalidf(s.px) && isvalidf(s.py) && isvalidf(s.pz);
  v = v && seg_unit(s.dix) && seg_unit(s.diy) && seg_unit(s.diz);
  v = v && seg_unit(s.dox) && seg_unit(s.doy) && seg_unit(s.doz);
  v = v && seg_unit(s.nx) && seg_unit(s.ny) && seg_unit(s.nz);
  v = v && isvalidf(s.pdfDirectionIn) && s.pdfDirectionIn >= 0.f;
  v = v && seg_nonneg3(s.sw) && seg_nonneg3(s.tw) && seg_nonneg3(s.dc) && seg_nonneg3(s.sc);
  v = v && isvalidf(s.miWeight) && s.miWeight >= 0.f && s.miWeight <= 1.0f;
  v = v && isvalidf(s.rr) && s.miWeight >= 0.f && s.rr <= 1.0f;
  v = v && isvalidf(s.eta) && s.eta >= 0.f;
  v = v && isvalidf(s.roughness) && s.roughness >= 0.f && s.roughness <= 1.f;
  return v;
}
// isValid(SampleData) (SampleData.h:25-46).
PGL_HD bool sample_record_valid(const PGLSampleRecord &d) {
  bool v = isvalidf(d.px) && isvalidf(d.py) && isvalidf(d.pz);
  v = v && isvalidf(d.dx) && isvalidf(d.dy) && isvalidf(d.dz);
  v = v && isvalidf(d.weight) && d.weight >= 0.f;
  v = v && isvalidf(d.pdf) && d.pdf > 0.f;
  v = v && isvalidf(d.distance) && d.distance > 0.f;
  return v;
}

}  // namespace pgl
