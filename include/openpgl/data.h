// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Sample records (reference: include/openpgl/data.h:21-119).
#pragma once

#ifdef __cplusplus
#include <cstdint>
#include <cstdlib>
#else
#include <stdint.h>
#include <stdlib.h>
#endif

#include "common.h"

struct PGLSampleData {
  enum Flags {
    ESplatted = 1 << 0,      // not a real scene intersection point
    EInsideVolume = 1 << 1   // the sample trains the volume field
  };
  pgl_point3f position;
  pgl_vec3f direction;
  float weight;
  float pdf;
  float distance;
  uint32_t flags;
};

struct PGLPathSegmentData {
  pgl_point3f position{0.f, 0.f, 0.f};
  pgl_vec3f directionIn{0.f, 1.f, 0.f};
  pgl_vec3f directionOut{1.f, 0.f, 0.f};
  pgl_vec3f normal{0.f, 0.f, 1.f};
  bool volumeScatter{false};
  float pdfDirectionIn{1.0f};
  bool isDelta{false};
  pgl_vec3f scatteringWeight{1.0f, 1.0f, 1.0f};
  pgl_vec3f transmittanceWeight{1.0f, 1.0f, 1.0f};
  pgl_vec3f directContribution{0.0f, 0.0f, 0.0f};
  float miWeight{1.0f};
  pgl_vec3f scatteredContribution{0.0f, 0.0f, 0.0f};
  float russianRouletteProbability{1.0f};
  float eta{1.0f};
  float roughness{1.0f};
  const void *regionPtr{nullptr};
};

struct PGLString {
  char *m_str{nullptr};
  size_t m_size{0};
};

#ifdef __cplusplus
extern "C" {
#endif
// replaces api.cpp:838-846
OPENPGL_CORE_INTERFACE void pglReleaseString(PGLString str);
#ifdef __cplusplus
}
#endif
