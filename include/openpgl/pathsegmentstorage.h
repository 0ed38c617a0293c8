// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Path segment storage (reference: include/openpgl/pathsegmentstorage.h:36-70):
// one path's segments in host memory and the training samples made from them
// (openpgl_gb300/csrc/pathsegments.cpp).  Many paths at once on the device:
// pglPathSegmentsPrepareSamplesDevice in openpgl_gb300.h.
#pragma once
#ifdef __cplusplus
#include <cstdint>
#include <cstdlib>
#else
#include <stdint.h>
#include <stdlib.h>
#endif
#include "common.h"
#include "data.h"
#include "region.h"
#include "samplestorage.h"
#ifdef __cplusplus
extern "C" {
struct PathSegmentStorage {};
struct PGLPathSegmentData;
#endif
typedef struct PathSegmentStorage *PGLPathSegmentStorage;
typedef struct PGLPathSegmentData *PGLPathSegment;

OPENPGL_CORE_INTERFACE PGLPathSegmentStorage pglNewPathSegmentStorage();
OPENPGL_CORE_INTERFACE void pglReleasePathSegmentStorage(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageReserve(PGLPathSegmentStorage s, size_t size);
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageClear(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE void pglPathSegmentSetMaxDistance(PGLPathSegmentStorage s, float maxDistance);
OPENPGL_CORE_INTERFACE float pglPathSegmentGetMaxDistance(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE int pglPathSegmentGetNumSegments(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE int pglPathSegmentGetNumSamples(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE size_t pglPathSegmentStoragePrepareSamples(PGLPathSegmentStorage s,
                                                                  const bool useNEEMiWeights = false,
                                                                  const bool guideDirectLight = false,
                                                                  const bool rrAffectsDirectContribution = true);
OPENPGL_CORE_INTERFACE pgl_vec3f pglPathSegmentStorageCalculatePixelEstimate(
    PGLPathSegmentStorage s, const bool rrAffectsDirectContribution = true);
OPENPGL_CORE_INTERFACE const PGLSampleData *pglPathSegmentStorageGetSamples(PGLPathSegmentStorage s, size_t &nSamples);
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageAddSample(PGLPathSegmentStorage s, PGLSampleData sample);
OPENPGL_CORE_INTERFACE PGLPathSegmentData *pglPathSegmentStorageNextSegment(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE void pglPathSegmentStorageAddSegment(PGLPathSegmentStorage s, PGLPathSegmentData segment);
OPENPGL_CORE_INTERFACE bool pglPathSegmentStorageValidateSamples(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE bool pglPathSegmentStorageValidateSegments(PGLPathSegmentStorage s);
OPENPGL_CORE_INTERFACE void pglPathSegmentStoragePropagateSamples(PGLPathSegmentStorage s,
                                                                  PGLSampleStorage sampleStorage,
                                                                  bool guideDirectLight = false,
                                                                  bool useNEEMiWeights = false,
                                                                  bool rrAffectsDirectContribution = true);
#ifdef __cplusplus
}
#endif
