// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Volume sampling distribution (reference: include/openpgl/volumesamplingdistribution.h:24-46;
// api.cpp:660-737).
#pragma once
#include "common.h"
#include "region.h"
#ifdef __cplusplus
extern "C" {
struct VolumeSamplingDistribution;
#endif
typedef struct VolumeSamplingDistribution *PGLVolumeSamplingDistribution;

OPENPGL_CORE_INTERFACE void pglReleaseVolumeSamplingDistribution(PGLVolumeSamplingDistribution d);
OPENPGL_CORE_INTERFACE pgl_vec3f pglVolumeSamplingDistributionSample(PGLVolumeSamplingDistribution d,
                                                                     pgl_point2f sample);
OPENPGL_CORE_INTERFACE float pglVolumeSamplingDistributionPDF(PGLVolumeSamplingDistribution d, pgl_vec3f direction);
OPENPGL_CORE_INTERFACE float pglVolumeSamplingDistributionSamplePDF(PGLVolumeSamplingDistribution d,
                                                                    pgl_point2f sample, pgl_vec3f &direction);
OPENPGL_CORE_INTERFACE float pglVolumeSamplingDistributionIncomingRadiancePDF(PGLVolumeSamplingDistribution d,
                                                                              pgl_vec3f direction);
OPENPGL_CORE_INTERFACE uint32_t pglVolumeSamplingDistributionGetId(PGLVolumeSamplingDistribution d);
OPENPGL_CORE_INTERFACE bool pglVolumeSamplingDistributionValidate(PGLVolumeSamplingDistribution d);
OPENPGL_CORE_INTERFACE void pglVolumeSamplingDistributionClear(PGLVolumeSamplingDistribution d);
OPENPGL_CORE_INTERFACE void pglVolumeSamplingDistributionApplySingleLobeHenyeyGreensteinProduct(
    PGLVolumeSamplingDistribution d, pgl_vec3f dir, const float meanCosine);
OPENPGL_CORE_INTERFACE bool pglVolumeSamplingDistributionSupportsApplySingleLobeHenyeyGreensteinProduct(
    PGLVolumeSamplingDistribution d);
OPENPGL_CORE_INTERFACE PGLRegion pglVolumeSamplingGetRegion(PGLVolumeSamplingDistribution d);
#ifdef __cplusplus
}
#endif
