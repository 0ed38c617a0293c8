// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Field statistics (reference: include/openpgl/fieldstatistics.h:21-27).
#pragma once
#include "common.h"
#include "data.h"
#ifdef __cplusplus
extern "C" {
struct FieldStatistics;
#endif
typedef struct FieldStatistics *PGLFieldStatistics;
// replace api.cpp:788-836
OPENPGL_CORE_INTERFACE void pglReleaseFieldStatistics(PGLFieldStatistics fieldStatistics);
OPENPGL_CORE_INTERFACE PGLString pglFieldStatisticsToString(PGLFieldStatistics fieldStatistics);
OPENPGL_CORE_INTERFACE PGLString pglFieldStatisticsHeaderCSVString(PGLFieldStatistics fieldStatistics);
OPENPGL_CORE_INTERFACE PGLString pglFieldStatisticsToCSVString(PGLFieldStatistics fieldStatistics);
#ifdef __cplusplus
}
#endif
