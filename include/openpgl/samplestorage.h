// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Sample storage (reference: include/openpgl/samplestorage.h:35-65; api.cpp:328-400).
#pragma once
#include "common.h"
#ifdef __cplusplus
#include <cstdint>
#include <cstdlib>
#else
#include <stdint.h>
#include <stdlib.h>
#endif
#ifdef __cplusplus
extern "C" {
struct SampleStorage {};
struct PGLSampleData;
#endif
typedef struct SampleStorage *PGLSampleStorage;

OPENPGL_CORE_INTERFACE PGLSampleStorage pglNewSampleStorage();
OPENPGL_CORE_INTERFACE PGLSampleStorage pglNewSampleStorageFromFile(const char *sampleStorageFileName);
OPENPGL_CORE_INTERFACE void pglReleaseSampleStorage(PGLSampleStorage sampleStorage);
OPENPGL_CORE_INTERFACE bool pglSampleStorageStoreToFile(PGLSampleStorage sampleStorage, const char *sampleStorageFileName);
OPENPGL_CORE_INTERFACE void pglSampleStorageAddSample(PGLSampleStorage sampleStorage, PGLSampleData &sample);
OPENPGL_CORE_INTERFACE void pglSampleStorageAddSamples(PGLSampleStorage sampleStorage, const PGLSampleData *samples,
                                                       size_t numSamples);
OPENPGL_CORE_INTERFACE void pglSampleStorageReserve(PGLSampleStorage sampleStorage, const size_t sizeSurface,
                                                    const size_t sizeVolume);
OPENPGL_CORE_INTERFACE void pglSampleStorageClear(PGLSampleStorage sampleStorage);
OPENPGL_CORE_INTERFACE void pglSampleStorageClearSurface(PGLSampleStorage sampleStorage);
OPENPGL_CORE_INTERFACE void pglSampleStorageClearVolume(PGLSampleStorage sampleStorage);
OPENPGL_CORE_INTERFACE size_t pglSampleStorageGetSizeSurface(PGLSampleStorage sampleStorage);
OPENPGL_CORE_INTERFACE size_t pglSampleStorageGetSizeVolume(PGLSampleStorage sampleStorage);
OPENPGL_CORE_INTERFACE PGLSampleData pglSampleStorageGetSampleSurface(PGLSampleStorage sampleStorage, const int idx);
OPENPGL_CORE_INTERFACE PGLSampleData pglSampleStorageGetSampleVolume(PGLSampleStorage sampleStorage, const int idx);
OPENPGL_CORE_INTERFACE bool pglSampleStorageValidate(PGLSampleStorage sampleStorage);
OPENPGL_CORE_INTERFACE bool pglSampleStorageCompare(PGLSampleStorage sampleStorageA, PGLSampleStorage sampleStorageB);
#ifdef __cplusplus
}
#endif
