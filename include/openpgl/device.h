// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Device (reference: include/openpgl/device.h:22-28; api.cpp:83-114).
#pragma once
#include "common.h"
#include "config.h"
#include "field.h"
#ifdef __cplusplus
extern "C" {
struct Device;
#endif
typedef struct Device *PGLDevice;

OPENPGL_CORE_INTERFACE PGLDevice pglNewDevice(PGL_DEVICE_TYPE deviceType, size_t numThreads);
OPENPGL_CORE_INTERFACE PGLField pglDeviceNewField(PGLDevice device, PGLFieldArguments args);
OPENPGL_CORE_INTERFACE PGLField pglDeviceNewFieldFromFile(PGLDevice device, const char *fieldFileName);
OPENPGL_CORE_INTERFACE void pglReleaseDevice(PGLDevice device);
#ifdef __cplusplus
}
#endif
