// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Opaque region handle (reference: include/openpgl/region.h).
#pragma once
#include "common.h"
#include "distribution.h"
#ifdef __cplusplus
extern "C" {
struct Region {};
#endif
typedef struct Region *PGLRegion;
#ifdef __cplusplus
}
#endif
