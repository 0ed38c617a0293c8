// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Umbrella header of the C API (reference: include/openpgl/openpgl.h).
#pragma once

#define OPENPGL_INLINE inline

#ifndef OPENPGL_DISABLE_ASSERTS
#include <assert.h>
#define OPENPGL_ASSERT(cond) assert(cond);
#else
#define OPENPGL_ASSERT(cond)
#endif

#include "common.h"
#include "data.h"
#include "device.h"
#include "field.h"
#include "fieldstatistics.h"
#include "pathsegmentstorage.h"
#include "region.h"
#include "samplestorage.h"
#include "surfacesamplingdistribution.h"
#include "volumesamplingdistribution.h"
