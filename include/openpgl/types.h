// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Spatial / directional representation types (reference: include/openpgl/types.h:3-13).
#pragma once

enum PGL_SPATIAL_STRUCTURE_TYPE { PGL_SPATIAL_STRUCTURE_KDTREE = 0 };

enum PGL_DIRECTIONAL_DISTRIBUTION_TYPE {
  PGL_DIRECTIONAL_DISTRIBUTION_PARALLAX_AWARE_VMM = 0,
  PGL_DIRECTIONAL_DISTRIBUTION_QUADTREE,
  PGL_DIRECTIONAL_DISTRIBUTION_VMM
};
