// Copyright 2021 Intel Corporation
// SPDX-License-Identifier: Apache-2.0
// (The declarations restate the Open PGL 0.6.0 C API header of the same name,
// which is licensed under Apache-2.0, so that code written against it builds
// unchanged.)
// Open PGL C API, common types.  Drop-in declarations matching the reference
// ABI (openpgl/include/openpgl/common.h:6-88); the implementation is the GPU
// library libopenpgl_gb300.so.
#pragma once

#if defined(_WIN32)
#define OPENPGL_CORE_INTERFACE __declspec(dllimport)
#else
#define OPENPGL_CORE_INTERFACE __attribute__((visibility("default")))
#endif

#define PGL_VECTOR_SIZE 4
#define PGL_VMM_MAX_COMPONENTS 32
#define PGL_VMM_MAX_KAPPA 320000.f

typedef struct {
  float x, y, z;
} pgl_vec3f;
typedef pgl_vec3f pgl_point3f;

typedef struct {
  float x, y;
} pgl_vec2f;
typedef pgl_vec2f pgl_point2f;

typedef struct {
  pgl_vec3f lower, upper;
} pgl_box3f;

#ifdef __cplusplus
inline void pglVec3f(pgl_vec3f &v, const float x, const float y, const float z) { v.x = x; v.y = y; v.z = z; }
inline void pglVec3fAdd(pgl_vec3f &a, const pgl_vec3f &b) { a.x += b.x; a.y += b.y; a.z += b.z; }
inline void pglVec2f(pgl_vec2f &v, const float x, const float y) { v.x = x; v.y = y; }
inline void pglVec2fAdd(pgl_vec2f &a, const pgl_vec2f &b) { a.x += b.x; a.y += b.y; }
inline void pglPoint3f(pgl_point3f &v, const float x, const float y, const float z) { pglVec3f(v, x, y, z); }
inline void pglPoint2f(pgl_point2f &v, const float x, const float y) { pglVec2f(v, x, y); }
inline void pglBox3f(pgl_box3f &b, const float lx, const float ly, const float lz, const float ux, const float uy,
                     const float uz) {
  pglVec3f(b.lower, lx, ly, lz);
  pglVec3f(b.upper, ux, uy, uz);
}
#endif
