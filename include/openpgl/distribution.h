// Opaque distribution / region handles (reference: include/openpgl/distribution.h).
#pragma once
#include "common.h"
#ifdef __cplusplus
extern "C" {
struct Region;
struct Distribution;
#endif
typedef struct Distribution *PGLDistribution;
typedef struct Region *PGLRegion;
#ifdef __cplusplus
}
#endif
