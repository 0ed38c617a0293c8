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
