/* Measures the x86 approximate-reciprocal instructions that the reference's
 * embree::rcp / embree::rsqrt start from (third-party/embreeSrc/common/math/
 * emath.h:61-85,129-145; simd/vfloat8_avx.h:254-290) and writes them as
 * lookup tables, so that the oracle and the GPU library can reproduce the
 * reference's results bit for bit on any machine (the GPU host is Arm).
 *
 * Measured facts (Intel, this generator checks them and fails otherwise):
 *   RCPSS / RCPPS  : output depends only on the top 11 mantissa bits; the
 *                    exponent only shifts the result.  2048 entries.
 *   RSQRTSS/RSQRTPS: output depends on exponent parity and the top 10
 *                    mantissa bits.  2 x 1024 entries.
 * Usage: gen_x86_tables <out.h> <array prefix>   (x86-64 hosts only)
 */
#include <immintrin.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint32_t bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float fl(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static float rcp1(float x) { return _mm_cvtss_f32(_mm_rcp_ss(_mm_set_ss(x))); }
static float rsq1(float x) { return _mm_cvtss_f32(_mm_rsqrt_ss(_mm_set_ss(x))); }

int main(int argc, char **argv) {
  if (argc < 3) { fprintf(stderr, "usage: %s out.h prefix\n", argv[0]); return 2; }
  /* verify the structural facts the tables rely on */
  for (uint32_t m = 0; m < (1u << 23); m++) {
    uint32_t a = bits(rcp1(fl((127u << 23) | m)));
    if (a != bits(rcp1(fl((127u << 23) | (m & ~0xFFFu))))) { fprintf(stderr, "rcp: more than 11 bits\n"); return 1; }
    if ((a & 0x7FFFFF) != (bits(rcp1(fl((100u << 23) | m))) & 0x7FFFFF)) { fprintf(stderr, "rcp: exponent dependence\n"); return 1; }
    for (uint32_t e = 127; e <= 128; e++) {
      uint32_t r = bits(rsq1(fl((e << 23) | m)));
      if (r != bits(rsq1(fl((e << 23) | (m & ~0x1FFFu))))) { fprintf(stderr, "rsqrt: more than 10 bits\n"); return 1; }
      if ((r & 0x7FFFFF) != (bits(rsq1(fl(((e + 20) << 23) | m))) & 0x7FFFFF)) { fprintf(stderr, "rsqrt: exponent dependence\n"); return 1; }
    }
  }
  FILE *f = fopen(argv[1], "w");
  if (!f) return 1;
  fprintf(f, "/* Generated by gen_x86_tables.c on an x86-64 host: bit patterns of RCPSS and\n"
             " * RSQRTSS for inputs 1.m (exponent 127) and 2*1.m (exponent 128), indexed by\n"
             " * the top 11 (rcp) or 10 (rsqrt) mantissa bits.  Data, not code. */\n#pragma once\n#include <stdint.h>\n");
  fprintf(f, "static const uint32_t %s_rcp_table[2048] = {\n", argv[2]);
  for (uint32_t i = 0; i < 2048; i++)
    fprintf(f, "0x%08x%s", bits(rcp1(fl((127u << 23) | (i << 12)))), (i % 8 == 7) ? ",\n" : ",");
  fprintf(f, "};\nstatic const uint32_t %s_rsqrt_table[2048] = {\n", argv[2]);
  for (uint32_t e = 127; e <= 128; e++)
    for (uint32_t i = 0; i < 1024; i++)
      fprintf(f, "0x%08x%s", bits(rsq1(fl((e << 23) | (i << 13)))), (i % 8 == 7) ? ",\n" : ",");
  fprintf(f, "};\n");
  fclose(f);
  return 0;
}
