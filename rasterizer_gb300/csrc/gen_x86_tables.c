/*
 * Generator for x86_tables.h: the result mantissas of the x86 approximate
 * reciprocal (RCPPS) and approximate reciprocal square root (RSQRTPS)
 * instructions, read from the instruction itself on the machine that runs it.
 *
 * The occluder rasteriser this library reproduces calls RCPPS on its hot path
 * (Rasterizer.cpp:218,223,456,717-727,981) and RSQRTPS in its occluder bake
 * (VectorMath.h:20-23).  Both instructions are approximations whose exact
 * outputs are vendor specific, so bit-exact results on a GPU (or on an Arm
 * host) need the measured tables.  On the Intel Xeon this was generated on:
 *
 *   RCPPS(x)   depends only on the sign, the exponent and the top 11 mantissa
 *              bits of x.  Table index = mantissa bits 22..12.
 *   RSQRTPS(x) depends only on the exponent parity and the top 10 mantissa
 *              bits.  Table index = (E & 1) << 11 | mantissa bits 22..12 (the
 *              low index bit is redundant; kept so both tables index alike).
 *
 * The emulation rules (special values, exponent arithmetic) are written next
 * to the consumers (x86_emu.cuh, oracle.c).  Running this program with
 * --verify checks those rules against the instruction for all 2^32 inputs.
 *
 * Build and run (x86-64 with AVX only):
 *   gcc -O2 -mavx2 gen_x86_tables.c -o gen && ./gen --verify > x86_tables.h
 */
#include <immintrin.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static uint32_t rcp_tab[2048];
static uint32_t rsqrt_tab[4096];

static uint32_t emu_rcp(uint32_t x)
{
  uint32_t s = x & 0x80000000u, E = (x >> 23) & 0xFF;
  if (E == 255) return (x & 0x7FFFFF) ? (x | 0x400000u) : s;
  if (E == 0) return s | 0x7F800000u;
  uint32_t t = rcp_tab[(x >> 12) & 0x7FF];
  int re = (int)((t >> 23) & 0xFF) + 127 - (int)E;
  return re <= 0 ? s : (s | ((uint32_t)re << 23) | (t & 0x7FFFFFu));
}

static uint32_t emu_rsqrt(uint32_t x)
{
  uint32_t s = x & 0x80000000u, E = (x >> 23) & 0xFF;
  if (E == 255 && (x & 0x7FFFFF)) return x | 0x400000u;
  if (E == 0) return s | 0x7F800000u;
  if (s) return 0xFFC00000u;
  if (E == 255) return 0;
  uint32_t p = E & 1, Eb = p ? 127 : 128;
  uint32_t t = rsqrt_tab[(p << 11) | ((x >> 12) & 0x7FF)];
  int re = (int)((t >> 23) & 0xFF) - ((int)E - (int)Eb) / 2;
  return ((uint32_t)re << 23) | (t & 0x7FFFFFu);
}

static int verify(uint64_t stride)
{
  uint64_t bad_rcp = 0, bad_rsqrt = 0;
  for (uint64_t b = 0; b <= 0xFFFFFFFFull - 7; b += stride) {
    __m256i xi = _mm256_setr_epi32((int)b, (int)(b + 1), (int)(b + 2), (int)(b + 3),
                                   (int)(b + 4), (int)(b + 5), (int)(b + 6), (int)(b + 7));
    uint32_t r[8], q[8];
    _mm256_storeu_si256((__m256i*)r, _mm256_castps_si256(_mm256_rcp_ps(_mm256_castsi256_ps(xi))));
    _mm256_storeu_si256((__m256i*)q, _mm256_castps_si256(_mm256_rsqrt_ps(_mm256_castsi256_ps(xi))));
    for (int k = 0; k < 8; ++k) {
      uint32_t x = (uint32_t)(b + k);
      bad_rcp += emu_rcp(x) != r[k];
      bad_rsqrt += emu_rsqrt(x) != q[k];
    }
  }
  fprintf(stderr, "verify: rcp mismatches %llu, rsqrt mismatches %llu over %s inputs\n",
          (unsigned long long)bad_rcp, (unsigned long long)bad_rsqrt, stride == 8 ? "all 2^32" : "sampled");
  return (bad_rcp || bad_rsqrt) ? 1 : 0;
}

int main(int argc, char** argv)
{
  for (uint32_t m = 0; m < 2048; ++m)
    rcp_tab[m] = f2u(_mm_cvtss_f32(_mm_rcp_ss(_mm_set_ss(u2f(0x3F800000u | (m << 12))))));
  for (uint32_t p = 0; p < 2; ++p)
    for (uint32_t m = 0; m < 2048; ++m) {
      uint32_t E = p ? 127 : 128;
      rsqrt_tab[(p << 11) | m] = f2u(_mm_cvtss_f32(_mm_rsqrt_ss(_mm_set_ss(u2f((E << 23) | (m << 12))))));
    }
  /* --verify: all 2^32 inputs; --sample: 8 consecutive inputs out of every 2053 */
  if (argc > 1 && strcmp(argv[1], "--verify") == 0 && verify(8) != 0) return 1;
  if (argc > 1 && strcmp(argv[1], "--sample") == 0 && verify(2053) != 0) return 1;

  printf("/* Generated by gen_x86_tables.c from the RCPPS/RSQRTPS instructions of an\n"
         " * Intel Xeon (x86-64).  Data, not code: see gen_x86_tables.c for the layout. */\n"
         "#pragma once\n#include <stdint.h>\n\n");
  printf("/* RCPPS(1.m) for m = top 11 mantissa bits; result exponent field is 126 or 127. */\n");
  printf("#define X86_RCP_TABLE_VALUES \\\n");
  for (int i = 0; i < 2048; ++i) printf("0x%08x,%s", rcp_tab[i], (i % 8 == 7) ? " \\\n" : "");
  printf("\n/* RSQRTPS: index (E&1)<<11 | top 11 mantissa bits; base exponent 127 (odd) or 128 (even). */\n");
  printf("#define X86_RSQRT_TABLE_VALUES \\\n");
  for (int i = 0; i < 4096; ++i) printf("0x%08x,%s", rsqrt_tab[i], (i % 8 == 7) ? " \\\n" : "");
  printf("\nstatic const uint32_t kX86RcpTable[2048] = {X86_RCP_TABLE_VALUES};\n");
  printf("static const uint32_t kX86RsqrtTable[4096] = {X86_RSQRT_TABLE_VALUES};\n");
  return 0;
}
