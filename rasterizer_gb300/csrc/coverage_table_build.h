// Builder of the 8x8 coverage-mask table (host code).
//
// 64 quantised edge slopes x 64 quantised edge offsets -> one 64-bit mask of
// the pixels of an 8x8 block lying on the inner side of the edge.  The table
// is built by sampling 2000 edge angles x 2000 offsets and OR-ing the covered
// samples into the entry each (angle, offset) quantises to, the method of
// Rasterizer.cpp:547-604, with its quantisers (Rasterizer.cpp:470-480,
// 496-506).  Mask bit layout: pixel (x, y) -> bit 8x + (y even ? 4 + y/2 :
// (y-1)/2), i.e. per byte x the even rows in the high nibble and the odd rows
// in the low nibble (Rasterizer.cpp:527-545, consumed at :1259-1267).
//
// The angles go through libm cosf/sinf, whose last bit may differ between
// hosts, so the library ships the table generated on x86-64
// (coverage_table.h) and this builder is kept to regenerate and check it.
#pragma once
#include <stdint.h>
#include <string.h>
#include <math.h>

namespace occ_table {

inline uint64_t pixel_bit_layout(uint64_t samples)
{
  uint64_t out = 0;
  for (int x = 0; x < 8; ++x)
    for (int y = 0; y < 8; ++y)
      if ((samples >> (8 * x + y)) & 1)
        out |= 1ull << (8 * x + ((y & 1) ? (y >> 1) : 4 + (y >> 1)));
  return out;
}

inline int32_t trunc_x86(float a)
{
  if (!(a > -2147483904.0f && a < 2147483648.0f)) return INT32_MIN;
  return (int32_t)a;
}

inline void build_coverage_table(int64_t* table)
{
  const int kOffsets = 64, kSlopes = 64;
  const float minEdgeOffset = -0.45f, maxOffset = 0.45f;
  memset(table, 0, sizeof(int64_t) * kOffsets * kSlopes);
  const uint32_t angular = 2000, offsets = 2000;
  for (uint32_t i = 0; i < angular; ++i) {
    float angle = -0.1f + 6.4f * (float)i / (float)(angular - 1);
    float nx = cosf(angle), ny = sinf(angle);
    float l = 1.0f / (fabsf(nx) + fabsf(ny));
    nx *= l;
    ny *= l;
    // slope quantiser of the table build: strict ny < 0 (the runtime one uses <=)
    const float smul = (kSlopes / 2 - 1) * 0.5f;
    const float sadd = smul + 0.5f;
    int32_t q = trunc_x86(fmaf(nx, smul, sadd));
    uint32_t yneg = (ny < 0.0f) ? 0xFFFFFFFFu : 0u;
    uint32_t slope = ((((uint32_t)q) << 1) - yneg) << 6;
    for (uint32_t j = 0; j < offsets; ++j) {
      float offset = -0.6f + 1.2f * (float)j / (float)(angular - 1);
      const float omul = (kOffsets - 1) / (maxOffset - minEdgeOffset);
      const float oadd = 0.5f - minEdgeOffset * omul;
      float lookup = offset * omul + oadd;
      int32_t oi = (int32_t)lookup;
      oi = oi < 0 ? 0 : (oi > kOffsets - 1 ? kOffsets - 1 : oi);
      uint64_t samples = 0;
      for (int x = 0; x < 8; ++x)
        for (int y = 0; y < 8; ++y) {
          float d = offset + (x - 3.5f) / 8.0f * nx + (y - 3.5f) / 8.0f * ny;
          if (d <= 0.0f) samples |= 1ull << (8 * x + y);
        }
      table[slope | (uint32_t)oi] |= (int64_t)pixel_bit_layout(samples);
    }
  }
}

}  // namespace occ_table
