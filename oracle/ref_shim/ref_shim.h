/*
 * Forced-include shim that lets gcc compile the reference occluder rasteriser's
 * own sources (Rasterizer.cpp, Occluder.cpp, QuadDecomposition.cpp,
 * SurfaceAreaHeuristic.cpp) unchanged, for use as the oracle on x86-64.
 * Test infrastructure only; nothing in the product includes it.
 *
 * It supplies the MSVC-isms those files use and maps the 32-byte-aligned AVX
 * loads/stores to unaligned forms: the reference applies them to
 * std::vector<__m128i> storage (Rasterizer.h:54, used at Rasterizer.cpp:1274-1284)
 * and to __m128 out[8] stack arrays (Rasterizer.cpp:428-431), which gcc only
 * aligns to 16 bytes.  The unaligned forms compute the same values.
 */
#pragma once
#include <immintrin.h>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <limits>
#include <algorithm>
#include <memory>
#include <vector>

#define __forceinline inline __attribute__((always_inline))

static inline void* _aligned_malloc(size_t size, size_t alignment)
{
  void* p = nullptr;
  if (posix_memalign(&p, alignment, size ? size : alignment) != 0) return nullptr;
  return p;
}

static inline unsigned char _BitScanForward(unsigned long* index, unsigned long mask)
{
  if (mask == 0) return 0;
  *index = (unsigned long)__builtin_ctzl(mask);
  return 1;
}

#define __debugbreak() abort()
#define _mm_cvtsi64x_si128 _mm_cvtsi64_si128
#define _mm256_load_si256 _mm256_loadu_si256
#define _mm256_store_si256 _mm256_storeu_si256
#define _mm256_store_ps _mm256_storeu_ps
