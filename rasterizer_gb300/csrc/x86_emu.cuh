// x86 SSE/AVX single-precision semantics for host and device code.
//
// The reference rasteriser's results depend on details of the x86 float
// instructions it uses, so bit-exact output on the GPU needs them spelled out:
//  * every add/sub/mul/div/fma is separately rounded (no contraction; this
//    file is compiled with --fmad=false and uses __f*_rn on the device),
//    and a fused multiply-add happens only where the reference writes
//    _mm*_fmadd/fmsub/fnmadd_ps;
//  * a NaN result keeps the first NaN operand (quieted); an invalid operation
//    (inf-inf, 0*inf, 0/0) gives the x86 default NaN 0xFFC00000.  The GPU's
//    own NaN is 0x7FFFFFFF; only the sign of a NaN can reach the output (the
//    depth packing shifts float bits), but the whole pattern is reproduced;
//  * minps/maxps return the second operand when the comparison is false;
//  * cvttps2dq returns 0x80000000 for NaN and out-of-range inputs;
//  * RCPPS comes from the instruction's measured table (x86_tables.h).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define X86_HD __host__ __device__ __forceinline__
#else
#define X86_HD inline
#endif

#include "x86_tables.h"

#if defined(__CUDACC__)
// Device copies of the RCPPS and RSQRTPS tables, indexed with data-dependent
// bits (global memory through the read-only path; the constant cache would
// serialise).
__device__ const uint32_t kDevRcpTable[2048] = {X86_RCP_TABLE_VALUES};
__device__ const uint32_t kDevRsqrtTable[4096] = {X86_RSQRT_TABLE_VALUES};
#endif

namespace x86 {

X86_HD uint32_t fu(float f)
{
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  __builtin_memcpy(&u, &f, 4);
  return u;
#endif
}

X86_HD float uf(uint32_t u)
{
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
#endif
}

X86_HD bool isnan_(float f) { return (fu(f) & 0x7FFFFFFFu) > 0x7F800000u; }
X86_HD float quiet(float f) { return uf(fu(f) | 0x00400000u); }
constexpr uint32_t kDefaultNaN = 0xFFC00000u;

X86_HD float nan2(float r, float a, float b)
{
  if (!isnan_(r)) return r;
  if (isnan_(a)) return quiet(a);
  if (isnan_(b)) return quiet(b);
  return uf(kDefaultNaN);
}

X86_HD float nan3(float r, float a, float b, float c)
{
  if (!isnan_(r)) return r;
  if (isnan_(a)) return quiet(a);
  if (isnan_(b)) return quiet(b);
  if (isnan_(c)) return quiet(c);
  return uf(kDefaultNaN);
}

// Raw IEEE operations, round to nearest even, never contracted.
X86_HD float radd(float a, float b)
{
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
X86_HD float rsub(float a, float b)
{
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
X86_HD float rmul(float a, float b)
{
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
X86_HD float rdiv(float a, float b)
{
#ifdef __CUDA_ARCH__
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
X86_HD float rfma(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}

// x86-exact operations (NaN rules included).
X86_HD float xadd(float a, float b) { return nan2(radd(a, b), a, b); }
X86_HD float xsub(float a, float b) { return nan2(rsub(a, b), a, b); }
X86_HD float xmul(float a, float b) { return nan2(rmul(a, b), a, b); }
X86_HD float xdiv(float a, float b) { return nan2(rdiv(a, b), a, b); }
// _mm_fmadd_ps(a,b,c) = a*b + c
X86_HD float xfmadd(float a, float b, float c) { return nan3(rfma(a, b, c), a, b, c); }
// _mm_fmsub_ps(a,b,c) = a*b - c
X86_HD float xfmsub(float a, float b, float c) { return nan3(rfma(a, b, uf(fu(c) ^ 0x80000000u)), a, b, c); }
// _mm_fnmadd_ps(a,b,c) = c - a*b
X86_HD float xfnmadd(float a, float b, float c) { return nan3(rfma(uf(fu(a) ^ 0x80000000u), b, c), a, b, c); }

X86_HD float xmin(float a, float b) { return a < b ? a : b; }
X86_HD float xmax(float a, float b) { return a > b ? a : b; }
X86_HD float fxor(float a, uint32_t m) { return uf(fu(a) ^ m); }
X86_HD float fabs_(float a) { return uf(fu(a) & 0x7FFFFFFFu); }
X86_HD uint32_t sign(float a) { return fu(a) & 0x80000000u; }

X86_HD float round_even(float a)
{
  if (isnan_(a)) return quiet(a);
#ifdef __CUDA_ARCH__
  return rintf(a);
#else
  return __builtin_rintf(a);
#endif
}

X86_HD float floor_(float a)
{
  if (isnan_(a)) return quiet(a);
#ifdef __CUDA_ARCH__
  return floorf(a);
#else
  return __builtin_floorf(a);
#endif
}

X86_HD int32_t cvtt(float a)
{
  if (!(a > -2147483904.0f && a < 2147483648.0f)) return INT32_MIN;
#ifdef __CUDA_ARCH__
  return __float2int_rz(a);
#else
  return (int32_t)a;
#endif
}

X86_HD float i2f(int32_t i)
{
#ifdef __CUDA_ARCH__
  return __int2float_rn(i);
#else
  return (float)i;
#endif
}

// RCPPS (verified for all 2^32 inputs against the instruction).
X86_HD float rcp(float a)
{
  uint32_t x = fu(a), s = x & 0x80000000u, E = (x >> 23) & 0xFF;
  if (E == 255) return uf((x & 0x7FFFFF) ? (x | 0x400000u) : s);
  if (E == 0) return uf(s | 0x7F800000u);
#ifdef __CUDA_ARCH__
  uint32_t t = __ldg(&kDevRcpTable[(x >> 12) & 0x7FF]);
#else
  uint32_t t = kX86RcpTable[(x >> 12) & 0x7FF];
#endif
  int re = (int)((t >> 23) & 0xFF) + 127 - (int)E;
  return uf(re <= 0 ? s : (s | ((uint32_t)re << 23) | (t & 0x7FFFFFu)));
}

// RSQRTPS (occluder bake; the host form verified for all 2^32 inputs).
X86_HD float rsqrt(float a)
{
  uint32_t x = fu(a), s = x & 0x80000000u, E = (x >> 23) & 0xFF;
  if (E == 255 && (x & 0x7FFFFF)) return uf(x | 0x400000u);
  if (E == 0) return uf(s | 0x7F800000u);
  if (s) return uf(kDefaultNaN);
  if (E == 255) return 0.0f;
  uint32_t p = E & 1, Eb = p ? 127 : 128;
#ifdef __CUDA_ARCH__
  uint32_t t = __ldg(&kDevRsqrtTable[(p << 11) | ((x >> 12) & 0x7FF)]);
#else
  uint32_t t = kX86RsqrtTable[(p << 11) | ((x >> 12) & 0x7FF)];
#endif
  int re = (int)((t >> 23) & 0xFF) - ((int)E - (int)Eb) / 2;
  return uf(((uint32_t)re << 23) | (t & 0x7FFFFFu));
}

// DPPS, imm8 = 0xFF: (a0*b0 + a1*b1) + (a2*b2 + a3*b3); imm8 = 0x7F: last product is +0.
X86_HD float dp4(const float* a, const float* b)
{
  float p0 = xmul(a[0], b[0]), p1 = xmul(a[1], b[1]), p2 = xmul(a[2], b[2]), p3 = xmul(a[3], b[3]);
  return xadd(xadd(p0, p1), xadd(p2, p3));
}
X86_HD float dp3(const float* a, const float* b)
{
  float p0 = xmul(a[0], b[0]), p1 = xmul(a[1], b[1]), p2 = xmul(a[2], b[2]);
  return xadd(xadd(p0, p1), xadd(p2, 0.0f));
}

// packDepthPremultiplied for one value: arithmetic >> 12 of the float bits,
// unsigned 16-bit saturation.
X86_HD uint32_t pack_depth(float d)
{
  int32_t v = (int32_t)fu(d) >> 12;
  return (uint32_t)(v < 0 ? 0 : (v > 65535 ? 65535 : v));
}

}  // namespace x86
