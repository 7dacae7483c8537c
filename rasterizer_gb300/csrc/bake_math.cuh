// Arithmetic of Occluder::bake (Occluder.cpp:7-181) shared by the host bake
// (bake.cpp) and the GPU bake (bake_gpu.cu), so that both produce the same
// bytes: every float operation separately rounded with the x86 NaN rules,
// RSQRTPS from the measured table (x86_emu.cuh).
#pragma once
#include <stdint.h>

#include "x86_emu.cuh"

namespace bake {

struct V4 {
  float v[4];
};

X86_HD V4 vsub(const V4& a, const V4& b)
{
  V4 r;
  for (int i = 0; i < 4; ++i) r.v[i] = x86::xsub(a.v[i], b.v[i]);
  return r;
}

X86_HD V4 vadd(const V4& a, const V4& b)
{
  V4 r;
  for (int i = 0; i < 4; ++i) r.v[i] = x86::xadd(a.v[i], b.v[i]);
  return r;
}

// cross product of the xyz lanes, w = a.w*b.w - a.w*b.w (VectorMath.h:6-12)
X86_HD V4 cross(const V4& a, const V4& b)
{
  using x86::xmul; using x86::xsub;
  V4 r;
  r.v[0] = xsub(xmul(a.v[1], b.v[2]), xmul(a.v[2], b.v[1]));
  r.v[1] = xsub(xmul(a.v[2], b.v[0]), xmul(a.v[0], b.v[2]));
  r.v[2] = xsub(xmul(a.v[0], b.v[1]), xmul(a.v[1], b.v[0]));
  r.v[3] = xsub(xmul(a.v[3], b.v[3]), xmul(a.v[3], b.v[3]));
  return r;
}

X86_HD V4 tri_normal(const V4& a, const V4& b, const V4& c) { return cross(vsub(b, a), vsub(c, a)); }

// v * RSQRTPS(dot3(v, v)) on all four lanes (VectorMath.h:20-23)
X86_HD V4 normalize(const V4& v)
{
  const float s = x86::rsqrt(x86::dp3(v.v, v.v));
  V4 r;
  for (int i = 0; i < 4; ++i) r.v[i] = x86::xmul(v.v[i], s);
  return r;
}

// A quad's normal for the k-means (Occluder.cpp:12-21)
X86_HD V4 quad_normal(const V4& v0, const V4& v1, const V4& v2, const V4& v3)
{
  return normalize(vadd(tri_normal(v0, v1, v2), tri_normal(v0, v2, v3)));
}

// The k-means seeds: the six axis directions (Occluder.cpp:23-29)
X86_HD V4 seed_centroid(int k)
{
  V4 c = {{0.0f, 0.0f, 0.0f, 0.0f}};
  const int axis[6] = {0, 1, 2, 1, 2, 0};
  c.v[axis[k]] = k < 3 ? 1.0f : -1.0f;
  return c;
}

// One packed vertex word: 11/11/10 bits of the position in the reference box
// (Occluder.cpp:111-150); inv = 1 / (refMax - refMin).
X86_HD uint32_t pack_vertex(const V4& p, const V4& lo, const V4& inv)
{
  using x86::cvtt; using x86::xfmadd; using x86::xmul; using x86::xsub;
  float r[3];
  for (int a = 0; a < 3; ++a) r[a] = xmul(xsub(p.v[a], lo.v[a]), inv.v[a]);
  const uint32_t X = (uint32_t)cvtt(xfmadd(r[0], 2047.0f, 0.5f)) - 1024u;  // _mm_sub_epi32 wraps
  const uint32_t Y = (uint32_t)cvtt(xfmadd(r[1], 2047.0f, 0.5f));
  const uint32_t Z = (uint32_t)cvtt(xfmadd(r[2], 1023.0f, 0.5f));
  return (X << 21) | (Y << 10) | Z;
}

}  // namespace bake
