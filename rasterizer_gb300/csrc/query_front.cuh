// Device-side queryVisibility front end (Rasterizer.cpp:123-273) and the
// arithmetic policies it runs under; shared by the rasteriser's kernels and the
// learned-selection feature kernel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "raster_types.h"
#include "x86_emu.cuh"

namespace occ {

// ---- arithmetic policies -------------------------------------------------------------
// ExactOps applies the x86 NaN rules to every result.  FastOps uses plain IEEE
// operations and only records whether any result was NaN: without a NaN the
// two are bit-identical, so callers run FastOps and fall back to ExactOps for
// the rare inputs that produce one.  LazyOps (below) records NaN only where
// the caller asks.

struct ExactOps {
  __device__ __forceinline__ float add(float a, float b) { return x86::xadd(a, b); }
  __device__ __forceinline__ float sub(float a, float b) { return x86::xsub(a, b); }
  __device__ __forceinline__ float mul(float a, float b) { return x86::xmul(a, b); }
  __device__ __forceinline__ float div(float a, float b) { return x86::xdiv(a, b); }
  __device__ __forceinline__ float fmadd(float a, float b, float c) { return x86::xfmadd(a, b, c); }
  __device__ __forceinline__ float fmsub(float a, float b, float c) { return x86::xfmsub(a, b, c); }
  __device__ __forceinline__ float fnmadd(float a, float b, float c) { return x86::xfnmadd(a, b, c); }
  __device__ __forceinline__ float round(float a) { return x86::round_even(a); }
  __device__ __forceinline__ float floor(float a) { return x86::floor_(a); }
  __device__ __forceinline__ float dp4(const float* a, const float* b)
  {
    return add(add(mul(a[0], b[0]), mul(a[1], b[1])), add(mul(a[2], b[2]), mul(a[3], b[3])));
  }
  __device__ __forceinline__ float chk(float r) { return r; }
};

// Plain IEEE operations without per-result checks; the caller checks with
// chk() every value that reaches an operation which does not propagate NaN
// (comparisons, min/max, sign and bit extraction, the reciprocal table).  Any
// NaN produced earlier reaches one of those through IEEE add/multiply/fma,
// which propagate NaN, so a clean flag still means no NaN anywhere.
struct LazyOps {
  bool nan = false;
  __device__ __forceinline__ float chk(float r)
  {
    nan |= r != r;
    return r;
  }
  __device__ __forceinline__ float add(float a, float b) { return x86::radd(a, b); }
  __device__ __forceinline__ float sub(float a, float b) { return x86::rsub(a, b); }
  __device__ __forceinline__ float mul(float a, float b) { return x86::rmul(a, b); }
  __device__ __forceinline__ float div(float a, float b) { return x86::rdiv(a, b); }
  __device__ __forceinline__ float fmadd(float a, float b, float c) { return x86::rfma(a, b, c); }
  __device__ __forceinline__ float floor(float a) { return floorf(a); }
  __device__ __forceinline__ float dp4(const float* a, const float* b)
  {
    return add(add(mul(a[0], b[0]), mul(a[1], b[1])), add(mul(a[2], b[2]), mul(a[3], b[3])));
  }
};

struct FastOps {
  bool nan = false;
  __device__ __forceinline__ float chk(float r)
  {
    nan |= r != r;
    return r;
  }
  __device__ __forceinline__ float add(float a, float b) { return chk(x86::radd(a, b)); }
  __device__ __forceinline__ float sub(float a, float b) { return chk(x86::rsub(a, b)); }
  __device__ __forceinline__ float mul(float a, float b) { return chk(x86::rmul(a, b)); }
  __device__ __forceinline__ float div(float a, float b) { return chk(x86::rdiv(a, b)); }
  __device__ __forceinline__ float fmadd(float a, float b, float c) { return chk(x86::rfma(a, b, c)); }
  __device__ __forceinline__ float fmsub(float a, float b, float c) { return chk(x86::rfma(a, b, -c)); }
  __device__ __forceinline__ float fnmadd(float a, float b, float c) { return chk(x86::rfma(-a, b, c)); }
  __device__ __forceinline__ float round(float a) { return chk(rintf(a)); }
  __device__ __forceinline__ float floor(float a) { return chk(floorf(a)); }
  __device__ __forceinline__ float dp4(const float* a, const float* b)
  {
    return add(add(mul(a[0], b[0]), mul(a[1], b[1])), add(mul(a[2], b[2]), mul(a[3], b[3])));
  }
};

// ---- queryVisibility front end (Rasterizer.cpp:123-273) ------------------------------

// The frustum half of the front end (Rasterizer.cpp:125-167): true when the
// box is outside one of the six planes.
template <class Ops>
__device__ __forceinline__ bool query_outside_t(Ops& o, const ViewDesc& V, const float* bmin, const float* bmax)
{
  using x86::fxor; using x86::sign; using x86::fu;
  float ext[4], ctr[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    ext[i] = o.sub(bmax[i], bmin[i]);
    ctr[i] = o.add(bmax[i], bmin[i]);
  }
  const float* row3 = V.rows + 12;
  uint32_t signs = 0;
#pragma unroll
  for (int p = 0; p < 6; ++p) {
    const float* rr = V.rows + 4 * (p >> 1);
    float plane[4], offs[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      plane[i] = (p & 1) ? o.sub(row3[i], rr[i]) : o.add(row3[i], rr[i]);
      offs[i] = o.add(ctr[i], fxor(ext[i], sign(plane[i])));
    }
    signs |= fu(o.chk(o.dp4(plane, offs)));  // the box's values and the planes all reach this sum
  }
  return (signs & 0x80000000u) != 0;
}

// The projection half (Rasterizer.cpp:169-273) for a box inside the frustum:
// 1 (visible, needs clipping) or 2 (screen rectangle + maxZ for query2D), 0
// for an empty rectangle.  minZOut (optional) receives the smallest packed
// corner depth.
template <class Ops>
__device__ __forceinline__ int query_project_t(Ops& o, const ViewDesc& V, const float* bmin, const float* bmax, uint32_t* rect,
                                               uint32_t* maxZOut, uint32_t* minZOut = nullptr)
{
  using x86::xmin; using x86::xmax; using x86::fxor; using x86::fu;
  using x86::cvtt; using x86::i2f; using x86::rcp; using x86::pack_depth;
  float ext[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) ext[i] = o.sub(bmax[i], bmin[i]);
  const float* col0 = V.cols;
  const float* col1 = V.cols + 4;
  const float* col2 = V.cols + 8;
  const float* col3 = V.cols + 12;
  float c[8][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float e0 = o.mul(col0[i], ext[0]), e1 = o.mul(col1[i], ext[1]), e2 = o.mul(col2[i], ext[2]);
    c[0][i] = o.fmadd(col0[i], bmin[0], o.fmadd(col1[i], bmin[1], o.fmadd(col2[i], bmin[2], col3[i])));
    c[1][i] = o.add(c[0][i], e0);
    c[2][i] = o.add(c[0][i], e1);
    c[4][i] = o.add(c[0][i], e2);
    c[3][i] = o.add(c[1][i], e1);
    c[5][i] = o.add(c[4][i], e0);
    c[6][i] = o.add(c[2][i], e2);
    c[7][i] = o.add(c[6][i], e0);
  }
  float m1[4] = {xmax(ext[0], ext[2]), xmax(ext[1], ext[3]), xmax(ext[2], ext[0]), xmax(ext[3], ext[1])};
  float me[4] = {xmax(m1[0], m1[1]), xmax(m1[1], m1[0]), xmax(m1[2], m1[3]), xmax(m1[3], m1[2])};
  bool close = false;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float eps = o.mul(me[i], 0.001f);
    close |= (o.chk(c[i][3]) < eps) || (o.chk(c[4 + i][3]) < eps);
  }
  if (close) return 1;
  float X[8], Y[8], Z[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    float iw = rcp(c[k][3]);
    X[k] = o.chk(o.mul(c[k][0], iw));
    Y[k] = o.chk(o.mul(c[k][1], iw));
    Z[k] = o.chk(o.mul(c[k][2], iw));
  }
  float mnX[4], mxX[4], mnY[4], mxY[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    mnX[i] = xmin(X[i], X[4 + i]);
    mxX[i] = xmax(X[i], X[4 + i]);
    mnY[i] = xmin(Y[i], Y[4 + i]);
    mxY[i] = xmax(Y[i], Y[4 + i]);
  }
  float mn[4] = {xmin(mnX[0], mnX[2]), xmin(mnY[0], mnY[2]), xmin(mnX[1], mnX[3]), xmin(mnY[1], mnY[3])};
  float mx[4] = {xmax(mxX[0], mxX[2]), xmax(mxY[0], mxY[2]), xmax(mxX[1], mxX[3]), xmax(mxY[1], mxY[3])};
  const float limX = i2f((int32_t)(V.width - 1)), limY = i2f((int32_t)(V.height - 1));
  const float lim[4] = {limX, limY, limX, limY};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    mn[i] = xmax(mn[i], 0.0f);
    mx[i] = fxor(xmin(mx[i], lim[i]), 0x80000000u);
  }
  float bf[4] = {xmin(mn[0], mn[2]), xmin(mx[0], mx[2]), xmin(mn[1], mn[3]), xmin(mx[1], mx[3])};
  int32_t b[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) b[i] = cvtt(o.floor(bf[i]));
  b[1] = (int32_t)(0u - (uint32_t)b[1]);
  b[3] = (int32_t)(0u - (uint32_t)b[3]);
  if (b[0] >= b[1] || b[2] >= b[3]) return 0;
  uint32_t maxZ = 0, minZ = 0xFFFFFFFFu;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint32_t z = pack_depth(Z[k]);
    maxZ = ::max(maxZ, z);
    minZ = ::min(minZ, z);
  }
  if (minZOut) *minZOut = minZ;  // farthest corner (not part of the reference's query)
  rect[0] = (uint32_t)b[0];
  rect[1] = (uint32_t)b[1];
  rect[2] = (uint32_t)b[2];
  rect[3] = (uint32_t)b[3];
  *maxZOut = maxZ;
  return 2;
}

// Returns 0 (not visible), 1 (visible, needs clipping) or 2 (rect + maxZ for query2D).
template <class Ops>
__device__ __forceinline__ int query_front_t(Ops& o, const ViewDesc& V, const float* bmin, const float* bmax, uint32_t* rect,
                                             uint32_t* maxZOut, uint32_t* minZOut = nullptr)
{
  if (query_outside_t(o, V, bmin, bmax)) return 0;
  return query_project_t(o, V, bmin, bmax, rect, maxZOut, minZOut);
}

static __device__ __noinline__ int query_front_exact(const ViewDesc& V, const float* bmin, const float* bmax, uint32_t* rect,
                                              uint32_t* maxZOut, uint32_t* minZOut)
{
  ExactOps o;
  return query_front_t(o, V, bmin, bmax, rect, maxZOut, minZOut);
}

// Returns 0 (not visible), 1 (visible, needs clipping) or 2 (rect + maxZ for query2D).
// minZOut (optional) receives the smallest packed corner depth.
__device__ __forceinline__ int query_front(const ViewDesc& V, const float* bmin, const float* bmax, uint32_t* rect,
                                           uint32_t* maxZOut, uint32_t* minZOut = nullptr)
{
  LazyOps f;
  const int st = query_front_t(f, V, bmin, bmax, rect, maxZOut, minZOut);
  if (!f.nan) return st;
  return query_front_exact(V, bmin, bmax, rect, maxZOut, minZOut);
}


}  // namespace occ
