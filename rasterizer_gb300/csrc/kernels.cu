// GPU occluder rasteriser and visibility queries (sm_103a).
//
// One flush runs these kernels over a batch of views (raster_types.h), each
// after the first a programmatic dependent of the one before:
//
//   k_chunk_gate  one CTA per view: gates the view's commands (the plain
//                 loop's queryVisibility of the occluder bounds,
//                 Rasterizer.cpp:123-281; k_gate does it for views of more
//                 than 1,024 commands, the selection kernels with a
//                 selector), then lists the chunks holding a drawn command
//                 with their rank in the view.
//   k_setup       one CTA per active 256-quad chunk: per-occluder prologue
//                 (Rasterizer.cpp:612-655), then one thread per quad does the
//                 vertex transform and quad setup (Rasterizer.cpp:660-1081)
//                 and counts the quad's rows, row-walk checkpoints and
//                 16x16-block super-tiles.
//   k_scan        order-preserving prefix sums of those counts.
//   k_fill        one CTA per active chunk: writes each super-tile's quad
//                 list in submission order and the (quad, row) list of the
//                 row walk.
//   k_walk_prep   the row walk, one thread per (quad, block row): the
//                 reference's incremental float adds along the row, storing
//                 the edge offsets and depth lanes every 8 block columns; then
//                 the tile preparation, one warp per 8x4-block tile: the
//                 clear, and the queue of raster units a listed quad reaches.
//   k_raster      a warp per queued unit of 8 x R blocks (k_raster_cta: a CTA
//                 of 128 per 8x2-block unit, for launches with few units):
//                 filters the super-tile list to the quads reaching the unit,
//                 computes (quad, block) fragments and merges them per block
//                 in list order (Rasterizer.cpp:1098-1292); each unit writes
//                 its block rows' minimum hiZ.
//   k_query       queryVisibility + query2D (Rasterizer.cpp:123-349): frustum
//                 test per box, survivors listed per warp and projected by
//                 full warps, boxes over more than a warp-tile of blocks
//                 tested by the whole warp (k_query_thread: one box per
//                 thread in place, for few boxes; boxes over more than two
//                 warp-tiles shared by the CTA's warps).
//
// Exactness: every float operation follows the reference's order and
// rounding (x86_emu.cuh); the block loop sees each quad's primitives in
// submission order with the hiZ early-out tested against the running hiZ.
// The only place the rasteriser and the reference differ in control flow is
// the convex-quad row early exit (Rasterizer.cpp:1161-1165): the blocks it
// skips fail the same range test it is triggered by, because each edge offset
// is a monotone sequence along a row (repeated addition of one constant), so
// the in-range blocks of a row form one interval.  Skipping them or testing
// them gives the same result.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <stdlib.h>

#include <mutex>

#include "coverage_table.h"
#include "query_front.cuh"
#include "raster_types.h"
#include "x86_emu.cuh"

namespace occ {

__device__ const unsigned long long kDevCoverage[4096] = {OCC_COVERAGE_TABLE_VALUES};

// Row-walk grid: a few CTAs per SM, grid-striding over the batch's rows.
static uint32_t g_walkBlocks = 152 * 8;
// Persistent grids of the setup / list-fill / raster kernels (resident CTAs x SMs),
// looping over the launch's active chunks and tiles.
static uint32_t g_sms = 152;
static uint32_t g_setupPerSm = 4, g_fillPerSm = 4;  // occupancy limits
static uint32_t g_rasterPerSm[3] = {6, 6, 4};        // per raster unit shape R = 1, 2, 4
static uint32_t g_rasterCtaPerSm = 8;                 // the 128-thread form

static uint32_t grid_of(uint32_t tuned, uint32_t limit, uint32_t work)
{
  const uint32_t perSm = tuned ? ::min(tuned, limit) : limit;
  return ::max(1u, ::min(work, perSm * g_sms));
}

// Programmatic dependent launch.  Every kernel of a flush after the first is
// launched with programmatic stream serialisation: it is scheduled as the
// CTAs of its predecessor exit, before that grid has completed, so its launch
// and whatever it does before pdl_wait overlap the predecessor's last CTAs.
// pdl_wait returns when the predecessor grid has completed and its memory
// operations are visible; nothing a predecessor writes is read before it.
// (No kernel signals its dependents earlier: CTAs waiting in pdl_wait slow
// the ones still working on their SM.)  Launched without the attribute,
// pdl_wait returns at once.  The environment variable OCC_PDL=0 launches
// every kernel plainly.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

static bool g_pdl = true;

// Primitive mode for the 8-bit configuration (area signs | W signs << 4),
// the classification of Rasterizer.cpp:30-64.
__device__ const uint8_t kDevModeTable[256] = {
#define CV kModeConvex
#define T0 kModeTriangle0
#define T1 kModeTriangle1
#define CR kModeConcaveRight
#define CL kModeConcaveLeft
#define CC kModeConcaveCenter
#define NO kModeCulled
  CV, T1, CL, T1, T0, NO, T0, NO,  CR, T1, NO, T1, T0, NO, T0, NO,
  CV, T1, CL, T1, T0, NO, T0, NO,  NO, T1, CC, T1, T0, NO, T0, NO,
  CV, NO, CL, T1, T0, NO, T0, NO,  CR, T1, CC, T1, T0, NO, NO, NO,
  CV, T1, CL, NO, T0, NO, T0, NO,  CR, T1, CC, T1, NO, NO, T0, NO,
  CV, T1, NO, T1, T0, NO, T0, NO,  CR, T1, CC, T1, T0, NO, T0, NO,
  NO, T1, CC, T1, T0, NO, T0, NO,  CC, T1, CC, T1, T0, NO, T0, NO,
  CV, T1, CL, T1, T0, NO, NO, NO,  CR, NO, CC, T1, T0, NO, T0, NO,
  T1, T1, T1, T1, NO, NO, NO, NO,  T1, T1, T1, NO, NO, NO, NO, NO,
  CV, T1, CL, T1, NO, NO, T0, NO,  CR, T1, CC, NO, T0, NO, T0, NO,
  CV, T1, CL, T1, T0, NO, NO, NO,  CR, NO, CC, T1, T0, NO, T0, NO,
  NO, T1, CL, T1, T0, NO, T0, NO,  CR, T1, CC, T1, T0, NO, T0, NO,
  CR, T1, NO, T1, T0, NO, T0, NO,  CR, T1, CC, T1, T0, NO, T0, NO,
  CV, T1, CL, NO, T0, NO, T0, NO,  CR, T1, CC, T1, NO, NO, T0, NO,
  T0, NO, T0, NO, T0, NO, T0, NO,  T0, NO, T0, NO, T0, NO, NO, NO,
  CL, T1, CL, T1, T0, NO, T0, NO,  NO, T1, CC, T1, T0, NO, T0, NO,
  NO, NO, NO, NO, NO, NO, NO, NO,  NO, NO, NO, NO, NO, NO, NO, NO,
#undef CV
#undef T0
#undef T1
#undef CR
#undef CL
#undef CC
#undef NO
};

// ---- constants (Rasterizer.cpp:9-17, written as their float values) -----------

__device__ __forceinline__ float kMaxInvW() { return __uint_as_float(0x5F7FFFFFu); }  // sqrtf(FLT_MAX)
constexpr float kOffsetMul = 70.0f;    // (64 - 1) / (0.45f - -0.45f)
constexpr float kOffsetAdd = 32.0f;    // 0.5f - -0.45f * 63 / 0.9f
constexpr float kCkRange = 63.0f;      // OFFSET_QUANTIZATION_FACTOR - 1
__device__ __forceinline__ float kSlopeMul() { return __uint_as_float(0x3E62BE2Cu); }  // 15.5f / 70.0f
constexpr float kSlopeAdd = 16.0f;     // (32 - 1) * 0.5f + 0.5f
__device__ __forceinline__ float kBboxMinAdd() { return __uint_as_float(0x3F1FFF2Eu); }  // 4.9999f / 8.0f
constexpr float kBboxMaxAdd = 1.375f;  // 11.0f / 8.0f

// ---- small device helpers -----------------------------------------------------------

__device__ __forceinline__ uint32_t vmax_u16x2(uint32_t a, uint32_t b)
{
  uint32_t d;
  asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

__device__ __forceinline__ uint32_t vmin_u16x2(uint32_t a, uint32_t b)
{
  uint32_t d;
  asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// _mm256_avg_epu16 on two packed pairs: (a + b + 1) >> 1 per 16-bit lane.
__device__ __forceinline__ uint32_t avg_u16x2(uint32_t a, uint32_t b)
{
  return (a | b) - (((a ^ b) >> 1) & 0x7FFF7FFFu);
}

// packDepthPremultiplied of two lanes (Rasterizer.cpp:508-525): each float's
// bits shifted right by 12 (arithmetic), saturated to [0, 65535] as
// _mm256_packus_epi32 does; lo -> bits 0..15, hi -> bits 16..31.  One
// saturating pack instruction: its first source fills the upper half.
__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
  uint32_t d;
  asm("cvt.pack.sat.u16.s32 %0, %1, %2;"
      : "=r"(d)
      : "r"((int32_t)__float_as_uint(hi) >> 12), "r"((int32_t)__float_as_uint(lo) >> 12));
  return d;
}

template <int NT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t& total, uint32_t* sm /* NT/32 */)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < NT / 32 ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NT / 32) sm[lane] = w;
  }
  __syncthreads();
  uint32_t prefix = warp > 0 ? sm[warp - 1] : 0;
  total = sm[NT / 32 - 1];
  __syncthreads();
  return prefix + x - v;
}

// query2D (Rasterizer.cpp:283-349), split by warp-tile.  The reference skips
// every block whose hiZ >= maxZ; a warp-tile whose minimum hiZ is >= maxZ is
// skipped as a whole, which skips exactly the same blocks.  The result is the
// OR over blocks, so tiles and blocks may be visited in any order.

// Per warp-tile, the minimum hiZ of each of its four block rows (tileHiz[4 t
// + r], 0xFFFF for rows outside the view); written by the raster unit that
// owns the row, or by the tile preparation for rows no unit is queued for.
__device__ __forceinline__ uint2 tile_rows(const ViewDesc& V, uint32_t t)
{
  return *reinterpret_cast<const uint2*>(V.tileHiz + 4 * (size_t)t);
}
__device__ __forceinline__ uint32_t row_min(const uint2 rm, uint32_t r)
{
  const uint32_t w = r & 2u ? rm.y : rm.x;
  return r & 1u ? w >> 16 : w & 0xFFFFu;
}
__device__ __forceinline__ uint32_t tile_min(const uint2 rm)
{
  const uint32_t m = vmin_u16x2(rm.x, rm.y);
  return ::min(m & 0xFFFFu, m >> 16);
}

// Two forms of each helper: kBatch loads what a step needs together (a block
// row's hiZ values, four pixel rows of a block) for the shortest chain of
// dependent loads, where few boxes are in flight (one view's boxes, a thread
// each); the other form loads one value at a time and stops at the first
// visible one, for the fewest instructions where many boxes keep the GPU busy.

// One block (bx, by) of the rectangle whose hiZ is below maxZ: visible if the
// rectangle covers it whole, else if any covered pixel has depth < maxZ
// (Rasterizer.cpp:303-344).
template <bool kBatch>
__device__ __forceinline__ bool query2d_open_block(const ViewDesc& V, uint32_t bx, uint32_t by, uint32_t minX,
                                                   uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ)
{
  int32_t sy = (int32_t)(minY - 8 * by);
  sy = sy < 0 ? 0 : sy;
  int32_t ey = (int32_t)(maxY - 8 * by);
  ey = ey > 7 ? 7 : ey;
  int32_t sx = (int32_t)(minX - bx * 8);
  sx = sx < 0 ? 0 : sx;
  int32_t ex = (int32_t)(maxX - bx * 8);
  ex = ex > 7 ? 7 : ex;
  if (sy == 0 && ey == 7 && sx == 0 && ex == 7) return true;
  const uint32_t mz2 = maxZ | (maxZ << 16);  // maxZ is a packed 16-bit depth
  // the reference's rowSelector as 16-bit lanes of the 4 row words
  uint32_t cm[4];
#pragma unroll
  for (int w = 0; w < 4; ++w)
    cm[w] = ((2 * w >= sx && 2 * w <= ex) ? 0x0000FFFFu : 0u) | ((2 * w + 1 >= sx && 2 * w + 1 <= ex) ? 0xFFFF0000u : 0u);
  const uint4* d = reinterpret_cast<const uint4*>(V.depth + (size_t)(by * V.blocksX + bx) * 64);
  // a pixel is visible where its depth < maxZ (Rasterizer.cpp:333-336)
  auto hit = [&](const uint4& row) {
    return ((__vcmpltu2(row.x, mz2) & cm[0]) | (__vcmpltu2(row.y, mz2) & cm[1]) | (__vcmpltu2(row.z, mz2) & cm[2]) |
            (__vcmpltu2(row.w, mz2) & cm[3])) != 0u;
  };
  if constexpr (!kBatch) {
    for (int32_t y = sy; y <= ey; ++y)
      if (hit(d[y])) return true;
  } else {
#pragma unroll
    for (int y0 = 0; y0 < 8; y0 += 4) {  // the block is one 128-byte line
      if (y0 > ey || y0 + 3 < sy) continue;
      uint4 row[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) row[k] = (y0 + k >= sy && y0 + k <= ey) ? d[y0 + k] : make_uint4(0, 0, 0, 0);
      bool any = false;
#pragma unroll
      for (int k = 0; k < 4; ++k) any |= y0 + k >= sy && y0 + k <= ey && hit(row[k]);
      if (any) return true;
    }
  }
  return false;
}

// One block of the rectangle: skipped if maxZ <= its hiZ, else as above.
template <bool kBatch>
__device__ __forceinline__ bool query2d_block(const ViewDesc& V, uint32_t bx, uint32_t by, uint32_t minX,
                                              uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ)
{
  if (maxZ <= (uint32_t)V.hiz[by * V.blocksX + bx]) return false;
  return query2d_open_block<kBatch>(V, bx, by, minX, maxX, minY, maxY, maxZ);
}

// Blocks of tile (tx, ty) inside the rectangle, rows whose minimum hiZ is
// >= maxZ skipped (all their blocks are); kBatch: a block row at a time, the
// row's hiZ values (at most 8) loaded together.  rm: the tile's row minima.
template <bool kBatch>
__device__ bool query2d_tile(const ViewDesc& V, uint32_t tx, uint32_t ty, uint2 rm, uint32_t minX, uint32_t maxX,
                             uint32_t minY, uint32_t maxY, uint32_t maxZ)
{
  const uint32_t bx0 = minX >> 3, bx1 = maxX >> 3, by0 = minY >> 3, by1 = maxY >> 3;
  const uint32_t ya = ::max(by0, ty * kTileH), yb = ::min(by1, ty * kTileH + kTileH - 1);
  const uint32_t xa = ::max(bx0, tx * kTileW), xb = ::min(bx1, tx * kTileW + kTileW - 1);
  for (uint32_t by = ya; by <= yb; ++by) {
    if (maxZ <= row_min(rm, by - ty * kTileH)) continue;
    if (!kBatch) {
      for (uint32_t bx = xa; bx <= xb; ++bx)
        if (query2d_block<false>(V, bx, by, minX, maxX, minY, maxY, maxZ)) return true;
      continue;
    }
    const uint16_t* h = V.hiz + by * V.blocksX + xa;
    uint32_t open = 0;
#pragma unroll
    for (uint32_t k = 0; k < (uint32_t)kTileW; ++k)
      if (xa + k <= xb && maxZ > (uint32_t)h[k]) open |= 1u << k;
    while (open) {
      const uint32_t k = (uint32_t)(__ffs(open) - 1);
      open &= open - 1;
      if (query2d_open_block<true>(V, xa + k, by, minX, maxX, minY, maxY, maxZ)) return true;
    }
  }
  return false;
}

template <bool kBatch>
__device__ bool query2d(const ViewDesc& V, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ)
{
  const uint32_t tilesX = (V.blocksX + kTileW - 1) / kTileW;
  const uint32_t tx0 = (minX >> 3) / kTileW, tx1 = (maxX >> 3) / kTileW;
  const uint32_t ty0 = (minY >> 3) / kTileH, ty1 = (maxY >> 3) / kTileH;
  for (uint32_t ty = ty0; ty <= ty1; ++ty)
    for (uint32_t tx = tx0; tx <= tx1; ++tx) {
      const uint2 rm = tile_rows(V, ty * tilesX + tx);
      if (maxZ <= tile_min(rm)) continue;
      if (query2d_tile<kBatch>(V, tx, ty, rm, minX, maxX, minY, maxY, maxZ)) return true;
    }
  return false;
}

// ---- per-occluder prologue (Rasterizer.cpp:612-655) ----------------------------------

struct CmdConst {
  float rows[4][4];  // output i's coefficients for (X word, Y word, Z word, 1)
  float c0, c1;      // Z = c1 * (1/W) + c0
  uint32_t draw, nc;
};

template <class Ops>
__device__ __forceinline__ void cmd_prologue_t(Ops& o, const ViewDesc& V, const Cmd& cmd, CmdConst& out)
{
  using x86::xmin; using x86::xmax; using x86::fxor; using x86::fabs_; using x86::sign; using x86::fu;
  using x86::cvtt; using x86::i2f; using x86::rcp; using x86::pack_depth; using x86::radd; using x86::rmul;
  float col[4][4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) col[j][i] = V.cols[4 * j + i];
  float ext[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) ext[i] = o.sub(cmd.refMax[i], cmd.refMin[i]);
  float c3[4], n0[4], n1[4], n2[4];
  const float s0 = o.mul(ext[0], __uint_as_float(0x2F801002u));  // 1.0f / (2047ull << 21)
  const float s1 = o.mul(ext[1], __uint_as_float(0x35001002u));  // 1.0f / (2047 << 10)
  const float s2 = o.mul(ext[2], __uint_as_float(0x3A802008u));  // 1.0f / 1023
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    c3[i] = o.fmadd(col[0][i], cmd.refMin[0], o.fmadd(col[1][i], cmd.refMin[1], o.fmadd(col[2][i], cmd.refMin[2], col[3][i])));
    n0[i] = o.mul(col[0][i], s0);
    n1[i] = o.mul(col[1][i], s1);
    n2[i] = o.mul(col[2][i], s2);
    c3[i] = o.fmadd(n0[i], 2147483648.0f, c3[i]);  // 1024ull << 21
    n1[i] = o.sub(n1[i], n0[i]);
    n2[i] = o.sub(n2[i], n0[i]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    out.rows[i][0] = n0[i];
    out.rows[i][1] = n1[i];
    out.rows[i][2] = n2[i];
    out.rows[i][3] = c3[i];
  }
  const float w[4] = {2097152.0f, 1024.0f, 1.0f, 1.0f};
  const float Za = out.rows[2][3], Zb = o.dp4(out.rows[2], w);
  const float Wa = out.rows[3][3], Wb = o.dp4(out.rows[3], w);
  const float c0 = o.div(o.sub(Za, Zb), o.sub(Wa, Wb));
  out.c0 = c0;
  out.c1 = o.fnmadd(c0, Wa, Za);
}

__device__ __noinline__ void cmd_prologue_exact(const ViewDesc& V, const Cmd& cmd, CmdConst& out)
{
  ExactOps o;
  cmd_prologue_t(o, V, cmd, out);
}

__device__ __forceinline__ void cmd_prologue(const ViewDesc& V, const Cmd& cmd, CmdConst& out)
{
  FastOps f;
  cmd_prologue_t(f, V, cmd, out);
  if (f.nan) cmd_prologue_exact(V, cmd, out);
}

// ---- quad setup (one SIMD lane of Rasterizer.cpp:660-1081) ---------------------------

template <class Ops>
__device__ __forceinline__ bool quad_setup_t(Ops& o, const ViewDesc& V, const uint32_t w4[4], const CmdConst& K,
                                             QuadRaster& R, QuadWalk& Wk)
{
  using x86::xmin; using x86::xmax; using x86::fxor; using x86::fabs_; using x86::sign; using x86::fu;
  using x86::cvtt; using x86::i2f; using x86::rcp; using x86::pack_depth; using x86::radd; using x86::rmul;
  const bool nc = K.nc != 0;
  float x[4], y[4], z[4], invW[4];
  uint32_t ws[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float Xf = i2f((int32_t)w4[j]);
    const float Yf = i2f((int32_t)(w4[j] & (2047u << 10)));
    const float Zf = i2f((int32_t)(w4[j] & 1023u));
    const float X = o.fmadd(Xf, K.rows[0][0], o.fmadd(Yf, K.rows[0][1], o.fmadd(Zf, K.rows[0][2], K.rows[0][3])));
    const float Y = o.fmadd(Xf, K.rows[1][0], o.fmadd(Yf, K.rows[1][1], o.fmadd(Zf, K.rows[1][2], K.rows[1][3])));
    const float W = o.fmadd(Xf, K.rows[3][0], o.fmadd(Yf, K.rows[3][1], o.fmadd(Zf, K.rows[3][2], K.rows[3][3])));
    invW[j] = nc ? xmin(kMaxInvW(), xmax(-kMaxInvW(), rcp(W))) : rcp(W);
    x[j] = o.mul(o.round(o.mul(X, invW[j])), 0.125f);
    y[j] = o.mul(o.round(o.mul(Y, invW[j])), 0.125f);
    ws[j] = nc ? sign(invW[j]) : 0u;
  }
  float eX[5], eY[5];
  eX[0] = o.sub(y[1], y[0]); eX[1] = o.sub(y[2], y[1]); eX[2] = o.sub(y[3], y[2]); eX[3] = o.sub(y[0], y[3]);
  eY[0] = o.sub(x[0], x[1]); eY[1] = o.sub(x[1], x[2]); eY[2] = o.sub(x[2], x[3]); eY[3] = o.sub(x[3], x[0]);
  const float area0 = o.fmsub(eX[0], eY[1], o.mul(eX[1], eY[0]));
  const float area1 = o.fmsub(eX[1], eY[2], o.mul(eX[2], eY[1]));
  const float area2 = o.fmsub(eX[2], eY[3], o.mul(eX[3], eY[2]));
  const float area3 = o.sub(o.add(area0, area2), area1);
  uint32_t cfg = 0;
  cfg |= (fxor(area0, ws[0] ^ ws[1] ^ ws[2]) <= 0.0f) ? 1u : 0u;
  cfg |= (fxor(area1, ws[1] ^ ws[2] ^ ws[3]) <= 0.0f) ? 2u : 0u;
  cfg |= (fxor(area2, ws[0] ^ ws[2] ^ ws[3]) <= 0.0f) ? 4u : 0u;
  cfg |= (fxor(area3, ws[1] ^ ws[0] ^ ws[3]) <= 0.0f) ? 8u : 0u;
  cfg |= (ws[0] >> 27) | (ws[1] >> 26) | (ws[2] >> 25) | (ws[3] >> 24);
  const int mode = kDevModeTable[cfg];
  if (mode == kModeCulled) return false;

  float minFx, minFy, maxFx, maxFy;
  if (nc) {
    // clipless bounding box (Rasterizer.cpp:820-909)
    const float infP = 10000.0f, infN = -10000.0f;
    float mPx[4], mPy[4], MPx[4], MPy[4], mNx[4], mNy[4], MNx[4], MNy[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      mPx[j] = ws[j] ? infP : x[j];
      mPy[j] = ws[j] ? infP : y[j];
      MPx[j] = fxor(mPx[j], ws[j]);
      MPy[j] = fxor(mPy[j], ws[j]);
      mNx[j] = ws[j] ? x[j] : infP;
      mNy[j] = ws[j] ? y[j] : infP;
      MNx[j] = ws[j] ? x[j] : infN;
      MNy[j] = ws[j] ? y[j] : infN;
    }
    const float minPx = xmin(xmin(mPx[0], mPx[1]), xmin(mPx[2], mPx[3]));
    const float minPy = xmin(xmin(mPy[0], mPy[1]), xmin(mPy[2], mPy[3]));
    const float maxPx = xmax(xmax(MPx[0], MPx[1]), xmax(MPx[2], MPx[3]));
    const float maxPy = xmax(xmax(MPy[0], MPy[1]), xmax(MPy[2], MPy[3]));
    const float minNx = xmin(xmin(mNx[0], mNx[1]), xmin(mNx[2], mNx[3]));
    const float minNy = xmin(xmin(mNy[0], mNy[1]), xmin(mNy[2], mNy[3]));
    const float maxNx = xmax(xmax(MNx[0], MNx[1]), xmax(MNx[2], MNx[3]));
    const float maxNy = xmax(xmax(MNy[0], MNy[1]), xmax(MNy[2], MNy[3]));
    const float incAx = (maxNx > minPx) ? infN : minPx;
    const float incAy = (maxNy > minPy) ? infN : minPy;
    const float incBx = (maxPx > minNx) ? infP : maxPx;
    const float incBy = (maxPy > minNy) ? infP : maxPy;
    minFx = xmin(incAx, incBx);
    minFy = xmin(incAy, incBy);
    maxFx = xmax(incAx, incBx);
    maxFy = xmax(incAy, incBy);
  } else {
    minFx = xmin(xmin(x[0], x[1]), xmin(x[2], x[3]));
    minFy = xmin(xmin(y[0], y[1]), xmin(y[2], y[3]));
    maxFx = xmax(xmax(x[0], x[1]), xmax(x[2], x[3]));
    maxFy = xmax(xmax(y[0], y[1]), xmax(y[2], y[3]));
  }
  int32_t minX = cvtt(o.add(minFx, kBboxMinAdd()));
  int32_t minY = cvtt(o.add(minFy, kBboxMinAdd()));
  int32_t maxX = cvtt(o.add(maxFx, kBboxMaxAdd));
  int32_t maxY = cvtt(o.add(maxFy, kBboxMaxAdd));
  minX = minX < 0 ? 0 : minX;
  minY = minY < 0 ? 0 : minY;
  maxX = maxX > (int32_t)V.blocksX ? (int32_t)V.blocksX : maxX;
  maxY = maxY > (int32_t)V.blocksY ? (int32_t)V.blocksY : maxY;
  if (!(maxX > minX && maxY > minY)) return false;

#pragma unroll
  for (int j = 0; j < 4; ++j) z[j] = o.fmadd(invW[j], K.c1, K.c0);
  float maxZ = xmax(xmax(z[0], z[1]), xmax(z[2], z[3]));
  if (nc && (ws[0] | ws[1] | ws[2] | ws[3])) maxZ = 1.0f;

  // depth plane of the larger triangle (Rasterizer.cpp:963-999)
  const bool t0 = mode == kModeTriangle0, t1 = mode == kModeTriangle1;
  bool greater = fabs_(area0) < fabs_(area2);
  greater = !t0 && (t1 || greater);
  const float a = greater ? area2 : area0;
  const float invArea = nc ? o.div(1.0f, a) : rcp(a);
  const float z12 = o.sub(z[1], z[2]), z20 = o.sub(z[2], z[0]), z30 = o.sub(z[3], z[0]);
  eX[4] = o.sub(y[0], y[2]);
  eY[4] = o.sub(x[2], x[0]);
  const float dx = greater ? o.fnmadd(z20, eX[3], o.mul(z30, eX[4])) : o.fmsub(z20, eX[1], o.mul(z12, eX[4]));
  const float dy = greater ? o.fnmadd(z20, eY[3], o.mul(z30, eY[4])) : o.fmsub(z20, eY[1], o.mul(z12, eY[4]));
  const float plane1 = o.mul(invArea, dx);
  const float plane2 = o.mul(invArea, dy);
  const float x0 = o.sub(x[0], i2f(minX));
  const float y0 = o.sub(y[0], i2f(minY));
  const float plane0 = o.fnmadd(x0, plane1, o.fnmadd(y0, plane2, z[0]));

  if (t0) { eX[2] = eX[4]; eY[2] = eY[4]; }
  if (t1) { eX[0] = fxor(eX[4], 0x80000000u); eY[0] = fxor(eY[4], 0x80000000u); }
  uint32_t flip[4] = {0, 0, 0, 0};
  if (nc) {
    flip[0] = ws[0] ^ (t1 ? ws[2] : ws[1]);
    flip[1] = ws[1] ^ ws[2];
    flip[2] = ws[2] ^ (t0 ? ws[0] : ws[3]);
    flip[3] = ws[0] ^ ws[3];
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) {  // normalizeEdge (Rasterizer.cpp:452-468)
    float invLen = rcp(o.add(fabs_(eX[e]), fabs_(eY[e])));
    invLen = o.mul(nc ? fxor(kOffsetMul, flip[e]) : kOffsetMul, invLen);
    eX[e] = o.mul(eX[e], invLen);
    eY[e] = o.mul(eY[e], invLen);
  }
  float off[4];
  off[0] = o.fnmadd(x0, eX[0], o.fnmadd(y0, eY[0], kOffsetAdd));
#pragma unroll
  for (int e = 1; e < 4; ++e) off[e] = o.fnmadd(x[e], eX[e], o.fnmadd(y[e], eY[e], kOffsetAdd));
#pragma unroll
  for (int e = 1; e < 4; ++e) off[e] = o.fmadd(i2f(minX), eX[e], off[e]);
#pragma unroll
  for (int e = 1; e < 4; ++e) off[e] = o.fmadd(i2f(minY), eY[e], off[e]);
#pragma unroll
  for (int e = 0; e < 4; ++e) {  // quantizeSlopeLookup (Rasterizer.cpp:482-493)
    const uint32_t yneg = (eY[e] <= 0.0f) ? 0xFFFFFFFFu : 0u;
    const uint32_t q = (uint32_t)cvtt(o.fmadd(eX[e], kSlopeMul(), kSlopeAdd));
    R.slope[e] = (uint16_t)(((((q << 1) - yneg) << 6)) & 4095u);
    R.nx[e] = eX[e];
    Wk.ny[e] = eY[e];
    Wk.off[e] = off[e];
  }
  R.minX = (uint16_t)minX;
  R.minY = (uint16_t)minY;
  R.maxX = (uint16_t)maxX;
  R.maxY = (uint16_t)maxY;
  R.maxZ = (uint16_t)pack_depth(maxZ);
  R.mode = (uint8_t)mode;
  R.Dx = plane1;
  R.Dy = plane2;
  Wk.plane0 = plane0;
  // Safe when no depth value along the walk can leave the finite range: then
  // plain IEEE adds give the x86 result bit for bit (no NaN can appear).
  const float span = i2f((maxX - minX) + (maxY - minY) + 4);
  const float bound = radd(fabs_(plane0), rmul(span, radd(fabs_(plane1), fabs_(plane2))));
  const bool safe = bound < 1e37f;  // false for NaN / inf inputs too
  R.flags = (uint8_t)((nc ? kQuadNearClip : 0) | (safe ? kQuadSafe : 0));
  return true;
}

__device__ __noinline__ bool quad_setup_exact(const ViewDesc& V, const uint32_t w4[4], const CmdConst& K,
                                              QuadRaster& R, QuadWalk& Wk)
{
  ExactOps o;
  return quad_setup_t(o, V, w4, K, R, Wk);
}

__device__ __forceinline__ bool quad_setup(const ViewDesc& V, const uint32_t w4[4], const CmdConst& K, QuadRaster& R,
                                           QuadWalk& Wk)
{
  FastOps f;
  const bool ok = quad_setup_t(f, V, w4, K, R, Wk);
  if (!f.nan) return ok;
  return quad_setup_exact(V, w4, K, R, Wk);
}

__device__ __forceinline__ uint32_t view_of_chunk(const FrameParams& P, uint32_t c) { return P.chunks[c].view; }

__device__ __forceinline__ uint32_t nck_of(const QuadRaster& R)
{
  return (uint32_t)((R.maxX - 1) >> 3) - (uint32_t)(R.minX >> 3) + 1u;
}

// ---- k_gate / k_chunk_gate ------------------------------------------------------------
// One thread per command: whether it is drawn and with which variant.  A gated
// command runs queryVisibility of its bounds against an empty buffer: drawn
// iff in the frustum and either near the camera plane or covering a nonempty
// screen rectangle with a nonzero depth bound; needs clipping iff near the
// camera plane.  With a selection, commands outside the view's top-K are not
// drawn.

__device__ __forceinline__ void gate_cmd(const FrameParams& P, uint32_t c)
{
  const Cmd& cmd = P.cmds[c];
  const ViewDesc& V = P.views[cmd.view];
  uint32_t draw = 1, nc = (cmd.flags & kCmdNearClip) ? 1u : 0u;
  if (cmd.flags & kCmdGated) {
    uint32_t rect[4], maxZ = 0;
    const int st = query_front(V, cmd.boundsMin, cmd.boundsMax, rect, &maxZ);
    draw = (st == 1 || (st == 2 && maxZ > 0)) ? 1u : 0u;
    nc = st == 1 ? 1u : 0u;
  }
  if (P.select && !P.select[c]) draw = 0;  // not among the view's top-K
  P.cmdDraw[c] = draw | (nc << 1);
}

__global__ void __launch_bounds__(256) k_gate(FrameParams P)
{
  pdl_wait();
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < P.numCmds) gate_cmd(P, c);
}

// Second pass of a selection, one warp per command: a candidate left out of
// the top-K is drawn if its bounds are still visible against the first pass's
// buffer (queryVisibility, as the reference's loop runs it before each
// rasterize, Main.cpp:192-206).  The lanes share the query2D over warp-tiles.
__global__ void __launch_bounds__(256) k_gate_second(FrameParams P)
{
  pdl_wait();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t c = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (c >= P.numCmds) return;  // whole warp
  const uint32_t first = P.cmdDraw[c] & 1u;
  uint32_t draw = 0, nc = 0;
  if (!first && P.cand[c]) {
    const Cmd& cmd = P.cmds[c];
    const ViewDesc& V = P.views[cmd.view];
    uint32_t rect[4], maxZ = 0;
    const int st = query_front(V, cmd.boundsMin, cmd.boundsMax, rect, &maxZ);  // same on every lane
    if (st == 1) {
      draw = nc = 1;
    } else if (st == 2) {
      const uint32_t tilesX = (V.blocksX + kTileW - 1) / kTileW;
      const uint32_t tx0 = (rect[0] >> 3) / kTileW, tx1 = (rect[1] >> 3) / kTileW;
      const uint32_t ty0 = (rect[2] >> 3) / kTileH, ty1 = (rect[3] >> 3) / kTileH;
      const uint32_t ntx = tx1 - tx0 + 1, nt = ntx * (ty1 - ty0 + 1);
      bool found = false;
      for (uint32_t t0 = 0; t0 < nt && !found; t0 += 32) {
        const uint32_t t = t0 + lane;
        bool hit = false;
        if (t < nt) {
          const uint32_t tx = tx0 + t % ntx, ty = ty0 + t / ntx;
          const uint2 rm = tile_rows(V, ty * tilesX + tx);
          if (maxZ > tile_min(rm)) hit = query2d_tile<false>(V, tx, ty, rm, rect[0], rect[1], rect[2], rect[3], maxZ);
        }
        found = __ballot_sync(0xFFFFFFFFu, hit) != 0;
      }
      draw = found ? 1u : 0u;
    }
  }
  if (lane == 0) P.cmdDraw[c] = draw | (nc << 1) | (first << 2);
}

// One CTA per view, one thread per chunk: chunks with a drawn command go to
// the active list (in any order: a chunk's outputs do not depend on where it
// is processed) and get their rank among the view's active chunks (chunk
// order), which indexes their totals and count-matrix columns; the others
// contribute no rows, checkpoints or list entries.
// With `gate` (views of at most kChunkGateThreads commands, no selection
// pass), the CTA first gates the view's commands itself, one per thread, in
// place of k_gate.  With `reset` (a launch of one view, so one CTA), thread 0
// resets the launch's counters in place of a memset before the launch.
constexpr uint32_t kChunkGateThreads = 1024;

__global__ void __launch_bounds__(kChunkGateThreads) k_chunk_gate(FrameParams P, uint32_t gate, uint32_t reset)
{
  __shared__ uint32_t s_scan[kChunkGateThreads / 32];
  __shared__ uint32_t s_base;
  pdl_wait();
  const uint32_t v = blockIdx.x, tid = threadIdx.x;
  const ViewDesc& V = P.views[v];
  if (reset && tid == 0) {  // before this thread's first atomic on activeChunks; the others are later kernels'
    P.header->activeChunks = 0;
    P.header->activeTiles = 0;
    P.header->tileCursor = 0;
  }
  if (gate) {
    if (tid < V.cmdCount) gate_cmd(P, V.cmdStart + tid);
    __syncthreads();  // the CTA's cmdDraw stores, visible to its threads
  }
  uint32_t n = 0;
  for (uint32_t i0 = 0; i0 < V.chunkCount; i0 += kChunkGateThreads) {
    const uint32_t i = i0 + tid, c = V.chunkStart + i;
    bool active = false;
    if (i < V.chunkCount) {
      const Chunk ch = P.chunks[c];
      for (uint32_t k = 0; k < ch.cmdCount && !active; ++k) active = (P.cmdDraw[ch.cmdFirst + k] & 1u) != 0;
    }
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan<kChunkGateThreads>(active ? 1u : 0u, tot, s_scan);
    if (tid == 0 && tot) s_base = atomicAdd(&P.header->activeChunks, tot);
    __syncthreads();
    if (active) {
      P.chunkRank[c] = n + ex;
      P.activeChunkList[s_base + ex] = c;
    }
    n += tot;
    __syncthreads();  // s_base is reused by the next round
  }
  if (tid == 0) P.viewActiveCount[v] = n;
}

// ---- k_setup -------------------------------------------------------------------------

__global__ void __launch_bounds__(kChunk) k_setup(FrameParams P)
{
  extern __shared__ uint32_t s_stCount[];
  __shared__ CmdConst s_cc[kMaxCmdPerChunk];
  __shared__ uint32_t s_cmdStart[kMaxCmdPerChunk];
  __shared__ uint32_t s_scan[kChunk / 32];
  __shared__ __align__(16) uint32_t s_words[kChunk * 4];  // the chunk's packed words (Occluder.cpp:153-156 layout)

  pdl_wait();
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const uint32_t nActive = P.header->activeChunks;
  for (uint32_t ai = blockIdx.x; ai < nActive; ai += gridDim.x) {
    const uint32_t c = P.activeChunkList[ai];
    const Chunk ch = P.chunks[c];
    const ViewDesc& V = P.views[ch.view];
    const uint32_t rank = P.chunkRank[c];
    const uint32_t nst = V.stX * V.stY;
    for (uint32_t i = tid; i < nst; i += kChunk) s_stCount[i] = 0;
    if (tid < ch.cmdCount) {
      const Cmd cmd = P.cmds[ch.cmdFirst + tid];
      const uint32_t dn = P.cmdDraw[ch.cmdFirst + tid];  // k_gate
      if (dn & 1u) cmd_prologue(V, cmd, s_cc[tid]);
      s_cc[tid].draw = dn & 1u;
      s_cc[tid].nc = dn >> 1;
      s_cmdStart[tid] = cmd.quadStart;
    }
    __syncthreads();

    // the chunk's packed words into shared memory, one coalesced 16-byte load
    // per thread: thread t loads vector t % 8 of the chunk's 8-quad group t / 8
    // (a group's 32 words are corner-major: word 8j + i is corner j of quad i).
    // A group lies in one command, the command of thread t's own quad too.
    const uint32_t g0 = (c << kChunkShift) + 8 * (tid >> 3);  // first quad of the group
    uint32_t k = 0;
    {
      uint32_t hi = ch.cmdCount - 1;  // last command starting at or before the group
      while (k < hi) {
        const uint32_t mid = (k + hi + 1) >> 1;
        if (s_cmdStart[mid] <= g0) k = mid; else hi = mid - 1;
      }
      if (8 * (tid >> 3) < ch.quadCount && s_cc[k].draw) {
        const Cmd& cmd = P.cmds[ch.cmdFirst + k];
        const uint4* src = reinterpret_cast<const uint4*>(P.pool + cmd.wordOffset + (g0 - cmd.quadStart) * 4);
        reinterpret_cast<uint4*>(s_words)[tid] = __ldg(src + (tid & 7));
      }
    }
    __syncthreads();
    const uint32_t q = (c << kChunkShift) + tid;
    QuadRaster R;
    QuadWalk Wk;
    bool valid = false;
    if (tid < ch.quadCount) {
      if (s_cc[k].draw) {
        uint32_t w4[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) w4[j] = s_words[(tid >> 3) * 32 + 8 * j + (tid & 7)];
        valid = quad_setup(V, w4, s_cc[k], R, Wk);
        Wk.pad[0] = ch.cmdFirst + k;  // command of this quad (win counts)
      }
    }
    uint32_t rows = 0, cks = 0;
    if (valid) {
      rows = (uint32_t)(R.maxY - R.minY);
      cks = rows * nck_of(R);
    } else {
      R = QuadRaster{};
      Wk = QuadWalk{};
    }
    uint32_t totRows, totCks;
    const uint32_t rowLocal = block_exclusive_scan<kChunk>(rows, totRows, s_scan);
    const uint32_t ckLocal = block_exclusive_scan<kChunk>(cks, totCks, s_scan);
    R.ckLocal = ckLocal;
    Wk.rowLocal = rowLocal;
    P.rec[q] = R;
    P.walk[q] = Wk;
    // super-tile counts, warp-aggregated: each round every lane offers its
    // next super-tile, lanes offering the same one add together (one atomic)
    {
      const uint32_t sh = V.stShift;
      const uint32_t sx0 = valid ? (uint32_t)R.minX >> sh : 0u, sx1 = valid ? (R.maxX - 1u) >> sh : 0u;
      const uint32_t sy1 = valid ? (R.maxY - 1u) >> sh : 0u;
      uint32_t sx = sx0, sy = valid ? (uint32_t)R.minY >> sh : 0u;
      bool pending = valid;
      while (__any_sync(0xFFFFFFFFu, pending)) {
        const uint32_t key = pending ? sy * V.stX + sx : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        if (pending && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&s_stCount[key], (uint32_t)__popc(peers));
        if (pending && ++sx > sx1) {
          sx = sx0;
          pending = ++sy <= sy1;
        }
      }
    }
    __syncthreads();
    for (uint32_t st = tid; st < nst; st += kChunk) P.mat[V.matBase + st * V.chunkCount + rank] = s_stCount[st];
    if (tid == 0) P.chunkTot[V.chunkStart + rank] = Totals{totRows, totCks, 0, 0};
    __syncthreads();  // shared arrays are reused by the next chunk
  }
}

// ---- k_scan ----------------------------------------------------------------------------
// CTAs [0, nst): one super-tile's chunk counts -> exclusive prefix in place, list length.
// CTAs [nst, nst + views): one view's chunk totals -> chunk bases.  The last CTA
// to finish lays the super-tile lists and the views' row/checkpoint ranges out
// back to back and checks the capacities.

// Inclusive prefix sum over the warp's lanes.
__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v, uint32_t lane)
{
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= (uint32_t)o) v += u;
  }
  return v;
}

__global__ void __launch_bounds__(256) k_scan(FrameParams P, uint32_t numSt)
{
  __shared__ uint32_t s_scan[8];
  __shared__ uint32_t s_last;
  pdl_wait();
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  // the first numViews CTAs: one view each (its chunk totals, block scans);
  // the others: one warp per super-tile (its row of the count matrix).  Few
  // CTAs in all, so that few arrive at the counter below.
  if (blockIdx.x < P.numViews) {
    const uint32_t v = blockIdx.x;
    const ViewDesc& V = P.views[v];
    const uint32_t na = V.chunkCount ? P.viewActiveCount[v] : 0u;  // active chunks, by rank
    uint32_t carryR = 0, carryC = 0;
    for (uint32_t i0 = 0; i0 < na; i0 += 256) {
      const uint32_t i = i0 + tid;
      const Totals t = i < na ? P.chunkTot[V.chunkStart + i] : Totals{0, 0, 0, 0};
      uint32_t totR, totC;
      const uint32_t exR = block_exclusive_scan<256>(t.rows, totR, s_scan);
      const uint32_t exC = block_exclusive_scan<256>(t.cks, totC, s_scan);
      if (i < na) P.chunkBase[V.chunkStart + i] = Totals{carryR + exR, carryC + exC, 0, 0};
      carryR += totR;
      carryC += totC;
    }
    if (tid == 0) P.viewTot[v] = Totals{carryR, carryC, 0, 0};
  }
  const uint32_t stride = (gridDim.x - P.numViews) * 8;
  for (uint32_t b = (blockIdx.x - P.numViews) * 8 + (tid >> 5); blockIdx.x >= P.numViews && b < numSt; b += stride) {
    uint32_t lo = 0, hi = P.numViews - 1;  // view owning super-tile b
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (P.views[mid].stBase <= b) lo = mid; else hi = mid - 1;
    }
    const ViewDesc& V = P.views[lo];
    // the row over the view's active chunks, by rank (chunk order); the other
    // entries are neither written nor read.  128 entries a step: four
    // coalesced loads in flight, then four warp scans.
    uint32_t* m = P.mat + V.matBase + (b - V.stBase) * V.chunkCount;
    const uint32_t na = V.chunkCount ? P.viewActiveCount[lo] : 0u;
    uint32_t carry = 0;
    for (uint32_t i0 = 0; i0 < na; i0 += 128) {
      uint32_t x[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t i = i0 + 32 * k + lane;
        x[k] = i < na ? m[i] : 0u;
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t i = i0 + 32 * k + lane;
        const uint32_t inc = warp_inclusive_scan(x[k], lane);
        if (i < na) m[i] = carry + inc - x[k];
        carry += __shfl_sync(0xFFFFFFFFu, inc, 31);
      }
    }
    if (lane == 0) P.stLen[b] = carry;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(&P.header->viewsDone, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // list starts: each thread sums a contiguous run of super-tiles, one block
  // scan of the run totals, then each thread writes its run's prefixes
  const uint32_t per = (numSt + 255) / 256, a0 = ::min(numSt, tid * per), a1 = ::min(numSt, a0 + per);
  uint32_t run = 0;
  for (uint32_t i = a0; i < a1; ++i) run += __ldcg(&P.stLen[i]);
  uint32_t carry;
  uint32_t pre = block_exclusive_scan<256>(run, carry, s_scan);
  for (uint32_t i = a0; i < a1; ++i) {
    P.stStart[i] = pre;
    pre += __ldcg(&P.stLen[i]);
  }
  uint32_t carryR = 0, carryC = 0;
  for (uint32_t i0 = 0; i0 < P.numViews; i0 += 256) {
    const uint32_t i = i0 + tid;
    Totals t = Totals{0, 0, 0, 0};
    if (i < P.numViews) {
      t.rows = __ldcg(&P.viewTot[i].rows);
      t.cks = __ldcg(&P.viewTot[i].cks);
    }
    uint32_t totR, totC;
    const uint32_t exR = block_exclusive_scan<256>(t.rows, totR, s_scan);
    const uint32_t exC = block_exclusive_scan<256>(t.cks, totC, s_scan);
    if (i < P.numViews) P.viewBase[i] = Totals{carryR + exR, carryC + exC, 0, 0};
    carryR += totR;
    carryC += totC;
  }
  if (tid == 0) {
    FrameHeader* H = P.header;
    H->totalRows = carryR;
    H->totalCks = carryC;
    H->totalSt = carry;
    H->overflow = (carryC > H->capCks ? 1u : 0u) | (carry > H->capSt ? 2u : 0u);
    H->sticky |= H->overflow;
    H->maxCks = ::max(H->maxCks, carryC);
    H->maxSt = ::max(H->maxSt, carry);
    H->viewsDone = 0;
  }
}

// ---- k_fill -------------------------------------------------------------------------

__global__ void __launch_bounds__(kChunk) k_fill(FrameParams P)
{
  extern __shared__ uint32_t s_dyn[];  // per union super-tile: 8 warp ballots + 8 warp prefixes
  __shared__ uint32_t s_rowLocal[kChunk];
  __shared__ int s_rect[4];
  pdl_wait();
  if (P.header->overflow) return;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t nActive = P.header->activeChunks;
  for (uint32_t ai = blockIdx.x; ai < nActive; ai += gridDim.x) {
    const uint32_t c = P.activeChunkList[ai];
    const Chunk ch = P.chunks[c];
    const ViewDesc& V = P.views[ch.view];
    const uint32_t rank = P.chunkRank[c];
    const uint32_t q = (c << kChunkShift) + tid;
    const QuadRaster R = P.rec[q];
    const bool valid = tid < ch.quadCount && R.minX < R.maxX;
    const Totals cb = P.chunkBase[V.chunkStart + rank];
    const uint32_t ckChunk = P.viewBase[ch.view].cks + cb.cks;
    if (valid) P.ckBase[q] = ckChunk + R.ckLocal;
    s_rowLocal[tid] = P.walk[q].rowLocal;  // this thread's quad only
    if (tid == 0) {
      s_rect[0] = 1 << 30; s_rect[1] = -1; s_rect[2] = 1 << 30; s_rect[3] = -1;
    }
    __syncthreads();
    int sx0 = 0, sx1 = -1, sy0 = 0, sy1 = -1;
    if (valid) {
      sx0 = (int)((uint32_t)R.minX >> V.stShift); sx1 = (int)((uint32_t)(R.maxX - 1) >> V.stShift);
      sy0 = (int)((uint32_t)R.minY >> V.stShift); sy1 = (int)((uint32_t)(R.maxY - 1) >> V.stShift);
      atomicMin(&s_rect[0], sx0); atomicMax(&s_rect[1], sx1);
      atomicMin(&s_rect[2], sy0); atomicMax(&s_rect[3], sy1);
    }
    __syncthreads();
    // super-tile lists in submission order: per super-tile of the chunk's union
    // rectangle, one ballot per warp, then a prefix over the 8 warps
    const int ux0 = s_rect[0], ux1 = s_rect[1], uy0 = s_rect[2], uy1 = s_rect[3];
    const int uw = ux1 - ux0 + 1;
    const int nu = ux1 >= ux0 ? uw * (uy1 - uy0 + 1) : 0;
    uint32_t* s_bal = s_dyn;                    // [nu][8]
    uint32_t* s_pre = s_dyn + (size_t)nu * 8;   // [nu][8]
    for (int u = 0; u < nu; ++u) {
      const int sx = ux0 + u % uw, sy = uy0 + u / uw;
      const bool flag = valid && sx >= sx0 && sx <= sx1 && sy >= sy0 && sy <= sy1;
      const uint32_t bal = __ballot_sync(0xFFFFFFFFu, flag);
      if (lane == 0) s_bal[u * 8 + warp] = bal;
    }
    __syncthreads();
    for (int u = tid; u < nu; u += kChunk) {
      // the chunk's first entry in super-tile u's list (one load latency for
      // all of them), plus the warps before
      const uint32_t st = (uint32_t)(uy0 + u / uw) * V.stX + (uint32_t)(ux0 + u % uw);
      uint32_t acc = P.stStart[V.stBase + st] + P.mat[V.matBase + st * V.chunkCount + rank];
#pragma unroll
      for (int w = 0; w < 8; ++w) {
        s_pre[u * 8 + w] = acc;
        acc += __popc(s_bal[u * 8 + w]);
      }
    }
    __syncthreads();
    if (valid) {
      const uint32_t lt = (1u << lane) - 1u;
      const uint4 entry = make_uint4(q, (uint32_t)R.minX | ((uint32_t)R.minY << 16),
                                     (uint32_t)R.maxX | ((uint32_t)R.maxY << 16), (uint32_t)R.maxZ);
      for (int sy = sy0; sy <= sy1; ++sy)
        for (int sx = sx0; sx <= sx1; ++sx) {
          const int u = (sy - uy0) * uw + (sx - ux0);
          P.stList[s_pre[u * 8 + warp] + __popc(s_bal[u * 8 + warp] & lt)] = entry;
        }
    }
    // rows of this chunk's quads -> (quad, row) entries for the row walk
    if (valid) {
      const uint32_t rowG = P.viewBase[ch.view].rows + cb.rows + s_rowLocal[tid];
      const uint32_t rows = (uint32_t)(R.maxY - R.minY);
      for (uint32_t i = 0; i < rows; ++i) P.rowOwner[rowG + i] = make_uint2(q, i);
    }
    __syncthreads();  // shared arrays are reused by the next chunk
  }
}

// ---- row walk (k_walk_prep) -------------------------------------------------------------
// One thread per (quad, block row) of the whole batch: the reference's
// incremental adds along the row (Rasterizer.cpp:1125-1146), storing the edge
// offsets and depth lanes at the quad's first column and every 8 block columns.

// Plain IEEE add where the quad's depth cannot overflow (x86-exact there),
// else the x86 rules; chosen per quad, outside the inner loops.
template <bool kSafe>
__device__ __forceinline__ float zadd(float a, float b)
{
  return kSafe ? x86::radd(a, b) : x86::xadd(a, b);
}
template <bool kSafe>
__device__ __forceinline__ float zfma(float a, float b, float c)
{
  return kSafe ? x86::rfma(a, b, c) : x86::xfmadd(a, b, c);
}

template <bool kSafe>
__device__ __forceinline__ void walk_row(const FrameParams& P, const QuadRaster& Q, const QuadWalk& Wk, uint32_t qq,
                                         uint32_t r)
{
  const float dsp = -0.4375f;  // -0.5f + 1.0f / 16.0f
  float depth[8], off[4];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float lx = dsp + 0.125f * (float)(k & 3);
    const float ly = dsp + 0.125f * (float)(k >> 2);
    depth[k] = x86::xfmadd(Q.Dx, lx, x86::xfmadd(Q.Dy, ly, Wk.plane0));
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) off[e] = Wk.off[e];
  for (uint32_t i = 0; i < r; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) depth[k] = zadd<kSafe>(depth[k], Q.Dy);
#pragma unroll
    for (int e = 0; e < 4; ++e) off[e] = x86::radd(off[e], Wk.ny[e]);
  }
  const uint32_t nck = nck_of(Q);
  float4* out = reinterpret_cast<float4*>(P.ck + (size_t)kCkFloats * (P.ckBase[qq] + r * nck));
  const uint32_t lastCk = ::max((uint32_t)Q.minX, (uint32_t)(Q.maxX - 1) & ~7u);
  for (uint32_t bx = Q.minX;; ++bx) {
    if (bx == Q.minX || (bx & 7u) == 0) {
      out[0] = make_float4(off[0], off[1], off[2], off[3]);
      out[1] = make_float4(depth[0], depth[1], depth[2], depth[3]);
      out[2] = make_float4(depth[4], depth[5], depth[6], depth[7]);
      out += 3;
    }
    if (bx == lastCk) break;
#pragma unroll
    for (int k = 0; k < 8; ++k) depth[k] = zadd<kSafe>(Q.Dx, depth[k]);
#pragma unroll
    for (int e = 0; e < 4; ++e) off[e] = x86::radd(Q.nx[e], off[e]);
  }
}

// The row walk's part of k_walk_prep: CTA `cta` of `ctas`, 256 threads,
// grid-striding over the batch's rows.
__device__ __forceinline__ void walk_rows(const FrameParams& P, uint32_t cta, uint32_t ctas)
{
  const uint32_t total = P.header->totalRows;
  for (uint32_t row = cta * 256 + threadIdx.x; row < total; row += ctas * 256) {
    const uint2 own = P.rowOwner[row];
    const QuadRaster Q = P.rec[own.x];
    const QuadWalk Wk = P.walk[own.x];
    if (Q.flags & kQuadSafe) walk_row<true>(P, Q, Wk, own.x, own.y);
    else walk_row<false>(P, Q, Wk, own.x, own.y);
  }
}

// ---- k_raster ------------------------------------------------------------------------
//
// Persistent warps, each on its own: a warp takes a queued raster unit of
// 8 x R blocks (R = 1, 2 or 4 block rows of an 8x4-block warp-tile) from the
// global queue, walks the unit's super-tile quad list in order, keeps the
// quads that overlap the unit and are not already hidden in an ordered local
// list, and turns them into (quad, block) fragments, 32 at a time: every lane
// computes one fragment (coverage mask, packed depth rows) into its slot in the
// warp's shared memory, then each block's lanes merge the fragments aimed at
// the block in list order with the reference's hiZ test, fast-clear overwrite
// and max-merge (Rasterizer.cpp:1148-1290).  A block is held by 32 / (8 R)
// lanes, each with 2 R of its pixel rows in registers.  Only warp-level
// synchronisation is used: units are latency chains (record loads, fragment
// arithmetic, the ordered merge), and up to 32 warps per SM overlap as many.

template <int R>
struct UnitShape {
  static constexpr int kBlocks = 8 * R;                  // blocks per unit
  static constexpr int kLanesPerBlock = 32 / kBlocks;    // 4, 2, 1
  static constexpr int kRowsPerLane = 8 / kLanesPerBlock;  // 2, 4, 8
};

constexpr int kRasterWarps = 4;                    // warps per CTA (they share nothing)
// resident CTAs per SM the register budget is sized for: 80 registers a
// thread at 1 or 2 block rows (no spills of the merge state), 128 at 4
template <int R>
constexpr int kRasterMinBlocks = R == 4 ? 4 : 6;
constexpr int kRasterThreads = 32 * kRasterWarps;
constexpr int kWarpListCap = 64;                   // listed quads buffered per warp
constexpr int kFragStride = 36;                    // words per fragment slot: rows move as 16-byte words

struct WarpRasterSmem {
  __align__(16) uint32_t frag[32 * kFragStride];  // one fragment slot per lane: 8 rows x 4 packed words
  uint32_t meta[32];                // per slot: maxZ << 16 | target block
  uint32_t fcmd[32];                // per slot: command within the view + 1 (win counting)
  uint32_t bmask[32];               // per block: slots aimed at it
  uint32_t hiz[32];                 // per block: current hiZ
  uint32_t lq[kWarpListCap];        // listed quad
  uint32_t lrect[kWarpListCap];     // its rectangle in the unit: x0 | y0 << 3 | w << 5 | h << 9
  uint32_t loff[kWarpListCap];      // its first fragment
};

// Row y of a fragment, masked by the coverage mask, into its slot.
__device__ __forceinline__ void put_row(uint32_t* dst, int y, uint64_t mask, uint32_t w0, uint32_t w1, uint32_t w2,
                                        uint32_t w3)
{
  if (mask != ~0ull) {
    const int bitpos = (y & 1) ? (y >> 1) : 4 + (y >> 1);
    const uint64_t bits = (mask >> bitpos) & 0x0101010101010101ull;
    const uint32_t lo = (uint32_t)bits * 0xFFu, hi = (uint32_t)(bits >> 32) * 0xFFu;
    w0 &= __byte_perm(lo, 0, 0x1100);
    w1 &= __byte_perm(lo, 0, 0x3322);
    w2 &= __byte_perm(hi, 0, 0x1100);
    w3 &= __byte_perm(hi, 0, 0x3322);
  }
  *reinterpret_cast<uint4*>(dst + 4 * y) = make_uint4(w0, w1, w2, w3);
}

// Fragment of quad Q at block (bx, by): packed depth rows with the coverage
// mask applied, written to dst.  Returns false if the reference would skip
// the block (convex quad outside the offset range, or an empty mask).
template <bool kSafe>
__device__ __forceinline__ bool make_fragment_t(const FrameParams& P, const QuadRaster& Q, uint32_t ckq,
                                                uint32_t bx, uint32_t by, uint32_t tx0, uint32_t* dst)
{
  const uint32_t cx = ::max((uint32_t)Q.minX, tx0);
  const uint32_t kk = (cx >> 3) - ((uint32_t)Q.minX >> 3);
  const uint32_t ckIdx = ckq + (by - Q.minY) * nck_of(Q) + kk;
  const float4* ck = reinterpret_cast<const float4*>(P.ck + (size_t)kCkFloats * ckIdx);
  const float4 o = __ldg(ck), d0 = __ldg(ck + 1), d1 = __ldg(ck + 2);
  float off[4] = {o.x, o.y, o.z, o.w};
  float depth[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
  for (uint32_t i = cx; i < bx; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) depth[k] = zadd<kSafe>(Q.Dx, depth[k]);
#pragma unroll
    for (int e = 0; e < 4; ++e) off[e] = x86::radd(Q.nx[e], off[e]);
  }
  uint64_t mask;
  if (Q.mode == kModeConvex) {
    if (off[0] >= kCkRange || off[1] >= kCkRange || off[2] >= kCkRange || off[3] >= kCkRange) return false;
    mask = ~0ull;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      int32_t oi = x86::cvtt(off[e]);
      oi = oi < 0 ? 0 : oi;
      mask &= __ldg(&kDevCoverage[(Q.slope[e] | (uint32_t)oi) & 4095u]);
    }
  } else {
    uint64_t L[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      int32_t oi = x86::cvtt(off[e]);
      oi = oi < 0 ? 0 : (oi > 63 ? 63 : oi);
      L[e] = __ldg(&kDevCoverage[(Q.slope[e] | (uint32_t)oi) & 4095u]);
    }
    switch (Q.mode) {
      case kModeTriangle0: mask = L[0] & L[1] & L[2]; break;
      case kModeTriangle1: mask = L[0] & L[2] & L[3]; break;
      case kModeConcaveRight: mask = (L[0] | L[3]) & (L[1] & L[2]); break;
      case kModeConcaveCenter:
        mask = (Q.flags & kQuadNearClip) ? ((L[0] & L[1]) | (L[2] & L[3])) : ((L[0] & L[3]) & (L[1] | L[2]));
        break;
      default: mask = (L[0] & L[3]) & (L[1] | L[2]); break;
    }
    if (!mask) return false;
  }
  // depth rows (Rasterizer.cpp:1241-1268): rows 0/1 from (depth, d1), rows 8/9
  // from (d8, d9), rows 2-7 by rounding averages of packed values; rows are
  // written to the slot as soon as they are known, to keep few registers live
  const float Dx = Q.Dx, Dy = Q.Dy;
  uint32_t r0[4], r1[4], r8[4], r9[4];
#pragma unroll
  for (int h = 0; h < 2; ++h) {  // depth lanes 0-3 give rows 0 and 8, lanes 4-7 rows 1 and 9
    float a[4], b[4], c[4], e[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a[k] = depth[4 * h + k];
      b[k] = zfma<kSafe>(Dx, 0.5f, a[k]);
      c[k] = zadd<kSafe>(Dy, a[k]);
      e[k] = zadd<kSafe>(Dy, b[k]);
    }
    uint32_t* ra = h ? r1 : r0;
    uint32_t* rb = h ? r9 : r8;
    ra[0] = pack2(a[0], a[1]); ra[1] = pack2(a[2], a[3]); ra[2] = pack2(b[0], b[1]); ra[3] = pack2(b[2], b[3]);
    rb[0] = pack2(c[0], c[1]); rb[1] = pack2(c[2], c[3]); rb[2] = pack2(e[0], e[1]); rb[3] = pack2(e[2], e[3]);
  }
  uint32_t r4[4], r5[4];
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    r4[w] = avg_u16x2(r0[w], r8[w]);
    r5[w] = avg_u16x2(r1[w], r9[w]);
  }
  put_row(dst, 2, mask, avg_u16x2(r0[0], r4[0]), avg_u16x2(r0[1], r4[1]), avg_u16x2(r0[2], r4[2]),
          avg_u16x2(r0[3], r4[3]));
  put_row(dst, 3, mask, avg_u16x2(r1[0], r5[0]), avg_u16x2(r1[1], r5[1]), avg_u16x2(r1[2], r5[2]),
          avg_u16x2(r1[3], r5[3]));
  put_row(dst, 0, mask, r0[0], r0[1], r0[2], r0[3]);
  put_row(dst, 1, mask, r1[0], r1[1], r1[2], r1[3]);
  put_row(dst, 6, mask, avg_u16x2(r4[0], r8[0]), avg_u16x2(r4[1], r8[1]), avg_u16x2(r4[2], r8[2]),
          avg_u16x2(r4[3], r8[3]));
  put_row(dst, 7, mask, avg_u16x2(r5[0], r9[0]), avg_u16x2(r5[1], r9[1]), avg_u16x2(r5[2], r9[2]),
          avg_u16x2(r5[3], r9[3]));
  put_row(dst, 4, mask, r4[0], r4[1], r4[2], r4[3]);
  put_row(dst, 5, mask, r5[0], r5[1], r5[2], r5[3]);
  return true;
}

// Computes the fragment and, if the reference would draw it, stores its 8
// rows of 4 packed words at dst (a fragment slot in shared memory).
template <bool kSafe>
__device__ __forceinline__ bool fragment_to(const FrameParams& P, const QuadRaster& Q, uint32_t ckq, uint32_t bx,
                                            uint32_t by, uint32_t tx0, uint32_t* dst)
{
  return make_fragment_t<kSafe>(P, Q, ckq, bx, by, tx0, dst);
}

// Quads whose depth may overflow are rare: their copy stays out of line so
// that the common path keeps its registers.  It reloads quad q's record
// itself: a record passed by reference would have to live in local memory
// on every path.
static __device__ __noinline__ bool fragment_to_unsafe(const FrameParams& P, uint32_t q, uint32_t ckq, uint32_t bx,
                                                       uint32_t by, uint32_t tx0, uint32_t* dst)
{
  const QuadRaster Q = P.rec[q];
  return fragment_to<false>(P, Q, ckq, bx, by, tx0, dst);
}

__device__ __forceinline__ bool make_fragment(const FrameParams& P, const QuadRaster& Q, uint32_t q, uint32_t ckq,
                                              uint32_t bx, uint32_t by, uint32_t tx0, uint32_t* dst)
{
  if (Q.flags & kQuadSafe) return fragment_to<true>(P, Q, ckq, bx, by, tx0, dst);
  return fragment_to_unsafe(P, q, ckq, bx, by, tx0, dst);
}

// Merges fragment slot `slot` into this lane's RPL pixel rows (from row0) of
// its block: the reference's hiZ test, fast-clear overwrite or max-merge with
// memory, and the block's new hiZ (minimum over the block's lanes,
// `groupMask`).  With kWins, own[r][i] holds the owners (command within the
// view + 1, or 0) of pixels 2i and 2i+1 of row r as two 16-bit halves.
template <int RPL, int LPB, bool kWins>
__device__ __forceinline__ void merge_slot(const ViewDesc& V, const WarpRasterSmem& S, uint32_t slot, uint32_t row0,
                                           uint32_t blk, uint32_t groupMask, uint32_t (&row)[RPL][4], uint32_t& hiz,
                                           bool& have, uint32_t (&own)[RPL][4])
{
  const uint32_t mz = S.meta[slot] >> 16;
  if (hiz >= mz) return;  // the reference's hiZ test (Rasterizer.cpp:1148-1152)
  const uint4* src = reinterpret_cast<const uint4*>(S.frag + slot * kFragStride + 4 * row0);
  const uint32_t c1 = kWins ? S.fcmd[slot] : 0u;
  if (hiz == 1) {
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const uint4 q = src[r];
      const uint32_t wr[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t w = wr[i];
        if (kWins) own[r][i] = ((w & 0xFFFFu) ? c1 : 0u) | ((w >> 16) ? (c1 << 16) : 0u);
        row[r][i] = w;
      }
    }
  } else {
    if (!have) {
      const uint4* d = reinterpret_cast<const uint4*>(V.depth + (size_t)blk * 64 + 8 * row0);
#pragma unroll
      for (int r = 0; r < RPL; ++r) {
        const uint4 a = d[r];
        row[r][0] = a.x; row[r][1] = a.y; row[r][2] = a.z; row[r][3] = a.w;
      }
    }
#pragma unroll
    for (int r = 0; r < RPL; ++r) {
      const uint4 q = src[r];
      const uint32_t wr[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t w = wr[i];
        if (kWins) {
          if ((w & 0xFFFFu) > (row[r][i] & 0xFFFFu)) own[r][i] = (own[r][i] & 0xFFFF0000u) | c1;
          if ((w >> 16) > (row[r][i] >> 16)) own[r][i] = (own[r][i] & 0xFFFFu) | (c1 << 16);
        }
        row[r][i] = vmax_u16x2(row[r][i], w);
      }
    }
  }
  have = true;
  uint32_t mn = 0xFFFFFFFFu;
#pragma unroll
  for (int r = 0; r < RPL; ++r) mn = vmin_u16x2(mn, vmin_u16x2(vmin_u16x2(row[r][0], row[r][1]), vmin_u16x2(row[r][2], row[r][3])));
#pragma unroll
  for (int o = 1; o < LPB; o <<= 1) mn = vmin_u16x2(mn, __shfl_xor_sync(groupMask, mn, o));
  hiz = ::min(mn & 0xFFFFu, mn >> 16);
}

// Per-lane state of one raster unit.
template <int R>
struct UnitState {
  static constexpr int RPL = UnitShape<R>::kRowsPerLane;
  uint32_t tx0, ty0, myBlock, row0, blk, groupMask, hiz;
  bool inView, have;
  uint32_t row[RPL][4];
  uint32_t own[RPL][4];
};

// Runs the buffered local list (n quads, F fragments) 32 fragments at a time.
template <int R, bool kWins>
__device__ __forceinline__ void raster_list(const FrameParams& P, const ViewDesc& V, WarpRasterSmem& S, uint32_t n,
                                            uint32_t F, uint32_t lane, UnitState<R>& U)
{
  using Sh = UnitShape<R>;
  for (uint32_t f0 = 0; f0 < F; f0 += 32) {
    const uint32_t f = f0 + lane;
    uint32_t meta = 0, target = 0;
    bool valid = false;
    if (f < F) {
      uint32_t lo = 0, hi = n - 1;  // last local quad whose first fragment is <= f
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (S.loff[mid] <= f) lo = mid; else hi = mid - 1;
      }
      const uint32_t k = f - S.loff[lo];
      const uint32_t rc = S.lrect[lo];
      const uint32_t rw = (rc >> 5) & 15u;
      const uint32_t rr = k / rw, cc = k - rr * rw;
      const uint32_t lx = (rc & 7u) + cc, ly = ((rc >> 3) & 3u) + rr;
      target = ly * kTileW + lx;
      const uint32_t q = S.lq[lo];
      const QuadRaster Q = P.rec[q];
      const uint32_t ckq = __ldg(P.ckBase + q);
      const uint32_t ownerHiz = S.hiz[target];
      // Early skip: hiZ only falls through the fast-clear overwrite (1 -> 0),
      // so a block with hiZ >= maxZ now still has it when this fragment's
      // turn comes, unless hiZ == 1 and maxZ == 1.
      const bool skip = ownerHiz >= Q.maxZ && !(ownerHiz == 1 && Q.maxZ == 1);
      if (!skip && make_fragment(P, Q, q, ckq, U.tx0 + lx, U.ty0 + ly, U.tx0, S.frag + lane * kFragStride)) {
        valid = true;
        meta = ((uint32_t)Q.maxZ << 16) | target;
        if (kWins) S.fcmd[lane] = P.walk[q].pad[0] - V.cmdStart + 1u;
      }
    }
    S.meta[lane] = meta;
    // slots aimed at each block: lanes with the same target form one group
    const uint32_t grp = __match_any_sync(0xFFFFFFFFu, valid ? target : 64u + lane);
    if (lane < (uint32_t)Sh::kBlocks) S.bmask[lane] = 0;
    __syncwarp();
    if (valid) S.bmask[target] = grp;
    __syncwarp();
    // merge, in slot order, the fragments aimed at this lane's block
    uint32_t mine = U.inView ? S.bmask[U.myBlock] : 0u;
    while (mine) {
      const uint32_t slot = __ffs(mine) - 1;
      mine &= mine - 1;
      merge_slot<Sh::kRowsPerLane, Sh::kLanesPerBlock, kWins>(V, S, slot, U.row0, U.blk, U.groupMask, U.row, U.hiz,
                                                              U.have, U.own);
    }
    if (U.row0 == 0) S.hiz[U.myBlock] = U.hiz;
    __syncwarp();
  }
}

// Pixels of one lane whose owners differ: runs of equal owners along the
// lane's n pixel pairs (own: 16-bit owner halves), one atomic per run.  Out
// of line: rare, and kept out of the kernel's hot instruction stream.
static __device__ __noinline__ void add_win_runs(uint32_t* wins, uint32_t cmdStart, const uint32_t* own, int n)
{
  uint32_t cur = 0, cnt = 0;
  for (int i = 0; i < 2 * n; ++i) {
    const uint32_t k = (own[i >> 1] >> (16 * (i & 1))) & 0xFFFFu;
    if (k != cur) {
      if (cur) atomicAdd(&wins[cmdStart + cur - 1], cnt);
      cur = k;
      cnt = 0;
    }
    ++cnt;
  }
  if (cur) atomicAdd(&wins[cmdStart + cur - 1], cnt);
}

// Per-pixel owners (global command + 1, or 0) of one lane's rows: all of them
// (the first pass) or the pixels this pass changed (the second pass).
static __device__ __noinline__ void write_owners(uint32_t* o, uint32_t cmdStart, const uint32_t* own, int rows,
                                                 bool all)
{
  for (int i = 0; i < 8 * rows; ++i) {
    const uint32_t k = (own[i >> 1] >> (16 * (i & 1))) & 0xFFFFu;
    if (all || k) o[i] = k ? cmdStart + k : 0u;
  }
}

// Adds the pixels this lane's rows won to their commands (wins) and writes
// the per-pixel owners.  A pixel is won by the command whose fragment set its
// final value (the fast-clear overwrite or a strictly larger max-merge).
template <int R>
__device__ __forceinline__ void count_wins(const FrameParams& P, const ViewDesc& V, const UnitState<R>& U,
                                           uint32_t lane)
{
  constexpr int RPL = UnitShape<R>::kRowsPerLane;
  const uint32_t k0 = U.own[0][0] & 0xFFFFu;
  bool same = true;
#pragma unroll
  for (int r = 0; r < RPL; ++r)
#pragma unroll
    for (int i = 0; i < 4; ++i) same &= U.own[r][i] == (k0 | (k0 << 16));
  if (__all_sync(0xFFFFFFFFu, same)) {
    // every lane's rows won by one command (the common case): one atomic per command
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, k0);
    if (k0 && lane == (uint32_t)(__ffs(peers) - 1))
      atomicAdd(&P.wins[V.cmdStart + k0 - 1], 8u * RPL * (uint32_t)__popc(peers));
  } else if (!same || (V.owner && U.inView)) {
    // a copy in local memory for the out-of-line paths (U.own stays in registers)
    uint32_t own[4 * RPL];
#pragma unroll
    for (int r = 0; r < RPL; ++r)
#pragma unroll
      for (int i = 0; i < 4; ++i) own[4 * r + i] = U.own[r][i];
    if (!same) add_win_runs(P.wins, V.cmdStart, own, 4 * RPL);
    else if (k0) atomicAdd(&P.wins[V.cmdStart + k0 - 1], 8u * RPL);
    if (V.owner && U.inView)
      write_owners(V.owner + (size_t)U.blk * 64 + 8 * U.row0, V.cmdStart, own, RPL, P.phase == 0);
  } else if (k0) {
    atomicAdd(&P.wins[V.cmdStart + k0 - 1], 8u * RPL);
  }
}

// One raster unit: queue record {warp-tile * 4 + first block row, view,
// first entry and length of the unit's super-tile list}.
template <int R, bool kWins>
__device__ __forceinline__ void raster_unit(const FrameParams& P, WarpRasterSmem& S, const uint4 rec, uint32_t lane)
{
  using Sh = UnitShape<R>;
  constexpr int RPL = Sh::kRowsPerLane, LPB = Sh::kLanesPerBlock;
  const ViewDesc& V = P.views[rec.y];
  UnitState<R> U;
  const uint32_t lt = (rec.x >> 2) - V.tileStart;
  U.tx0 = (lt % V.tilesX) * kTileW;
  U.ty0 = (lt / V.tilesX) * kTileH + (rec.x & 3u);
  U.myBlock = lane / LPB;
  U.row0 = (lane % LPB) * RPL;
  const uint32_t bx = U.tx0 + (U.myBlock & 7u), by = U.ty0 + (U.myBlock >> 3);
  U.inView = bx < V.blocksX && by < V.blocksY;
  U.blk = U.inView ? by * V.blocksX + bx : 0u;
  U.groupMask = LPB == 1 ? (1u << lane) : (((1u << LPB) - 1u) << (lane & ~(uint32_t)(LPB - 1)));
  const bool clearing = (V.flags & kViewClear) != 0 && P.phase == 0;
  U.hiz = clearing ? 1u : (U.inView ? (uint32_t)V.hiz[U.blk] : 0xFFFFu);
  U.have = false;
#pragma unroll
  for (int r = 0; r < RPL; ++r)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      U.row[r][i] = 0;
      U.own[r][i] = 0;
    }
  if (U.row0 == 0) S.hiz[U.myBlock] = U.hiz;
  __syncwarp();
  const uint32_t listLen = rec.w;
  const uint4* list = P.stList + rec.z;
  const uint32_t below = (1u << lane) - 1u;
  uint32_t n = 0, F = 0;
  // 32 list entries per round, one per lane, appended to the local list in
  // list order unless they miss the unit or are already hidden in every
  // block they touch here
#pragma unroll 1
  for (uint32_t base = 0; base < listLen; base += 32) {
    const uint4 e = base + lane < listLen ? __ldg(list + base + lane) : make_uint4(0, 0, 0, 0);
    const uint32_t qx0 = e.y & 0xFFFFu, qy0 = e.y >> 16, qx1 = e.z & 0xFFFFu, qy1 = e.z >> 16;
    const uint32_t x0 = ::max(qx0, U.tx0), x1 = ::min(qx1, U.tx0 + kTileW);
    const uint32_t y0 = ::max(qy0, U.ty0), y1 = ::min(qy1, U.ty0 + R);
    bool o = x0 < x1 && y0 < y1;  // padding entries have an empty box
    if (o) {
      // hidden if every block it touches here already has hiZ >= its maxZ
      // (exact for the rest of the list: see raster_list)
      const uint32_t mz = e.w;
      bool hidden = true;
      for (uint32_t yy = y0 - U.ty0; yy < y1 - U.ty0 && hidden; ++yy)
        for (uint32_t xx = x0 - U.tx0; xx < x1 - U.tx0; ++xx) {
          const uint32_t h = S.hiz[yy * kTileW + xx];
          if (!(h >= mz && !(h == 1 && mz == 1))) {
            hidden = false;
            break;
          }
        }
      o = !hidden;
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, o);
    if (!bal) continue;
    const uint32_t nf = o ? (x1 - x0) * (y1 - y0) : 0u;
    const uint32_t incl = warp_inclusive_scan(nf, lane);
    if (o) {
      const uint32_t pos = n + __popc(bal & below);
      S.lq[pos] = e.x;
      S.lrect[pos] = (x0 - U.tx0) | ((y0 - U.ty0) << 3) | ((x1 - x0) << 5) | ((y1 - y0) << 9);
      S.loff[pos] = F + incl - nf;
    }
    n += __popc(bal);
    F += __shfl_sync(0xFFFFFFFFu, incl, 31);
    __syncwarp();
    if (n > (uint32_t)(kWarpListCap - 32)) {  // the next round may append 32
      raster_list<R, kWins>(P, V, S, n, F, lane, U);
      n = 0;
      F = 0;
    }
  }
  if (n > 0) raster_list<R, kWins>(P, V, S, n, F, lane, U);
  if (U.inView) {
    if ((clearing || U.have) && U.row0 == 0) V.hiz[U.blk] = (uint16_t)U.hiz;
    uint4* d = reinterpret_cast<uint4*>(V.depth + (size_t)U.blk * 64 + 8 * U.row0);
    if (U.have) {
#pragma unroll
      for (int r = 0; r < RPL; ++r) d[r] = make_uint4(U.row[r][0], U.row[r][1], U.row[r][2], U.row[r][3]);
    } else if (clearing && (V.flags & kViewZeroDepth)) {
#pragma unroll
      for (int r = 0; r < RPL; ++r) d[r] = make_uint4(0, 0, 0, 0);
    }
  }
  // the unit's block rows' minimum hiZ (its lanes are block-major, 8 R blocks)
  {
    uint32_t h = U.inView ? U.hiz : 0xFFFFu;
#pragma unroll
    for (int o = 1; o < 32 / R; o <<= 1) h = ::min(h, __shfl_xor_sync(0xFFFFFFFFu, h, o));
    if (lane % (32 / R) == 0) V.tileHiz[4 * (size_t)lt + (rec.x & 3u) + lane / (32 / R)] = (uint16_t)h;
  }
  if (kWins) count_wins<R>(P, V, U, lane);
}

// ---- tile preparation (k_walk_prep) --------------------------------------------------
// One warp per warp-tile (8x4 blocks, one lane per block): applies the view's
// clear (hiZ := 1, Rasterizer.cpp:107-121) to every block, then either queues
// the tile's raster units of R block rows for the raster kernel (a quad of
// its super-tile list reaches the unit; long lists are not checked) or
// finishes them here: no quad touches them, so their hiZ is final (and with
// kViewZeroDepth their depth is zeroed).  The block rows of the unqueued
// units get their minimum hiZ here, the others from their raster unit.

__device__ __forceinline__ uint32_t view_of_tile(const FrameParams& P, uint32_t wt)
{
  uint32_t lo = 0, hi = P.numViews - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (P.views[mid].tileStart <= wt) lo = mid; else hi = mid - 1;
  }
  return lo;
}

constexpr uint32_t kPrepScanMax = 256;  // lists up to this length are checked against the tile

__device__ __forceinline__ uint32_t raster_rows(const FrameParams& P)
{
  return P.tune.rasterRows ? P.tune.rasterRows : kDefaultRasterRows;
}

// Per-row minima of a warp-tile from one warp: `h` is this lane's block hiZ
// (lane = row * 8 + column; 0xFFFF outside the view), rows `rows` (bit r =
// row r) are stored.
__device__ __forceinline__ void store_tile_rows(const ViewDesc& V, uint32_t lt, uint32_t h, uint32_t rows,
                                                uint32_t lane)
{
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) h = ::min(h, __shfl_xor_sync(0xFFFFFFFFu, h, o));
  const uint32_t r = lane >> 3;
  if ((lane & 7u) == 0 && ((rows >> r) & 1u)) V.tileHiz[4 * (size_t)lt + r] = (uint16_t)h;
}

// CTA `cta` of the tile preparation: warps over warp-tiles cta * 8 ...
__device__ __forceinline__ void tile_prep(const FrameParams& P, uint32_t cta)
{
  __shared__ uint32_t s_n, s_base;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t wt = cta * 8 + warp;
  const uint32_t R = raster_rows(P), units = kTileH / R, all = (1u << units) - 1u;
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  uint32_t queue = 0, slot = 0, v = 0;  // queue: bit u = raster unit u of the tile
  uint32_t listStart = 0, listLen = 0;
  if (wt < P.numTiles) {
    v = view_of_tile(P, wt);
    const ViewDesc& V = P.views[v];
    const uint32_t lt = wt - V.tileStart;
    const uint32_t tx0 = (lt % V.tilesX) * kTileW, ty0 = (lt / V.tilesX) * kTileH;
    const uint32_t bx = tx0 + (lane & 7), by = ty0 + (lane >> 3);
    const bool inView = bx < V.blocksX && by < V.blocksY;
    const uint32_t blk = inView ? by * V.blocksX + bx : 0;
    const bool clearing = (V.flags & kViewClear) != 0 && P.phase == 0;
    if (clearing) {
      if (inView) V.hiz[blk] = 1;
      if (lt == 0 && lane < 8) V.hiz[V.blocksX * V.blocksY + lane] = 1;  // padding entries
    }
    const uint32_t s = V.stBase + (ty0 >> V.stShift) * V.stX + (tx0 >> V.stShift);
    const uint32_t len = V.cmdCount ? P.stLen[s] : 0u;
    listLen = len;
    listStart = len ? P.stStart[s] : 0u;
    if (len > kPrepScanMax) {
      queue = all;
    } else if (len) {
      // queue a unit only if a quad of the super-tile list reaches it
      const uint4* list = P.stList + P.stStart[s];
      for (uint32_t i0 = 0; i0 < len && queue != all; i0 += 32) {
        uint32_t hit = 0;
        if (i0 + lane < len) {
          const uint4 e = __ldg(list + i0 + lane);
          if ((e.y & 0xFFFFu) < tx0 + kTileW && (e.z & 0xFFFFu) > tx0)
            for (uint32_t u = 0; u < units; ++u) {
              const uint32_t uy0 = ty0 + u * R;
              if ((e.y >> 16) < uy0 + R && (e.z >> 16) > uy0) hit |= 1u << u;
            }
        }
        queue |= __reduce_or_sync(0xFFFFFFFFu, hit);
      }
    }
    if (clearing && (V.flags & kViewZeroDepth) && queue != all) {
      // block rows of the units left unqueued: 8 blocks (1 KB) per row, 32 B per lane
      const uint32_t nbx = ::min((uint32_t)kTileW, V.blocksX - tx0);
      for (uint32_t r = 0; r < (uint32_t)kTileH; ++r)
        if (!((queue >> (r / R)) & 1u) && ty0 + r < V.blocksY && lane / 4 < nbx) {
          uint4* d = reinterpret_cast<uint4*>(V.depth + ((size_t)(ty0 + r) * V.blocksX + tx0) * 64) + 2 * lane;
          d[0] = make_uint4(0, 0, 0, 0);
          d[1] = make_uint4(0, 0, 0, 0);
        }
    }
    // rows of the units left unqueued are final: their minima now
    uint32_t rows = 0;
    for (uint32_t r = 0; r < (uint32_t)kTileH; ++r)
      if (!((queue >> (r / R)) & 1u)) rows |= 1u << r;
    if (rows) store_tile_rows(V, lt, inView ? (clearing ? 1u : (uint32_t)V.hiz[blk]) : 0xFFFFu, rows, lane);
    if (lane == 0 && queue) slot = atomicAdd(&s_n, (uint32_t)__popc(queue));
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_n) s_base = atomicAdd(&P.header->activeTiles, s_n);
  __syncthreads();
  if (lane == 0 && queue) {
    uint32_t k = s_base + slot;
    for (uint32_t u = 0; u < units; ++u)
      if (queue & (1u << u)) P.activeTileList[k++] = make_uint4(wt * 4 + u * R, v, listStart, listLen);
  }
}

// The two stages between the list fill and the raster, in one launch: CTAs
// [0, walkCtas) walk the batch's rows (grid-striding), the others prepare 8
// warp-tiles each as the walk's CTAs retire.
__global__ void __launch_bounds__(256) k_walk_prep(FrameParams P, uint32_t walkCtas)
{
  pdl_wait();
  if (P.header->overflow) return;
  if (blockIdx.x < walkCtas) walk_rows(P, blockIdx.x, walkCtas);
  else tile_prep(P, blockIdx.x - walkCtas);
}

// ---- k_raster -------------------------------------------------------------------------
// Persistent CTAs of kRasterWarps independent warps; each warp takes queued
// raster units a few at a time from the global queue (dynamic: heavy units
// vary a lot) and rasterises them one after the other (raster_unit).

template <int R, bool kWins>
__global__ void __launch_bounds__(kRasterThreads, kRasterMinBlocks<R>) k_raster(FrameParams P)
{
  __shared__ WarpRasterSmem S[kRasterWarps];
  pdl_wait();
  if (P.header->overflow) return;
  const uint32_t lane = threadIdx.x & 31;
  WarpRasterSmem& W = S[threadIdx.x >> 5];
  const uint32_t nActive = P.header->activeTiles;
  const uint32_t chunk = P.tune.rasterChunk ? P.tune.rasterChunk : 1u;  // units per fetch
  uint32_t i = 0;
  if (lane == 0) i = atomicAdd(&P.header->tileCursor, chunk);
  i = __shfl_sync(0xFFFFFFFFu, i, 0);
  while (i < nActive) {
    uint32_t nxt = 0;
    if (lane == 0) nxt = atomicAdd(&P.header->tileCursor, chunk);  // next fetch, ahead of time
    const uint32_t end = ::min(i + chunk, nActive);
    for (uint32_t j = i; j < end; ++j) {
      const uint4 rec = __ldg(P.activeTileList + j);
      raster_unit<R, kWins>(P, W, rec, lane);
    }
    i = __shfl_sync(0xFFFFFFFFu, nxt, 0);
  }
}

// ---- k_raster_cta: four warps per raster unit ------------------------------------------
//
// The other raster form: one CTA of 128 threads per unit of 8 x R blocks (R
// = 1 or 2), thread t owning pixel row t%8 of block t/8 (the threads past the
// unit's 8 R blocks hold none).  The CTA filters the unit's super-tile list
// 256 entries a round and computes 128 fragments a round, so a unit with a
// long list or many fragments finishes four times sooner than on one warp;
// the price is CTA barriers between the phases.  Views with few units and
// long lists (one large view) favour it; batches of many views favour the
// warp form.  Units of one block row halve a unit's fragments (the filter
// still reads the whole list): shorter chains for the heaviest units.

constexpr int kCtaUnitBlocks = kTileW * 2;               // blocks of the largest unit (8 x 2)
constexpr int kCtaThreads = 8 * kCtaUnitBlocks;          // one thread per block row: 128
constexpr int kCtaMinBlocks = 8;
constexpr int kCtaListCap = 512;                         // listed quads buffered per unit
constexpr int kCtaScanPerRound = 2 * kCtaThreads;
constexpr int kCtaMaskWords = kCtaThreads / 32;

struct CtaRasterSmem {
  uint32_t lq[kCtaListCap];      // quad index
  uint32_t lrect[kCtaListCap];   // quad rect within the unit: x0 | y0 << 3 | w << 5 | h << 9
  uint32_t loff[kCtaListCap];    // first fragment of each listed quad
  __align__(16) uint32_t frag[kCtaThreads * kFragStride];
  uint32_t meta[kCtaThreads];    // per fragment slot: maxZ << 16 | target block
  uint32_t fcmd[kCtaThreads];    // per fragment slot: command (win counting only)
  uint32_t bmask[kCtaUnitBlocks][kCtaMaskWords];  // per block: fragment slots aimed at it
  uint32_t hiz[kCtaUnitBlocks];  // per block: current hiZ
  uint32_t scan[kCtaThreads / 32];
  uint32_t rowMin[kCtaThreads / 32];  // per warp: minimum final hiZ of its 4 blocks
};

// Merges fragment slot `slot` into this thread's pixel row of its block (the
// reference's hiZ test, fast-clear overwrite or max-merge) and the block's new
// hiZ over its eight threads (`groupMask`).  With kWins, own[x] tracks the
// command (+1) that produced pixel x's value.
template <bool kWins>
__device__ __forceinline__ void merge_slot_row(const ViewDesc& V, const CtaRasterSmem& S, uint32_t slot, uint32_t py,
                                               uint32_t blk, uint32_t groupMask, uint32_t (&row)[4], uint32_t& hiz,
                                               bool& have, uint32_t (&own)[8])
{
  const uint32_t mz = S.meta[slot] >> 16;
  if (hiz >= mz) return;  // the reference's hiZ test (Rasterizer.cpp:1148-1152)
  const uint4 q = *reinterpret_cast<const uint4*>(S.frag + slot * kFragStride + 4 * py);
  const uint32_t src[4] = {q.x, q.y, q.z, q.w};
  const uint32_t c1 = kWins ? S.fcmd[slot] + 1 : 0u;
  if (hiz == 1) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (kWins) {
        own[2 * i] = (src[i] & 0xFFFFu) ? c1 : 0u;
        own[2 * i + 1] = (src[i] >> 16) ? c1 : 0u;
      }
      row[i] = src[i];
    }
  } else {
    if (!have) {
      const uint4 a = *reinterpret_cast<const uint4*>(V.depth + (size_t)blk * 64 + 8 * py);
      row[0] = a.x; row[1] = a.y; row[2] = a.z; row[3] = a.w;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (kWins) {
        if ((src[i] & 0xFFFFu) > (row[i] & 0xFFFFu)) own[2 * i] = c1;
        if ((src[i] >> 16) > (row[i] >> 16)) own[2 * i + 1] = c1;
      }
      row[i] = vmax_u16x2(row[i], src[i]);
    }
  }
  have = true;
  uint32_t mn = vmin_u16x2(vmin_u16x2(row[0], row[1]), vmin_u16x2(row[2], row[3]));
  mn = vmin_u16x2(mn, __shfl_xor_sync(groupMask, mn, 1));
  mn = vmin_u16x2(mn, __shfl_xor_sync(groupMask, mn, 2));
  mn = vmin_u16x2(mn, __shfl_xor_sync(groupMask, mn, 4));
  hiz = ::min(mn & 0xFFFFu, mn >> 16);
}

// Runs the listed quads (n of them, F fragments) kCtaThreads fragments a round.
template <bool kWins>
__device__ __forceinline__ void raster_list_cta(const FrameParams& P, const ViewDesc& V, CtaRasterSmem& S, uint32_t n,
                                                uint32_t F, uint32_t tx0, uint32_t ty0, uint32_t tid, uint32_t blk,
                                                bool inView, uint32_t (&row)[4], uint32_t& hiz, bool& have,
                                                uint32_t (&own)[8])
{
  const uint32_t lane = tid & 31;
  const uint32_t py = tid & 7;  // pixel row owned by this thread
  const uint32_t myBlock = tid >> 3;
  const uint32_t groupMask = 0xFFu << (lane & ~7u);
  for (uint32_t f0 = 0; f0 < F; f0 += kCtaThreads) {
    if (tid < kCtaUnitBlocks * kCtaMaskWords) (&S.bmask[0][0])[tid] = 0;
    const uint32_t f = f0 + tid;
    uint32_t target = 0, q = 0, bx = 0, by = 0;
    const bool haveF = f < F;
    if (haveF) {
      uint32_t lo = 0, hi = n - 1;  // last listed quad whose first fragment is <= f
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (S.loff[mid] <= f) lo = mid; else hi = mid - 1;
      }
      const uint32_t k = f - S.loff[lo];
      const uint32_t rc = S.lrect[lo];
      const uint32_t rw = (rc >> 5) & 15u;
      const uint32_t rr = k / rw, cc = k - rr * rw;
      const uint32_t lx = (rc & 7u) + cc, ly = ((rc >> 3) & 3u) + rr;
      target = ly * kTileW + lx;
      bx = tx0 + lx;
      by = ty0 + ly;
      q = S.lq[lo];
    }
    __syncthreads();  // bmask cleared
    uint32_t meta = 0;
    if (haveF) {
      const QuadRaster Q = P.rec[q];
      const uint32_t ckq = __ldg(P.ckBase + q);
      const uint32_t ownerHiz = S.hiz[target];
      // early skip (see raster_list): exact, hiZ only falls through the fast-clear overwrite
      const bool skip = ownerHiz >= Q.maxZ && !(ownerHiz == 1 && Q.maxZ == 1);
      if (!skip && make_fragment(P, Q, q, ckq, bx, by, tx0, S.frag + tid * kFragStride)) {
        meta = ((uint32_t)Q.maxZ << 16) | target;
        if (kWins) S.fcmd[tid] = P.walk[q].pad[0];
        atomicOr(&S.bmask[target][tid >> 5], 1u << lane);
      }
    }
    S.meta[tid] = meta;
    __syncthreads();
    // merge, in slot order, the fragments aimed at this thread's block
    if (inView) {
#pragma unroll 1
      for (int wd = 0; wd < kCtaMaskWords; ++wd) {
        uint32_t mine = S.bmask[myBlock][wd];
        while (mine) {
          const uint32_t slot = 32u * wd + __ffs(mine) - 1;
          mine &= mine - 1;
          merge_slot_row<kWins>(V, S, slot, py, blk, groupMask, row, hiz, have, own);
        }
      }
      if (py == 0) S.hiz[myBlock] = hiz;
    }
    __syncthreads();
  }
}

// One unit of 8 x R blocks (queue record as raster_unit's; first block row a
// multiple of R).
template <int R, bool kWins>
__device__ __forceinline__ void raster_unit_cta(const FrameParams& P, CtaRasterSmem& S, const uint4 rec)
{
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const ViewDesc& V = P.views[rec.y];
  const uint32_t lt = (rec.x >> 2) - V.tileStart;
  const uint32_t tx0 = (lt % V.tilesX) * kTileW, ty0 = (lt / V.tilesX) * kTileH + (rec.x & 3u);
  const uint32_t myBlock = tid >> 3, py = tid & 7;
  const uint32_t bx = tx0 + (myBlock & 7), by = ty0 + (myBlock >> 3);
  const bool inView = myBlock < 8u * R && bx < V.blocksX && by < V.blocksY;
  const uint32_t blk = inView ? by * V.blocksX + bx : 0;
  const bool clearing = (V.flags & kViewClear) != 0 && P.phase == 0;
  uint32_t hiz = clearing ? 1u : (inView ? (uint32_t)V.hiz[blk] : 0xFFFFu);
  bool have = false;
  uint32_t row[4] = {0, 0, 0, 0};
  uint32_t own[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const uint32_t listLen = rec.w;
  const uint4* list = P.stList + rec.z;
  if (py == 0 && myBlock < 8u * R) S.hiz[myBlock] = hiz;
  __syncthreads();
  uint32_t n = 0, F = 0;
  // kCtaScanPerRound list entries per round (two consecutive ones per thread),
  // listed in list order unless already hidden in every block they touch;
  // one scan of (fragments << 16 | quads) places both
  for (uint32_t base = 0; base < listLen; base += kCtaScanPerRound) {
    uint4 e[2];
    bool ov[2];
    uint32_t rect[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const uint32_t idx = base + 2 * tid + k;
      e[k] = idx < listLen ? __ldg(list + idx) : make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const uint32_t qx0 = e[k].y & 0xFFFFu, qy0 = e[k].y >> 16, qx1 = e[k].z & 0xFFFFu, qy1 = e[k].z >> 16;
      const uint32_t x0 = ::max(qx0, tx0), x1 = ::min(qx1, tx0 + kTileW);
      const uint32_t y0 = ::max(qy0, ty0), y1 = ::min(qy1, ty0 + R);
      bool o = x0 < x1 && y0 < y1;  // padding entries have an empty box
      if (o) {
        const uint32_t mz = e[k].w;
        bool hidden = true;
        for (uint32_t yy = y0 - ty0; yy < y1 - ty0 && hidden; ++yy)
          for (uint32_t xx = x0 - tx0; xx < x1 - tx0; ++xx) {
            const uint32_t h = S.hiz[yy * kTileW + xx];
            if (!(h >= mz && !(h == 1 && mz == 1))) {
              hidden = false;
              break;
            }
          }
        o = !hidden;
      }
      ov[k] = o;
      rect[k] = (x0 - tx0) | ((y0 - ty0) << 3) | ((x1 - x0) << 5) | ((y1 - y0) << 9);
    }
    uint32_t fr[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) fr[k] = ov[k] ? ((rect[k] >> 5) & 15u) * ((rect[k] >> 9) & 7u) : 0u;
    const uint32_t cnt = (ov[0] ? 1u : 0u) + (ov[1] ? 1u : 0u);
    uint32_t tot;  // per round at most 256 quads and 4,096 fragments: the halves do not carry
    const uint32_t ex = block_exclusive_scan<kCtaThreads>(cnt | ((fr[0] + fr[1]) << 16), tot, S.scan);
    uint32_t pos = n + (ex & 0xFFFFu), fpos = F + (ex >> 16);
#pragma unroll
    for (int k = 0; k < 2; ++k)
      if (ov[k]) {
        S.lq[pos] = e[k].x;
        S.lrect[pos] = rect[k];
        S.loff[pos] = fpos;
        ++pos;
        fpos += fr[k];
      }
    n += tot & 0xFFFFu;
    F += tot >> 16;
    __syncthreads();
    if (n > (uint32_t)(kCtaListCap - kCtaScanPerRound) || (base + kCtaScanPerRound >= listLen && n > 0)) {
      raster_list_cta<kWins>(P, V, S, n, F, tx0, ty0, tid, blk, inView, row, hiz, have, own);
      n = 0;
      F = 0;
    }
  }
  if (inView) {
    if ((clearing || have) && py == 0) V.hiz[blk] = (uint16_t)hiz;
    uint4* d = reinterpret_cast<uint4*>(V.depth + (size_t)blk * 64 + 8 * py);
    if (have) *d = make_uint4(row[0], row[1], row[2], row[3]);
    else if (clearing && (V.flags & kViewZeroDepth)) *d = make_uint4(0, 0, 0, 0);
  }
  {
    uint32_t h = inView ? hiz : 0xFFFFu;
#pragma unroll
    for (int o = 8; o < 32; o <<= 1) h = ::min(h, __shfl_xor_sync(0xFFFFFFFFu, h, o));  // 4 blocks
    if (lane == 0) S.rowMin[tid >> 5] = h;
  }
  if (kWins) {
    // pixels won per command: one atomic per distinct command per warp when
    // every row has one owner (the common case), else per warp and pixel column
    bool same = true;
#pragma unroll
    for (int x = 1; x < 8; ++x) same &= own[x] == own[0];
    if (__all_sync(0xFFFFFFFFu, same)) {
      const uint32_t key = inView ? own[0] : 0u;
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
      if (key && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&P.wins[key - 1], 8u * (uint32_t)__popc(peers));
    } else {
#pragma unroll
      for (int x = 0; x < 8; ++x) {
        const uint32_t key = inView ? own[x] : 0u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        if (key && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&P.wins[key - 1], (uint32_t)__popc(peers));
      }
    }
    if (V.owner && inView) {
      uint32_t* o = V.owner + (size_t)blk * 64 + 8 * py;
      if (P.phase == 0) {
        reinterpret_cast<uint4*>(o)[0] = make_uint4(own[0], own[1], own[2], own[3]);
        reinterpret_cast<uint4*>(o)[1] = make_uint4(own[4], own[5], own[6], own[7]);
      } else {
#pragma unroll
        for (int x = 0; x < 8; ++x)
          if (own[x]) o[x] = own[x];  // pixels the second pass changed
      }
    }
  }
}

// Persistent CTAs taking queued units of 8 x R blocks one at a time; the next
// record is copied with cp.async while the current unit is rasterised.
template <int R, bool kWins>
__global__ void __launch_bounds__(kCtaThreads, kCtaMinBlocks) k_raster_cta(FrameParams P)
{
  __shared__ CtaRasterSmem S;
  __shared__ uint32_t s_next;
  __shared__ __align__(16) uint4 s_rec[2];  // this unit's queue record and the next one's
  pdl_wait();
  if (P.header->overflow) return;
  const uint32_t nActive = P.header->activeTiles;
  const uint32_t chunk = P.tune.rasterChunk ? P.tune.rasterChunk : 1u;  // units per fetch
  if (threadIdx.x == 0) {
    const uint32_t i0 = atomicAdd(&P.header->tileCursor, chunk);
    s_next = i0;
    if (i0 < nActive) s_rec[0] = P.activeTileList[i0];
  }
  __syncthreads();
  uint32_t i = s_next, buf = 0;
  while (i < nActive) {
    uint32_t nxt = 0;
    if (threadIdx.x == 0) nxt = atomicAdd(&P.header->tileCursor, chunk);  // next fetch, ahead of time
    const uint32_t end = ::min(i + chunk, nActive);
    for (uint32_t j = i; j < end; ++j) {
      const uint4 rec = s_rec[buf];
      if (threadIdx.x == 0) {
        // the next unit's record, copied while this one is rasterised (the
        // buffer it lands in was last read before the previous unit's barrier)
        const uint32_t k = j + 1 < end ? j + 1 : nxt;
        if (k < nActive) {
          const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s_rec[buf ^ 1u]);
          asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(P.activeTileList + k) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
      }
      raster_unit_cta<R, kWins>(P, S, rec);
      if (threadIdx.x == 0) asm volatile("cp.async.wait_all;" ::: "memory");
      __syncthreads();  // shared state is reused by the next unit; the next record has landed
      if (threadIdx.x < (uint32_t)R) {  // the unit's block rows' minimum hiZ (warps 2r, 2r + 1)
        const ViewDesc& V = P.views[rec.y];
        const uint32_t r = threadIdx.x;
        V.tileHiz[4 * (size_t)((rec.x >> 2) - V.tileStart) + (rec.x & 3u) + r] =
            (uint16_t)::min(S.rowMin[2 * r], S.rowMin[2 * r + 1]);
      }
      buf ^= 1u;
    }
    if (threadIdx.x == 0) s_next = nxt;
    __syncthreads();
    i = s_next;
  }
}

// Recomputes the per-warp-tile row minima of one view's hiZ (after hiZ was
// written from the host).  One warp per tile.
__global__ void __launch_bounds__(128) k_tile_hiz(const uint16_t* hiz, uint16_t* tileHiz, uint32_t blocksX,
                                                  uint32_t blocksY, uint32_t tilesX, uint32_t tiles)
{
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t t = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (t >= tiles) return;
  const uint32_t bx = (t % tilesX) * kTileW + (lane & 7), by = (t / tilesX) * kTileH + (lane >> 3);
  uint32_t m = (bx < blocksX && by < blocksY) ? hiz[by * blocksX + bx] : 0xFFFFu;
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) m = ::min(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
  if ((lane & 7u) == 0) tileHiz[4 * (size_t)t + (lane >> 3)] = (uint16_t)m;  // per block row
}

// ---- k_query -------------------------------------------------------------------------

// Front-end status -> visibility for boxes with small rectangles (query2D per
// thread); `big` marks the ones left to the CTA's warps (collect_big).  Small means at most
// a warp-tile's worth of blocks where the warp's lanes are full (kFull, the
// survivor lists of k_query), at most two warp-tiles where many lanes idle.
template <bool kFull>
__device__ __forceinline__ void query_resolve(const ViewDesc& V, int st, const uint32_t* rect, uint32_t maxZ, bool& vis,
                                              bool& nc, bool& big)
{
  if (st == 1) {
    vis = true;
    nc = true;
  } else if (st == 2) {
    if (kFull) {
      const uint32_t nb = ((rect[1] >> 3) - (rect[0] >> 3) + 1) * ((rect[3] >> 3) - (rect[2] >> 3) + 1);
      big = nb > (uint32_t)(kTileW * kTileH);
    } else {
      const uint32_t ntx = (rect[1] >> 3) / kTileW - (rect[0] >> 3) / kTileW + 1;
      const uint32_t nty = (rect[3] >> 3) / kTileH - (rect[2] >> 3) / kTileH + 1;
      big = ntx * nty > 2;
    }
    if (!big) vis = query2d<!kFull>(V, rect[0], rect[1], rect[2], rect[3], maxZ);
  }
}

// Boxes with large rectangles are collected per CTA and tested after the
// CTA's other boxes by all of its warps, in pieces of 32 warp-tiles a warp at
// a time (a warp testing its own large boxes one after the other, or one box
// whole, would leave the few warps holding the heaviest to set the stage's
// time).  All 32 lanes; a box that does not fit the CTA's list is tested by
// its own warp at once (returns its visibility in `vis`).
constexpr uint32_t kBigPerCta = 256;

struct BigBoxes {
  uint4 box[kBigPerCta];           // {slot, minX | maxX << 16, minY | maxY << 16, maxZ}
  uint32_t pieceStart[kBigPerCta];  // first piece of each box (pieces of 32 warp-tiles)
  uint32_t found[kBigPerCta / 32];  // bit per box: visible (its other pieces are skipped)
  uint32_t scan[8];
  uint32_t count, next;
};

__device__ __forceinline__ bool query_big_box(const ViewDesc& V, uint32_t minX, uint32_t maxX, uint32_t minY,
                                              uint32_t maxY, uint32_t mz, uint32_t lane);
__device__ __forceinline__ bool query_big_round(const ViewDesc& V, uint32_t minX, uint32_t maxX, uint32_t minY,
                                                uint32_t maxY, uint32_t mz, uint32_t t0, uint32_t lane);
__device__ __forceinline__ uint32_t query_view(const FrameParams& P, uint32_t slot, uint32_t lo, uint32_t hi);

__device__ __forceinline__ void collect_big(const FrameParams& P, BigBoxes& B, bool big, uint32_t slot,
                                            uint32_t view, const uint32_t* rect, uint32_t maxZ, uint32_t lane,
                                            bool& vis)
{
  const uint32_t m = __ballot_sync(0xFFFFFFFFu, big);
  if (!m) return;
  uint32_t base = 0;
  if (lane == 0) base = atomicAdd(&B.count, (uint32_t)__popc(m));
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  const uint32_t at = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
  if (big && at < kBigPerCta)
    B.box[at] = make_uint4(slot, rect[0] | (rect[1] << 16), rect[2] | (rect[3] << 16), maxZ);
  uint32_t over = __ballot_sync(0xFFFFFFFFu, big && at >= kBigPerCta);
  while (over) {
    const int j = __ffs(over) - 1;
    over &= over - 1;
    const uint32_t r0 = __shfl_sync(0xFFFFFFFFu, rect[0], j), r1 = __shfl_sync(0xFFFFFFFFu, rect[1], j);
    const uint32_t r2 = __shfl_sync(0xFFFFFFFFu, rect[2], j), r3 = __shfl_sync(0xFFFFFFFFu, rect[3], j);
    const uint32_t mz = __shfl_sync(0xFFFFFFFFu, maxZ, j), vj = __shfl_sync(0xFFFFFFFFu, view, j);
    const bool found = query_big_box(P.views[vj], r0, r1, r2, r3, mz, lane);
    if ((int)lane == j) vis = found;
  }
}

// Warp-tiles of a box's rectangle.
__device__ __forceinline__ uint32_t big_tiles(const uint4& e)
{
  const uint32_t bx0 = (e.y & 0xFFFFu) >> 3, bx1 = (e.y >> 16) >> 3, by0 = (e.z & 0xFFFFu) >> 3, by1 = (e.z >> 16) >> 3;
  return (bx1 / kTileW - bx0 / kTileW + 1) * (by1 / kTileH - by0 / kTileH + 1);
}

// After the CTA barrier that follows every collect_big, all 256 threads of
// the CTA: each large box is cut into pieces of 32 warp-tiles (offsets by a
// CTA scan), and the warps take the pieces one at a time; a visible piece
// marks its box found (its pieces not yet taken are skipped) and sets bit
// (slot - slot0) of the CTA's bit array `bits`.
__device__ __forceinline__ void test_big(const FrameParams& P, BigBoxes& B, uint32_t slot0, uint32_t* bits,
                                         uint32_t tid)
{
  const uint32_t n = ::min(B.count, kBigPerCta), lane = tid & 31;
  if (n == 0) return;  // the same for every thread
  const uint32_t pieces = tid < n ? (big_tiles(B.box[tid]) + 31) / 32 : 0u;
  uint32_t total;
  const uint32_t first = block_exclusive_scan<256>(pieces, total, B.scan);
  if (tid < n) B.pieceStart[tid] = first;
  if (tid < kBigPerCta / 32) B.found[tid] = 0;
  __syncthreads();
  for (;;) {
    uint32_t i = 0;
    if (lane == 0) i = atomicAdd(&B.next, 1u);
    i = __shfl_sync(0xFFFFFFFFu, i, 0);
    if (i >= total) break;
    uint32_t lo = 0, hi = n - 1;  // the box of piece i
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (B.pieceStart[mid] <= i) lo = mid; else hi = mid - 1;
    }
    if ((B.found[lo >> 5] >> (lo & 31u)) & 1u) continue;
    const uint4 e = B.box[lo];
    const ViewDesc& V = P.views[query_view(P, e.x, 0, P.numViews - 1)];
    const uint32_t t0 = 32u * (i - B.pieceStart[lo]);
    if (query_big_round(V, e.y & 0xFFFFu, e.y >> 16, e.z & 0xFFFFu, e.z >> 16, e.w, t0, lane) && lane == 0) {
      atomicOr(&B.found[lo >> 5], 1u << (lo & 31u));
      atomicOr(bits + ((e.x - slot0) >> 5), 1u << (e.x & 31u));
    }
  }
}

// query2D of one box with a large rectangle by the whole warp, 32 of its
// warp-tiles from tile t0 (query_big_round) or all of them: one tile per
// lane, after their minimum hiZ (a tile whose minimum is >= maxZ holds no
// block the reference would read).  When few of the 32 tiles pass, each is
// then tested one block per lane (a tile has 8 x 4 = 32 blocks); when many
// pass, each lane tests its own tile's blocks in sequence.  Returns the same
// on every lane.
constexpr uint32_t kBigSplitMax = 4;  // tiles passing a round, at most, tested a block per lane

__device__ __forceinline__ bool query_big_round(const ViewDesc& V, uint32_t minX, uint32_t maxX, uint32_t minY,
                                                uint32_t maxY, uint32_t mz, uint32_t t0, uint32_t lane)
{
  const uint32_t tilesX = (V.blocksX + kTileW - 1) / kTileW;
  const uint32_t bx0 = minX >> 3, bx1 = maxX >> 3, by0 = minY >> 3, by1 = maxY >> 3;
  const uint32_t tx0 = bx0 / kTileW, ty0 = by0 / kTileH;
  const uint32_t ntx = bx1 / kTileW - tx0 + 1, nt = ntx * (by1 / kTileH - ty0 + 1);
  {
    const uint32_t t = t0 + lane;
    uint32_t tx = 0, ty = 0;
    uint2 rm = make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
    bool open = false;
    if (t < nt) {
      tx = tx0 + t % ntx;
      ty = ty0 + t / ntx;
      rm = tile_rows(V, ty * tilesX + tx);
      open = mz > tile_min(rm);
    }
    uint32_t openMask = __ballot_sync(0xFFFFFFFFu, open);
    if ((uint32_t)__popc(openMask) > kBigSplitMax) {
      const bool hit = open && query2d_tile<true>(V, tx, ty, rm, minX, maxX, minY, maxY, mz);
      return __ballot_sync(0xFFFFFFFFu, hit) != 0;
    }
    while (openMask) {
      const uint32_t tt = t0 + (uint32_t)(__ffs(openMask) - 1);
      openMask &= openMask - 1;
      const uint32_t bx = (tx0 + tt % ntx) * kTileW + (lane & (kTileW - 1));
      const uint32_t by = (ty0 + tt / ntx) * kTileH + lane / kTileW;
      const bool hit = bx >= bx0 && bx <= bx1 && by >= by0 && by <= by1 &&
                       query2d_block<true>(V, bx, by, minX, maxX, minY, maxY, mz);
      if (__ballot_sync(0xFFFFFFFFu, hit)) return true;
    }
  }
  return false;
}

__device__ __forceinline__ bool query_big_box(const ViewDesc& V, uint32_t minX, uint32_t maxX, uint32_t minY,
                                              uint32_t maxY, uint32_t mz, uint32_t lane)
{
  const uint32_t nt = big_tiles(make_uint4(0, minX | (maxX << 16), minY | (maxY << 16), 0));
  for (uint32_t t0 = 0; t0 < nt; t0 += 32)
    if (query_big_round(V, minX, maxX, minY, maxY, mz, t0, lane)) return true;
  return false;
}

// Boxes with large rectangles in k_query: the whole warp tests one box at a time, its
// warp-tiles 32 at a time, one per lane, after their minimum hiZ (a tile whose
// minimum is >= maxZ holds no block the reference would read).  kSplit: each
// tile that passes is then tested one block per lane (a tile has 8 x 4 = 32
// blocks; best when the lanes are full); otherwise its lane tests the tile's
// blocks itself (fewer steps in sequence: best when few boxes keep the GPU
// busy).  Called by all 32 lanes.
template <bool kSplit>
__device__ __forceinline__ void query_big_boxes(const FrameParams& P, bool big, const uint32_t* rect, uint32_t maxZ,
                                                uint32_t view, uint32_t lane, bool& vis)
{
  uint32_t bigMask = __ballot_sync(0xFFFFFFFFu, big);
  while (bigMask) {
    const int j = __ffs(bigMask) - 1;
    bigMask &= bigMask - 1;
    const uint32_t minX = __shfl_sync(0xFFFFFFFFu, rect[0], j), maxX = __shfl_sync(0xFFFFFFFFu, rect[1], j);
    const uint32_t minY = __shfl_sync(0xFFFFFFFFu, rect[2], j), maxY = __shfl_sync(0xFFFFFFFFu, rect[3], j);
    const uint32_t mz = __shfl_sync(0xFFFFFFFFu, maxZ, j), vj = __shfl_sync(0xFFFFFFFFu, view, j);
    const ViewDesc& V = P.views[vj];
    const uint32_t tilesX = (V.blocksX + kTileW - 1) / kTileW;
    const uint32_t bx0 = minX >> 3, bx1 = maxX >> 3, by0 = minY >> 3, by1 = maxY >> 3;
    const uint32_t tx0 = bx0 / kTileW, ty0 = by0 / kTileH;
    const uint32_t ntx = bx1 / kTileW - tx0 + 1, nt = ntx * (by1 / kTileH - ty0 + 1);
    bool found = false;
    for (uint32_t t0 = 0; t0 < nt && !found; t0 += 32) {
      const uint32_t t = t0 + lane;
      bool open = false;
      if (t < nt) {
        const uint32_t tx = tx0 + t % ntx, ty = ty0 + t / ntx;
        const uint2 rm = tile_rows(V, ty * tilesX + tx);
        open = mz > tile_min(rm);
        if (!kSplit && open) open = query2d_tile<false>(V, tx, ty, rm, minX, maxX, minY, maxY, mz);
      }
      if (!kSplit) {
        found = __ballot_sync(0xFFFFFFFFu, open) != 0;
        continue;
      }
      uint32_t openMask = __ballot_sync(0xFFFFFFFFu, open);
      while (openMask && !found) {
        const uint32_t tt = t0 + (uint32_t)(__ffs(openMask) - 1);
        openMask &= openMask - 1;
        const uint32_t bx = (tx0 + tt % ntx) * kTileW + (lane & (kTileW - 1));
        const uint32_t by = (ty0 + tt / ntx) * kTileH + lane / kTileW;
        const bool hit = bx >= bx0 && bx <= bx1 && by >= by0 && by <= by1 &&
                         query2d_block<false>(V, bx, by, minX, maxX, minY, maxY, mz);
        found = __ballot_sync(0xFFFFFFFFu, hit) != 0;
      }
    }
    if ((int)lane == j) vis = found;
  }
}

// The view owning query slot `slot`, searched in [lo, hi].
__device__ __forceinline__ uint32_t query_view(const FrameParams& P, uint32_t slot, uint32_t lo, uint32_t hi)
{
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (P.views[mid].queryStart <= slot) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One thread per query slot, the whole front end and query2D in place: the
// fastest form when there are too few slots to keep the GPU busy after
// compaction (a single view's 100k boxes).
__global__ void __launch_bounds__(256, 4) k_query_thread(FrameParams P)
{
  __shared__ BigBoxes s_big;
  __shared__ uint32_t s_vis[8];
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_big.count = s_big.next = 0;
  if (threadIdx.x < 8) s_vis[threadIdx.x] = 0;
  bool vis = false, nc = false, big = false;
  uint32_t rect[4] = {0, 0, 0, 0}, maxZ = 0, view = 0;
  // the box's projection reads only the view table and the boxes, written
  // before the launch: it may run while the raster's last CTAs finish
  int st = 0;
  bool have = false;
  if (slot < P.numQuerySlots) {
    view = query_view(P, slot, 0, P.numViews - 1);
    const ViewDesc& V = P.views[view];
    if (slot - V.queryStart < V.queryCount) {
      const float4 a = P.qmin[slot], b = P.qmax[slot];
      const float bmin[4] = {a.x, a.y, a.z, a.w}, bmax[4] = {b.x, b.y, b.z, b.w};
      st = query_front(V, bmin, bmax, rect, &maxZ);
      have = true;
    }
  }
  pdl_wait();
  if (P.header->overflow) return;  // the same for every thread
  __syncthreads();                 // s_big and s_vis set
  if (have) query_resolve<false>(P.views[view], st, rect, maxZ, vis, nc, big);
  collect_big(P, s_big, big, slot, view, rect, maxZ, lane, vis);
  const uint32_t vb = __ballot_sync(0xFFFFFFFFu, vis), nb = __ballot_sync(0xFFFFFFFFu, nc);
  __syncthreads();
  test_big(P, s_big, blockIdx.x * blockDim.x, s_vis, threadIdx.x);
  __syncthreads();
  if (lane == 0 && slot < P.numQuerySlots) {
    P.visBits[slot >> 5] = vb | s_vis[warp];
    P.ncBits[slot >> 5] = nb;
  }
}

// Each warp takes `rounds` x 32 consecutive query slots.  It tests every box
// against the six frustum planes, queues the boxes inside (and those whose
// arithmetic met a NaN) in its own shared-memory list, then projects them and
// runs query2D 32 at a time with its lanes full (most boxes of a view are
// outside its frustum: without the list most lanes would idle through the
// projection).  Warps never wait for one another.  CTAs run from the last
// slots to the first: the views rasterised last are the likeliest still in L2.
__global__ void __launch_bounds__(256, 6) k_query(FrameParams P, uint32_t rounds)
{
  __shared__ uint32_t s_slot[8][32 * kQueryRounds], s_view[8][32 * kQueryRounds];
  __shared__ uint32_t s_vis[8][kQueryRounds], s_nc[8][kQueryRounds];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t first = ((gridDim.x - 1 - blockIdx.x) * 8 + warp) * 32 * rounds;
  if (first >= P.numQuerySlots) return;
  if (lane < rounds) {
    s_vis[warp][lane] = 0;
    s_nc[warp][lane] = 0;
  }
  // the views of the warp's first and last slot bound every lane's search
  const uint32_t edge = lane ? ::min(first + 32 * rounds - 1, P.numQuerySlots - 1) : first;
  const uint32_t ev = lane < 2 ? query_view(P, edge, 0, P.numViews - 1) : 0u;
  const uint32_t vlo = __shfl_sync(0xFFFFFFFFu, ev, 0), vhi = __shfl_sync(0xFFFFFFFFu, ev, 1);
  uint32_t n = 0;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t slot = first + 32 * r + lane;
    bool keep = false, exact = false;
    uint32_t view = 0;
    if (slot < P.numQuerySlots) {
      view = query_view(P, slot, vlo, vhi);
      const ViewDesc& V = P.views[view];
      if (slot - V.queryStart < V.queryCount) {
        const float4 a = P.qmin[slot], b = P.qmax[slot];
        const float bmin[4] = {a.x, a.y, a.z, a.w}, bmax[4] = {b.x, b.y, b.z, b.w};
        LazyOps f;
        const bool outside = query_outside_t(f, V, bmin, bmax);
        exact = f.nan;  // redone in full under the x86 NaN rules
        keep = !outside || exact;
      }
    }
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, keep);
    if (keep) {
      const uint32_t at = n + (uint32_t)__popc(m & ((1u << lane) - 1u));
      s_slot[warp][at] = slot;
      s_view[warp][at] = view | (exact ? 0x80000000u : 0u);
    }
    n += (uint32_t)__popc(m);
  }
  // the frustum tests above read only the view table and the boxes, written
  // before the launch; the rest reads the rasterised hiZ
  pdl_wait();
  if (P.header->overflow) return;
  __syncwarp();
  for (uint32_t base = 0; base < n; base += 32) {
    const uint32_t k = base + lane;
    bool vis = false, nc = false, big = false;
    uint32_t rect[4] = {0, 0, 0, 0}, maxZ = 0, v = 0, sl = first;
    if (k < n) {
      sl = s_slot[warp][k];
      const uint32_t e = s_view[warp][k];
      v = e & 0x7FFFFFFFu;
      const ViewDesc& V = P.views[v];
      const float4 a = P.qmin[sl], b = P.qmax[sl];
      const float bmin[4] = {a.x, a.y, a.z, a.w}, bmax[4] = {b.x, b.y, b.z, b.w};
      int st;
      if (e >> 31) {
        st = query_front_exact(V, bmin, bmax, rect, &maxZ, nullptr);
      } else {
        LazyOps g;
        st = query_project_t(g, V, bmin, bmax, rect, &maxZ);
        if (g.nan) st = query_front_exact(V, bmin, bmax, rect, &maxZ, nullptr);
      }
      query_resolve<true>(V, st, rect, maxZ, vis, nc, big);
    }
    query_big_boxes<true>(P, big, rect, maxZ, v, lane, vis);
    const uint32_t w = (sl - first) >> 5, bit = 1u << (sl & 31u);
    if (vis) atomicOr(&s_vis[warp][w], bit);
    if (nc) atomicOr(&s_nc[warp][w], bit);
  }
  __syncwarp();
  if (lane < rounds) {
    const uint32_t w = (first >> 5) + lane;
    if (32 * w < P.numQuerySlots) {
      P.visBits[w] = s_vis[warp][lane];
      P.ncBits[w] = s_nc[warp][lane];
    }
  }
}

__global__ void k_query2d(const ViewDesc* V, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY,
                          uint32_t maxZ, uint32_t* out)
{
  *out = query2d<true>(*V, minX, maxX, minY, maxY, maxZ) ? 1u : 0u;
}

// ---- readBackDepth (Rasterizer.cpp:351-399) ---------------------------------------------

// readBackDepth (Rasterizer.cpp:351-399) and the values it computes on the way
// to its RGBA bytes, one pixel per thread, row-major output; cleared blocks
// (hiZ == 1) give zero in every format.
__global__ void __launch_bounds__(256) k_read_back(const uint16_t* depth, const uint16_t* hiz, uint32_t width,
                                                   uint32_t height, uint32_t blocksX, int format, void* out)
{
  const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t py = blockIdx.y;
  if (px >= width || py >= height) return;
  const uint32_t bx = px >> 3, by = py >> 3, blk = by * blocksX + bx;
  const size_t o = (size_t)py * width + px;
  const bool cleared = hiz[blk] == 1;
  const uint32_t v = cleared ? 0u : depth[(size_t)blk * 64 + 8 * (py & 7) + (px & 7)];
  if (format == kReadBackPackedU16) {
    static_cast<uint16_t*>(out)[o] = (uint16_t)v;
    return;
  }
  const float d = x86::rmul(__uint_as_float(v << 12), 3.9623753e+28f);  // :378-379
  if (format == kReadBackDepthF32) {
    static_cast<float*>(out)[o] = cleared ? 0.0f : d;
    return;
  }
  const float lin = x86::rdiv(0.5f, x86::rsub(1000.25f, x86::rmul(x86::rsub(1.0f, d), 999.75f)));  // :381
  if (format == kReadBackLinearF32) {
    static_cast<float*>(out)[o] = cleared ? 0.0f : lin;
    return;
  }
  uchar4 res = make_uchar4(0, 0, 0, 0);
  if (!cleared) {
    const float s = x86::rmul(25600.0f, lin);
    // static_cast<uint32_t>(float) on x86-64: 64-bit truncation, low 32 bits
    const uint32_t di = (s > -9.2233720e18f && s < 9.2233720e18f) ? (uint32_t)(unsigned long long)__float2ll_rz(s) : 0u;
    res = make_uchar4((unsigned char)(di / 100), (unsigned char)(di % 256), 0, 255);
  }
  static_cast<uchar4*>(out)[o] = res;
}

// ---- launchers -------------------------------------------------------------------------

// The frame's kernels in order; with `ev`, an event is recorded before the
// first stage and after each of the six stages (setup, scan, list fill, row
// walk, raster, query), also for stages that do not run.
// NVTX ranges naming the frame's stages on the host timeline of a profiler
// (the launches a stage issues sit inside its range).
struct StageRanges {
  int open = -1;
  void next(int i)
  {
    static const char* const kNames[6] = {"occ setup", "occ scan", "occ list fill", "occ row walk", "occ raster",
                                          "occ query"};
    if (open >= 0) nvtxRangePop();
    open = i < 6 ? i : -1;
    if (open >= 0) nvtxRangePushA(kNames[i]);
  }
  ~StageRanges()
  {
    if (open >= 0) nvtxRangePop();
  }
};

// Launches `kernel` on `stream`; with `pdl`, as a programmatic dependent of
// the kernel before it (pdl_wait).
template <typename... KArgs, typename... Args>
static cudaError_t launch_k(bool pdl, void (*kernel)(KArgs...), uint32_t grid, uint32_t block, size_t smem,
                            cudaStream_t stream, Args... args)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1u : 0u;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

static cudaError_t flush_stages(const FrameParams& P, uint32_t numSt, uint32_t maxStPerView, bool doRaster,
                                bool doQuery, cudaStream_t stream, cudaEvent_t* ev)
{
  StageRanges ranges;
  auto mark = [&](int i) {
    if (ev) cudaEventRecord(ev[i], stream);
    ranges.next(i);
  };
  // the first kernel follows the counter reset (a memset) in plain stream
  // order; each later one is a programmatic dependent of the kernel before it
  // (none when events are recorded between the stages)
  bool chained = false;
  cudaError_t e = cudaSuccess;
  auto go = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
    chained = g_pdl && ev == nullptr;
  };
  mark(0);
  // activeChunks, activeTiles, tileCursor: reset by the chunk gate when it is
  // one CTA (one view), else by a memset before the launch
  const bool resetInGate = doRaster && P.numChunks && P.numViews == 1;
  if (doRaster && !resetInGate) {
    e = cudaMemsetAsync(&P.header->activeChunks, 0, kHeaderResetWords * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
  }
  if (doRaster) {
    if (P.numChunks) {
      // the gating: k_gate_second for a selection's second pass; k_select_view
      // did it with fusedSelect; else k_chunk_gate itself (views of at most
      // kChunkGateThreads commands) or k_gate
      const bool inChunkGate = !P.phase && !P.fusedSelect && P.maxViewCmds <= kChunkGateThreads;
      if (P.phase) go(launch_k(chained, k_gate_second, (P.numCmds + 7) / 8, 256, 0, stream, P));
      else if (!P.fusedSelect && !inChunkGate)
        go(launch_k(chained, k_gate, (P.numCmds + 255) / 256, 256, 0, stream, P));
      go(launch_k(chained, k_chunk_gate, P.numViews, kChunkGateThreads, 0, stream, P, inChunkGate ? 1u : 0u,
                  resetInGate ? 1u : 0u));
      go(launch_k(chained, k_setup, grid_of(P.tune.setupPerSm, g_setupPerSm, P.numChunks), kChunk,
                  (size_t)maxStPerView * sizeof(uint32_t), stream, P));
    }
  }
  mark(1);
  if (doRaster)
    go(launch_k(chained, k_scan, P.numViews + ::max(1u, ::min((numSt + 7) / 8, 4 * g_sms)), 256, 0, stream, P,
                numSt));
  mark(2);
  if (doRaster && P.numChunks)
    go(launch_k(chained, k_fill, grid_of(P.tune.fillPerSm, g_fillPerSm, P.numChunks), kChunk,
                (size_t)maxStPerView * 64, stream, P));
  mark(3);
  // raster form: a warp per unit of R block rows, or a CTA per unit of 8 x R
  // blocks (R = 1 unless tuned to 2) when the launch has few units (a warp
  // would leave most of the GPU idle and long lists in sequence)
  FrameParams Q = P;
  uint32_t threads = P.tune.rasterThreads;
  if (!threads) threads = P.numTiles * 2u < 4u * g_sms * g_rasterPerSm[1] * kRasterWarps ? 128u : 32u;
  Q.tune.rasterThreads = threads;
  Q.tune.rasterRows = threads == 128u ? (P.tune.rasterRows == 2u ? 2u : kDefaultCtaRows)
                                      : (P.tune.rasterRows ? P.tune.rasterRows : kDefaultRasterRows);
  if (doRaster && (P.numChunks || P.numTiles)) {
    // tile preparation and the row walk, one launch
    const uint32_t prep = (Q.numTiles + 7) / 8;
    const uint32_t walk = P.numChunks ? (P.tune.walkPerSm ? P.tune.walkPerSm * g_sms : g_walkBlocks) : 0u;
    go(launch_k(chained, k_walk_prep, walk + prep, 256, 0, stream, Q, walk));
  }
  mark(4);
  if (doRaster && P.numTiles) {
    const uint32_t R = Q.tune.rasterRows;
    const uint32_t units = Q.numTiles * (kTileH / R);
    const bool w = Q.wins != nullptr;
    if (threads == 128u) {
      const uint32_t grid = grid_of(Q.tune.rasterPerSm, g_rasterCtaPerSm, units);
      void (*k)(FrameParams) = R == 1 ? (w ? k_raster_cta<1, true> : k_raster_cta<1, false>)
                                      : (w ? k_raster_cta<2, true> : k_raster_cta<2, false>);
      go(launch_k(chained, k, grid, kCtaThreads, 0, stream, Q));
    } else {
      const uint32_t shape = R == 1 ? 0u : (R == 2 ? 1u : 2u);
      const uint32_t grid = grid_of(Q.tune.rasterPerSm, g_rasterPerSm[shape], (units + kRasterWarps - 1) / kRasterWarps);
      void (*k)(FrameParams) = R == 1 ? (w ? k_raster<1, true> : k_raster<1, false>)
                               : R == 4 ? (w ? k_raster<4, true> : k_raster<4, false>)
                                        : (w ? k_raster<2, true> : k_raster<2, false>);
      go(launch_k(chained, k, grid, kRasterThreads, 0, stream, Q));
    }
  }
  mark(5);
  if (doQuery && P.numQuerySlots) {
    const uint32_t ctas = (P.numQuerySlots + 255) / 256, wave = g_sms * 6;
    uint32_t rounds = P.tune.queryRounds;
    if (rounds == 0)  // by slot count: the warp lists pay once the slots fill the GPU a few times over
      rounds = ctas < 4 * wave ? kQueryPerThread : ::min(kQueryRounds, ::max(1u, ctas / (6 * wave)));
    if (rounds == kQueryPerThread || rounds > kQueryRounds)
      go(launch_k(chained, k_query_thread, ctas, 256, 0, stream, P));
    else
      go(launch_k(chained, k_query, (ctas + rounds - 1) / rounds, 256, 0, stream, P, rounds));
  }

  mark(6);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_flush(const FrameParams& P, uint32_t numSt, uint32_t maxStPerView, bool doRaster,
                         bool doQuery, cudaStream_t stream)
{
  return flush_stages(P, numSt, maxStPerView, doRaster, doQuery, stream, nullptr);
}

cudaError_t launch_flush_timed(const FrameParams& P, uint32_t numSt, uint32_t maxStPerView, bool doRaster,
                               bool doQuery, cudaStream_t stream, cudaEvent_t* ev)
{
  return flush_stages(P, numSt, maxStPerView, doRaster, doQuery, stream, ev);
}

cudaError_t launch_read_back(const uint16_t* depth, const uint16_t* hiz, uint32_t width, uint32_t height,
                             int format, void* out, cudaStream_t stream)
{
  dim3 grid((width + 255) / 256, height);
  k_read_back<<<grid, 256, 0, stream>>>(depth, hiz, width, height, width / 8, format, out);
  return cudaGetLastError();
}

cudaError_t launch_query2d(const ViewDesc* view, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY,
                           uint32_t maxZ, uint32_t* out, cudaStream_t stream)
{
  k_query2d<<<1, 1, 0, stream>>>(view, minX, maxX, minY, maxY, maxZ, out);
  return cudaGetLastError();
}

cudaError_t launch_tile_hiz(const uint16_t* hiz, uint16_t* tileHiz, uint32_t blocksX, uint32_t blocksY,
                            cudaStream_t stream)
{
  const uint32_t tilesX = (blocksX + kTileW - 1) / kTileW, tilesY = (blocksY + kTileH - 1) / kTileH;
  const uint32_t tiles = tilesX * tilesY;
  k_tile_hiz<<<(tiles + 3) / 4, 128, 0, stream>>>(hiz, tileHiz, blocksX, blocksY, tilesX, tiles);
  return cudaGetLastError();
}

// Dynamic shared memory of k_setup (4 B per super-tile of the largest view)
// and k_fill (64 B per super-tile) may exceed the 48 KB default.
cudaError_t set_kernel_attributes()
{
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
  g_sms = (uint32_t)sms;
  g_walkBlocks = (uint32_t)sms * 8;
  const char* pdl = getenv("OCC_PDL");
  g_pdl = !(pdl && pdl[0] == '0');
  cudaError_t e = cudaFuncSetAttribute(k_setup, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kMaxStPerView * 4));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_fill, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kMaxStPerView * 64));
  if (e != cudaSuccess) return e;
  // persistent grids: resident CTAs per SM at the largest dynamic shared memory used
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_setup, kChunk, kMaxStPerView * 4) == cudaSuccess && nb > 0)
    g_setupPerSm = (uint32_t)nb;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fill, kChunk, kMaxStPerView * 16) == cudaSuccess && nb > 0)
    g_fillPerSm = (uint32_t)nb;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_raster<1, true>, kRasterThreads, 0) == cudaSuccess && nb > 0)
    g_rasterPerSm[0] = (uint32_t)nb;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_raster<2, true>, kRasterThreads, 0) == cudaSuccess && nb > 0)
    g_rasterPerSm[1] = (uint32_t)nb;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_raster<4, true>, kRasterThreads, 0) == cudaSuccess && nb > 0)
    g_rasterPerSm[2] = (uint32_t)nb;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_raster_cta<2, true>, kCtaThreads, 0) == cudaSuccess && nb > 0)
    g_rasterCtaPerSm = (uint32_t)nb;
  return cudaSuccess;
}

// Occupancy limits (resident CTAs per SM) of the persistent kernels -- setup,
// list fill, raster at unit rows 1, 2 and 4, the 128-thread raster form --
// and the SM count.
void tuning_limits(uint32_t out[7])
{
  out[0] = g_setupPerSm;
  out[1] = g_fillPerSm;
  out[2] = g_rasterPerSm[0];
  out[3] = g_rasterPerSm[1];
  out[4] = g_rasterPerSm[2];
  out[5] = g_rasterCtaPerSm;
  out[6] = g_sms;
}

// ---- cull labels ---------------------------------------------------------------------------
// One thread per query slot, after k_query: a box with a screen rectangle that
// the frame culls (an occlusion cull) credits the owners of a 4x4 grid of
// sample pixels in its rectangle, one count each (training labels of the
// occluder selector: how many culled boxes an occluder's pixels hide).

__global__ void __launch_bounds__(256) k_cull_labels(FrameParams P)
{
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= P.numQuerySlots) return;
  uint32_t lo = 0, hi = P.numViews - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (P.views[mid].queryStart <= slot) lo = mid; else hi = mid - 1;
  }
  const ViewDesc& V = P.views[lo];
  if (!V.owner || slot - V.queryStart >= V.queryCount) return;
  if ((P.visBits[slot >> 5] >> (slot & 31)) & 1u) return;  // visible
  const float4 a = P.qmin[slot], b = P.qmax[slot];
  const float bmin[4] = {a.x, a.y, a.z, a.w}, bmax[4] = {b.x, b.y, b.z, b.w};
  uint32_t rect[4], maxZ = 0;
  if (query_front(V, bmin, bmax, rect, &maxZ) != 2) return;  // outside the frustum: not an occlusion cull
  for (uint32_t j = 0; j < 4; ++j) {
    const uint32_t y = rect[2] + (uint32_t)(((uint64_t)(rect[3] - rect[2]) * (2 * j + 1)) / 8);
    for (uint32_t i = 0; i < 4; ++i) {
      const uint32_t x = rect[0] + (uint32_t)(((uint64_t)(rect[1] - rect[0]) * (2 * i + 1)) / 8);
      const uint32_t o = V.owner[(size_t)((y >> 3) * V.blocksX + (x >> 3)) * 64 + 8 * (y & 7) + (x & 7)];
      if (o) atomicAdd(&P.cullCount[o - 1], 1u);
    }
  }
}

cudaError_t launch_cull_labels(const FrameParams& P, cudaStream_t stream)
{
  if (P.numQuerySlots) k_cull_labels<<<(P.numQuerySlots + 255) / 256, 256, 0, stream>>>(P);
  return cudaGetLastError();
}

// ---- queries without device allocation -------------------------------------------------
//
// Callers that must not allocate device memory -- frame loops with a fixed
// memory budget that reserve everything at start-up, or engines that forbid
// cudaMalloc/cudaFree on their frame thread because both can synchronise and
// stall the whole device -- still need to test boxes against a rasterizer.
// For them occ_raster_query_batch_noalloc stages the boxes and the result bits
// in the fixed array below instead of in per-context buffers that grow on
// demand.  It is called from an ordinary host thread (it makes CUDA calls and
// waits for the bits), not from a host function on a stream.
//
// The array holds at most kNoAllocMaxQueries boxes (about 2 MiB in all) and
// lives on every GPU that loads this library until the process exits.  All
// calls on a device share it and it keeps the last call's contents; nothing in
// it needs clearing, because each call writes every word it later reads.
// Calls whose work overlaps on the GPU (several host threads, several streams)
// race on the array and must be serialised by the caller.

struct NoAllocScratch {
  ViewDesc view;
  float4 qmin[kNoAllocMaxQueries];
  float4 qmax[kNoAllocMaxQueries];
  uint32_t vis[kNoAllocMaxQueries / 32];
  uint32_t nc[kNoAllocMaxQueries / 32];
};

static __device__ __align__(256) unsigned char g_queryScratch[sizeof(NoAllocScratch)];

// Same queries as k_query for one view, staged in the fixed array.
__global__ void __launch_bounds__(256) k_query_noalloc(NoAllocScratch* S, uint32_t n)
{
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31;
  const ViewDesc& V = S->view;
  bool vis = false, nc = false;
  if (slot < n) {
    const float4 a = S->qmin[slot], b = S->qmax[slot];
    const float bmin[4] = {a.x, a.y, a.z, a.w}, bmax[4] = {b.x, b.y, b.z, b.w};
    uint32_t rect[4], maxZ = 0;
    const int st = query_front(V, bmin, bmax, rect, &maxZ);
    if (st == 1) {
      vis = true;
      nc = true;
    } else if (st == 2) {
      vis = query2d<true>(V, rect[0], rect[1], rect[2], rect[3], maxZ);
    }
  }
  const uint32_t vb = __ballot_sync(0xFFFFFFFFu, vis), nb = __ballot_sync(0xFFFFFFFFu, nc);
  if (lane == 0 && slot < ((n + 31) & ~31u)) {
    S->vis[slot >> 5] = vb;
    S->nc[slot >> 5] = nb;
  }
}

// Device address of the fixed array, looked up once per device with that
// device current (a host-side reference to g_queryScratch is only a stand-in
// for the symbol, not a device address).
static void* g_queryScratchAddr[64];
static std::mutex g_queryScratchLock;

static cudaError_t query_scratch_address(int device, NoAllocScratch** out)
{
  if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> guard(g_queryScratchLock);
  if (!g_queryScratchAddr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_queryScratch);
    if (e != cudaSuccess) return e;
    g_queryScratchAddr[device] = p;
  }
  *out = static_cast<NoAllocScratch*>(g_queryScratchAddr[device]);
  return cudaSuccess;
}

// Stages boxes and bits in the fixed array; no device memory is allocated.
// The caller has made `device` current and checked n <= kNoAllocMaxQueries.
cudaError_t query_noalloc(int device, const ViewDesc& view, uint32_t n, const float* mins, const float* maxs,
                          uint32_t* visibleBits, uint32_t* needsClippingBits, cudaStream_t stream)
{
  NoAllocScratch* S = nullptr;
  cudaError_t e = query_scratch_address(device, &S);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(&S->view, &view, sizeof(ViewDesc), cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
  if (n) {
    if ((e = cudaMemcpyAsync(S->qmin, mins, (size_t)n * 16, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(S->qmax, maxs, (size_t)n * 16, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
    k_query_noalloc<<<(n + 255) / 256, 256, 0, stream>>>(S, n);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const size_t words = (n + 31) / 32;
    if (visibleBits && (e = cudaMemcpyAsync(visibleBits, S->vis, words * 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
      return e;
    if (needsClippingBits &&
        (e = cudaMemcpyAsync(needsClippingBits, S->nc, words * 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
      return e;
  }
  return cudaStreamSynchronize(stream);
}

}  // namespace occ
