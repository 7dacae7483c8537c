/*
 * CPU oracle: scalar restatement of the reference occluder rasteriser
 * (SoftwareRasterizer/Rasterizer.cpp).  TEST INFRASTRUCTURE ONLY -- see oracle.h.
 *
 * The reference works on 8 quads at a time in AVX2 registers.  Each lane's
 * arithmetic is independent, so this restatement walks the quads of a packet
 * one at a time in lane order (the order Rasterizer.cpp:1090 visits them) and
 * keeps every operation of one lane, in the reference's order and rounding.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "x86_tables.h"

/* ---- x86 single-precision semantics -------------------------------------- */

typedef union { float f; uint32_t u; int32_t i; } fbits;

static inline uint32_t fu(float f) { fbits b; b.f = f; return b.u; }
static inline float uf(uint32_t u) { fbits b; b.u = u; return b.f; }
static inline int is_nan(float f) { return (fu(f) & 0x7FFFFFFFu) > 0x7F800000u; }
static inline float quiet(float f) { return uf(fu(f) | 0x00400000u); }
static const uint32_t kDefaultNaN = 0xFFC00000u; /* x86 "QNaN floating-point indefinite" */

/* Result of an arithmetic op with x86 NaN rules: a NaN operand propagates
 * (first one in source order, quieted); an invalid operation gives the
 * default NaN.  IEEE results are otherwise identical on every host. */
static inline float nan2(float r, float a, float b)
{
  if (!is_nan(r)) return r;
  if (is_nan(a)) return quiet(a);
  if (is_nan(b)) return quiet(b);
  return uf(kDefaultNaN);
}
static inline float nan3(float r, float a, float b, float c)
{
  if (!is_nan(r)) return r;
  if (is_nan(a)) return quiet(a);
  if (is_nan(b)) return quiet(b);
  if (is_nan(c)) return quiet(c);
  return uf(kDefaultNaN);
}
static inline float xadd(float a, float b) { return nan2(a + b, a, b); }
static inline float xsub(float a, float b) { return nan2(a - b, a, b); }
static inline float xmul(float a, float b) { return nan2(a * b, a, b); }
static inline float xdiv(float a, float b) { return nan2(a / b, a, b); }
/* _mm_fmadd_ps(a,b,c) = a*b+c, _mm_fmsub_ps = a*b-c, _mm_fnmadd_ps = c-a*b; one rounding. */
static inline float xfmadd(float a, float b, float c) { return nan3(fmaf(a, b, c), a, b, c); }
static inline float xfmsub(float a, float b, float c) { return nan3(fmaf(a, b, -c), a, b, c); }
static inline float xfnmadd(float a, float b, float c) { return nan3(fmaf(-a, b, c), a, b, c); }
/* minps/maxps: the second operand when the comparison is false (incl. NaN). */
static inline float xmin(float a, float b) { return a < b ? a : b; }
static inline float xmax(float a, float b) { return a > b ? a : b; }
static inline float xxor(float a, uint32_t m) { return uf(fu(a) ^ m); }
static inline float xabs(float a) { return uf(fu(a) & 0x7FFFFFFFu); }
static inline uint32_t sgn(float a) { return fu(a) & 0x80000000u; }
/* roundps: nearest-even / toward -inf; NaN stays (quieted). */
static inline float xround(float a) { return is_nan(a) ? quiet(a) : rintf(a); }
static inline float xfloor(float a) { return is_nan(a) ? quiet(a) : floorf(a); }
/* cvttps2dq: truncate; NaN and out-of-range give 0x80000000. */
static inline int32_t xcvtt(float a)
{
  if (!(a > -2147483904.0f && a < 2147483648.0f)) return INT32_MIN;
  return (int32_t)a;
}
/* RCPPS from the measured table (x86_tables.h); exhaustively verified rules. */
static inline float xrcp(float a)
{
  uint32_t x = fu(a), s = x & 0x80000000u, E = (x >> 23) & 0xFF;
  if (E == 255) return uf((x & 0x7FFFFF) ? (x | 0x400000u) : s);
  if (E == 0) return uf(s | 0x7F800000u);
  uint32_t t = kX86RcpTable[(x >> 12) & 0x7FF];
  int re = (int)((t >> 23) & 0xFF) + 127 - (int)E;
  return uf(re <= 0 ? s : (s | ((uint32_t)re << 23) | (t & 0x7FFFFFu)));
}
/* DPPS with imm8 = 0xFF (sum of all four products) per the Intel SDM:
 * (p0 + p1) + (p2 + p3), result broadcast. */
static inline float xdp4(const float* a, const float* b)
{
  float p0 = xmul(a[0], b[0]), p1 = xmul(a[1], b[1]), p2 = xmul(a[2], b[2]), p3 = xmul(a[3], b[3]);
  return xadd(xadd(p0, p1), xadd(p2, p3));
}
/* packDepthPremultiplied for one lane: float bits >> 12 (arithmetic), then
 * unsigned saturation to 16 bits (Rasterizer.cpp:508-525). */
static inline uint16_t pack_depth(float d)
{
  int32_t v = (int32_t)fu(d) >> 12;
  return (uint16_t)(v < 0 ? 0 : (v > 65535 ? 65535 : v));
}
static inline uint16_t avg16(uint16_t a, uint16_t b) { return (uint16_t)(((uint32_t)a + b + 1) >> 1); }

/* ---- constants (Rasterizer.cpp:9-17) --------------------------------------- */

#define OFFSET_Q 64
#define SLOPE_Q 64
static const float kBias = 2.5237386e-29f;     /* floatCompressionBias */
static const float kMinEdgeOffset = -0.45f;

enum { Culled = 0, Triangle0, Triangle1, ConcaveRight, ConcaveLeft, ConcaveCenter, Convex };

/* Primitive mode per 8-bit configuration: bits 0-3 = area of triangle k is
 * <= 0 (k = 0..3, triangles (0,1,2), (1,2,3), (2,3,0), (3,0,1)), bits 4-7 =
 * vertex k has W < 0.  Same classification as Rasterizer.cpp:30-64. */
static const uint8_t kModeTable[256] = {
#define CV Convex
#define T0 Triangle0
#define T1 Triangle1
#define CR ConcaveRight
#define CL ConcaveLeft
#define CC ConcaveCenter
#define NO Culled
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

struct orc_raster {
  uint32_t width, height, blocksX, blocksY;
  int wrap16;
  float mvp[16]; /* prebaked columns (Rasterizer.cpp:100-104) */
  float raw[16]; /* rows of the transposed input (Rasterizer.cpp:86-89) */
  int64_t table[OFFSET_Q * SLOPE_Q];
  uint16_t* depth; /* width*height, 8x8 blocks of 8 rows x 8 pixels, block-major */
  uint16_t* hiz;   /* blocks + 8 */
  uint32_t hizCount;
  uint64_t counters[5];
  orc_raster* scratch; /* never drawn into; used by orc_frame_plain */
};

/* ---- coverage-mask table (Rasterizer.cpp:470-480, 496-506, 527-604) -------- */

static uint64_t transpose_mask(uint64_t m)
{
  /* sample (x, y) at bit 8x+y  ->  bit 8x + (y even ? 4 + y/2 : (y-1)/2) */
  uint64_t out = 0;
  for (int x = 0; x < 8; ++x)
    for (int y = 0; y < 8; ++y)
      if ((m >> (8 * x + y)) & 1) out |= 1ull << (8 * x + ((y & 1) ? (y >> 1) : 4 + (y >> 1)));
  return out;
}

static void build_table(int64_t* table)
{
  memset(table, 0, sizeof(int64_t) * OFFSET_Q * SLOPE_Q);
  const uint32_t angular = 2000, offsets = 2000;
  const float maxOffset = -kMinEdgeOffset;
  for (uint32_t i = 0; i < angular; ++i) {
    float angle = -0.1f + 6.4f * (float)i / (float)(angular - 1);
    float nx = cosf(angle), ny = sinf(angle);
    float l = 1.0f / (fabsf(nx) + fabsf(ny));
    nx *= l;
    ny *= l;
    /* slope index with the table-build quantiser (strict ny < 0) */
    const float smul = (SLOPE_Q / 2 - 1) * 0.5f;
    const float sadd = smul + 0.5f;
    int32_t q = xcvtt(fmaf(nx, smul, sadd));
    uint32_t yneg = (ny < 0.0f) ? 0xFFFFFFFFu : 0u;
    uint32_t slope = (((uint32_t)q << 1) - yneg) << 6;
    for (uint32_t j = 0; j < offsets; ++j) {
      float offset = -0.6f + 1.2f * (float)j / (float)(angular - 1);
      const float omul = (OFFSET_Q - 1) / (maxOffset - kMinEdgeOffset);
      const float oadd = 0.5f - kMinEdgeOffset * omul;
      float lookup = offset * omul + oadd;
      int32_t oi = (int32_t)lookup;
      if (oi < 0) oi = 0;
      if (oi > OFFSET_Q - 1) oi = OFFSET_Q - 1;
      uint64_t block = 0;
      for (int x = 0; x < 8; ++x)
        for (int y = 0; y < 8; ++y) {
          float d = offset + (x - 3.5f) / 8.0f * nx + (y - 3.5f) / 8.0f * ny;
          if (d <= 0.0f) block |= 1ull << (8 * x + y);
        }
      table[slope | (uint32_t)oi] |= (int64_t)transpose_mask(block);
    }
  }
}

/* ---- lifetime -------------------------------------------------------------- */

orc_raster* orc_create(uint32_t width, uint32_t height, const int64_t* table)
{
  if (width % 8 || height % 8 || !width || !height) return NULL;
  orc_raster* r = (orc_raster*)calloc(1, sizeof(orc_raster));
  r->width = width;
  r->height = height;
  r->blocksX = width / 8;
  r->blocksY = height / 8;
  r->wrap16 = 1;
  r->hizCount = r->blocksX * r->blocksY + 8;
  r->depth = (uint16_t*)calloc((size_t)width * height, 2);
  r->hiz = (uint16_t*)calloc(r->hizCount, 2);
  if (table) memcpy(r->table, table, sizeof(r->table));
  else build_table(r->table);
  return r;
}

void orc_destroy(orc_raster* r)
{
  if (!r) return;
  orc_destroy(r->scratch);
  free(r->depth);
  free(r->hiz);
  free(r);
}

void orc_set_block_index_wrap(orc_raster* r, int wrap16) { r->wrap16 = wrap16 ? 1 : 0; }

/* Rasterizer.cpp:76-105 */
void orc_set_mvp(orc_raster* r, const float* m)
{
  /* rows of the transposed matrix: row i = (m[i], m[4+i], m[8+i], m[12+i]) */
  float row[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) row[i][j] = m[4 * j + i];
  memcpy(r->raw, row, sizeof(row));
  const float sx = (float)r->width * 0.5f - 4.0f;
  const float sy = (float)r->height * 0.5f - 4.0f;
  const float sz = 0.5f * kBias;
  float baked[4][4];
  for (int j = 0; j < 4; ++j) {
    baked[0][j] = xmul(xadd(row[0][j], row[3][j]), sx);
    baked[1][j] = xmul(xadd(row[1][j], row[3][j]), sy);
    baked[2][j] = xmul(xsub(row[3][j], row[2][j]), sz);
    baked[3][j] = row[3][j];
  }
  /* stored as columns: mvp[4*j + i] = baked[i][j] */
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r->mvp[4 * j + i] = baked[i][j];
}

/* Rasterizer.cpp:107-121: only hiZ is reset; depth keeps its stale contents. */
void orc_clear(orc_raster* r)
{
  for (uint32_t i = 0; i < r->hizCount; ++i) r->hiz[i] = 1;
  memset(r->counters, 0, sizeof(r->counters));
}

/* ---- rasterize<possiblyNearClipped> (Rasterizer.cpp:606-1295) -------------- */

typedef struct {
  int mode;
  int32_t minX, minY, rangeX, rangeY;
  uint16_t maxZ;
  float plane[3];          /* depth at block origin, d/dx, d/dy (block units) */
  float nx[4], ny[4], off[4];
  uint32_t slope[4];
} QuadSetup;

/* Per-occluder prologue (Rasterizer.cpp:612-655). rows[i] = output i's
 * coefficients for (X word, Y word, Z word, 1); c0/c1 give Z from 1/W. */
static void occluder_prologue(const orc_raster* r, const float* refMin, const float* refMax,
                              float rows[4][4], float* c0out, float* c1out)
{
  float col[4][4];
  for (int j = 0; j < 4; ++j)
    for (int i = 0; i < 4; ++i) col[j][i] = r->mvp[4 * j + i];
  float ext[4];
  for (int i = 0; i < 4; ++i) ext[i] = xsub(refMax[i], refMin[i]);
  float c3[4];
  for (int i = 0; i < 4; ++i)
    c3[i] = xfmadd(col[0][i], refMin[0], xfmadd(col[1][i], refMin[1], xfmadd(col[2][i], refMin[2], col[3][i])));
  const float s0 = xmul(ext[0], 1.0f / (float)(2047ull << 21));
  const float s1 = xmul(ext[1], 1.0f / (float)(2047 << 10));
  const float s2 = xmul(ext[2], 1.0f / (float)1023);
  float n0[4], n1[4], n2[4];
  for (int i = 0; i < 4; ++i) {
    n0[i] = xmul(col[0][i], s0);
    n1[i] = xmul(col[1][i], s1);
    n2[i] = xmul(col[2][i], s2);
  }
  for (int i = 0; i < 4; ++i) c3[i] = xfmadd(n0[i], (float)(1024ull << 21), c3[i]);
  for (int i = 0; i < 4; ++i) {
    n1[i] = xsub(n1[i], n0[i]);
    n2[i] = xsub(n2[i], n0[i]);
  }
  for (int i = 0; i < 4; ++i) {
    rows[i][0] = n0[i];
    rows[i][1] = n1[i];
    rows[i][2] = n2[i];
    rows[i][3] = c3[i];
  }
  const float w[4] = {(float)(1 << 21), (float)(1 << 10), 1.0f, 1.0f};
  float Za = rows[2][3], Zb = xdp4(rows[2], w);
  float Wa = rows[3][3], Wb = xdp4(rows[3], w);
  float c0 = xdiv(xsub(Za, Zb), xsub(Wa, Wb));
  *c0out = c0;
  *c1out = xfnmadd(c0, Wa, Za);
}

/* Setup of one quad (one SIMD lane of Rasterizer.cpp:660-1081). Returns 0 if
 * the quad is culled or outside the frustum. */
static int quad_setup(const orc_raster* r, const uint32_t* w4, float rows[4][4], float c0, float c1,
                      int nc, QuadSetup* s)
{
  const uint32_t maskY = 2047u << 10, maskZ = 1023u;
  float X[4], Y[4], W[4], invW[4], x[4], y[4], z[4];
  uint32_t ws[4];
  for (int j = 0; j < 4; ++j) {
    float Xf = (float)(int32_t)w4[j];
    float Yf = (float)(int32_t)(w4[j] & maskY);
    float Zf = (float)(int32_t)(w4[j] & maskZ);
    X[j] = xfmadd(Xf, rows[0][0], xfmadd(Yf, rows[0][1], xfmadd(Zf, rows[0][2], rows[0][3])));
    Y[j] = xfmadd(Xf, rows[1][0], xfmadd(Yf, rows[1][1], xfmadd(Zf, rows[1][2], rows[1][3])));
    W[j] = xfmadd(Xf, rows[3][0], xfmadd(Yf, rows[3][1], xfmadd(Zf, rows[3][2], rows[3][3])));
  }
  const float maxInvW = sqrtf(FLT_MAX);
  for (int j = 0; j < 4; ++j) {
    invW[j] = nc ? xmin(maxInvW, xmax(-maxInvW, xrcp(W[j]))) : xrcp(W[j]);
    x[j] = xmul(xround(xmul(X[j], invW[j])), 0.125f);
    y[j] = xmul(xround(xmul(Y[j], invW[j])), 0.125f);
    ws[j] = nc ? sgn(invW[j]) : 0u;
  }
  float eX[5], eY[5];
  eX[0] = xsub(y[1], y[0]); eX[1] = xsub(y[2], y[1]); eX[2] = xsub(y[3], y[2]); eX[3] = xsub(y[0], y[3]);
  eY[0] = xsub(x[0], x[1]); eY[1] = xsub(x[1], x[2]); eY[2] = xsub(x[2], x[3]); eY[3] = xsub(x[3], x[0]);
  float area0 = xfmsub(eX[0], eY[1], xmul(eX[1], eY[0]));
  float area1 = xfmsub(eX[1], eY[2], xmul(eX[2], eY[1]));
  float area2 = xfmsub(eX[2], eY[3], xmul(eX[3], eY[2]));
  float area3 = xsub(xadd(area0, area2), area1);
  /* area signs (zero counts as back-facing); flipped per vertex with W < 0 */
  uint32_t cfg = 0;
  cfg |= (xxor(area0, ws[0] ^ ws[1] ^ ws[2]) <= 0.0f) ? 1u : 0u;
  cfg |= (xxor(area1, ws[1] ^ ws[2] ^ ws[3]) <= 0.0f) ? 2u : 0u;
  cfg |= (xxor(area2, ws[0] ^ ws[2] ^ ws[3]) <= 0.0f) ? 4u : 0u;
  cfg |= (xxor(area3, ws[1] ^ ws[0] ^ ws[3]) <= 0.0f) ? 8u : 0u;
  if (nc) cfg |= (ws[0] >> 27) | (ws[1] >> 26) | (ws[2] >> 25) | (ws[3] >> 24);
  int mode = kModeTable[cfg];
  if (mode == Culled) return 0;

  float minFx, minFy, maxFx, maxFy;
  if (nc) {
    /* clipless bounding box (Rasterizer.cpp:820-909) */
    const float infP = 10000.0f, infN = -10000.0f;
    float mPx[4], mPy[4], MPx[4], MPy[4], mNx[4], mNy[4], MNx[4], MNy[4];
    for (int j = 0; j < 4; ++j) {
      mPx[j] = ws[j] ? infP : x[j];
      mPy[j] = ws[j] ? infP : y[j];
      MPx[j] = xxor(mPx[j], ws[j]);
      MPy[j] = xxor(mPy[j], ws[j]);
      mNx[j] = ws[j] ? x[j] : infP;
      mNy[j] = ws[j] ? y[j] : infP;
      MNx[j] = ws[j] ? x[j] : infN;
      MNy[j] = ws[j] ? y[j] : infN;
    }
    float minPx = xmin(xmin(mPx[0], mPx[1]), xmin(mPx[2], mPx[3]));
    float minPy = xmin(xmin(mPy[0], mPy[1]), xmin(mPy[2], mPy[3]));
    float maxPx = xmax(xmax(MPx[0], MPx[1]), xmax(MPx[2], MPx[3]));
    float maxPy = xmax(xmax(MPy[0], MPy[1]), xmax(MPy[2], MPy[3]));
    float minNx = xmin(xmin(mNx[0], mNx[1]), xmin(mNx[2], mNx[3]));
    float minNy = xmin(xmin(mNy[0], mNy[1]), xmin(mNy[2], mNy[3]));
    float maxNx = xmax(xmax(MNx[0], MNx[1]), xmax(MNx[2], MNx[3]));
    float maxNy = xmax(xmax(MNy[0], MNy[1]), xmax(MNy[2], MNy[3]));
    float incAx = (maxNx > minPx) ? infN : minPx;
    float incAy = (maxNy > minPy) ? infN : minPy;
    float incBx = (maxPx > minNx) ? infP : maxPx;
    float incBy = (maxPy > minNy) ? infP : maxPy;
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
  int32_t minX = xcvtt(xadd(minFx, 4.9999f / 8.0f));
  int32_t minY = xcvtt(xadd(minFy, 4.9999f / 8.0f));
  int32_t maxX = xcvtt(xadd(maxFx, 11.0f / 8.0f));
  int32_t maxY = xcvtt(xadd(maxFy, 11.0f / 8.0f));
  if (minX < 0) minX = 0;
  if (minY < 0) minY = 0;
  if (maxX > (int32_t)r->blocksX) maxX = (int32_t)r->blocksX;
  if (maxY > (int32_t)r->blocksY) maxY = (int32_t)r->blocksY;
  if (!(maxX > minX && maxY > minY)) return 0;

  for (int j = 0; j < 4; ++j) z[j] = xfmadd(invW[j], c1, c0);
  float maxZ = xmax(xmax(z[0], z[1]), xmax(z[2], z[3]));
  if (nc && (ws[0] | ws[1] | ws[2] | ws[3])) maxZ = 1.0f;

  /* depth plane of the larger-area triangle (Rasterizer.cpp:963-999) */
  int t0 = mode == Triangle0, t1 = mode == Triangle1;
  int greater = xabs(area0) < xabs(area2);
  greater = !t0 && (t1 || greater);
  float a = greater ? area2 : area0;
  float invArea = nc ? xdiv(1.0f, a) : xrcp(a);
  float z12 = xsub(z[1], z[2]), z20 = xsub(z[2], z[0]), z30 = xsub(z[3], z[0]);
  eX[4] = xsub(y[0], y[2]);
  eY[4] = xsub(x[2], x[0]);
  float dx = greater ? xfnmadd(z20, eX[3], xmul(z30, eX[4])) : xfmsub(z20, eX[1], xmul(z12, eX[4]));
  float dy = greater ? xfnmadd(z20, eY[3], xmul(z30, eY[4])) : xfmsub(z20, eY[1], xmul(z12, eY[4]));
  float plane1 = xmul(invArea, dx);
  float plane2 = xmul(invArea, dy);
  float x0 = xsub(x[0], (float)minX);
  float y0 = xsub(y[0], (float)minY);
  float plane0 = xfnmadd(x0, plane1, xfnmadd(y0, plane2, z[0]));

  /* triangle modes swap in the diagonal edge (Rasterizer.cpp:1001-1005) */
  if (t0) { eX[2] = eX[4]; eY[2] = eY[4]; }
  if (t1) { eX[0] = xxor(eX[4], 0x80000000u); eY[0] = xxor(eY[4], 0x80000000u); }
  uint32_t flip[4] = {0, 0, 0, 0};
  if (nc) {
    flip[0] = ws[0] ^ (t1 ? ws[2] : ws[1]);
    flip[1] = ws[1] ^ ws[2];
    flip[2] = ws[2] ^ (t0 ? ws[0] : ws[3]);
    flip[3] = ws[0] ^ ws[3];
  }
  /* normalizeEdge (Rasterizer.cpp:452-468) */
  const float maxOffset = -kMinEdgeOffset;
  const float nmul = (OFFSET_Q - 1) / (maxOffset - kMinEdgeOffset);
  for (int e = 0; e < 4; ++e) {
    float invLen = xrcp(xadd(xabs(eX[e]), xabs(eY[e])));
    float mul = nc ? xxor(nmul, flip[e]) : nmul;
    invLen = xmul(mul, invLen);
    eX[e] = xmul(eX[e], invLen);
    eY[e] = xmul(eY[e], invLen);
  }
  const float add = 0.5f - kMinEdgeOffset * (OFFSET_Q - 1) / (maxOffset - kMinEdgeOffset);
  float off[4];
  off[0] = xfnmadd(x0, eX[0], xfnmadd(y0, eY[0], add));
  off[1] = xfnmadd(x[1], eX[1], xfnmadd(y[1], eY[1], add));
  off[2] = xfnmadd(x[2], eX[2], xfnmadd(y[2], eY[2], add));
  off[3] = xfnmadd(x[3], eX[3], xfnmadd(y[3], eY[3], add));
  for (int e = 1; e < 4; ++e) off[e] = xfmadd((float)minX, eX[e], off[e]);
  for (int e = 1; e < 4; ++e) off[e] = xfmadd((float)minY, eY[e], off[e]);
  /* quantizeSlopeLookup, runtime form (Rasterizer.cpp:482-493) */
  const float smul = (SLOPE_Q / 2 - 1) * 0.5f / ((OFFSET_Q - 1) / (maxOffset - kMinEdgeOffset));
  const float sadd = (SLOPE_Q / 2 - 1) * 0.5f + 0.5f;
  for (int e = 0; e < 4; ++e) {
    uint32_t yneg = (eY[e] <= 0.0f) ? 0xFFFFFFFFu : 0u;
    uint32_t q = (uint32_t)xcvtt(xfmadd(eX[e], smul, sadd));
    s->slope[e] = ((q << 1) - yneg) << 6;
  }
  s->mode = mode;
  s->minX = minX;
  s->minY = minY;
  s->rangeX = maxX - minX;
  s->rangeY = maxY - minY;
  s->maxZ = pack_depth(maxZ);
  s->plane[0] = plane0;
  s->plane[1] = plane1;
  s->plane[2] = plane2;
  for (int e = 0; e < 4; ++e) {
    s->nx[e] = eX[e];
    s->ny[e] = eY[e];
    s->off[e] = off[e];
  }
  return 1;
}

/* Per-block loop of one quad (Rasterizer.cpp:1098-1292). */
static void quad_raster(orc_raster* r, const QuadSetup* s, int nc)
{
  const float dsp = -0.5f + 1.0f / 16.0f;
  const float lx[8] = {dsp + 0.0f, dsp + 0.125f, dsp + 0.25f, dsp + 0.375f,
                       dsp + 0.0f, dsp + 0.125f, dsp + 0.25f, dsp + 0.375f};
  const float ly[8] = {dsp, dsp, dsp, dsp, dsp + 0.125f, dsp + 0.125f, dsp + 0.125f, dsp + 0.125f};
  const float Dx = s->plane[1], Dy = s->plane[2];
  float lineDepth[8], lineOff[4];
  for (int k = 0; k < 8; ++k) lineDepth[k] = xfmadd(Dx, lx[k], xfmadd(Dy, ly[k], s->plane[0]));
  for (int e = 0; e < 4; ++e) lineOff[e] = s->off[e];

  uint32_t bX = r->blocksX;
  uint32_t first = r->wrap16 ? (((uint32_t)s->minY * bX) & 0xFFFFu) + (uint32_t)s->minX
                             : (uint32_t)s->minY * bX + (uint32_t)s->minX;
  for (int32_t by = 0; by < s->rangeY; ++by) {
    float off[4], depth[8];
    memcpy(off, lineOff, sizeof(off));
    memcpy(depth, lineDepth, sizeof(depth));
    int anyHit = 0;
    for (int32_t bx = 0; bx < s->rangeX; ++bx) {
      uint32_t blk = first + (uint32_t)by * bX + (uint32_t)bx;
      uint16_t hiZ = r->hiz[blk];
      r->counters[2]++;
      int draw = 1;
      uint64_t mask = 0;
      if (hiZ >= s->maxZ) {
        r->counters[3]++;
        draw = 0;
      } else if (s->mode == Convex) {
        int outside = 0;
        for (int e = 0; e < 4; ++e) outside |= off[e] >= (float)(OFFSET_Q - 1);
        if (outside) {
          if (anyHit) break;
          draw = 0;
        } else {
          anyHit = 1;
          mask = ~0ull;
          for (int e = 0; e < 4; ++e) {
            int32_t o = xcvtt(off[e]);
            if (o < 0) o = 0;
            mask &= (uint64_t)r->table[(s->slope[e] | (uint32_t)o) & 4095u];
          }
        }
      } else {
        uint64_t L[4];
        for (int e = 0; e < 4; ++e) {
          int32_t o = xcvtt(off[e]);
          if (o < 0) o = 0;
          if (o > OFFSET_Q - 1) o = OFFSET_Q - 1;
          L[e] = (uint64_t)r->table[(s->slope[e] | (uint32_t)o) & 4095u];
        }
        switch (s->mode) {
          case Triangle0: mask = L[0] & L[1] & L[2]; break;
          case Triangle1: mask = L[0] & L[2] & L[3]; break;
          case ConcaveRight: mask = (L[0] | L[3]) & (L[1] & L[2]); break;
          default:
            if (nc) { mask = (L[0] & L[1]) | (L[2] & L[3]); break; }
            /* fall through */
          case ConcaveLeft: mask = (L[0] & L[3]) & (L[1] | L[2]); break;
        }
        if (!mask) draw = 0;
      }
      if (draw) {
        float d0[8], d1[8], d8[8], d9[8];
        uint16_t row[10][8];
        for (int k = 0; k < 8; ++k) {
          d0[k] = depth[k];
          d1[k] = xfmadd(Dx, 0.5f, d0[k]);
          d8[k] = xadd(Dy, d0[k]);
          d9[k] = xadd(Dy, d1[k]);
        }
        /* rows 0,1 from (d0,d1); rows 8,9 from (d8,d9); lanes 0-3 even row, 4-7 odd */
        for (int k = 0; k < 4; ++k) {
          row[0][k] = pack_depth(d0[k]);     row[0][k + 4] = pack_depth(d1[k]);
          row[1][k] = pack_depth(d0[k + 4]); row[1][k + 4] = pack_depth(d1[k + 4]);
          row[8][k] = pack_depth(d8[k]);     row[8][k + 4] = pack_depth(d9[k]);
          row[9][k] = pack_depth(d8[k + 4]); row[9][k + 4] = pack_depth(d9[k + 4]);
        }
        for (int x = 0; x < 8; ++x) {
          row[4][x] = avg16(row[0][x], row[8][x]);
          row[5][x] = avg16(row[1][x], row[9][x]);
          row[2][x] = avg16(row[0][x], row[4][x]);
          row[3][x] = avg16(row[1][x], row[5][x]);
          row[6][x] = avg16(row[4][x], row[8][x]);
          row[7][x] = avg16(row[5][x], row[9][x]);
        }
        uint16_t* out = r->depth + (size_t)blk * 64;
        uint16_t mn = 0xFFFF;
        for (int yy = 0; yy < 8; ++yy)
          for (int x = 0; x < 8; ++x) {
            uint16_t v = row[yy][x];
            int bit = 8 * x + ((yy & 1) ? (yy >> 1) : 4 + (yy >> 1));
            if (mask != ~0ull && !((mask >> bit) & 1)) v = 0;
            if (hiZ != 1 && out[8 * yy + x] > v) v = out[8 * yy + x];
            out[8 * yy + x] = v;
            if (v < mn) mn = v;
          }
        r->hiz[blk] = mn;
        r->counters[4]++;
      }
      for (int k = 0; k < 8; ++k) depth[k] = xadd(Dx, depth[k]);
      for (int e = 0; e < 4; ++e) off[e] = xadd(s->nx[e], off[e]);
    }
    for (int k = 0; k < 8; ++k) lineDepth[k] = xadd(lineDepth[k], Dy);
    for (int e = 0; e < 4; ++e) lineOff[e] = xadd(lineOff[e], s->ny[e]);
  }
}

/* Setup of every quad of one occluder without rasterising (statistics for the
 * tests and benchmarks): per valid quad minX, minY, maxX, maxY (blocks,
 * [min, max)), maxZ, mode.  Returns the number of valid quads written. */
uint32_t orc_setup_dump(orc_raster* r, const uint32_t* packed, uint32_t packetCount, const float* refMin,
                        const float* refMax, int nearClip, int32_t* out6)
{
  float rows[4][4], c0, c1;
  occluder_prologue(r, refMin, refMax, rows, &c0, &c1);
  uint32_t n = 0;
  for (uint32_t p = 0; p + 4 <= packetCount; p += 4) {
    const uint32_t* base = packed + (size_t)p * 8;
    for (int q = 0; q < 8; ++q) {
      uint32_t w4[4] = {base[q], base[8 + q], base[16 + q], base[24 + q]};
      QuadSetup s;
      if (!quad_setup(r, w4, rows, c0, c1, nearClip, &s)) continue;
      int32_t* o = out6 + 6 * n++;
      o[0] = s.minX; o[1] = s.minY; o[2] = s.minX + s.rangeX; o[3] = s.minY + s.rangeY; o[4] = s.maxZ; o[5] = s.mode;
    }
  }
  return n;
}

void orc_rasterize(orc_raster* r, const uint32_t* packed, uint32_t packetCount, const float* refMin,
                   const float* refMax, int nearClip)
{
  float rows[4][4], c0, c1;
  occluder_prologue(r, refMin, refMax, rows, &c0, &c1);
  for (uint32_t p = 0; p + 4 <= packetCount; p += 4) {
    const uint32_t* base = packed + (size_t)p * 8;
    for (int q = 0; q < 8; ++q) {
      uint32_t w4[4] = {base[q], base[8 + q], base[16 + q], base[24 + q]};
      QuadSetup s;
      r->counters[0]++;
      if (!quad_setup(r, w4, rows, c0, c1, nearClip, &s)) continue;
      r->counters[1]++;
      quad_raster(r, &s, nearClip);
    }
  }
}

/* ---- queryVisibility / query2D (Rasterizer.cpp:123-349) -------------------- */

int orc_query2d(const orc_raster* r, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ)
{
  uint32_t bx0 = minX / 8, bx1 = maxX / 8, by0 = minY / 8, by1 = maxY / 8;
  for (uint32_t by = by0; by <= by1; ++by) {
    int32_t sy = (int32_t)(minY - 8 * by); if (sy < 0) sy = 0;
    int32_t ey = (int32_t)(maxY - 8 * by); if (ey > 7) ey = 7;
    int interiorLine = sy == 0 && ey == 7;
    for (uint32_t bx = bx0; bx <= bx1; ++bx) {
      uint32_t blk = by * r->blocksX + bx;
      if (maxZ <= r->hiz[blk]) continue;
      int32_t sx = (int32_t)(minX - bx * 8); if (sx < 0) sx = 0;
      int32_t ex = (int32_t)(maxX - bx * 8); if (ex > 7) ex = 7;
      if (interiorLine && sx == 0 && ex == 7) return 1;
      const uint16_t* d = r->depth + (size_t)blk * 64;
      for (int32_t yy = sy; yy <= ey; ++yy)
        for (int32_t x = sx; x <= ex; ++x)
          if (d[8 * yy + x] < maxZ) return 1;
    }
  }
  return 0;
}

int orc_query(orc_raster* r, const float* bmin, const float* bmax, int* needsClipping)
{
  float ext[4], ctr[4];
  for (int i = 0; i < 4; ++i) {
    ext[i] = xsub(bmax[i], bmin[i]);
    ctr[i] = xadd(bmax[i], bmin[i]);
  }
  const float* row0 = r->raw;
  const float* row1 = r->raw + 4;
  const float* row2 = r->raw + 8;
  const float* row3 = r->raw + 12;
  uint32_t signs = 0;
  for (int p = 0; p < 6; ++p) {
    const float* rr = p < 2 ? row0 : (p < 4 ? row1 : row2);
    float plane[4], offs[4];
    for (int i = 0; i < 4; ++i) {
      plane[i] = (p & 1) ? xsub(row3[i], rr[i]) : xadd(row3[i], rr[i]);
      offs[i] = xadd(ctr[i], xxor(ext[i], sgn(plane[i])));
    }
    signs |= fu(xdp4(plane, offs));
  }
  if (signs & 0x80000000u) return 0;

  const float* col0 = r->mvp;
  const float* col1 = r->mvp + 4;
  const float* col2 = r->mvp + 8;
  const float* col3 = r->mvp + 12;
  float e0[4], e1[4], e2[4], c[8][4];
  for (int i = 0; i < 4; ++i) {
    e0[i] = xmul(col0[i], ext[0]);
    e1[i] = xmul(col1[i], ext[1]);
    e2[i] = xmul(col2[i], ext[2]);
    c[0][i] = xfmadd(col0[i], bmin[0], xfmadd(col1[i], bmin[1], xfmadd(col2[i], bmin[2], col3[i])));
  }
  for (int i = 0; i < 4; ++i) {
    c[1][i] = xadd(c[0][i], e0[i]);
    c[2][i] = xadd(c[0][i], e1[i]);
    c[4][i] = xadd(c[0][i], e2[i]);
    c[3][i] = xadd(c[1][i], e1[i]);
    c[5][i] = xadd(c[4][i], e0[i]);
    c[6][i] = xadd(c[2][i], e2[i]);
    c[7][i] = xadd(c[6][i], e0[i]);
  }
  /* SoA: X[k], Y[k], Z[k], W[k] for corner k */
  float X[8], Y[8], Z[8], W[8];
  for (int k = 0; k < 8; ++k) { X[k] = c[k][0]; Y[k] = c[k][1]; Z[k] = c[k][2]; W[k] = c[k][3]; }
  /* per-lane near-plane epsilon (Rasterizer.cpp:205-207) */
  float m1[4] = {xmax(ext[0], ext[2]), xmax(ext[1], ext[3]), xmax(ext[2], ext[0]), xmax(ext[3], ext[1])};
  float me[4] = {xmax(m1[0], m1[1]), xmax(m1[1], m1[0]), xmax(m1[2], m1[3]), xmax(m1[3], m1[2])};
  int close = 0;
  for (int i = 0; i < 4; ++i) {
    float eps = xmul(me[i], 0.001f);
    close |= (W[i] < eps) || (W[4 + i] < eps);
  }
  if (close) { *needsClipping = 1; return 1; }
  *needsClipping = 0;
  for (int i = 0; i < 4; ++i) {
    float iw = xrcp(W[i]);
    X[i] = xmul(X[i], iw); Y[i] = xmul(Y[i], iw); Z[i] = xmul(Z[i], iw);
    float iw2 = xrcp(W[4 + i]);
    X[4 + i] = xmul(X[4 + i], iw2); Y[4 + i] = xmul(Y[4 + i], iw2); Z[4 + i] = xmul(Z[4 + i], iw2);
  }
  float mnX[4], mxX[4], mnY[4], mxY[4];
  for (int i = 0; i < 4; ++i) {
    mnX[i] = xmin(X[i], X[4 + i]); mxX[i] = xmax(X[i], X[4 + i]);
    mnY[i] = xmin(Y[i], Y[4 + i]); mxY[i] = xmax(Y[i], Y[4 + i]);
  }
  /* horizontal reductions in the reference's lane order (Rasterizer.cpp:236-247) */
  float mn[4] = {xmin(mnX[0], mnX[2]), xmin(mnY[0], mnY[2]), xmin(mnX[1], mnX[3]), xmin(mnY[1], mnY[3])};
  float mx[4] = {xmax(mxX[0], mxX[2]), xmax(mxY[0], mxY[2]), xmax(mxX[1], mxX[3]), xmax(mxY[1], mxY[3])};
  const float lim[4] = {(float)(r->width - 1), (float)(r->height - 1), (float)(r->width - 1), (float)(r->height - 1)};
  for (int i = 0; i < 4; ++i) {
    mn[i] = xmax(mn[i], 0.0f);
    mx[i] = xmin(mx[i], lim[i]);
    mx[i] = xxor(mx[i], 0x80000000u);
  }
  float bf[4] = {xmin(mn[0], mn[2]), xmin(mx[0], mx[2]), xmin(mn[1], mn[3]), xmin(mx[1], mx[3])};
  int32_t b[4];
  for (int i = 0; i < 4; ++i) b[i] = xcvtt(xfloor(bf[i]));
  b[1] = (int32_t)(0u - (uint32_t)b[1]);
  b[3] = (int32_t)(0u - (uint32_t)b[3]);
  if (b[0] >= b[1] || b[2] >= b[3]) return 0;
  uint16_t maxZ = 0;
  for (int i = 0; i < 4; ++i) {
    uint16_t a = pack_depth(Z[i]), bb = pack_depth(Z[4 + i]);
    if (a > maxZ) maxZ = a;
    if (bb > maxZ) maxZ = bb;
  }
  return orc_query2d(r, (uint32_t)b[0], (uint32_t)b[1], (uint32_t)b[2], (uint32_t)b[3], maxZ);
}

void orc_query_batch(orc_raster* r, uint32_t n, const float* mins, const float* maxs, uint8_t* vis, uint8_t* nc)
{
  for (uint32_t i = 0; i < n; ++i) {
    int c = 0;
    vis[i] = (uint8_t)orc_query(r, mins + 4 * i, maxs + 4 * i, &c);
    nc[i] = (uint8_t)c;
  }
}

/* ---- read-back (Rasterizer.cpp:351-399) ------------------------------------ */

void orc_read_back(const orc_raster* r, uint8_t* rgba)
{
  const float invBias = 3.9623753e+28f;
  for (uint32_t by = 0; by < r->blocksY; ++by)
    for (uint32_t bx = 0; bx < r->blocksX; ++bx) {
      uint32_t blk = by * r->blocksX + bx;
      for (uint32_t yy = 0; yy < 8; ++yy) {
        uint8_t* dest = rgba + 4 * ((size_t)8 * bx + (size_t)r->width * (8 * by + yy));
        if (r->hiz[blk] == 1) { memset(dest, 0, 32); continue; }
        for (uint32_t x = 0; x < 8; ++x) {
          float depth = xmul(uf((uint32_t)r->depth[(size_t)blk * 64 + 8 * yy + x] << 12), invBias);
          float lin = xdiv(2 * 0.25f, xsub(0.25f + 1000.0f, xmul(xsub(1.0f, depth), 1000.0f - 0.25f)));
          float s = xmul((float)(100 * 256), lin);
          uint32_t d = (s >= 0.0f && s < 4294967296.0f) ? (uint32_t)(uint64_t)s : 0u;
          dest[4 * x + 0] = (uint8_t)(d / 100);
          dest[4 * x + 1] = (uint8_t)(d % 256);
          dest[4 * x + 2] = 0;
          dest[4 * x + 3] = 255;
        }
      }
    }
}

/* The values readBackDepth computes on the way to its bytes (:378-381), row-major,
   0 in cleared blocks: format 1 float linDepth, 2 float depth, 3 u16 packed depth. */
void orc_read_back_values(const orc_raster* r, int format, void* out)
{
  const float invBias = 3.9623753e+28f;
  for (uint32_t y = 0; y < r->height; ++y)
    for (uint32_t x = 0; x < r->width; ++x) {
      const uint32_t blk = (y >> 3) * r->blocksX + (x >> 3);
      const size_t o = (size_t)y * r->width + x;
      const int cleared = r->hiz[blk] == 1;
      const uint32_t v = cleared ? 0u : r->depth[(size_t)blk * 64 + 8 * (y & 7) + (x & 7)];
      const float depth = xmul(uf(v << 12), invBias);
      const float lin = xdiv(2 * 0.25f, xsub(0.25f + 1000.0f, xmul(xsub(1.0f, depth), 1000.0f - 0.25f)));
      if (format == 3) ((uint16_t*)out)[o] = (uint16_t)v;
      else if (format == 2) ((float*)out)[o] = cleared ? 0.0f : depth;
      else ((float*)out)[o] = cleared ? 0.0f : lin;
    }
}

void orc_read_depth(const orc_raster* r, uint16_t* out) { memcpy(out, r->depth, (size_t)r->width * r->height * 2); }
uint32_t orc_read_hiz(const orc_raster* r, uint16_t* out)
{
  if (out) memcpy(out, r->hiz, (size_t)r->hizCount * 2);
  return r->hizCount;
}
void orc_read_table(const orc_raster* r, int64_t* out) { memcpy(out, r->table, sizeof(r->table)); }
void orc_write_depth(orc_raster* r, const uint16_t* in) { memcpy(r->depth, in, (size_t)r->width * r->height * 2); }
void orc_write_hiz(orc_raster* r, const uint16_t* in) { memcpy(r->hiz, in, (size_t)r->hizCount * 2); }
void orc_read_counters(const orc_raster* r, uint64_t* out5) { memcpy(out5, r->counters, sizeof(r->counters)); }

void orc_frame_plain(orc_raster* r, uint32_t n, const uint32_t* const* occ_packed, const uint32_t* occ_packets,
                     const float* occ_ref, const float* occ_bounds, const float* mvp, uint8_t* flags)
{
  if (!r->scratch) r->scratch = orc_create(r->width, r->height, r->table);
  orc_clear(r);
  orc_set_mvp(r, mvp);
  orc_set_mvp(r->scratch, mvp);
  for (uint32_t k = 0; k < n; ++k) {
    int nc = 0;
    int vis = orc_query(r->scratch, occ_bounds + 8 * k, occ_bounds + 8 * k + 4, &nc);
    if (flags) flags[k] = (uint8_t)((vis ? 1 : 0) | (nc ? 2 : 0));
    if (!vis) continue;
    orc_rasterize(r, occ_packed[k], occ_packets[k], occ_ref + 8 * k, occ_ref + 8 * k + 4, nc);
  }
}

/* Main.cpp:181-206: front-to-back order by squared centre distance, each
 * occluder queried against the live buffer before it is drawn. */
typedef struct {
  float d;
  uint32_t k;
} dist_key;

static int cmp_dist(const void* a, const void* b)
{
  const dist_key* x = (const dist_key*)a;
  const dist_key* y = (const dist_key*)b;
  if (x->d < y->d) return -1;
  if (y->d < x->d) return 1;
  return x->k < y->k ? -1 : (x->k > y->k ? 1 : 0);
}

void orc_frame_gated(orc_raster* r, uint32_t n, const uint32_t* const* occ_packed, const uint32_t* occ_packets,
                     const float* occ_ref, const float* occ_bounds, const float* occ_centers, const float* eye,
                     const float* mvp, uint32_t* order_out, uint8_t* flags)
{
  dist_key* keys = (dist_key*)malloc(sizeof(dist_key) * (n ? n : 1));
  for (uint32_t k = 0; k < n; ++k) {
    /* _mm_dp_ps(d, d, 0x7f): x, y, z products, w masked to +0 */
    const float d[4] = {xsub(occ_centers[4 * k], eye[0]), xsub(occ_centers[4 * k + 1], eye[1]),
                        xsub(occ_centers[4 * k + 2], eye[2]), 0.0f};
    keys[k].d = xdp4(d, d);
    keys[k].k = k;
  }
  qsort(keys, n, sizeof(dist_key), cmp_dist);
  orc_clear(r);
  orc_set_mvp(r, mvp);
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t k = keys[i].k;
    if (order_out) order_out[i] = k;
    int nc = 0;
    const int vis = orc_query(r, occ_bounds + 8 * k, occ_bounds + 8 * k + 4, &nc);
    if (flags) flags[k] = (uint8_t)((vis ? 1 : 0) | (nc ? 2 : 0));
    if (vis) orc_rasterize(r, occ_packed[k], occ_packets[k], occ_ref + 8 * k, occ_ref + 8 * k + 4, nc);
  }
  free(keys);
}
