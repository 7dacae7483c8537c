// Learned occluder selection (sm_103a): per-occluder features, a small MLP
// scored with BF16 tensor-core MMA, per-view top-K, and the MLP's training
// kernels (forward with saved activations, backward, Adam).
//
// The reference draws every occluder that passes its visibility test, nearest
// first (Main.cpp:184-206).  Here an MLP 16 -> 64 -> 64 -> 1 scores each
// occluder of a view from screen-space and depth features of its bounds and
// from the pixels it won in the previous frame; the top K of each view's
// candidates are rasterised.  Dropping occluders only leaves depth farther
// (max-merge of a subset), so culls can only be lost, not gained.
//
// The network is tiny, so inference uses warp-level mma.sync m16n8k16 tiles
// (bf16 inputs, fp32 accumulation) chained in registers; training runs the
// same forward, then a backward and an Adam update on CUDA cores in fp32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "query_front.cuh"
#include "raster_types.h"

namespace occ {

constexpr int kParams = kHidden * kFeatures + kHidden + kHidden * kHidden + kHidden + kHidden + 1;  // 5313
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kHidden * kFeatures, kOffW2 = kOffB1 + kHidden,
              kOffB2 = kOffW2 + kHidden * kHidden, kOffW3 = kOffB2 + kHidden, kOffB3 = kOffW3 + kHidden;

// ---- features ------------------------------------------------------------------------------
// One thread per command.  Features (all roughly in [0, 1]):
//  0 passes the gating test      1 near-clipped (no screen rectangle)
//  2 log2(1 + rect pixels) / log2(1 + W*H)   3 rect pixels / (W*H)
//  4 rect centre x / W           5 rect centre y / H
//  6 nearest corner's packed depth / 65535   7 farthest corner's packed depth / 65535
//  8 log2(1 + distance of the bounds centre to the eye) / 12
//  9 log2(1 + quads) / 9         10 log2(1 + bounds diagonal) / 8
// 11 feature 8 rescaled to [0, 1] over the view's candidates (0 = nearest)   (k_view_norm)
// 12 rect pixels / the largest rect of the view's candidates                 (k_view_norm)
// 13 log2(1 + previous-launch wins) / log2(1 + W*H)
// 14 drawn in the previous launch
// 15 rank in the view's nearest-first order over its candidates, 0 = nearest,
//    1 = farthest (non-candidates 1)                                        (k_view_norm)
// Features 13-14 need win counting; without it they are 0.

// Eye position of a view: clip x = clip y = clip w = 0 (rows hold the
// matrix's columns, clip_i = rows[i] . (p, 1)), by Cramer's rule.
__device__ __forceinline__ void view_eye(const ViewDesc& V, float e[3])
{
  const float* r = V.rows;
  const float a00 = r[0], a01 = r[1], a02 = r[2], b0 = -r[3];
  const float a10 = r[4], a11 = r[5], a12 = r[6], b1 = -r[7];
  const float a20 = r[12], a21 = r[13], a22 = r[14], b2 = -r[15];
  const float c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22, c02 = a10 * a21 - a11 * a20;
  const float det = a00 * c00 + a01 * c01 + a02 * c02;
  if (!(fabsf(det) > 1e-30f)) {
    e[0] = e[1] = e[2] = 0.0f;
    return;
  }
  const float inv = 1.0f / det;
  e[0] = (b0 * c00 + a01 * (a12 * b2 - b1 * a22) + a02 * (b1 * a21 - a11 * b2)) * inv;
  e[1] = (a00 * (b1 * a22 - a12 * b2) + b0 * c01 + a02 * (a10 * b2 - b1 * a20)) * inv;
  e[2] = (a00 * (a11 * b2 - b1 * a21) + a01 * (b1 * a20 - a10 * b2) + b0 * c02) * inv;
}

__global__ void __launch_bounds__(256) k_features(FrameParams P, uint32_t numCmds)
{
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= numCmds) return;
  const Cmd& cmd = P.cmds[c];
  const ViewDesc& V = P.views[cmd.view];
  uint32_t rect[4] = {0, 0, 0, 0}, maxZ = 0, minZ = 0;
  const int st = query_front(V, cmd.boundsMin, cmd.boundsMax, rect, &maxZ, &minZ);
  const bool cand = st == 1 || (st == 2 && maxZ > 0);
  const float W = (float)V.width, H = (float)V.height, WH = W * H;
  float area = 0, cx = 0, cy = 0, rw = 0, rh = 0;
  if (st == 2) {
    rw = (float)(rect[1] - rect[0] + 1);
    rh = (float)(rect[3] - rect[2] + 1);
    area = rw * rh;
    cx = 0.5f * (float)(rect[0] + rect[1]) / W;
    cy = 0.5f * (float)(rect[2] + rect[3]) / H;
  } else if (st == 1) {
    area = WH;
    cx = cy = 0.5f;
    maxZ = 65535u;
    minZ = 0u;
  }
  float eye[3], d2 = 0.0f, diag2 = 0.0f;
  view_eye(V, eye);
  for (int i = 0; i < 3; ++i) {
    const float m = 0.5f * (cmd.boundsMin[i] + cmd.boundsMax[i]) - eye[i];
    const float e = cmd.boundsMax[i] - cmd.boundsMin[i];
    d2 += m * m;
    diag2 += e * e;
  }
  const uint32_t prev = P.wins ? P.wins[c] : 0u;
  if (P.wins) P.wins[c] = 0;  // this launch accumulates afresh
  const float lwh = log2f(1.0f + WH);
  float* f = P.feat + (size_t)c * kFeatures;
  f[0] = cand ? 1.0f : 0.0f;
  f[1] = st == 1 ? 1.0f : 0.0f;
  f[2] = log2f(1.0f + area) / lwh;
  f[3] = area / WH;
  f[4] = cx;
  f[5] = cy;
  f[6] = (float)maxZ / 65535.0f;
  f[7] = (float)minZ / 65535.0f;
  f[8] = log2f(1.0f + sqrtf(d2)) / 12.0f;
  f[9] = log2f(1.0f + (float)cmd.quadCount) / 9.0f;
  f[10] = log2f(1.0f + sqrtf(diag2)) / 8.0f;
  f[11] = 0.0f;  // k_view_norm
  f[12] = 0.0f;
  f[13] = log2f(1.0f + (float)prev) / lwh;
  f[14] = (P.cmdDraw[c] & 5u) ? 1.0f : 0.0f;  // drawn by either pass of the previous launch (k_gate)
  f[15] = 1.0f;  // k_view_norm: rank in the view's nearest-first order
  P.cand[c] = cand ? 1 : 0;
}

constexpr uint32_t kRankMaxCmds = 2048;  // views ranked exactly (larger: the normalised distance)

// Features 11, 12 and 15 of view v from its candidates (a CTA of 256
// threads): distance rescaled over the candidates, area relative to the
// largest, and the rank in the reference's nearest-first order (Main.cpp:
// 184-190: centre distance to the eye, equal distances in command order)
// over the candidates, 0 = nearest, 1 = farthest.
__device__ __forceinline__ void view_norm(const FrameParams& P, uint32_t v)
{
  __shared__ float s_red[3][8];
  __shared__ float s_dist[kRankMaxCmds];  // the view's candidates' distances (non-candidates: +inf)
  __shared__ uint32_t s_ncand;
  const ViewDesc& V = P.views[v];
  const uint32_t c0 = V.cmdStart, n = V.cmdCount;
  float dmin = 3.0e38f, dmax = -3.0e38f, amax = 0.0f;
  for (uint32_t i = threadIdx.x; i < n; i += 256) {
    if (!P.cand[c0 + i]) continue;
    const float* f = P.feat + (size_t)(c0 + i) * kFeatures;
    dmin = fminf(dmin, f[8]);
    dmax = fmaxf(dmax, f[8]);
    amax = fmaxf(amax, f[3]);
  }
  for (int o = 16; o; o >>= 1) {
    dmin = fminf(dmin, __shfl_xor_sync(0xFFFFFFFFu, dmin, o));
    dmax = fmaxf(dmax, __shfl_xor_sync(0xFFFFFFFFu, dmax, o));
    amax = fmaxf(amax, __shfl_xor_sync(0xFFFFFFFFu, amax, o));
  }
  const uint32_t w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_red[0][w] = dmin;
    s_red[1][w] = dmax;
    s_red[2][w] = amax;
  }
  __syncthreads();
  for (int k = 0; k < 8; ++k) {
    dmin = fminf(dmin, s_red[0][k]);
    dmax = fmaxf(dmax, s_red[1][k]);
    amax = fmaxf(amax, s_red[2][k]);
  }
  const float span = dmax - dmin;
  const bool exact = n <= kRankMaxCmds;
  if (threadIdx.x == 0) s_ncand = 0;
  __syncthreads();
  uint32_t nc = 0;
  for (uint32_t i = threadIdx.x; i < n; i += 256) {
    const bool cand = P.cand[c0 + i] != 0;
    nc += cand ? 1u : 0u;
    if (exact) s_dist[i] = cand ? P.feat[(size_t)(c0 + i) * kFeatures + 8] : __int_as_float(0x7F800000);
  }
  atomicAdd(&s_ncand, nc);
  __syncthreads();
  const float rankScale = s_ncand > 1 ? 1.0f / (float)(s_ncand - 1) : 0.0f;
  for (uint32_t i = threadIdx.x; i < n; i += 256) {
    float* f = P.feat + (size_t)(c0 + i) * kFeatures;
    if (P.cand[c0 + i]) {
      f[11] = span > 0.0f ? (f[8] - dmin) / span : 0.0f;
      f[12] = amax > 0.0f ? f[3] / amax : 0.0f;
      if (exact) {
        const float d = s_dist[i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < n; ++j) rank += (s_dist[j] < d || (s_dist[j] == d && j < i)) ? 1u : 0u;
        f[15] = (float)rank * rankScale;
      } else {
        f[15] = f[11];
      }
    } else {
      f[11] = 1.0f;
      f[12] = 0.0f;
      f[15] = 1.0f;
    }
  }
}

// One CTA per view: features 11, 12 and 15 (win counting without a selector).
__global__ void __launch_bounds__(256) k_view_norm(FrameParams P) { view_norm(P, blockIdx.x); }

// ---- MLP forward: mma.sync m16n8k16, bf16 x bf16 -> fp32 ------------------------------------

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// The network's weights in shared memory (bf16 pairs for the MMA operands).
struct MlpSmem {
  uint32_t w1[kHidden * kFeatures / 2];
  uint32_t w2[kHidden * kHidden / 2];
  float b1[kHidden], b2[kHidden], w3[kHidden];
};

__device__ __forceinline__ void mlp_load(MlpSmem& W, const MlpDevice* __restrict__ mlp)
{
  for (int i = threadIdx.x; i < kHidden * kFeatures / 2; i += blockDim.x)
    W.w1[i] = reinterpret_cast<const uint32_t*>(mlp->w1t)[i];
  for (int i = threadIdx.x; i < kHidden * kHidden / 2; i += blockDim.x)
    W.w2[i] = reinterpret_cast<const uint32_t*>(mlp->w2t)[i];
  for (int i = threadIdx.x; i < kHidden; i += blockDim.x) {
    W.b1[i] = mlp->b1[i];
    W.b2[i] = mlp->b2[i];
    W.w3[i] = mlp->w3[i];
  }
}

// Scores rows [tile*16, tile*16+16) of M rows of kFeatures floats (one warp).
// The warp's lane (g = lane/4, t = lane%4) holds, per the m16n8k16 fragment
// layout, rows g and g+8 and columns 2t, 2t+1 of every 8-column tile.  Layer
// 1's fp32 accumulators become layer 2's bf16 A fragments in registers.  With
// h1/h2/xb non-null the activations are saved for the backward pass.
__device__ __forceinline__ void mlp_tile(const MlpSmem& W, float b3, uint32_t tile, const float* __restrict__ feat,
                                         uint32_t M, float* __restrict__ score, float* h1out, float* h2out,
                                         float* xout)
{
  const uint32_t lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t* s_w1 = W.w1;
  const uint32_t* s_w2 = W.w2;
  const float* s_b1 = W.b1;
  const float* s_b2 = W.b2;
  const float* s_w3 = W.w3;
  const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
  auto x = [&](uint32_t r, uint32_t k) -> float { return r < M ? feat[(size_t)r * kFeatures + k] : 0.0f; };
  uint32_t a[4];
  a[0] = pack_bf16x2(x(r0, 2 * t), x(r0, 2 * t + 1));
  a[1] = pack_bf16x2(x(r1, 2 * t), x(r1, 2 * t + 1));
  a[2] = pack_bf16x2(x(r0, 8 + 2 * t), x(r0, 9 + 2 * t));
  a[3] = pack_bf16x2(x(r1, 8 + 2 * t), x(r1, 9 + 2 * t));
  if (xout) {
    const uint32_t ks[4] = {2 * t, 2 * t + 1, 8 + 2 * t, 9 + 2 * t};
    for (int i = 0; i < 4; ++i) {
      if (r0 < M) xout[(size_t)r0 * kFeatures + ks[i]] = bf16_round(x(r0, ks[i]));
      if (r1 < M) xout[(size_t)r1 * kFeatures + ks[i]] = bf16_round(x(r1, ks[i]));
    }
  }
  // layer 1: 8 column tiles of 8
  float h1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    h1[j][0] = h1[j][1] = h1[j][2] = h1[j][3] = 0.0f;
    const uint32_t n = 8 * j + g;
    mma_bf16_16816(h1[j], a, s_w1[(n * kFeatures + 2 * t) / 2], s_w1[(n * kFeatures + 8 + 2 * t) / 2]);
    const float c0 = s_b1[8 * j + 2 * t], c1 = s_b1[8 * j + 2 * t + 1];
    h1[j][0] = fmaxf(h1[j][0] + c0, 0.0f);
    h1[j][1] = fmaxf(h1[j][1] + c1, 0.0f);
    h1[j][2] = fmaxf(h1[j][2] + c0, 0.0f);
    h1[j][3] = fmaxf(h1[j][3] + c1, 0.0f);
  }
  // layer 2: A fragments from layer 1's accumulators, 4 k-chunks of 16
  uint32_t a2[4][4];
#pragma unroll
  for (int kc = 0; kc < 4; ++kc) {
    a2[kc][0] = pack_bf16x2(h1[2 * kc][0], h1[2 * kc][1]);
    a2[kc][1] = pack_bf16x2(h1[2 * kc][2], h1[2 * kc][3]);
    a2[kc][2] = pack_bf16x2(h1[2 * kc + 1][0], h1[2 * kc + 1][1]);
    a2[kc][3] = pack_bf16x2(h1[2 * kc + 1][2], h1[2 * kc + 1][3]);
  }
  if (h1out) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t col = 8 * j + 2 * t;
      if (r0 < M) {
        h1out[(size_t)r0 * kHidden + col] = bf16_round(h1[j][0]);
        h1out[(size_t)r0 * kHidden + col + 1] = bf16_round(h1[j][1]);
      }
      if (r1 < M) {
        h1out[(size_t)r1 * kHidden + col] = bf16_round(h1[j][2]);
        h1out[(size_t)r1 * kHidden + col + 1] = bf16_round(h1[j][3]);
      }
    }
  }
  float p0 = 0.0f, p1 = 0.0f;  // layer 3 partial dot products for rows r0, r1
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const uint32_t n = 8 * j + g;
#pragma unroll
    for (int kc = 0; kc < 4; ++kc)
      mma_bf16_16816(acc, a2[kc], s_w2[(n * kHidden + 16 * kc + 2 * t) / 2],
                     s_w2[(n * kHidden + 16 * kc + 8 + 2 * t) / 2]);
    const uint32_t col = 8 * j + 2 * t;
    const float v0 = fmaxf(acc[0] + s_b2[col], 0.0f), v1 = fmaxf(acc[1] + s_b2[col + 1], 0.0f);
    const float v2 = fmaxf(acc[2] + s_b2[col], 0.0f), v3 = fmaxf(acc[3] + s_b2[col + 1], 0.0f);
    p0 += v0 * s_w3[col] + v1 * s_w3[col + 1];
    p1 += v2 * s_w3[col] + v3 * s_w3[col + 1];
    if (h2out) {
      if (r0 < M) {
        h2out[(size_t)r0 * kHidden + col] = v0;
        h2out[(size_t)r0 * kHidden + col + 1] = v1;
      }
      if (r1 < M) {
        h2out[(size_t)r1 * kHidden + col] = v2;
        h2out[(size_t)r1 * kHidden + col + 1] = v3;
      }
    }
  }
  p0 += __shfl_xor_sync(0xFFFFFFFFu, p0, 1);
  p0 += __shfl_xor_sync(0xFFFFFFFFu, p0, 2);
  p1 += __shfl_xor_sync(0xFFFFFFFFu, p1, 1);
  p1 += __shfl_xor_sync(0xFFFFFFFFu, p1, 2);
  if (t == 0) {
    if (r0 < M) score[r0] = p0 + b3;
    if (r1 < M) score[r1] = p1 + b3;
  }
}

// Scores M rows: one warp per 16-row tile.
__global__ void __launch_bounds__(128) k_mlp_forward(const float* __restrict__ feat, uint32_t M,
                                                     const MlpDevice* __restrict__ mlp, float* __restrict__ score,
                                                     float* h1out, float* h2out, float* xout)
{
  __shared__ MlpSmem W;
  mlp_load(W, mlp);
  __syncthreads();
  const float b3 = mlp->b3;
  const uint32_t warpsTotal = gridDim.x * (blockDim.x >> 5);
  for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < M; tile += warpsTotal)
    mlp_tile(W, b3, tile, feat, M, score, h1out, h2out, xout);
}

// ---- per-view top-K --------------------------------------------------------------------------
// One CTA per view: K = max(1, ceil(fraction * candidates)) highest scores
// (ties by command order) are selected; everything else is not rasterised.

__device__ __forceinline__ uint32_t score_key(float s)
{
  const uint32_t b = __float_as_uint(s);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);  // monotone in s
}

__device__ __forceinline__ uint32_t block_count(bool p, uint32_t* sm)
{
  const uint32_t w = __popc(__ballot_sync(0xFFFFFFFFu, p));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = w;
  __syncthreads();
  uint32_t total = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) total += sm[i];
  __syncthreads();
  return total;
}

__device__ __forceinline__ uint32_t block_exclusive_scan256(uint32_t v, uint32_t& total, uint32_t* sm /* 8 */)
{
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += t;
  }
  if (lane == 31) sm[warp] = x;
  __syncthreads();
  uint32_t prefix = 0;
  total = 0;
  for (uint32_t w = 0; w < 8; ++w) {
    if (w < warp) prefix += sm[w];
    total += sm[w];
  }
  __syncthreads();
  return prefix + x - v;
}

// The top-K of view v (a CTA of 256 threads).
__device__ __forceinline__ void topk_view(const FrameParams& P, uint32_t v)
{
  __shared__ uint32_t s_red[8];
  __shared__ uint32_t s_hist[256];
  __shared__ uint32_t s_pick[2];
  const ViewDesc& V = P.views[v];
  const uint32_t c0 = V.cmdStart, n = V.cmdCount;
  uint32_t ncand = 0;
  for (uint32_t i0 = 0; i0 < n; i0 += 256) {
    const uint32_t i = i0 + threadIdx.x;
    ncand += block_count(i < n && P.cand[c0 + i], s_red);
  }
  if (ncand == 0) {
    for (uint32_t i = threadIdx.x; i < n; i += 256) P.select[c0 + i] = 0;
    return;
  }
  uint32_t K = (uint32_t)ceilf(P.selectFrac * (float)ncand);
  K = K < 1 ? 1 : (K > ncand ? ncand : K);
  // radix select, 8 bits at a time from the top: T = the K-th largest key
  uint32_t T = 0, above = 0;  // keys > the current prefix range already counted
  for (int shift = 24; shift >= 0; shift -= 8) {
    s_hist[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t hiMask = shift == 24 ? 0u : (0xFFFFFFFFu << (shift + 8));
    for (uint32_t i = threadIdx.x; i < n; i += 256)
      if (P.cand[c0 + i]) {
        const uint32_t key = score_key(P.score[c0 + i]);
        if ((key & hiMask) == (T & hiMask)) atomicAdd(&s_hist[(key >> shift) & 255u], 1u);
      }
    __syncthreads();
    // largest digit d with above + count(digits >= d) >= K: thread t holds
    // digit 255 - t, an inclusive scan over t counts the digits >= it
    if (threadIdx.x == 0) {
      s_pick[0] = 0;
      s_pick[1] = above;
    }
    const uint32_t v = s_hist[255 - threadIdx.x];
    uint32_t tot;
    const uint32_t incl = block_exclusive_scan256(v, tot, s_red) + v;
    if (above + incl >= K && above + incl - v < K) {
      s_pick[0] = 255 - threadIdx.x;
      s_pick[1] = above + incl - v;  // keys above this digit (within the prefix) plus the earlier ones
    }
    __syncthreads();
    T |= s_pick[0] << shift;
    above = s_pick[1];
    __syncthreads();
  }
  // `above` keys are > T; the remaining K - above come from the ties at T, in command order
  uint32_t needEq = K - above, seenEq = 0;
  for (uint32_t i0 = 0; i0 < n; i0 += 256) {
    const uint32_t i = i0 + threadIdx.x;
    bool c = false, eq = false;
    uint32_t key = 0;
    if (i < n && P.cand[c0 + i]) {
      key = score_key(P.score[c0 + i]);
      c = true;
      eq = key == T;
    }
    // rank of this tie among the ties, in command order
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, eq);
    if (lane == 0) s_red[threadIdx.x >> 5] = __popc(bal);
    __syncthreads();
    uint32_t before = seenEq;
    for (uint32_t w = 0; w < (threadIdx.x >> 5); ++w) before += s_red[w];
    before += __popc(bal & ((1u << lane) - 1u));
    uint32_t tot = 0;
    for (int w = 0; w < 8; ++w) tot += s_red[w];
    __syncthreads();
    seenEq += tot;
    if (i < n) P.select[c0 + i] = (c && (key > T || (eq && before < needEq))) ? 1 : 0;
  }
}

// One CTA per view: its top-K.
__global__ void __launch_bounds__(256) k_topk(FrameParams P) { topk_view(P, blockIdx.x); }

// Selection after k_features, one CTA per view: features 11 and 12, the
// network's scores of the view's commands (a warp per 16 rows), the top-K,
// and each command's draw flags as k_gate would set them (a gated command is
// drawn if it is a candidate -- feature 0, the same visibility test -- and
// among the top K, with the near-clip variant if its test said so -- feature
// 1), so the frame needs no k_gate.
__global__ void __launch_bounds__(256) k_select_view(FrameParams P)
{
  __shared__ MlpSmem W;
  const uint32_t v = blockIdx.x;
  mlp_load(W, P.mlp);
  view_norm(P, v);
  __syncthreads();  // the view's features and the weights
  const ViewDesc& V = P.views[v];
  const float b3 = P.mlp->b3;
  for (uint32_t tile = threadIdx.x >> 5; tile * 16 < V.cmdCount; tile += blockDim.x >> 5)
    mlp_tile(W, b3, tile, P.feat + (size_t)V.cmdStart * kFeatures, V.cmdCount, P.score + V.cmdStart, nullptr, nullptr,
             nullptr);
  __syncthreads();  // the view's scores
  topk_view(P, v);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < V.cmdCount; i += blockDim.x) {
    const uint32_t c = V.cmdStart + i;
    const uint32_t flags = P.cmds[c].flags;
    uint32_t draw = 1, nc = (flags & kCmdNearClip) ? 1u : 0u;
    if (flags & kCmdGated) {
      const float* f = P.feat + (size_t)c * kFeatures;
      draw = f[0] != 0.0f ? 1u : 0u;
      nc = f[1] != 0.0f ? 1u : 0u;
    }
    if (!P.select[c]) draw = 0;
    P.cmdDraw[c] = draw | (nc << 1);
  }
}

// ---- training: backward and Adam ---------------------------------------------------------------

// Listwise loss, one warp per group of rows (one view in one frame): the
// scores' softmax over the group against the target distribution t of the
// group; loss = -sum_groups sum_i t_i log p_i / G, ds_i = (p_i - t_i) / G.
// err2 receives each row's loss term scaled by B / G, so that the common
// reduction (sum / B) yields the loss.
__global__ void __launch_bounds__(256) k_listwise_ds(const float* __restrict__ score, const float* __restrict__ target,
                                                     const uint32_t* __restrict__ groupStart, uint32_t G, uint32_t B,
                                                     float* ds, float* err2)
{
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t g = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (g >= G) return;
  const uint32_t a = groupStart[g], b = groupStart[g + 1];
  float mx = -3.0e38f;
  for (uint32_t i = a + lane; i < b; i += 32) mx = fmaxf(mx, score[i]);
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
  float z = 0.0f;
  for (uint32_t i = a + lane; i < b; i += 32) z += expf(score[i] - mx);
  for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(0xFFFFFFFFu, z, o);
  const float lz = logf(z), invG = 1.0f / (float)G;
  for (uint32_t i = a + lane; i < b; i += 32) {
    const float lp = score[i] - mx - lz;
    ds[i] = (expf(lp) - target[i]) * invG;
    err2[i] = -target[i] * lp * ((float)B * invG);
  }
}

// Per row: ds = 2 (s - t) / B (mean squared error; with haveDs, ds is given),
// dh2 = ds w3 (h2 > 0), dh1 = (dh2 W2) (h1 > 0).
__global__ void __launch_bounds__(128) k_mlp_backward_rows(const float* __restrict__ score,
                                                           const float* __restrict__ target, uint32_t B,
                                                           const MlpDevice* __restrict__ mlp,
                                                           const float* __restrict__ h1, const float* __restrict__ h2,
                                                           float* ds, float* dh1, float* dh2, float* err2, bool haveDs)
{
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B) return;
  float d;
  if (haveDs) {
    d = ds[r];
  } else {
    const float e = score[r] - target[r];
    d = 2.0f * e / (float)B;
    ds[r] = d;
    err2[r] = e * e;
  }
  float g2[kHidden];
#pragma unroll 8
  for (int n = 0; n < kHidden; ++n) {
    g2[n] = h2[(size_t)r * kHidden + n] > 0.0f ? d * mlp->w3[n] : 0.0f;
    dh2[(size_t)r * kHidden + n] = g2[n];
  }
  for (int k = 0; k < kHidden; ++k) {
    float acc = 0.0f;
    if (h1[(size_t)r * kHidden + k] > 0.0f) {
#pragma unroll 8
      for (int n = 0; n < kHidden; ++n) acc += g2[n] * __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(mlp->w2t)[n * kHidden + k]);
    }
    dh1[(size_t)r * kHidden + k] = acc;
  }
}

// Gradient of every parameter (and the squared errors in slot kParams), summed
// over the rows of one row block [r0, r1) in row order: partial[rb][p].
__device__ __forceinline__ float grad_term(uint32_t p, uint32_t r, const float* __restrict__ xb,
                                           const float* __restrict__ h1, const float* __restrict__ h2,
                                           const float* __restrict__ ds, const float* __restrict__ dh1,
                                           const float* __restrict__ dh2, const float* __restrict__ err2)
{
  if (p < (uint32_t)kOffB1) {
    const uint32_t n = p / kFeatures, k = p % kFeatures;
    return dh1[(size_t)r * kHidden + n] * xb[(size_t)r * kFeatures + k];
  }
  if (p < (uint32_t)kOffW2) return dh1[(size_t)r * kHidden + (p - kOffB1)];
  if (p < (uint32_t)kOffB2) {
    const uint32_t q = p - kOffW2, n = q / kHidden, k = q % kHidden;
    return dh2[(size_t)r * kHidden + n] * h1[(size_t)r * kHidden + k];
  }
  if (p < (uint32_t)kOffW3) return dh2[(size_t)r * kHidden + (p - kOffB2)];
  if (p < (uint32_t)kOffB3) return ds[r] * h2[(size_t)r * kHidden + (p - kOffW3)];
  if (p == (uint32_t)kOffB3) return ds[r];
  return err2[r];
}

__global__ void __launch_bounds__(128) k_mlp_grad_partial(uint32_t B, uint32_t rowsPerBlock,
                                                          const float* __restrict__ xb, const float* __restrict__ h1,
                                                          const float* __restrict__ h2, const float* __restrict__ ds,
                                                          const float* __restrict__ dh1, const float* __restrict__ dh2,
                                                          const float* __restrict__ err2, float* partial)
{
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > (uint32_t)kParams) return;
  const uint32_t r0 = blockIdx.y * rowsPerBlock, r1 = ::min(B, r0 + rowsPerBlock);
  float acc = 0.0f;
  for (uint32_t r = r0; r < r1; ++r) acc += grad_term(p, r, xb, h1, h2, ds, dh1, dh2, err2);
  partial[(size_t)blockIdx.y * (kParams + 1) + p] = acc;
}

// Sums the row blocks in order (deterministic); slot kParams becomes the loss.
__global__ void __launch_bounds__(128) k_mlp_grad_final(uint32_t B, uint32_t blocks, const float* __restrict__ partial,
                                                        float* grad)
{
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > (uint32_t)kParams) return;
  float acc = 0.0f;
  for (uint32_t b = 0; b < blocks; ++b) acc += partial[(size_t)b * (kParams + 1) + p];
  grad[p] = p == (uint32_t)kParams ? acc / (float)B : acc;
}

// Writes the kernels' copy of the weights (bf16 matrices) from the fp32 master.
__global__ void k_mlp_publish(const float* __restrict__ params, MlpDevice* mlp)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (uint32_t)(kHidden * kFeatures))
    reinterpret_cast<__nv_bfloat16*>(mlp->w1t)[i] = __float2bfloat16_rn(params[kOffW1 + i]);
  if (i < (uint32_t)(kHidden * kHidden))
    reinterpret_cast<__nv_bfloat16*>(mlp->w2t)[i] = __float2bfloat16_rn(params[kOffW2 + i]);
  if (i < (uint32_t)kHidden) {
    mlp->b1[i] = params[kOffB1 + i];
    mlp->b2[i] = params[kOffB2 + i];
    mlp->w3[i] = params[kOffW3 + i];
  }
  if (i == 0) mlp->b3 = params[kOffB3];
}

__global__ void k_adam(float* params, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                       float eps, float bc1, float bc2)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint32_t)kParams) return;
  const float g = grad[i];
  const float mi = beta1 * m[i] + (1.0f - beta1) * g;
  const float vi = beta2 * v[i] + (1.0f - beta2) * g * g;
  m[i] = mi;
  v[i] = vi;
  params[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// ---- launchers -------------------------------------------------------------------------------

cudaError_t launch_selection(const FrameParams& P, uint32_t numCmds, bool useMlp, cudaStream_t stream)
{
  if (numCmds) k_features<<<(numCmds + 255) / 256, 256, 0, stream>>>(P, numCmds);
  if (numCmds) {
    if (useMlp && P.fusedSelect) {
      k_select_view<<<P.numViews, 256, 0, stream>>>(P);
    } else {
      k_view_norm<<<P.numViews, 256, 0, stream>>>(P);
      if (useMlp) {
        const uint32_t tiles = (numCmds + 15) / 16;
        k_mlp_forward<<<(tiles + 3) / 4, 128, 0, stream>>>(P.feat, numCmds, P.mlp, P.score, nullptr, nullptr, nullptr);
        k_topk<<<P.numViews, 256, 0, stream>>>(P);
      }
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_mlp_forward(const float* feat, uint32_t M, const MlpDevice* mlp, float* score, float* h1, float* h2,
                               float* xb, cudaStream_t stream)
{
  const uint32_t tiles = (M + 15) / 16;
  if (M) k_mlp_forward<<<(tiles + 3) / 4, 128, 0, stream>>>(feat, M, mlp, score, h1, h2, xb);
  return cudaGetLastError();
}

uint32_t mlp_grad_blocks(uint32_t B) { return ::min(64u, (B + 63) / 64); }

cudaError_t launch_mlp_backward(const float* score, const float* target, uint32_t B, const MlpDevice* mlp,
                                const float* xb, const float* h1, const float* h2, float* ds, float* dh1, float* dh2,
                                float* err2, float* partial, float* grad, cudaStream_t stream,
                                const uint32_t* groupStart, uint32_t groups)
{
  if (groupStart) k_listwise_ds<<<(groups + 7) / 8, 256, 0, stream>>>(score, target, groupStart, groups, B, ds, err2);
  k_mlp_backward_rows<<<(B + 127) / 128, 128, 0, stream>>>(score, target, B, mlp, h1, h2, ds, dh1, dh2, err2,
                                                           groupStart != nullptr);
  const uint32_t nb = mlp_grad_blocks(B), rows = (B + nb - 1) / nb;
  const dim3 grid((kParams + 1 + 127) / 128, nb);
  k_mlp_grad_partial<<<grid, 128, 0, stream>>>(B, rows, xb, h1, h2, ds, dh1, dh2, err2, partial);
  k_mlp_grad_final<<<(kParams + 1 + 127) / 128, 128, 0, stream>>>(B, nb, partial, grad);
  return cudaGetLastError();
}

cudaError_t launch_mlp_publish(const float* params, MlpDevice* mlp, cudaStream_t stream)
{
  k_mlp_publish<<<(kHidden * kHidden + 255) / 256, 256, 0, stream>>>(params, mlp);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* params, const float* grad, float* m, float* v, float lr, uint32_t step,
                        cudaStream_t stream)
{
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
  k_adam<<<(kParams + 255) / 256, 256, 0, stream>>>(params, grad, m, v, lr, b1, b2, 1e-8f, bc1, bc2);
  return cudaGetLastError();
}

int mlp_param_count() { return kParams; }

}  // namespace occ
