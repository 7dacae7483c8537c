// SurfaceAreaHeuristic::generateBatches (SurfaceAreaHeuristic.cpp:10-104) on
// the GPU: the same batches, byte for byte, as the host restatement
// (bake.cpp, sah_recurse) and the reference.
//
// The reference recurses depth first; each call sorts its range of quad
// indices stably by the box centre along x, then y, then z (each sort starts
// from the order the previous one left), evaluates the split cost at every
// multiple of the split granularity after each sort, keeps the first
// strictly cheaper split in the order (axis, index), and sorts the range
// stably by the chosen axis again.  The outcome of a call depends only on its
// range, so all ranges of one recursion depth are processed together here:
//
//   * every stable sort is one LSD radix sort of (range id, centre key)
//     pairs over the whole index array (ranges are contiguous and numbered in
//     position order, so a range's elements stay in its positions; ranges
//     already final sort by their id alone and keep their order);
//   * the surface areas of the prefix and suffix unions are segmented
//     min/max scans (exact in any association: only the sign of a zero
//     coordinate can differ, which changes no cost comparison);
//   * the first strictly cheaper (axis, index) is a 64-bit atomicMin of
//     (cost in an order-preserving integer form, axis, index) per range.
//
// Batches come out in the reference's depth-first order because a left
// child's positions precede its sibling's: the final ranges in position order
// are the batches.  Centres are compared as the reference compares them
// (`<` on floats, the two zeros equal); a NaN centre makes the reference's
// comparison inconsistent and its order that of its library's merge sort, so
// such inputs are refused (the host bake handles them).
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "sah_scratch.h"

namespace occ {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 2048 elements per CTA
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t order_key(float f)
{
  uint32_t u = f == 0.0f ? 0u : __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// centres (lo + hi) and their keys; the identity order
__global__ void k_sah_prep(const float* aabbs, uint32_t n, float4* lo, float4* hi, uint32_t* mk, uint32_t* idx,
                           uint32_t* flag)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = reinterpret_cast<const float4*>(aabbs)[2 * (size_t)i];
  const float4 b = reinterpret_cast<const float4*>(aabbs)[2 * (size_t)i + 1];
  lo[i] = a;
  hi[i] = b;
  const float c[3] = {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
  bool nan = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    nan |= c[k] != c[k];
    mk[(size_t)k * n + i] = order_key(c[k]);
  }
  if (nan) atomicOr(flag, 1u);
  idx[i] = i;
}

// range of every position: the last range starting at or before it
__global__ void k_sah_rng(const uint32_t* starts, uint32_t numRanges, uint32_t n, uint32_t* rng)
{
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  uint32_t lo = 0, hi = numRanges - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (starts[mid] <= p) lo = mid; else hi = mid - 1;
  }
  rng[p] = lo;
}

__global__ void k_sah_keys(const uint32_t* idx, const uint32_t* rng, const int8_t* rangeAxis, const uint32_t* mk,
                           uint32_t n, unsigned long long* key)
{
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t r = rng[p];
  const int a = rangeAxis[r];
  key[p] = ((unsigned long long)r << 32) | (a >= 0 ? mk[(size_t)a * n + idx[p]] : 0u);
}

// ---- stable LSD radix sort of (key, index) pairs, 8 bits a pass ---------------------

__global__ void __launch_bounds__(kSortThreads) k_rs_hist(const unsigned long long* key, uint32_t n, uint32_t shift,
                                                        uint32_t* hist, uint32_t tiles)
{
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * kSortTile;
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const uint32_t p = base + r * kSortThreads + threadIdx.x;
    if (p < n) atomicAdd(&cnt[(key[p] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

// exclusive prefix sum of `total` counts in place (digit-major: every tile's
// share of digit d follows all of digit d - 1), one CTA
__global__ void __launch_bounds__(1024) k_rs_scan(uint32_t* v, uint32_t total)
{
  __shared__ uint32_t part[1024];
  const uint32_t t = threadIdx.x;
  const uint32_t per = (total + 1023) / 1024;
  const uint32_t a = t * per, b = min(a + per, total);
  uint32_t s = 0;
  for (uint32_t i = a; i < b; ++i) s += v[i];
  part[t] = s;
  __syncthreads();
  for (uint32_t o = 1; o < 1024; o <<= 1) {
    const uint32_t x = t >= o ? part[t - o] : 0u;
    __syncthreads();
    part[t] += x;
    __syncthreads();
  }
  uint32_t run = part[t] - s;
  for (uint32_t i = a; i < b; ++i) {
    const uint32_t c = v[i];
    v[i] = run;
    run += c;
  }
}

// Each CTA places its tile's elements in position order: within a round of
// 256 elements, lanes with the same digit are ranked by __match_any_sync and
// warps by their counts; rounds follow one another.
__global__ void __launch_bounds__(kSortThreads) k_rs_scatter(const unsigned long long* keyIn, const uint32_t* valIn,
                                                           unsigned long long* keyOut, uint32_t* valOut, uint32_t n,
                                                           uint32_t shift, const uint32_t* offs, uint32_t tiles)
{
  __shared__ uint32_t cnt[kSortThreads / 32][256];
  __shared__ uint32_t run[256];
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  run[t] = 0;
  const uint32_t base = blockIdx.x * kSortTile;
  for (int r = 0; r < kSortItems; ++r) {
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) cnt[w][t] = 0;
    __syncthreads();
    const uint32_t p = base + r * kSortThreads + t;
    const bool valid = p < n;
    unsigned long long k = 0;
    uint32_t v = 0, d = 0;
    if (valid) {
      k = keyIn[p];
      v = valIn[p];
      d = (uint32_t)(k >> shift) & 255u;
    }
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 0x100u + lane);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) cnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t off = run[d] + rank;
      for (uint32_t w = 0; w < warp; ++w) off += cnt[w][d];
      const uint32_t dst = offs[d * tiles + blockIdx.x] + off;
      keyOut[dst] = k;
      valOut[dst] = v;
    }
    __syncthreads();
    uint32_t add = 0;
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) add += cnt[w][t];
    run[t] += add;
    __syncthreads();
  }
}

// ---- segmented surface-area scans ----------------------------------------------------

struct SegBox {
  float lx, ly, lz, hx, hy, hz;
  bool start;  // the segment holds a range start
};

__device__ __forceinline__ SegBox seg_empty()
{
  const float inf = __int_as_float(0x7F800000);
  return SegBox{inf, inf, inf, -inf, -inf, -inf, false};
}

// Aabb::include: _mm_min_ps / _mm_max_ps
__device__ __forceinline__ void seg_grow(SegBox& a, const SegBox& b)
{
  a.lx = a.lx < b.lx ? a.lx : b.lx;
  a.ly = a.ly < b.ly ? a.ly : b.ly;
  a.lz = a.lz < b.lz ? a.lz : b.lz;
  a.hx = a.hx > b.hx ? a.hx : b.hx;
  a.hy = a.hy > b.hy ? a.hy : b.hy;
  a.hz = a.hz > b.hz ? a.hz : b.hz;
}

// (a then b): b alone if b starts a segment, else the union
__device__ __forceinline__ SegBox seg_combine(const SegBox& a, const SegBox& b)
{
  if (b.start) return b;
  SegBox c = a;
  seg_grow(c, b);
  c.start = a.start;
  return c;
}

// Aabb::surfaceArea (VectorMath.h:57-62): DPPS 0x7F of the extents with their
// yzx shuffle, (ex*ey + ey*ez) + (ez*ex + 0)
__device__ __forceinline__ float seg_area(const SegBox& b)
{
  const float ex = __fsub_rn(b.hx, b.lx), ey = __fsub_rn(b.hy, b.ly), ez = __fsub_rn(b.hz, b.lz);
  return __fadd_rn(__fadd_rn(__fmul_rn(ex, ey), __fmul_rn(ey, ez)), __fadd_rn(__fmul_rn(ez, ex), 0.0f));
}

// Position q of the scan in direction dir (0: left to right, 1: right to left)
// and whether it starts its range in that direction.
__device__ __forceinline__ uint32_t scan_pos(uint32_t j, uint32_t n, int dir) { return dir ? n - 1 - j : j; }

__device__ __forceinline__ SegBox scan_elem(const SahScratch& S, const uint32_t* idx, uint32_t q, int dir)
{
  const uint32_t r = S.rng[q];
  const bool start = dir ? (q + 1 == S.starts[r + 1]) : (q == S.starts[r]);
  const uint32_t i = idx[q];
  const float4 a = S.lo[i], b = S.hi[i];
  return SegBox{a.x, a.y, a.z, b.x, b.y, b.z, start};
}

// per tile: the segmented aggregate of its elements in scan order
__global__ void __launch_bounds__(kScanThreads) k_sah_scan_reduce(SahScratch S, const uint32_t* idx, uint32_t n,
                                                                  int dir)
{
  __shared__ SegBox part[kScanThreads];
  const uint32_t t = threadIdx.x;
  SegBox acc = seg_empty();
  const uint32_t j0 = blockIdx.x * kScanTile + t * kScanItems;
  for (int k = 0; k < kScanItems; ++k)
    if (j0 + k < n) acc = seg_combine(acc, scan_elem(S, idx, scan_pos(j0 + k, n, dir), dir));
  part[t] = acc;
  __syncthreads();
  if (t == 0) {
    SegBox a = seg_empty();
    for (int k = 0; k < kScanThreads; ++k) a = seg_combine(a, part[k]);
    S.aggLo[blockIdx.x] = make_float4(a.lx, a.ly, a.lz, a.start ? 1.0f : 0.0f);
    S.aggHi[blockIdx.x] = make_float4(a.hx, a.hy, a.hz, 0.0f);
  }
}

// exclusive segmented scan of the tile aggregates in place (one thread: a few
// hundred tiles)
__global__ void k_sah_scan_tiles(SahScratch S, uint32_t tiles)
{
  SegBox acc = seg_empty();
  for (uint32_t b = 0; b < tiles; ++b) {
    const float4 l = S.aggLo[b], h = S.aggHi[b];
    const SegBox x{l.x, l.y, l.z, h.x, h.y, h.z, l.w != 0.0f};
    S.aggLo[b] = make_float4(acc.lx, acc.ly, acc.lz, 0.0f);
    S.aggHi[b] = make_float4(acc.hx, acc.hy, acc.hz, 0.0f);
    acc = seg_combine(acc, x);
  }
}

// every position's area, the tile's carry-in applied
__global__ void __launch_bounds__(kScanThreads) k_sah_scan_apply(SahScratch S, const uint32_t* idx, uint32_t n,
                                                                 int dir, float* area)
{
  __shared__ SegBox part[kScanThreads];
  const uint32_t t = threadIdx.x;
  const uint32_t j0 = blockIdx.x * kScanTile + t * kScanItems;
  SegBox mine = seg_empty();
  for (int k = 0; k < kScanItems; ++k)
    if (j0 + k < n) mine = seg_combine(mine, scan_elem(S, idx, scan_pos(j0 + k, n, dir), dir));
  part[t] = mine;
  __syncthreads();
  // the thread's carry-in: the tile's carry, then the threads before it
  const float4 l = S.aggLo[blockIdx.x], h = S.aggHi[blockIdx.x];
  SegBox acc{l.x, l.y, l.z, h.x, h.y, h.z, false};
  for (uint32_t k = 0; k < t; ++k) acc = seg_combine(acc, part[k]);
  for (int k = 0; k < kScanItems; ++k)
    if (j0 + k < n) {
      const uint32_t q = scan_pos(j0 + k, n, dir);
      acc = seg_combine(acc, scan_elem(S, idx, q, dir));
      area[q] = seg_area(acc);
    }
}

// split costs at every multiple of the granularity (SurfaceAreaHeuristic.cpp:44-62)
__global__ void k_sah_cost(SahScratch S, uint32_t n, uint32_t gran, uint32_t axis)
{
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const uint32_t r = S.rng[q];
  if (S.rangeAxis[r] < 0) return;
  const uint32_t start = S.starts[r], len = S.starts[r + 1] - start, s = q - start;
  if (s < gran || s % gran != 0 || s >= len - gran) return;
  const float cost = __fadd_rn(__fmul_rn(S.left[q - 1], __int2float_rn((int)s)),
                               __fmul_rn(S.right[q], __int2float_rn((int)(len - s))));
  if (!(cost < __int_as_float(0x7F800000))) return;  // the reference's best starts at +inf (strict <)
  const unsigned long long k = ((unsigned long long)order_key(cost) << 32) | ((unsigned long long)axis << 30) | s;
  atomicMin(&S.best[r], k);
}

static uint32_t blocks_of(uint32_t n, uint32_t per) { return (n + per - 1) / per; }

// One stable sort of (key, idx) by the low `bits` bits of the key; the result
// is in buffers [cur] after the call (cur is updated).
static cudaError_t radix_sort(SahScratch& S, uint32_t n, uint32_t bits, int& cur, cudaStream_t st)
{
  const uint32_t tiles = blocks_of(n, kSortTile);
  for (uint32_t shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<tiles, kSortThreads, 0, st>>>(S.key[cur], n, shift, S.hist, tiles);
    k_rs_scan<<<1, 1024, 0, st>>>(S.hist, 256 * tiles);
    k_rs_scatter<<<tiles, kSortThreads, 0, st>>>(S.key[cur], S.idx[cur], S.key[cur ^ 1], S.idx[cur ^ 1], n, shift,
                                                 S.hist, tiles);
    cur ^= 1;
  }
  return cudaGetLastError();
}

static uint32_t bits_for(uint32_t v)
{
  uint32_t b = 0;
  while (b < 32 && (v >> b)) ++b;
  return b;
}

// The whole recursion.  aabbs: device, n x 8 floats; flat: device, n indices;
// offsets (host) receives the batch boundaries.  Returns 0, 1 (a NaN centre:
// not handled here) or -1 with `err` set.
int sah_generate_device(SahScratch& S, uint32_t n, const float* aabbs, uint32_t target, uint32_t gran,
                        uint32_t* flat, std::vector<uint32_t>& offsets, cudaStream_t st, std::string& err)
{
  auto cuda = [&](cudaError_t e) {
    if (e != cudaSuccess) err = cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  const uint32_t tb = 256;
  if (!cuda(cudaMemsetAsync(S.flag, 0, 4, st))) return -1;
  k_sah_prep<<<blocks_of(n, tb), tb, 0, st>>>(aabbs, n, S.lo, S.hi, S.mk, S.idx[0], S.flag);
  uint32_t nanSeen = 0;
  if (!cuda(cudaMemcpyAsync(&nanSeen, S.flag, 4, cudaMemcpyDeviceToHost, st)) || !cuda(cudaStreamSynchronize(st)))
    return -1;
  if (nanSeen) return 1;
  int cur = 0;
  // ranges in position order: start, and whether the recursion still splits it
  std::vector<uint32_t> starts{0u, n};
  std::vector<uint8_t> active{1};
  std::vector<int8_t> axisOf;
  std::vector<unsigned long long> best;
  const uint32_t scanTiles = blocks_of(n, kScanTile);
  for (;;) {
    const uint32_t nr = (uint32_t)active.size();
    bool any = false;
    for (uint8_t a : active) any |= a != 0;
    if (!any) break;
    if (!cuda(cudaMemcpyAsync(S.starts, starts.data(), (nr + 1) * 4, cudaMemcpyHostToDevice, st))) return -1;
    k_sah_rng<<<blocks_of(n, tb), tb, 0, st>>>(S.starts, nr, n, S.rng);
    best.assign(nr, ~0ull);
    if (!cuda(cudaMemcpyAsync(S.best, best.data(), nr * 8, cudaMemcpyHostToDevice, st))) return -1;
    const uint32_t keyBits = 32 + bits_for(nr - 1);
    axisOf.assign(nr, -1);
    for (uint32_t axis = 0; axis < 3; ++axis) {
      // stable sort of every active range by this axis's centres
      for (uint32_t r = 0; r < nr; ++r) axisOf[r] = active[r] ? (int8_t)axis : (int8_t)-1;
      if (!cuda(cudaMemcpyAsync(S.rangeAxis, axisOf.data(), nr, cudaMemcpyHostToDevice, st))) return -1;
      k_sah_keys<<<blocks_of(n, tb), tb, 0, st>>>(S.idx[cur], S.rng, S.rangeAxis, S.mk, n, S.key[cur]);
      if (!cuda(radix_sort(S, n, keyBits, cur, st))) return -1;
      for (int dir = 0; dir < 2; ++dir) {
        k_sah_scan_reduce<<<scanTiles, kScanThreads, 0, st>>>(S, S.idx[cur], n, dir);
        k_sah_scan_tiles<<<1, 1, 0, st>>>(S, scanTiles);
        k_sah_scan_apply<<<scanTiles, kScanThreads, 0, st>>>(S, S.idx[cur], n, dir, dir ? S.right : S.left);
      }
      k_sah_cost<<<blocks_of(n, tb), tb, 0, st>>>(S, n, gran, axis);
      if (!cuda(cudaGetLastError())) return -1;
    }
    if (!cuda(cudaMemcpyAsync(best.data(), S.best, nr * 8, cudaMemcpyDeviceToHost, st)) ||
        !cuda(cudaStreamSynchronize(st)))
      return -1;
    // sort again by the chosen axis; the split ranges' halves
    std::vector<uint32_t> nstarts;
    std::vector<uint8_t> nactive;
    for (uint32_t r = 0; r < nr; ++r) {
      const uint32_t a = starts[r], len = starts[r + 1] - a;
      const bool split = active[r] && best[r] != ~0ull;
      axisOf[r] = split ? (int8_t)((best[r] >> 30) & 3u) : (int8_t)-1;
      nstarts.push_back(a);
      if (!split) {
        nactive.push_back(0);  // a batch (no split found: the range stays whole)
        continue;
      }
      // a half of at least targetSize quads recurses; the recursion keeps a
      // range of at most two granules whole and unsorted (no split exists)
      const uint32_t s = (uint32_t)(best[r] & 0x3FFFFFFFu);
      const auto recurse = [&](uint32_t m) { return m >= target && m > 2 * gran ? (uint8_t)1 : (uint8_t)0; };
      nactive.push_back(recurse(s));
      nstarts.push_back(a + s);
      nactive.push_back(recurse(len - s));
    }
    if (!cuda(cudaMemcpyAsync(S.rangeAxis, axisOf.data(), nr, cudaMemcpyHostToDevice, st))) return -1;
    k_sah_keys<<<blocks_of(n, tb), tb, 0, st>>>(S.idx[cur], S.rng, S.rangeAxis, S.mk, n, S.key[cur]);
    if (!cuda(radix_sort(S, n, keyBits, cur, st))) return -1;
    nstarts.push_back(n);
    starts.swap(nstarts);
    active.swap(nactive);
  }
  if (!cuda(cudaMemcpyAsync(flat, S.idx[cur], (size_t)n * 4, cudaMemcpyDeviceToDevice, st)) ||
      !cuda(cudaStreamSynchronize(st)))
    return -1;
  offsets.assign(starts.begin(), starts.end());
  return 0;
}

}  // namespace occ
