// Occluder::bake (Occluder.cpp:7-181) on the GPU, many occluders per launch:
// for occluders whose vertices change at run time (moving or deforming
// geometry), so that they can be baked again where the vertices already are.
// The bytes equal the host bake's (bake.cpp; both use bake_math.cuh), which
// equal the reference's.
//
// One CTA per occluder:
//   1. quad normals (thread per quad);
//   2. up to ten k-means rounds around the six axis directions: assignment
//      thread per quad; each centroid's component sums in quad order (the
//      reference adds the normals one after another, so one thread per
//      (centroid, component) keeps that order), normalised;
//   3. quads grouped by centroid, quad order kept within a group;
//   4. 11/11/10 packing, thread per output word;
//   5. bounds over the input vertices with minps/maxps: per-lane runs over
//      contiguous ranges, merged in range order (the earlier value wins a tie,
//      as in the reference's running minimum), w = 1, centre.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bake_math.cuh"
#include "raster_types.h"

namespace occ {

using bake::V4;

constexpr int kBakeThreads = 256;

__device__ __forceinline__ V4 load_v4(const float4* p)
{
  const float4 a = p[0];
  return V4{{a.x, a.y, a.z, a.w}};
}

// minps / maxps as the reference's running bounds use them: x op y keeps y
// unless x < y (x > y), so a NaN x is skipped and a tie keeps y.
__device__ __forceinline__ float run_min(float x, float y) { return x < y ? x : y; }
__device__ __forceinline__ float run_max(float x, float y) { return x > y ? x : y; }

__global__ void __launch_bounds__(kBakeThreads) k_bake(const BakeJob* jobs, const float4* vertices, float4* normals,
                                                       uint32_t* cluster, uint32_t* order, uint32_t* packed,
                                                       float* bounds)
{
  __shared__ V4 s_centroid[6];
  __shared__ float s_sum[6][4];
  __shared__ uint32_t s_count[6], s_base[6];
  __shared__ float s_lo[32][4], s_hi[32][4];
  const BakeJob J = jobs[blockIdx.x];
  const uint32_t tid = threadIdx.x;
  const uint32_t nv = J.vertexCount, nq = nv / 4, q0 = J.vertexStart / 4;
  const float4* vtx = vertices + J.vertexStart;
  float4* nrm = normals + q0;
  uint32_t* cl = cluster + q0;
  uint32_t* ord = order + q0;

  // 1. normals; every quad starts in cluster 0 (Occluder.cpp:31)
  for (uint32_t q = tid; q < nq; q += kBakeThreads) {
    const V4 n = bake::quad_normal(load_v4(vtx + 4 * q), load_v4(vtx + 4 * q + 1), load_v4(vtx + 4 * q + 2),
                                   load_v4(vtx + 4 * q + 3));
    nrm[q] = make_float4(n.v[0], n.v[1], n.v[2], n.v[3]);
    cl[q] = 0;
  }
  if (tid < 6) s_centroid[tid] = bake::seed_centroid((int)tid);
  __syncthreads();

  // 2. k-means (Occluder.cpp:33-78)
  bool changed = true;
  for (int iter = 0; iter < 10 && changed; ++iter) {
    bool mine = false;
    for (uint32_t q = tid; q < nq; q += kBakeThreads) {
      const float4 f = nrm[q];
      const float n[4] = {f.x, f.y, f.z, f.w};
      float best = -__int_as_float(0x7F800000);
      uint32_t bestK = 0;
      for (uint32_t k = 0; k < 6; ++k) {
        const float d = x86::dp3(s_centroid[k].v, n);
        if (d >= best) {  // COMISS: false when unordered
          best = d;
          bestK = k;
        }
      }
      if (cl[q] != bestK) {
        cl[q] = bestK;
        mine = true;
      }
    }
    changed = __syncthreads_or(mine) != 0;
    if (tid < 24) {
      const uint32_t k = tid >> 2, a = tid & 3;
      float acc = 0.0f;
      for (uint32_t q = 0; q < nq; ++q)
        if (cl[q] == k) acc = x86::xadd(acc, reinterpret_cast<const float*>(nrm + q)[a]);
      s_sum[k][a] = acc;
    }
    __syncthreads();
    if (tid < 6) s_centroid[tid] = bake::normalize(V4{{s_sum[tid][0], s_sum[tid][1], s_sum[tid][2], s_sum[tid][3]}});
    __syncthreads();
  }

  // 3. quads by centroid, in quad order within each (Occluder.cpp:80-92)
  if (tid < 6) {
    uint32_t c = 0;
    for (uint32_t q = 0; q < nq; ++q) c += cl[q] == tid;
    s_count[tid] = c;
  }
  __syncthreads();
  if (tid < 6) {
    uint32_t b = 0;
    for (uint32_t k = 0; k < tid; ++k) b += s_count[k];
    for (uint32_t q = 0; q < nq; ++q)
      if (cl[q] == tid) ord[b++] = q;
  }
  __syncthreads();

  // 4. packing: word w of the occluder is vertex j of quad order[8g + l],
  //    g = w / 32, j = (w / 8) % 4, l = w % 8 (Occluder.cpp:104-157)
  const V4 lo{{J.refMin[0], J.refMin[1], J.refMin[2], J.refMin[3]}};
  V4 inv;
  for (int i = 0; i < 4; ++i) inv.v[i] = x86::xdiv(1.0f, x86::xsub(J.refMax[i], J.refMin[i]));
  uint32_t* out = packed + J.vertexStart;
  for (uint32_t w = tid; w < nv; w += kBakeThreads) {
    const uint32_t g = w >> 5, j = (w >> 3) & 3, l = w & 7;
    out[w] = bake::pack_vertex(load_v4(vtx + 4 * ord[8 * g + l] + j), lo, inv);
  }

  // 5. bounds (Occluder.cpp:159-178): warp 0, lane i runs over the i-th
  //    contiguous range of vertices, then the ranges merge in order
  if (tid < 32) {
    const uint32_t per = (nv + 31) / 32, b0 = ::min(nv, tid * per), b1 = ::min(nv, b0 + per);
    float mn[4], mx[4];
    for (int a = 0; a < 4; ++a) {
      mn[a] = __int_as_float(0x7F800000);
      mx[a] = -__int_as_float(0x7F800000);
    }
    for (uint32_t i = b0; i < b1; ++i) {
      const float4 p = vtx[i];
      const float v[4] = {p.x, p.y, p.z, p.w};
      for (int a = 0; a < 4; ++a) {
        mn[a] = run_min(v[a], mn[a]);
        mx[a] = run_max(v[a], mx[a]);
      }
    }
    for (int a = 0; a < 4; ++a) {
      s_lo[tid][a] = mn[a];
      s_hi[tid][a] = mx[a];
    }
    __syncwarp();
    if (tid < 4) {
      // ranges in order; a later range's value replaces the running one only
      // if strictly smaller (larger), as vertex by vertex
      float m = s_lo[0][tid], M = s_hi[0][tid];
      for (int r = 1; r < 32; ++r) {
        m = run_min(s_lo[r][tid], m);
        M = run_max(s_hi[r][tid], M);
      }
      if (tid == 3) m = M = 1.0f;  // w = 1 (Occluder.cpp:171-173)
      float* B = bounds + 20 * (size_t)blockIdx.x;
      B[tid] = J.refMin[tid];
      B[4 + tid] = J.refMax[tid];
      B[8 + tid] = m;
      B[12 + tid] = M;
      B[16 + tid] = x86::xmul(x86::xadd(M, m), 0.5f);
    }
  }
}

cudaError_t launch_bake(const BakeJob* jobs, uint32_t count, const float4* vertices, float4* normals,
                        uint32_t* cluster, uint32_t* order, uint32_t* packed, float* bounds, cudaStream_t stream)
{
  if (!count) return cudaSuccess;
  k_bake<<<count, kBakeThreads, 0, stream>>>(jobs, vertices, normals, cluster, order, packed, bounds);
  return cudaGetLastError();
}

}  // namespace occ
