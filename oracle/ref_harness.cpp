/*
 * Headless C harness over the reference occluder rasteriser's own sources
 * (SoftwareRasterizer/{Rasterizer,Occluder,QuadDecomposition,SurfaceAreaHeuristic}.cpp),
 * compiled unchanged with gcc -mavx2 -mfma -ffp-contract=off and ref_shim.h.
 *
 * TEST INFRASTRUCTURE ONLY.  It exists to pin the portable oracle (oracle.c)
 * and the library's host bake against the reference itself on x86-64.  It
 * replaces the Win32 demo driver (Main.cpp), whose scene-building steps
 * (Main.cpp:86-128) and per-frame loop (Main.cpp:181-206) are restated here
 * as plain C entry points for ctypes.
 */
#define private public /* read-back of the depth buffer, hiZ and mask table */
#include "Rasterizer.h"
#undef private
#include "Occluder.h"
#include "QuadDecomposition.h"
#include "SurfaceAreaHeuristic.h"
#include "VectorMath.h"

#include <chrono>
#include <cstdio>

namespace {

__m128 load4(const float* p) { return _mm_loadu_ps(p); }
void store4(float* p, __m128 v) { _mm_storeu_ps(p, v); }

struct Scene {
  std::vector<std::unique_ptr<Occluder>> occluders;
  std::vector<uint32_t> quadIndices;  // after decomposition and padding
  std::vector<std::vector<uint32_t>> batches;
};

Occluder makeOccluder(const uint32_t* packed, uint32_t packetCount, const float* refMin, const float* refMax)
{
  Occluder o;
  o.m_vertexData = reinterpret_cast<__m256i*>(const_cast<uint32_t*>(packed));
  o.m_packetCount = packetCount;
  o.m_refMin = load4(refMin);
  o.m_refMax = load4(refMax);
  o.m_boundsMin = o.m_boundsMax = o.m_center = _mm_setzero_ps();
  return o;
}

}  // namespace

extern "C" {

/* ---- bake pipeline, one stage at a time ---------------------------------- */

uint32_t ref_decompose(const uint32_t* idx, uint32_t nidx, const float* verts, uint32_t nverts, uint32_t* out)
{
  std::vector<uint32_t> indices(idx, idx + nidx);
  std::vector<__m128> vertices(nverts);
  for (uint32_t i = 0; i < nverts; ++i) vertices[i] = load4(verts + 4 * i);
  std::vector<uint32_t> quads = QuadDecomposition::decompose(indices, vertices);
  std::copy(quads.begin(), quads.end(), out);
  return (uint32_t)quads.size();
}

uint32_t ref_sah(const float* aabbs, uint32_t n, uint32_t targetSize, uint32_t granularity,
                 uint32_t* flat, uint32_t* offsets)
{
  std::vector<Aabb> boxes(n);
  for (uint32_t i = 0; i < n; ++i) {
    boxes[i].m_min = load4(aabbs + 8 * i);
    boxes[i].m_max = load4(aabbs + 8 * i + 4);
  }
  auto batches = SurfaceAreaHeuristic::generateBatches(boxes, targetSize, granularity);
  uint32_t pos = 0;
  for (size_t b = 0; b < batches.size(); ++b) {
    offsets[b] = pos;
    for (uint32_t q : batches[b]) flat[pos++] = q;
  }
  offsets[batches.size()] = pos;
  return (uint32_t)batches.size();
}

/* vertices: nverts float4 (multiple of 16).  packed_out: nverts uint32 words. */
uint32_t ref_bake(const float* verts, uint32_t nverts, const float* refMin, const float* refMax,
                  uint32_t* packed_out, float* boundsMin, float* boundsMax, float* center)
{
  std::vector<__m128> vertices(nverts);
  for (uint32_t i = 0; i < nverts; ++i) vertices[i] = load4(verts + 4 * i);
  auto occ = Occluder::bake(vertices, load4(refMin), load4(refMax));
  std::memcpy(packed_out, occ->m_vertexData, (size_t)occ->m_packetCount * 32);
  store4(boundsMin, occ->m_boundsMin);
  store4(boundsMax, occ->m_boundsMax);
  store4(center, occ->m_center);
  uint32_t packets = occ->m_packetCount;
  free(occ->m_vertexData);
  return packets;
}

/* ---- whole scene as the demo builds it (Main.cpp:86-128) ------------------ */

void* ref_scene_build(const uint32_t* idx, uint32_t nidx, const float* verts, uint32_t nverts)
{
  auto* scene = new Scene;
  std::vector<uint32_t> indices(idx, idx + nidx);
  std::vector<__m128> vertices(nverts);
  for (uint32_t i = 0; i < nverts; ++i) vertices[i] = load4(verts + 4 * i);

  indices = QuadDecomposition::decompose(indices, vertices);
  while (indices.size() % 32 != 0) indices.push_back(indices[0]);

  std::vector<Aabb> quadAabbs;
  for (size_t q = 0; q < indices.size() / 4; ++q) {
    Aabb aabb;
    for (int k = 0; k < 4; ++k) aabb.include(vertices[indices[4 * q + k]]);
    quadAabbs.push_back(aabb);
  }
  scene->batches = SurfaceAreaHeuristic::generateBatches(quadAabbs, 512, 8);

  Aabb refAabb;
  for (auto v : vertices) refAabb.include(v);

  for (const auto& batch : scene->batches) {
    std::vector<__m128> batchVertices;
    for (auto q : batch)
      for (int k = 0; k < 4; ++k) batchVertices.push_back(vertices[indices[q * 4 + k]]);
    scene->occluders.push_back(Occluder::bake(batchVertices, refAabb.m_min, refAabb.m_max));
  }
  scene->quadIndices = std::move(indices);
  return scene;
}

uint32_t ref_scene_count(void* s) { return (uint32_t)static_cast<Scene*>(s)->occluders.size(); }

uint32_t ref_scene_quad_indices(void* s, uint32_t* out)
{
  auto* scene = static_cast<Scene*>(s);
  if (out) std::copy(scene->quadIndices.begin(), scene->quadIndices.end(), out);
  return (uint32_t)scene->quadIndices.size();
}

uint32_t ref_scene_batch(void* s, uint32_t i, uint32_t* out)
{
  auto& b = static_cast<Scene*>(s)->batches[i];
  if (out) std::copy(b.begin(), b.end(), out);
  return (uint32_t)b.size();
}

/* Returns packetCount (number of 32-byte vectors); copies packed words if packed != NULL. */
uint32_t ref_scene_occluder(void* s, uint32_t i, uint32_t* packed, float* refMin, float* refMax,
                            float* bmin, float* bmax, float* center)
{
  const Occluder& o = *static_cast<Scene*>(s)->occluders[i];
  if (packed) std::memcpy(packed, o.m_vertexData, (size_t)o.m_packetCount * 32);
  if (refMin) store4(refMin, o.m_refMin);
  if (refMax) store4(refMax, o.m_refMax);
  if (bmin) store4(bmin, o.m_boundsMin);
  if (bmax) store4(bmax, o.m_boundsMax);
  if (center) store4(center, o.m_center);
  return o.m_packetCount;
}

void ref_scene_free(void* s)
{
  auto* scene = static_cast<Scene*>(s);
  for (auto& o : scene->occluders) free(o->m_vertexData);  // the reference never frees it
  delete scene;
}

/* ---- rasterizer ---------------------------------------------------------- */

void* ref_raster_create(uint32_t w, uint32_t h) { return new Rasterizer(w, h); }
void ref_raster_destroy(void* r) { delete static_cast<Rasterizer*>(r); }
void ref_raster_set_mvp(void* r, const float* m) { static_cast<Rasterizer*>(r)->setModelViewProjection(m); }
void ref_raster_clear(void* r) { static_cast<Rasterizer*>(r)->clear(); }

/* packed must be 32-byte aligned (the reference stream-loads it). */
void ref_raster_rasterize(void* r, const uint32_t* packed, uint32_t packetCount,
                          const float* refMin, const float* refMax, int nearClip)
{
  Occluder o = makeOccluder(packed, packetCount, refMin, refMax);
  if (nearClip) static_cast<Rasterizer*>(r)->rasterize<true>(o);
  else static_cast<Rasterizer*>(r)->rasterize<false>(o);
}

void ref_raster_rasterize_scene(void* r, void* s, uint32_t i, int nearClip)
{
  const Occluder& o = *static_cast<Scene*>(s)->occluders[i];
  if (nearClip) static_cast<Rasterizer*>(r)->rasterize<true>(o);
  else static_cast<Rasterizer*>(r)->rasterize<false>(o);
}

int ref_raster_query(void* r, const float* bmin, const float* bmax, int* needsClipping)
{
  bool nc = false;
  bool v = static_cast<Rasterizer*>(r)->queryVisibility(load4(bmin), load4(bmax), nc);
  *needsClipping = nc ? 1 : 0;
  return v ? 1 : 0;
}

void ref_raster_query_batch(void* r, uint32_t n, const float* mins, const float* maxs, uint8_t* vis, uint8_t* nc)
{
  auto* R = static_cast<Rasterizer*>(r);
  for (uint32_t i = 0; i < n; ++i) {
    bool c = false;
    vis[i] = R->queryVisibility(load4(mins + 4 * i), load4(maxs + 4 * i), c) ? 1 : 0;
    nc[i] = c ? 1 : 0;
  }
}

int ref_raster_query2d(void* r, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ)
{
  return static_cast<Rasterizer*>(r)->query2D(minX, maxX, minY, maxY, maxZ) ? 1 : 0;
}

void ref_raster_read_depth(void* r, uint16_t* out)
{
  auto* R = static_cast<Rasterizer*>(r);
  std::memcpy(out, R->m_depthBuffer.data(), R->m_depthBuffer.size() * 16);
}

uint32_t ref_raster_read_hiz(void* r, uint16_t* out)
{
  auto* R = static_cast<Rasterizer*>(r);
  if (out) std::memcpy(out, R->m_hiZ.data(), R->m_hiZ.size() * 2);
  return (uint32_t)R->m_hiZ.size();
}

void ref_raster_read_table(void* r, int64_t* out)
{
  auto* R = static_cast<Rasterizer*>(r);
  std::memcpy(out, R->m_precomputedRasterTables.data(), R->m_precomputedRasterTables.size() * 8);
}

void ref_raster_read_back(void* r, uint8_t* rgba) { static_cast<Rasterizer*>(r)->readBackDepth(rgba); }

/*
 * One frame of the plain all-occluder loop (the parity mode): for each
 * occluder in submission order, queryVisibility of its bounds on `scratch`
 * (a rasterizer that is never drawn into) gives the frustum cull and the
 * near-clip variant; visible occluders are rasterised into `r`.
 * Mirrors Main.cpp:181-206 without the distance sort and without gating on
 * the live buffer.  flags[i] = visible | needsClipping << 1.
 */
void ref_frame_plain(void* r, void* scratch, void* s, const uint32_t* order, uint32_t n,
                     const float* mvp, uint8_t* flags)
{
  auto* R = static_cast<Rasterizer*>(r);
  auto* S = static_cast<Rasterizer*>(scratch);
  auto* scene = static_cast<Scene*>(s);
  R->clear();
  R->setModelViewProjection(mvp);
  S->setModelViewProjection(mvp);
  for (uint32_t k = 0; k < n; ++k) {
    const Occluder& o = *scene->occluders[order ? order[k] : k];
    bool nc = false;
    bool vis = S->queryVisibility(o.m_boundsMin, o.m_boundsMax, nc);
    if (flags) flags[k] = (vis ? 1 : 0) | (nc ? 2 : 0);
    if (!vis) continue;
    if (nc) R->rasterize<true>(o);
    else R->rasterize<false>(o);
  }
}

/*
 * Main.cpp's own gated loop (Main.cpp:181-206): sort occluders front to back by
 * squared distance of their centre to the eye, then query each against the
 * live buffer before rasterising it.  Order dependent; CPU-baseline variant.
 */
void ref_frame_gated(void* r, void* s, const float* mvp, const float* eye)
{
  auto* R = static_cast<Rasterizer*>(r);
  auto* scene = static_cast<Scene*>(s);
  __m128 cam = load4(eye);
  R->clear();
  R->setModelViewProjection(mvp);
  std::vector<Occluder*> occ;
  for (auto& o : scene->occluders) occ.push_back(o.get());
  std::sort(occ.begin(), occ.end(), [&](const Occluder* a, const Occluder* b) {
    __m128 d1 = _mm_sub_ps(a->m_center, cam), d2 = _mm_sub_ps(b->m_center, cam);
    return _mm_comilt_ss(_mm_dp_ps(d1, d1, 0x7f), _mm_dp_ps(d2, d2, 0x7f));
  });
  for (Occluder* o : occ) {
    bool nc = false;
    if (R->queryVisibility(o->m_boundsMin, o->m_boundsMax, nc)) {
      if (nc) R->rasterize<true>(*o);
      else R->rasterize<false>(*o);
    }
  }
}

/* Timed loop of plain frames + queries; returns seconds for `frames` frames. */
double ref_time_plain(void* r, void* scratch, void* s, uint32_t nframes, const float* mvps,
                      uint32_t nq, const float* mins, const float* maxs, uint8_t* vis, uint8_t* nc)
{
  auto* scene = static_cast<Scene*>(s);
  uint32_t n = (uint32_t)scene->occluders.size();
  auto t0 = std::chrono::steady_clock::now();
  for (uint32_t f = 0; f < nframes; ++f) {
    ref_frame_plain(r, scratch, s, nullptr, n, mvps + 16 * f, nullptr);
    if (nq) ref_raster_query_batch(r, nq, mins, maxs, vis, nc);
  }
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
