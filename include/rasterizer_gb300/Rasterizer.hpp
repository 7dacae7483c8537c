// C++ facade with the reference's class names and signatures
// (SoftwareRasterizer/Rasterizer.h:10-61, Occluder.h:7-21,
// QuadDecomposition.h:5-10, SurfaceAreaHeuristic.h:5-12) over the C ABI of
// librasterizer_gb300.  Header only; link with -lrasterizer_gb300.
//
// Differences a caller of the reference sees:
//  * a Context (one GPU, one CUDA stream) is passed to the Rasterizer and to
//    Occluder::upload;
//  * vectors are Vec4 (four floats) instead of __m128; with SSE available the
//    __m128 overloads are provided too;
//  * rasterize() is deferred: the next query, read-back or flush runs the
//    pending work on the GPU in one batch (results are those of immediate
//    execution);
//  * errors throw gb300::Error instead of asserting.
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../rasterizer_gb300.h"

#if defined(__SSE__) || defined(_M_X64)
#include <xmmintrin.h>
#define GB300_HAVE_M128 1
#endif

namespace gb300 {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& where) : std::runtime_error(where + ": " + occ_last_error()), status(s) {}
};

inline void check(int s, const char* where)
{
  if (s != OCC_OK) throw Error(s, where);
}

struct Vec4 {
  float v[4];
};

class Context {
 public:
  explicit Context(int device = 0) { check(occ_ctx_create(device, &h_), "occ_ctx_create"); }
  ~Context() { occ_ctx_destroy(h_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  occ_ctx handle() const { return h_; }
  void synchronize() { check(occ_ctx_synchronize(h_), "occ_ctx_synchronize"); }

 private:
  occ_ctx h_ = nullptr;
};

// Occluder::bake output (Occluder.h:7-21): packed 11/11/10 words, 8 quads per
// 4 vectors, quantisation box, bounds with w = 1.
struct Occluder {
  static std::unique_ptr<Occluder> bake(const std::vector<Vec4>& vertices, Vec4 refMin, Vec4 refMax)
  {
    auto o = std::make_unique<Occluder>();
    o->m_vertexData.resize(vertices.size());
    check(occ_occluder_bake(&vertices[0].v[0], (uint32_t)vertices.size(), refMin.v, refMax.v, o->m_vertexData.data(),
                            &o->m_packetCount, o->m_boundsMin.v, o->m_boundsMax.v, o->m_center.v),
          "occ_occluder_bake");
    o->m_vertexData.resize((size_t)o->m_packetCount * 8);
    o->m_refMin = refMin;
    o->m_refMax = refMax;
    return o;
  }

  // Copies the packed data to the GPU once per context.
  occ_occluder upload(Context& ctx) const
  {
    if (m_uploadedTo != ctx.handle()) {
      check(occ_occluder_upload(ctx.handle(), m_vertexData.data(), m_packetCount, m_refMin.v, m_refMax.v,
                                m_boundsMin.v, m_boundsMax.v, &m_id),
            "occ_occluder_upload");
      m_uploadedTo = ctx.handle();
    }
    return m_id;
  }

  Vec4 m_center{}, m_refMin{}, m_refMax{}, m_boundsMin{}, m_boundsMax{};
  std::vector<uint32_t> m_vertexData;
  uint32_t m_packetCount = 0;

 private:
  mutable occ_ctx m_uploadedTo = nullptr;
  mutable occ_occluder m_id = 0;
};

// The reference demo's mesh files (Main.cpp:56-84): dir/VertexBuffer.bin and
// dir/IndexBuffer.bin.
inline void loadMeshBin(const std::string& dir, std::vector<Vec4>& vertices, std::vector<uint32_t>& indices)
{
  const std::string vp = dir + "/VertexBuffer.bin", ip = dir + "/IndexBuffer.bin";
  uint32_t nv = 0, ni = 0;
  check(occ_mesh_load_bin(vp.c_str(), ip.c_str(), nullptr, &nv, nullptr, &ni), "occ_mesh_load_bin");
  vertices.resize(nv ? nv : 1);
  indices.resize(ni ? ni : 1);
  check(occ_mesh_load_bin(vp.c_str(), ip.c_str(), &vertices[0].v[0], &nv, indices.data(), &ni), "occ_mesh_load_bin");
  vertices.resize(nv);
  indices.resize(ni);
}

// The demo's scene preparation in one call (Main.cpp:86-128): decomposition,
// padding, SAH batches (targetSize, splitGranularity), one Occluder::bake per
// batch in the box of all vertices.
inline std::vector<std::unique_ptr<Occluder>> bakeScene(const std::vector<Vec4>& vertices,
                                                        const std::vector<uint32_t>& indices, uint32_t targetSize = 512,
                                                        uint32_t splitGranularity = 8)
{
  const uint32_t quads = (uint32_t)(indices.size() / 3) + 7;
  const uint32_t capCount = quads / 8 + 1;
  const uint64_t capWords = 4ull * quads;
  std::vector<uint32_t> counts(capCount), packed(capWords ? capWords : 1);
  std::vector<float> bounds(20 * (size_t)capCount);
  uint32_t n = 0;
  uint64_t words = 0;
  check(occ_scene_bake(vertices.empty() ? nullptr : &vertices[0].v[0], (uint32_t)vertices.size(),
                       indices.empty() ? nullptr : indices.data(), (uint32_t)indices.size(), targetSize,
                       splitGranularity, capCount, capWords, &n, &words, counts.data(), packed.data(), bounds.data()),
        "occ_scene_bake");
  std::vector<std::unique_ptr<Occluder>> out;
  size_t pos = 0;
  for (uint32_t k = 0; k < n; ++k) {
    auto o = std::make_unique<Occluder>();
    o->m_packetCount = counts[k];
    o->m_vertexData.assign(packed.begin() + pos, packed.begin() + pos + 8 * (size_t)counts[k]);
    pos += 8 * (size_t)counts[k];
    Vec4* dst[5] = {&o->m_refMin, &o->m_refMax, &o->m_boundsMin, &o->m_boundsMax, &o->m_center};
    for (int j = 0; j < 5; ++j) std::memcpy(dst[j]->v, &bounds[20 * (size_t)k + 4 * j], 16);
    out.push_back(std::move(o));
  }
  return out;
}

// Baked occluders of a scene in one file, and back.
inline void saveOccluders(const std::string& path, const std::vector<std::unique_ptr<Occluder>>& occluders)
{
  std::vector<uint32_t> counts;
  std::vector<const uint32_t*> packed;
  std::vector<float> bounds;
  for (const auto& o : occluders) {
    counts.push_back(o->m_packetCount);
    packed.push_back(o->m_vertexData.data());
    for (const Vec4* b : {&o->m_refMin, &o->m_refMax, &o->m_boundsMin, &o->m_boundsMax, &o->m_center})
      bounds.insert(bounds.end(), b->v, b->v + 4);
  }
  check(occ_occluders_save(path.c_str(), (uint32_t)occluders.size(), counts.data(), packed.data(), bounds.data()),
        "occ_occluders_save");
}

inline std::vector<std::unique_ptr<Occluder>> loadOccluders(const std::string& path)
{
  uint32_t n = 0;
  uint64_t words = 0;
  check(occ_occluders_file_info(path.c_str(), &n, &words), "occ_occluders_file_info");
  std::vector<uint32_t> counts(n ? n : 1), packed(words ? words : 1);
  std::vector<float> bounds(20 * (size_t)(n ? n : 1));
  check(occ_occluders_load(path.c_str(), n, words, counts.data(), packed.data(), bounds.data()), "occ_occluders_load");
  std::vector<std::unique_ptr<Occluder>> out;
  size_t pos = 0;
  for (uint32_t k = 0; k < n; ++k) {
    auto o = std::make_unique<Occluder>();
    o->m_packetCount = counts[k];
    o->m_vertexData.assign(packed.begin() + pos, packed.begin() + pos + 8 * (size_t)counts[k]);
    pos += 8 * (size_t)counts[k];
    Vec4* dst[5] = {&o->m_refMin, &o->m_refMax, &o->m_boundsMin, &o->m_boundsMax, &o->m_center};
    for (int j = 0; j < 5; ++j) std::memcpy(dst[j]->v, &bounds[20 * (size_t)k + 4 * j], 16);
    out.push_back(std::move(o));
  }
  return out;
}

// Occluder::bake on the GPU for many occluders at once (device pointers; see
// occ_occluders_bake_device), asynchronous on the context's stream, and the
// registration of a device-resident packed occluder (occ_occluder_upload_device).
inline void bakeOnDevice(Context& ctx, const std::vector<uint32_t>& vertexStart, const float* dVertices,
                         const std::vector<float>& refBoxes, uint32_t* dPacked, float* dBounds)
{
  check(occ_occluders_bake_device(ctx.handle(), (uint32_t)(vertexStart.size() - 1), dVertices, vertexStart.data(),
                                  refBoxes.data(), dPacked, dBounds),
        "occ_occluders_bake_device");
}

inline occ_occluder uploadFromDevice(Context& ctx, const uint32_t* dPacked, uint32_t packetCount, const float bounds[20])
{
  occ_occluder id = 0;
  check(occ_occluder_upload_device(ctx.handle(), dPacked, packetCount, bounds, &id), "occ_occluder_upload_device");
  return id;
}

class Rasterizer {
 public:
  Rasterizer(Context& ctx, uint32_t width, uint32_t height) : ctx_(ctx), w_(width), h_(height)
  {
    check(occ_raster_create(ctx.handle(), width, height, &r_), "occ_raster_create");
  }
  ~Rasterizer() { occ_raster_destroy(r_); }
  Rasterizer(const Rasterizer&) = delete;
  Rasterizer& operator=(const Rasterizer&) = delete;

  void setModelViewProjection(const float* matrix) { check(occ_raster_set_mvp(r_, matrix), "occ_raster_set_mvp"); }
  void clear() { check(occ_raster_clear(r_), "occ_raster_clear"); }

  template <bool possiblyNearClipped>
  void rasterize(const Occluder& occluder)
  {
    check(occ_raster_rasterize(r_, occluder.upload(ctx_), possiblyNearClipped ? 1 : 0), "occ_raster_rasterize");
  }

  bool queryVisibility(Vec4 boundsMin, Vec4 boundsMax, bool& needsClipping)
  {
    int v = 0, c = 0;
    check(occ_raster_query_visibility(r_, boundsMin.v, boundsMax.v, &v, &c), "occ_raster_query_visibility");
    needsClipping = c != 0;
    return v != 0;
  }

#ifdef GB300_HAVE_M128
  bool queryVisibility(__m128 boundsMin, __m128 boundsMax, bool& needsClipping)
  {
    Vec4 a, b;
    _mm_storeu_ps(a.v, boundsMin);
    _mm_storeu_ps(b.v, boundsMax);
    return queryVisibility(a, b, needsClipping);
  }
#endif

  bool query2D(uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ) const
  {
    int v = 0;
    check(occ_raster_query2d(r_, minX, maxX, minY, maxY, maxZ, &v), "occ_raster_query2d");
    return v != 0;
  }

  void readBackDepth(void* target) const { check(occ_raster_read_back_depth(r_, target), "occ_raster_read_back_depth"); }
  // OCC_READBACK_* format: width*height elements of 4 (RGBA8, float) or 2 (u16) bytes
  void readBack(int format, void* target) const { check(occ_raster_read_back(r_, format, target), "occ_raster_read_back"); }

  // Batch form of queryVisibility: one bit per box (bit i%32 of word i/32).
  void queryVisibilityBatch(uint32_t n, const Vec4* mins, const Vec4* maxs, uint32_t* visibleBits,
                            uint32_t* needsClippingBits)
  {
    check(occ_raster_query_batch(r_, n, &mins[0].v[0], &maxs[0].v[0], visibleBits, needsClippingBits),
          "occ_raster_query_batch");
  }

  void flush() { check(occ_raster_flush(r_), "occ_raster_flush"); }
  occ_raster handle() const { return r_; }

 private:
  Context& ctx_;
  occ_raster r_ = nullptr;
  uint32_t w_, h_;
};

// The learned occluder selector (replaces the distance-sorted loop of
// Main.cpp:184-206): an MLP scoring each occluder of a view.
class OccluderSelector {
 public:
  explicit OccluderSelector(Context& ctx, uint32_t seed = 0) { check(occ_mlp_create(ctx.handle(), seed, &m_), "occ_mlp_create"); }
  ~OccluderSelector() { occ_mlp_destroy(m_); }
  OccluderSelector(const OccluderSelector&) = delete;
  OccluderSelector& operator=(const OccluderSelector&) = delete;
  static uint32_t paramCount() { return (uint32_t)occ_mlp_param_count(); }
  std::vector<float> params() const
  {
    std::vector<float> p(paramCount());
    check(occ_mlp_get_params(m_, p.data()), "occ_mlp_get_params");
    return p;
  }
  void setParams(const std::vector<float>& p) { check(occ_mlp_set_params(m_, p.data()), "occ_mlp_set_params"); }
  // one listwise Adam step: rows in groups [groupStart[g], groupStart[g+1])
  float trainStepListwise(uint32_t n, const float* features, const float* targets, const std::vector<uint32_t>& groupStart,
                          float lr)
  {
    float loss = 0;
    check(occ_mlp_train_step_listwise(m_, n, features, targets, (uint32_t)groupStart.size() - 1, groupStart.data(), lr,
                                      &loss),
          "occ_mlp_train_step_listwise");
    return loss;
  }
  occ_mlp handle() const { return m_; }

 private:
  occ_mlp m_ = nullptr;
};

// Many views prepared once and launched as one CUDA graph per frame.
class Batch {
 public:
  struct View {
    Rasterizer* raster;
    const float* mvp;                          // float[16]
    std::vector<const Occluder*> occluders;
    std::vector<uint8_t> flags;                // OCC_GATED / OCC_NEAR_CLIP per occluder (empty: all 0)
    std::vector<Vec4> queryMins, queryMaxs;
  };

  Batch(Context& ctx, const std::vector<View>& views) : views_(views.size())
  {
    std::vector<occ_view_work> w(views.size());
    for (size_t i = 0; i < views.size(); ++i) {
      const View& v = views[i];
      std::vector<occ_occluder>& ids = ids_.emplace_back();
      for (const Occluder* o : v.occluders) ids.push_back(o->upload(ctx));
      occ_view_work& x = w[i];
      std::memset(&x, 0, sizeof(x));
      x.raster = v.raster->handle();
      x.mvp = v.mvp;
      x.clear = 1;
      x.numOccluders = (uint32_t)ids.size();
      x.occluders = ids.data();
      x.flags = v.flags.empty() ? nullptr : v.flags.data();
      x.numQueries = (uint32_t)v.queryMins.size();
      x.queryMins = x.numQueries ? &v.queryMins[0].v[0] : nullptr;
      x.queryMaxs = x.numQueries ? &v.queryMaxs[0].v[0] : nullptr;
      queries_.push_back(x.numQueries);
    }
    check(occ_batch_prepare(ctx.handle(), (uint32_t)w.size(), w.data(), &b_), "occ_batch_prepare");
  }
  ~Batch() { occ_batch_destroy(b_); }
  Batch(const Batch&) = delete;
  Batch& operator=(const Batch&) = delete;

  void setModelViewProjection(uint32_t view, const float* m) { check(occ_batch_set_mvp(b_, view, m), "occ_batch_set_mvp"); }
  // top `fraction` of each view's candidates by the selector's score
  void setSelection(OccluderSelector* selector, float fraction, bool trackWins = true)
  {
    check(occ_batch_set_selection(b_, selector ? selector->handle() : nullptr, fraction, trackWins ? 1 : 0),
          "occ_batch_set_selection");
  }
  void setSecondPass(bool enable) { check(occ_batch_set_second_pass(b_, enable ? 1 : 0), "occ_batch_set_second_pass"); }
  void autotune(uint32_t iterations = 5) { check(occ_batch_autotune(b_, iterations, nullptr, nullptr, nullptr), "occ_batch_autotune"); }
  // launch shapes in occ_batch_autotune's layout (0 = default)
  void setTuning(const uint32_t tune[OCC_TUNING_FIELDS]) { check(occ_batch_set_tuning(b_, tune), "occ_batch_set_tuning"); }
  void launch() { check(occ_batch_launch(b_), "occ_batch_launch"); }
  // false if a launch since the last check outgrew the scratch (grown now: run the frame again)
  bool check_capacity()
  {
    const int s = occ_batch_check(b_);
    if (s == OCC_ERR_CAPACITY) return false;
    check(s, "occ_batch_check");
    return true;
  }
  // visibility bits of one view's boxes (bit i%32 of word i/32)
  void results(uint32_t view, std::vector<uint32_t>& visibleBits, std::vector<uint32_t>& needsClippingBits)
  {
    const size_t nw = (queries_.at(view) + 31) / 32;
    visibleBits.resize(nw);
    needsClippingBits.resize(nw);
    check(occ_batch_results(b_, view, visibleBits.data(), needsClippingBits.data()), "occ_batch_results");
  }
  occ_batch handle() const { return b_; }

 private:
  occ_batch b_ = nullptr;
  size_t views_;
  std::vector<std::vector<occ_occluder>> ids_;
  std::vector<uint32_t> queries_;
};

struct QuadDecomposition {
  static std::vector<uint32_t> decompose(const std::vector<uint32_t>& indices, const std::vector<Vec4>& vertices)
  {
    std::vector<uint32_t> out(4 * (indices.size() / 3) + 4);
    uint32_t n = 0;
    check(occ_quad_decompose(indices.data(), (uint32_t)indices.size(), &vertices[0].v[0], (uint32_t)vertices.size(),
                             out.data(), &n),
          "occ_quad_decompose");
    out.resize(n);
    return out;
  }
};

struct Aabb {
  Vec4 m_min{}, m_max{};
};

struct SurfaceAreaHeuristic {
  static std::vector<std::vector<uint32_t>> generateBatches(const std::vector<Aabb>& aabbs, uint32_t targetSize,
                                                            uint32_t splitGranularity)
  {
    const uint32_t n = (uint32_t)aabbs.size();
    std::vector<float> flatBoxes((size_t)n * 8);
    for (uint32_t i = 0; i < n; ++i) {
      std::memcpy(&flatBoxes[8 * (size_t)i], aabbs[i].m_min.v, 16);
      std::memcpy(&flatBoxes[8 * (size_t)i + 4], aabbs[i].m_max.v, 16);
    }
    std::vector<uint32_t> flat(n + 1), offsets(n + 2);
    uint32_t nb = 0;
    check(occ_sah_generate_batches(flatBoxes.data(), n, targetSize, splitGranularity, flat.data(), offsets.data(), &nb),
          "occ_sah_generate_batches");
    std::vector<std::vector<uint32_t>> out(nb);
    for (uint32_t b = 0; b < nb; ++b) out[b].assign(flat.begin() + offsets[b], flat.begin() + offsets[b + 1]);
    return out;
  }
};

}  // namespace gb300
