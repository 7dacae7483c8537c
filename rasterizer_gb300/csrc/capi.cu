// C ABI of the GB300 occluder rasteriser: contexts, occluder storage,
// rasterizer targets, deferred command lists, batches and CUDA graphs.
// Host-side float math here (setModelViewProjection) is compiled with
// -ffp-contract=off and goes through x86_emu.cuh, like the kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/rasterizer_gb300.h"
#include "coverage_table.h"
#include "coverage_table_build.h"
#include "raster_types.h"
#include "sah_scratch.h"
#include "x86_emu.cuh"

namespace occ {
cudaError_t launch_flush(const FrameParams& P, uint32_t numSt, uint32_t maxStPerView, bool doRaster,
                         bool doQuery, cudaStream_t stream);
cudaError_t launch_read_back(const uint16_t* depth, const uint16_t* hiz, uint32_t width, uint32_t height,
                             int format, void* out, cudaStream_t stream);
cudaError_t launch_flush_timed(const FrameParams& P, uint32_t numSt, uint32_t maxStPerView, bool doRaster,
                               bool doQuery, cudaStream_t stream, cudaEvent_t* ev);
cudaError_t set_kernel_attributes();
cudaError_t launch_selection(const FrameParams& P, uint32_t numCmds, bool useMlp, cudaStream_t stream);
cudaError_t launch_mlp_forward(const float* feat, uint32_t M, const MlpDevice* mlp, float* score, float* h1, float* h2,
                               float* xb, cudaStream_t stream);
cudaError_t launch_mlp_backward(const float* score, const float* target, uint32_t B, const MlpDevice* mlp,
                                const float* xb, const float* h1, const float* h2, float* ds, float* dh1, float* dh2,
                                float* err2, float* partial, float* grad, cudaStream_t stream,
                                const uint32_t* groupStart = nullptr, uint32_t groups = 0);
uint32_t mlp_grad_blocks(uint32_t B);
cudaError_t launch_mlp_publish(const float* params, MlpDevice* mlp, cudaStream_t stream);
cudaError_t launch_cull_labels(const FrameParams& P, cudaStream_t stream);
void tuning_limits(uint32_t out[7]);
cudaError_t launch_adam(float* params, const float* grad, float* m, float* v, float lr, uint32_t step,
                        cudaStream_t stream);
int mlp_param_count();
cudaError_t query_noalloc(int device, const ViewDesc& view, uint32_t n, const float* mins, const float* maxs,
                          uint32_t* visibleBits, uint32_t* needsClippingBits, cudaStream_t stream);
cudaError_t launch_tile_hiz(const uint16_t* hiz, uint16_t* tileHiz, uint32_t blocksX, uint32_t blocksY,
                            cudaStream_t stream);
cudaError_t launch_query2d(const ViewDesc* view, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY,
                           uint32_t maxZ, uint32_t* out, cudaStream_t stream);
int set_error(int code, const char* msg);
cudaError_t launch_bake(const BakeJob* jobs, uint32_t count, const float4* vertices, float4* normals,
                        uint32_t* cluster, uint32_t* order, uint32_t* packed, float* bounds, cudaStream_t stream);
int sah_generate_device(SahScratch& S, uint32_t n, const float* aabbs, uint32_t target, uint32_t gran,
                        uint32_t* flat, std::vector<uint32_t>& offsets, cudaStream_t st, std::string& err);
}  // namespace occ

using namespace occ;

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg)
{
  g_error = msg;
  return code;
}

}  // namespace

// The message occ_last_error returns, for the host-only sources (files.cpp).
int occ::set_error(int code, const char* msg)
{
  return fail(code, msg);
}

namespace {

#define OCC_CUDA(call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return fail(OCC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define OCC_CHECK(call)         \
  do {                          \
    int s_ = (call);            \
    if (s_ != OCC_OK) return s_; \
  } while (0)

uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release()
  {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  // grows to at least m elements; contents are not kept
  int reserve(size_t m)
  {
    if (m <= n && p) return OCC_OK;
    release();
    size_t want = std::max<size_t>(m, 1);
    cudaError_t e = cudaMalloc(&p, want * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(OCC_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    n = want;
    return OCC_OK;
  }
};

template <class T>
struct PinBuf {
  T* p = nullptr;
  size_t n = 0;
  PinBuf() = default;
  PinBuf(const PinBuf&) = delete;
  PinBuf& operator=(const PinBuf&) = delete;
  ~PinBuf()
  {
    if (p) cudaFreeHost(p);
  }
  int reserve(size_t m)
  {
    if (m <= n && p) return OCC_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    size_t want = std::max<size_t>(m, 1);
    cudaError_t e = cudaMallocHost(&p, want * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(OCC_ERR_OUT_OF_MEMORY, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    n = want;
    return OCC_OK;
  }
};

struct OccluderRec {
  uint32_t wordOffset, packetCount;
  float refMin[4], refMax[4], boundsMin[4], boundsMax[4];
};

struct PendingCmd {
  uint32_t occ;
  uint32_t flags;
};

// Scratch of one frame batch (grows, never shrinks).
struct FrameScratch {
  DevBuf<uint8_t> tables;  // views | cmds | chunks
  DevBuf<QuadRaster> rec;
  DevBuf<QuadWalk> walk;
  DevBuf<Totals> chunkTot, chunkBase, viewTot, viewBase;
  DevBuf<uint32_t> mat, stStart, stLen, cmdDraw, ckBase, activeChunks, viewActive, viewActiveCount;
  DevBuf<uint4> activeTiles;
  DevBuf<uint4> stList;
  DevBuf<float> ck;
  DevBuf<uint2> rowOwner;  // sized like the checkpoints (a row has at least one)
  DevBuf<FrameHeader> header;
  DevBuf<float4> qmin, qmax;
  DevBuf<uint32_t> visBits, ncBits;
  uint32_t capCks = 0, capSt = 0;
};

}  // namespace

struct occ_raster_s;

struct occ_ctx_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  DevBuf<uint32_t> pool;  // packed occluder words
  size_t poolWords = 0;
  std::vector<OccluderRec> occluders;
  FrameScratch scratch;
  PinBuf<uint8_t> stage;  // host staging for tables / queries
  PinBuf<uint8_t> readback;
  cudaEvent_t stageFree = nullptr;  // signalled when the last upload from `stage` finished
  DevBuf<int64_t> table;
  // GPU bake: job table and per-quad scratch (normals, cluster, order)
  DevBuf<BakeJob> bakeJobs;
  DevBuf<float4> bakeNormals;
  DevBuf<uint32_t> bakeCluster, bakeOrder;
  DevBuf<uint8_t> sah;  // GPU SAH batching scratch (sah_gpu.cu), grown on demand
};

struct occ_raster_s {
  occ_ctx_s* ctx = nullptr;
  uint32_t width = 0, height = 0, blocksX = 0, blocksY = 0;
  DevBuf<uint16_t> depth, hiz, tileHiz;
  DevBuf<uint32_t> owner;  // per pixel: command + 1 of its final value (cull labels only)
  float cols[16] = {};
  float rows[16] = {};
  bool clearPending = false;
  std::vector<PendingCmd> pending;
  std::vector<uint8_t> lastFlags;  // gated results of the last flush, per command
};

namespace {

// Rasterizer::setModelViewProjection (Rasterizer.cpp:76-105).
void bake_mvp(const float* m, uint32_t width, uint32_t height, float cols[16], float rows[16])
{
  using namespace x86;
  float row[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) row[i][j] = m[4 * j + i];
  std::memcpy(rows, row, sizeof(row));
  const float sx = (float)width * 0.5f - 4.0f;
  const float sy = (float)height * 0.5f - 4.0f;
  const float sz = 0.5f * 2.5237386e-29f;
  float baked[4][4];
  for (int j = 0; j < 4; ++j) {
    baked[0][j] = xmul(xadd(row[0][j], row[3][j]), sx);
    baked[1][j] = xmul(xadd(row[1][j], row[3][j]), sy);
    baked[2][j] = xmul(xsub(row[3][j], row[2][j]), sz);
    baked[3][j] = row[3][j];
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) cols[4 * j + i] = baked[i][j];
}

// One view of a batch as the host lays it out.
struct ViewJob {
  occ_raster_s* r;
  const PendingCmd* cmds;
  uint32_t ncmds;
  bool clear;
  uint32_t nq;
  const float* hmin;  // host query boxes (or null)
  const float* hmax;
  const void* dmin;   // device query boxes (single-view zero-copy path)
  const void* dmax;
  uint32_t* hvis;     // host outputs
  uint32_t* hnc;
  void* dvis;         // device outputs
  void* dnc;
};

struct BatchLayout {
  std::vector<ViewDesc> views;
  std::vector<Cmd> cmds;
  std::vector<Chunk> chunks;
  uint32_t numSt = 0, maxStPerView = 0, numTiles = 0, matSize = 0, querySlots = 0;
  uint32_t totalQuads = 0;
};

// stShift: super-tile edge 1 << stShift blocks (3 or 4); a view whose grid
// of such super-tiles would exceed kMaxStPerView takes 16-block super-tiles.
int build_layout(occ_ctx_s* ctx, const std::vector<ViewJob>& jobs, BatchLayout& L, uint32_t stShift = 4)
{
  uint32_t quadBase = 0, chunkBase = 0, tileBase = 0, stBase = 0, matBase = 0, queryBase = 0;
  for (size_t v = 0; v < jobs.size(); ++v) {
    const ViewJob& J = jobs[v];
    occ_raster_s* r = J.r;
    ViewDesc V{};
    V.depth = r->depth.p;
    V.hiz = r->hiz.p;
    V.tileHiz = r->tileHiz.p;
    V.width = r->width;
    V.height = r->height;
    V.blocksX = r->blocksX;
    V.blocksY = r->blocksY;
    std::memcpy(V.cols, r->cols, sizeof(V.cols));
    std::memcpy(V.rows, r->rows, sizeof(V.rows));
    V.cmdStart = (uint32_t)L.cmds.size();
    V.cmdCount = J.ncmds;
    uint32_t q = quadBase;
    for (uint32_t i = 0; i < J.ncmds; ++i) {
      const PendingCmd& pc = J.cmds[i];
      if (pc.occ >= ctx->occluders.size()) return fail(OCC_ERR_INVALID_ARG, "unknown occluder id");
      const OccluderRec& o = ctx->occluders[pc.occ];
      Cmd c{};
      c.view = (uint32_t)v;
      c.wordOffset = o.wordOffset;
      c.quadStart = q;
      c.quadCount = o.packetCount * 2;
      c.flags = pc.flags;
      std::memcpy(c.refMin, o.refMin, 16);
      std::memcpy(c.refMax, o.refMax, 16);
      std::memcpy(c.boundsMin, o.boundsMin, 16);
      std::memcpy(c.boundsMax, o.boundsMax, 16);
      q += c.quadCount;
      L.cmds.push_back(c);
    }
    const uint32_t nq = q - quadBase;
    V.chunkStart = chunkBase;
    V.chunkCount = div_up(nq, kChunk);
    uint32_t ci = V.cmdStart;  // first command overlapping each chunk
    for (uint32_t k = 0; k < V.chunkCount; ++k) {
      Chunk ch{};
      ch.view = (uint32_t)v;
      ch.localIndex = k;
      const uint32_t c0 = quadBase + k * kChunk;
      const uint32_t c1 = std::min(c0 + kChunk, q);
      ch.quadCount = c1 - c0;
      while (ci + 1 < V.cmdStart + V.cmdCount && L.cmds[ci + 1].quadStart <= c0) ++ci;
      ch.cmdFirst = ci;
      uint32_t cj = ci;
      while (cj + 1 < V.cmdStart + V.cmdCount && L.cmds[cj + 1].quadStart < c1) ++cj;
      ch.cmdCount = cj - ci + 1;
      if (ch.cmdCount > (uint32_t)kMaxCmdPerChunk) return fail(OCC_ERR_INVALID_ARG, "too many commands per chunk");
      L.chunks.push_back(ch);
    }
    quadBase += V.chunkCount * kChunk;
    chunkBase += V.chunkCount;
    V.tilesX = div_up(r->blocksX, kTileW);
    V.tilesY = div_up(r->blocksY, kTileH);
    V.tileStart = tileBase;
    tileBase += V.tilesX * V.tilesY;
    uint32_t sh = stShift;
    if ((size_t)div_up(r->blocksX, 1u << sh) * div_up(r->blocksY, 1u << sh) > (size_t)kMaxStPerView) sh = 4;
    V.stShift = sh;
    V.stX = div_up(r->blocksX, 1u << sh);
    V.stY = div_up(r->blocksY, 1u << sh);
    V.stBase = stBase;
    stBase += V.stX * V.stY;
    L.maxStPerView = std::max(L.maxStPerView, V.stX * V.stY);
    V.matBase = matBase;
    matBase += V.stX * V.stY * V.chunkCount;
    V.queryStart = queryBase;
    V.queryCount = J.nq;
    queryBase += div_up(J.nq, 32) * 32;
    V.flags = J.clear ? kViewClear : 0;
    L.views.push_back(V);
  }
  L.numSt = stBase;
  L.numTiles = tileBase;
  L.matSize = matBase;
  L.querySlots = queryBase;
  L.totalQuads = quadBase;
  return OCC_OK;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Runs one batch: uploads the tables, launches the kernels, reads results.
// With sync, retries with larger scratch if the first attempt overflowed.
int run_batch(occ_ctx_s* ctx, FrameScratch& S, std::vector<ViewJob>& jobs, bool sync)
{
  BatchLayout L;
  OCC_CHECK(build_layout(ctx, jobs, L));
  const uint32_t nv = (uint32_t)L.views.size();
  const size_t offViews = 0;
  const size_t offCmds = align_up(offViews + nv * sizeof(ViewDesc), 256);
  const size_t offChunks = align_up(offCmds + L.cmds.size() * sizeof(Cmd), 256);
  const size_t tablesBytes = align_up(offChunks + L.chunks.size() * sizeof(Chunk), 256);
  bool anyHostQuery = false, anyRaster = false;
  for (auto& J : jobs) {
    anyHostQuery |= J.nq && J.hmin;
    anyRaster |= J.ncmds || J.clear;
  }
  const size_t offQMin = tablesBytes;
  const size_t offQMax = offQMin + (anyHostQuery ? (size_t)L.querySlots * 16 : 0);
  const size_t offHdr = align_up(offQMax + (anyHostQuery ? (size_t)L.querySlots * 16 : 0), 64);
  const size_t stageBytes = offHdr + 64;

  // host staging (wait until the previous upload from it has finished)
  OCC_CUDA(cudaEventSynchronize(ctx->stageFree));
  OCC_CHECK(ctx->stage.reserve(stageBytes));
  uint8_t* st = ctx->stage.p;
  std::memcpy(st + offViews, L.views.data(), nv * sizeof(ViewDesc));
  if (!L.cmds.empty()) std::memcpy(st + offCmds, L.cmds.data(), L.cmds.size() * sizeof(Cmd));
  if (!L.chunks.empty()) std::memcpy(st + offChunks, L.chunks.data(), L.chunks.size() * sizeof(Chunk));
  if (anyHostQuery) {
    std::memset(st + offQMin, 0, (size_t)L.querySlots * 32);
    for (size_t v = 0; v < jobs.size(); ++v)
      if (jobs[v].nq && jobs[v].hmin) {
        std::memcpy(st + offQMin + (size_t)L.views[v].queryStart * 16, jobs[v].hmin, (size_t)jobs[v].nq * 16);
        std::memcpy(st + offQMax + (size_t)L.views[v].queryStart * 16, jobs[v].hmax, (size_t)jobs[v].nq * 16);
      }
  }

  // device scratch
  OCC_CHECK(S.tables.reserve(tablesBytes));
  OCC_CHECK(S.rec.reserve(L.totalQuads));
  OCC_CHECK(S.walk.reserve(L.totalQuads));
  OCC_CHECK(S.ckBase.reserve(L.totalQuads));
  OCC_CHECK(S.chunkTot.reserve(L.chunks.size()));
  OCC_CHECK(S.chunkBase.reserve(L.chunks.size()));
  OCC_CHECK(S.viewTot.reserve(nv));
  OCC_CHECK(S.viewBase.reserve(nv));
  OCC_CHECK(S.mat.reserve(L.matSize));
  OCC_CHECK(S.stStart.reserve(L.numSt));
  OCC_CHECK(S.stLen.reserve(L.numSt));
  OCC_CHECK(S.cmdDraw.reserve(L.cmds.size()));
  OCC_CHECK(S.activeChunks.reserve(L.chunks.size()));
  OCC_CHECK(S.viewActive.reserve(L.chunks.size()));
  OCC_CHECK(S.viewActiveCount.reserve(nv));
  OCC_CHECK(S.activeTiles.reserve((size_t)L.numTiles * kMaxUnitsPerTile));
  if (S.header.n == 0) {
    OCC_CHECK(S.header.reserve(1));
    OCC_CUDA(cudaMemsetAsync(S.header.p, 0, sizeof(FrameHeader), ctx->stream));
    OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  if (S.capSt < L.totalQuads * 2 + 1024) S.capSt = L.totalQuads * 2 + 1024;
  if (S.capCks < L.totalQuads * 2 + 4096) S.capCks = L.totalQuads * 2 + 4096;
  uint32_t querySlots = L.querySlots;
  if (anyHostQuery) {
    OCC_CHECK(S.qmin.reserve(querySlots));
    OCC_CHECK(S.qmax.reserve(querySlots));
  }
  bool hostBits = false;
  for (auto& J : jobs) hostBits |= J.nq && (J.hvis || J.hnc);
  if (hostBits || anyHostQuery) {
    OCC_CHECK(S.visBits.reserve(querySlots / 32 + 1));
    OCC_CHECK(S.ncBits.reserve(querySlots / 32 + 1));
  }

  OCC_CUDA(cudaMemcpyAsync(S.tables.p, st, tablesBytes, cudaMemcpyHostToDevice, ctx->stream));
  if (anyHostQuery) {
    OCC_CUDA(cudaMemcpyAsync(S.qmin.p, st + offQMin, (size_t)querySlots * 16, cudaMemcpyHostToDevice, ctx->stream));
    OCC_CUDA(cudaMemcpyAsync(S.qmax.p, st + offQMax, (size_t)querySlots * 16, cudaMemcpyHostToDevice, ctx->stream));
  }
  OCC_CUDA(cudaEventRecord(ctx->stageFree, ctx->stream));

  for (int attempt = 0; attempt < 4; ++attempt) {
    OCC_CHECK(S.stList.reserve(S.capSt));
    OCC_CHECK(S.ck.reserve((size_t)S.capCks * kCkFloats));
    OCC_CHECK(S.rowOwner.reserve(S.capCks));
    // overflow := 0 and the capacities; totals are recomputed, viewsDone is reset by
    // the kernels themselves and the sticky overflow bit is kept
    uint32_t* hs = reinterpret_cast<uint32_t*>(st + offHdr);
    hs[0] = 0;
    hs[1] = S.capCks;
    hs[2] = S.capSt;
    OCC_CUDA(cudaMemcpyAsync(&S.header.p->overflow, hs, 12, cudaMemcpyHostToDevice, ctx->stream));

    FrameParams P{};
    P.views = reinterpret_cast<const ViewDesc*>(S.tables.p + offViews);
    P.numViews = nv;
    P.numCmds = (uint32_t)L.cmds.size();
    for (const auto& Vd : L.views) P.maxViewCmds = std::max(P.maxViewCmds, Vd.cmdCount);
    P.matSize = L.matSize;
    P.activeChunkList = S.activeChunks.p;
    P.chunkRank = S.viewActive.p;
    P.viewActiveCount = S.viewActiveCount.p;
    P.activeTileList = S.activeTiles.p;
    P.cmds = reinterpret_cast<const Cmd*>(S.tables.p + offCmds);
    P.chunks = reinterpret_cast<const Chunk*>(S.tables.p + offChunks);
    P.numChunks = (uint32_t)L.chunks.size();
    P.numTiles = L.numTiles;
    P.numQuerySlots = querySlots;
    P.pool = ctx->pool.p;
    P.rec = S.rec.p;
    P.walk = S.walk.p;
    P.ckBase = S.ckBase.p;
    P.chunkTot = S.chunkTot.p;
    P.chunkBase = S.chunkBase.p;
    P.mat = S.mat.p;
    P.stStart = S.stStart.p;
    P.stLen = S.stLen.p;
    P.viewTot = S.viewTot.p;
    P.viewBase = S.viewBase.p;
    P.stList = S.stList.p;
    P.ck = S.ck.p;
    P.rowOwner = S.rowOwner.p;
    P.header = S.header.p;
    P.cmdDraw = S.cmdDraw.p;
    if (anyHostQuery) {
      P.qmin = S.qmin.p;
      P.qmax = S.qmax.p;
    } else if (jobs.size() == 1 && jobs[0].dmin) {
      P.qmin = static_cast<const float4*>(jobs[0].dmin);
      P.qmax = static_cast<const float4*>(jobs[0].dmax);
    }
    if (jobs.size() == 1 && jobs[0].dvis) {
      P.visBits = static_cast<uint32_t*>(jobs[0].dvis);
      P.ncBits = static_cast<uint32_t*>(jobs[0].dnc);
    } else {
      P.visBits = S.visBits.p;
      P.ncBits = S.ncBits.p;
    }
    const bool doQuery = querySlots > 0 && P.qmin != nullptr;
    OCC_CUDA(launch_flush(P, L.numSt, L.maxStPerView, anyRaster, doQuery, ctx->stream));
    if (!sync) return OCC_OK;

    // read back header, command flags and result bits
    const size_t nCmd = L.cmds.size();
    const size_t rbBytes = sizeof(FrameHeader) + nCmd * 4 + (size_t)(querySlots / 32) * 8 + 64;
    OCC_CHECK(ctx->readback.reserve(rbBytes));
    uint8_t* rb = ctx->readback.p;
    OCC_CUDA(cudaMemcpyAsync(rb, S.header.p, sizeof(FrameHeader), cudaMemcpyDeviceToHost, ctx->stream));
    if (nCmd) OCC_CUDA(cudaMemcpyAsync(rb + sizeof(FrameHeader), S.cmdDraw.p, nCmd * 4, cudaMemcpyDeviceToHost, ctx->stream));
    uint32_t* bitsOut = reinterpret_cast<uint32_t*>(rb + sizeof(FrameHeader) + nCmd * 4);
    if (doQuery && P.visBits == S.visBits.p) {
      OCC_CUDA(cudaMemcpyAsync(bitsOut, S.visBits.p, (size_t)(querySlots / 32) * 4, cudaMemcpyDeviceToHost, ctx->stream));
      OCC_CUDA(cudaMemcpyAsync(bitsOut + querySlots / 32, S.ncBits.p, (size_t)(querySlots / 32) * 4,
                               cudaMemcpyDeviceToHost, ctx->stream));
    }
    OCC_CUDA(cudaStreamSynchronize(ctx->stream));
    FrameHeader Hr;
    std::memcpy(&Hr, rb, sizeof(Hr));
    if (anyRaster && Hr.overflow) {
      S.capCks = std::max(S.capCks, Hr.totalCks + Hr.totalCks / 4 + 1024);
      S.capSt = std::max(S.capSt, Hr.totalSt + Hr.totalSt / 4 + 1024);
      continue;
    }
    const uint32_t* draw = reinterpret_cast<const uint32_t*>(rb + sizeof(FrameHeader));
    for (size_t v = 0; v < jobs.size(); ++v) {
      const ViewDesc& V = L.views[v];
      jobs[v].r->lastFlags.assign(V.cmdCount, 0);
      for (uint32_t i = 0; i < V.cmdCount; ++i) jobs[v].r->lastFlags[i] = (uint8_t)draw[V.cmdStart + i];
      if (doQuery && P.visBits == S.visBits.p && jobs[v].nq) {
        const uint32_t w0 = V.queryStart / 32, nw = div_up(jobs[v].nq, 32);
        if (jobs[v].hvis) std::memcpy(jobs[v].hvis, bitsOut + w0, nw * 4);
        if (jobs[v].hnc) std::memcpy(jobs[v].hnc, bitsOut + querySlots / 32 + w0, nw * 4);
      }
    }
    return OCC_OK;
  }
  return fail(OCC_ERR_CAPACITY, "scratch capacity still exceeded after retries");
}

int flush_raster(occ_raster_s* r, const ViewJob* withQueries)
{
  std::vector<ViewJob> jobs(1);
  ViewJob& J = jobs[0];
  if (withQueries) J = *withQueries;
  J.r = r;
  J.cmds = r->pending.data();
  J.ncmds = (uint32_t)r->pending.size();
  J.clear = r->clearPending;
  if (!J.ncmds && !J.clear && !J.nq) return OCC_OK;
  const bool sync = !(withQueries && withQueries->dvis);
  int s = run_batch(r->ctx, r->ctx->scratch, jobs, sync);
  if (s == OCC_OK) {
    r->pending.clear();
    r->clearPending = false;
  }
  return s;
}

}  // namespace

// ==== exported API =======================================================================

extern "C" {

const char* occ_last_error(void) { return g_error.c_str(); }
int occ_version(void) { return 1; }

int occ_ctx_create(int device, occ_ctx* out)
{
  if (!out) return fail(OCC_ERR_INVALID_ARG, "null out");
  auto ctx = std::make_unique<occ_ctx_s>();
  ctx->device = device;
  OCC_CUDA(cudaSetDevice(device));
  OCC_CUDA(set_kernel_attributes());
  OCC_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  OCC_CUDA(cudaEventCreateWithFlags(&ctx->stageFree, cudaEventDisableTiming));
  OCC_CUDA(cudaEventRecord(ctx->stageFree, ctx->stream));
  *out = ctx.release();
  return OCC_OK;
}

int occ_ctx_destroy(occ_ctx ctx)
{
  if (!ctx) return OCC_OK;
  cudaStreamSynchronize(ctx->stream);
  cudaEventDestroy(ctx->stageFree);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return OCC_OK;
}

int occ_ctx_synchronize(occ_ctx ctx)
{
  if (!ctx) return fail(OCC_ERR_INVALID_ARG, "null ctx");
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  return OCC_OK;
}

void* occ_ctx_stream(occ_ctx ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int occ_occluder_upload(occ_ctx ctx, const uint32_t* packed, uint32_t packetCount, const float refMin[4],
                        const float refMax[4], const float boundsMin[4], const float boundsMax[4], occ_occluder* out)
{
  if (!ctx || !packed || !refMin || !refMax || !boundsMin || !boundsMax || !out)
    return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (packetCount == 0 || packetCount % 4 != 0)
    return fail(OCC_ERR_INVALID_ARG, "packetCount must be a positive multiple of 4 (8 quads per packet group)");
  const size_t words = (size_t)packetCount * 8;
  if (ctx->poolWords + words > 0xFFFFFFFFull) return fail(OCC_ERR_CAPACITY, "occluder pool exceeds 2^32 words");
  if (ctx->poolWords + words > ctx->pool.n) {
    size_t cap = std::max<size_t>(ctx->pool.n * 2, ctx->poolWords + words);
    cap = std::max<size_t>(cap, 1 << 16);
    uint32_t* np = nullptr;
    cudaError_t e = cudaMalloc(&np, cap * 4);
    if (e != cudaSuccess) return fail(OCC_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    if (ctx->poolWords) OCC_CUDA(cudaMemcpyAsync(np, ctx->pool.p, ctx->poolWords * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    OCC_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->pool.release();
    ctx->pool.p = np;
    ctx->pool.n = cap;
  }
  OCC_CUDA(cudaMemcpyAsync(ctx->pool.p + ctx->poolWords, packed, words * 4, cudaMemcpyHostToDevice, ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  OccluderRec rec{};
  rec.wordOffset = (uint32_t)ctx->poolWords;
  rec.packetCount = packetCount;
  std::memcpy(rec.refMin, refMin, 16);
  std::memcpy(rec.refMax, refMax, 16);
  std::memcpy(rec.boundsMin, boundsMin, 16);
  std::memcpy(rec.boundsMax, boundsMax, 16);
  ctx->poolWords += words;
  ctx->occluders.push_back(rec);
  *out = (occ_occluder)(ctx->occluders.size() - 1);
  return OCC_OK;
}

int occ_occluders_bake_device(occ_ctx ctx, uint32_t count, const float* vertices, const uint32_t* vertexStart,
                              const float* refBoxes, uint32_t* packed, float* bounds)
{
  if (!ctx || (count && (!vertices || !vertexStart || !refBoxes || !packed || !bounds)))
    return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (!count) return OCC_OK;
  if (vertexStart[0] != 0) return fail(OCC_ERR_INVALID_ARG, "vertexStart[0] must be 0");
  std::vector<BakeJob> jobs(count);
  for (uint32_t k = 0; k < count; ++k) {
    if (vertexStart[k + 1] <= vertexStart[k] || (vertexStart[k + 1] - vertexStart[k]) % 32 != 0)
      return fail(OCC_ERR_INVALID_ARG, "each occluder needs a positive multiple of 32 vertices (8 quads per packet)");
    jobs[k].vertexStart = vertexStart[k];
    jobs[k].vertexCount = vertexStart[k + 1] - vertexStart[k];
    std::memcpy(jobs[k].refMin, refBoxes + 8 * (size_t)k, 16);
    std::memcpy(jobs[k].refMax, refBoxes + 8 * (size_t)k + 4, 16);
  }
  const size_t quads = vertexStart[count] / 4;
  OCC_CHECK(ctx->bakeJobs.reserve(count));
  OCC_CHECK(ctx->bakeNormals.reserve(quads));
  OCC_CHECK(ctx->bakeCluster.reserve(quads));
  OCC_CHECK(ctx->bakeOrder.reserve(quads));
  OCC_CUDA(cudaMemcpyAsync(ctx->bakeJobs.p, jobs.data(), count * sizeof(BakeJob), cudaMemcpyHostToDevice, ctx->stream));
  OCC_CUDA(launch_bake(ctx->bakeJobs.p, count, reinterpret_cast<const float4*>(vertices), ctx->bakeNormals.p,
                       ctx->bakeCluster.p, ctx->bakeOrder.p, packed, bounds, ctx->stream));
  return OCC_OK;
}

int occ_sah_generate_batches_device(occ_ctx ctx, const float* aabbs, uint32_t n, uint32_t targetSize,
                                    uint32_t splitGranularity, uint32_t* flat, uint32_t* offsets,
                                    uint32_t* numBatches)
{
  if (!ctx || !offsets || !numBatches || !splitGranularity || (n && (!aabbs || !flat)))
    return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (n >= (1u << 30)) return fail(OCC_ERR_INVALID_ARG, "at most 2^30 - 1 boxes");
  if (reinterpret_cast<uintptr_t>(aabbs) % 16 != 0)
    return fail(OCC_ERR_INVALID_ARG, "aabbs must be 16-byte aligned (rows of two float4)");
  if (n <= 2 * splitGranularity) {  // as occ_sah_generate_batches: one batch
    std::vector<uint32_t> iota(n);
    for (uint32_t i = 0; i < n; ++i) iota[i] = i;
    if (n) OCC_CUDA(cudaMemcpyAsync(flat, iota.data(), (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    OCC_CUDA(cudaStreamSynchronize(ctx->stream));
    offsets[0] = 0;
    offsets[1] = n;
    *numBatches = n ? 1 : 0;
    return OCC_OK;
  }
  // carve the scratch (256-byte aligned pieces)
  const size_t tiles = (n + 2047) / 2048;
  const size_t sizes[] = {16 * (size_t)n, 16 * (size_t)n, 12 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n,
                          8 * (size_t)n, 8 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n,
                          4 * 256 * tiles, 4 * ((size_t)n + 1), (size_t)n, 8 * (size_t)n, 16 * tiles,
                          16 * tiles, 4};
  size_t total = 0;
  for (size_t z : sizes) total += align_up(z, 256);
  OCC_CHECK(ctx->sah.reserve(total));
  uint8_t* p = ctx->sah.p;
  void* piece[17];
  for (int k = 0; k < 17; ++k) {
    piece[k] = p;
    p += align_up(sizes[k], 256);
  }
  SahScratch S;
  S.lo = static_cast<float4*>(piece[0]);
  S.hi = static_cast<float4*>(piece[1]);
  S.mk = static_cast<uint32_t*>(piece[2]);
  S.idx[0] = static_cast<uint32_t*>(piece[3]);
  S.idx[1] = static_cast<uint32_t*>(piece[4]);
  S.key[0] = static_cast<unsigned long long*>(piece[5]);
  S.key[1] = static_cast<unsigned long long*>(piece[6]);
  S.rng = static_cast<uint32_t*>(piece[7]);
  S.left = static_cast<float*>(piece[8]);
  S.right = static_cast<float*>(piece[9]);
  S.hist = static_cast<uint32_t*>(piece[10]);
  S.starts = static_cast<uint32_t*>(piece[11]);
  S.rangeAxis = static_cast<int8_t*>(piece[12]);
  S.best = static_cast<unsigned long long*>(piece[13]);
  S.aggLo = static_cast<float4*>(piece[14]);
  S.aggHi = static_cast<float4*>(piece[15]);
  S.flag = static_cast<uint32_t*>(piece[16]);
  std::vector<uint32_t> offs;
  std::string err;
  const int st = sah_generate_device(S, n, aabbs, targetSize, splitGranularity, flat, offs, ctx->stream, err);
  if (st < 0) return fail(OCC_ERR_CUDA, "occ_sah_generate_batches_device: " + err);
  if (st > 0)
    return fail(OCC_ERR_UNSUPPORTED, "a box centre is NaN: the reference's order for it comes from its library's "
                                     "merge sort; use occ_sah_generate_batches");
  std::copy(offs.begin(), offs.end(), offsets);
  *numBatches = (uint32_t)offs.size() - 1;
  return OCC_OK;
}

int occ_occluder_upload_device(occ_ctx ctx, const uint32_t* packed, uint32_t packetCount, const float bounds[20],
                               occ_occluder* out)
{
  if (!ctx || !packed || !bounds || !out) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (packetCount == 0 || packetCount % 4 != 0)
    return fail(OCC_ERR_INVALID_ARG, "packetCount must be a positive multiple of 4 (8 quads per packet group)");
  const size_t words = (size_t)packetCount * 8;
  if (ctx->poolWords + words > 0xFFFFFFFFull) return fail(OCC_ERR_CAPACITY, "occluder pool exceeds 2^32 words");
  if (ctx->poolWords + words > ctx->pool.n) {
    size_t cap = std::max<size_t>(ctx->pool.n * 2, ctx->poolWords + words);
    cap = std::max<size_t>(cap, 1 << 16);
    uint32_t* np = nullptr;
    cudaError_t e = cudaMalloc(&np, cap * 4);
    if (e != cudaSuccess) return fail(OCC_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    if (ctx->poolWords) OCC_CUDA(cudaMemcpyAsync(np, ctx->pool.p, ctx->poolWords * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    OCC_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->pool.release();
    ctx->pool.p = np;
    ctx->pool.n = cap;
  }
  OCC_CUDA(cudaMemcpyAsync(ctx->pool.p + ctx->poolWords, packed, words * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  OccluderRec rec{};
  rec.wordOffset = (uint32_t)ctx->poolWords;
  rec.packetCount = packetCount;
  std::memcpy(rec.refMin, bounds, 16);
  std::memcpy(rec.refMax, bounds + 4, 16);
  std::memcpy(rec.boundsMin, bounds + 8, 16);
  std::memcpy(rec.boundsMax, bounds + 12, 16);
  ctx->poolWords += words;
  ctx->occluders.push_back(rec);
  *out = (occ_occluder)(ctx->occluders.size() - 1);
  return OCC_OK;
}

int occ_occluder_count(occ_ctx ctx, uint32_t* count)
{
  if (!ctx || !count) return fail(OCC_ERR_INVALID_ARG, "null argument");
  *count = (uint32_t)ctx->occluders.size();
  return OCC_OK;
}

int occ_raster_create(occ_ctx ctx, uint32_t width, uint32_t height, occ_raster* out)
{
  if (!ctx || !out) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (width == 0 || height == 0 || width % 8 || height % 8)
    return fail(OCC_ERR_INVALID_ARG, "width and height must be positive multiples of 8");
  if (width > 65528 || height > 65528) return fail(OCC_ERR_INVALID_ARG, "width/height above 65528");
  if ((size_t)div_up(width / 8, kSuperTile) * div_up(height / 8, kSuperTile) > (size_t)kMaxStPerView)
    return fail(OCC_ERR_UNSUPPORTED, "view too large: more than 3072 binning super-tiles (128x128 pixels each)");
  auto r = std::make_unique<occ_raster_s>();
  r->ctx = ctx;
  r->width = width;
  r->height = height;
  r->blocksX = width / 8;
  r->blocksY = height / 8;
  const size_t blocks = (size_t)r->blocksX * r->blocksY;
  OCC_CHECK(r->depth.reserve((size_t)width * height));
  OCC_CHECK(r->hiz.reserve(blocks + 8));
  const size_t tiles = (size_t)div_up(r->blocksX, kTileW) * div_up(r->blocksY, kTileH);
  OCC_CHECK(r->tileHiz.reserve((size_t)tiles * 4));  // the minimum hiZ of each tile's 4 block rows
  // the reference value-initialises both (Rasterizer.cpp:70-71)
  OCC_CUDA(cudaMemsetAsync(r->depth.p, 0, (size_t)width * height * 2, ctx->stream));
  OCC_CUDA(cudaMemsetAsync(r->hiz.p, 0, (blocks + 8) * 2, ctx->stream));
  OCC_CUDA(cudaMemsetAsync(r->tileHiz.p, 0, (size_t)tiles * 8, ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = r.release();
  return OCC_OK;
}

int occ_raster_destroy(occ_raster r)
{
  if (!r) return OCC_OK;
  cudaStreamSynchronize(r->ctx->stream);
  delete r;
  return OCC_OK;
}

int occ_raster_set_mvp(occ_raster r, const float matrix[16])
{
  if (!r || !matrix) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (!r->pending.empty()) OCC_CHECK(flush_raster(r, nullptr));  // pending commands use the old matrix
  bake_mvp(matrix, r->width, r->height, r->cols, r->rows);
  return OCC_OK;
}

int occ_raster_clear(occ_raster r)
{
  if (!r) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (!r->pending.empty()) OCC_CHECK(flush_raster(r, nullptr));
  r->clearPending = true;
  return OCC_OK;
}

int occ_raster_rasterize(occ_raster r, occ_occluder occ, int possiblyNearClipped)
{
  if (!r) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (occ >= r->ctx->occluders.size()) return fail(OCC_ERR_INVALID_ARG, "unknown occluder id");
  r->pending.push_back(PendingCmd{occ, possiblyNearClipped ? kCmdNearClip : 0u});
  return OCC_OK;
}

int occ_raster_rasterize_many(occ_raster r, uint32_t n, const occ_occluder* occ, const uint8_t* flags)
{
  if (!r || (n && !occ)) return fail(OCC_ERR_INVALID_ARG, "null argument");
  for (uint32_t i = 0; i < n; ++i)
    if (occ[i] >= r->ctx->occluders.size()) return fail(OCC_ERR_INVALID_ARG, "unknown occluder id");
  for (uint32_t i = 0; i < n; ++i)
    r->pending.push_back(PendingCmd{occ[i], flags ? (uint32_t)(flags[i] & (kCmdNearClip | kCmdGated)) : 0u});
  return OCC_OK;
}

int occ_raster_flush(occ_raster r)
{
  if (!r) return fail(OCC_ERR_INVALID_ARG, "null argument");
  return flush_raster(r, nullptr);
}

int occ_raster_command_flags(occ_raster r, uint32_t n, uint8_t* out)
{
  if (!r || (n && !out)) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (n > r->lastFlags.size()) return fail(OCC_ERR_INVALID_ARG, "more flags requested than commands flushed");
  std::memcpy(out, r->lastFlags.data(), n);
  return OCC_OK;
}

int occ_raster_query_batch(occ_raster r, uint32_t n, const float* mins, const float* maxs, uint32_t* visibleBits,
                           uint32_t* needsClippingBits)
{
  if (!r || (n && (!mins || !maxs))) return fail(OCC_ERR_INVALID_ARG, "null argument");
  ViewJob J{};
  J.nq = n;
  J.hmin = mins;
  J.hmax = maxs;
  J.hvis = visibleBits;
  J.hnc = needsClippingBits;
  return flush_raster(r, &J);
}

int occ_raster_query_visibility(occ_raster r, const float boundsMin[4], const float boundsMax[4], int* visible,
                                int* needsClipping)
{
  if (!visible || !needsClipping) return fail(OCC_ERR_INVALID_ARG, "null argument");
  uint32_t v = 0, c = 0;
  OCC_CHECK(occ_raster_query_batch(r, 1, boundsMin, boundsMax, &v, &c));
  *visible = (int)(v & 1);
  *needsClipping = (int)(c & 1);
  return OCC_OK;
}

int occ_raster_query_batch_device(occ_raster r, uint32_t n, const void* dMins, const void* dMaxs,
                                  void* dVisibleBits, void* dNeedsClippingBits)
{
  if (!r || (n && (!dMins || !dMaxs || !dVisibleBits || !dNeedsClippingBits)))
    return fail(OCC_ERR_INVALID_ARG, "null argument");
  ViewJob J{};
  J.nq = n;
  J.dmin = dMins;
  J.dmax = dMaxs;
  J.dvis = dVisibleBits;
  J.dnc = dNeedsClippingBits;
  return flush_raster(r, &J);
}

int occ_raster_query_batch_noalloc(occ_raster r, uint32_t n, const float* mins, const float* maxs,
                                   uint32_t* visibleBits, uint32_t* needsClippingBits)
{
  if (!r || (n && (!mins || !maxs))) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (n > kNoAllocMaxQueries)
    return fail(OCC_ERR_INVALID_ARG, "occ_raster_query_batch_noalloc takes at most 65536 boxes per call");
  if (!r->pending.empty() || r->clearPending)
    return fail(OCC_ERR_INVALID_ARG, "rasterisation is pending: call occ_raster_flush first (it may allocate)");
  ViewDesc V{};
  V.depth = r->depth.p;
  V.hiz = r->hiz.p;
  V.tileHiz = r->tileHiz.p;
  V.width = r->width;
  V.height = r->height;
  V.blocksX = r->blocksX;
  V.blocksY = r->blocksY;
  std::memcpy(V.cols, r->cols, sizeof(V.cols));
  std::memcpy(V.rows, r->rows, sizeof(V.rows));
  V.queryCount = n;
  int prev = 0;
  OCC_CUDA(cudaGetDevice(&prev));
  if (prev != r->ctx->device) OCC_CUDA(cudaSetDevice(r->ctx->device));
  const cudaError_t e = query_noalloc(r->ctx->device, V, n, mins, maxs, visibleBits, needsClippingBits, r->ctx->stream);
  if (prev != r->ctx->device) cudaSetDevice(prev);
  if (e != cudaSuccess) return fail(OCC_ERR_CUDA, std::string("occ_raster_query_batch_noalloc: ") + cudaGetErrorString(e));
  return OCC_OK;
}

int occ_raster_query2d(occ_raster r, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ,
                       int* visible)
{
  if (!r || !visible) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (minX > maxX || minY > maxY || maxX >= r->width || maxY >= r->height)
    return fail(OCC_ERR_INVALID_ARG, "rectangle outside the buffer");
  OCC_CHECK(flush_raster(r, nullptr));
  occ_ctx_s* ctx = r->ctx;
  ViewDesc V{};
  V.depth = r->depth.p;
  V.hiz = r->hiz.p;
  V.tileHiz = r->tileHiz.p;
  V.width = r->width;
  V.height = r->height;
  V.blocksX = r->blocksX;
  V.blocksY = r->blocksY;
  DevBuf<uint8_t> tmp;
  OCC_CHECK(tmp.reserve(sizeof(ViewDesc) + 16));
  OCC_CUDA(cudaMemcpyAsync(tmp.p, &V, sizeof(V), cudaMemcpyHostToDevice, ctx->stream));
  uint32_t* dout = reinterpret_cast<uint32_t*>(tmp.p + sizeof(ViewDesc));
  OCC_CUDA(launch_query2d(reinterpret_cast<const ViewDesc*>(tmp.p), minX, maxX, minY, maxY, maxZ, dout, ctx->stream));
  uint32_t hv = 0;
  OCC_CUDA(cudaMemcpyAsync(&hv, dout, 4, cudaMemcpyDeviceToHost, ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  *visible = (int)hv;
  return OCC_OK;
}

static_assert(kReadBackRgba8 == OCC_READBACK_RGBA8 && kReadBackLinearF32 == OCC_READBACK_LINEAR_F32 &&
                  kReadBackDepthF32 == OCC_READBACK_DEPTH_F32 && kReadBackPackedU16 == OCC_READBACK_PACKED_U16,
              "read-back format codes");

int occ_raster_read_back(occ_raster r, int format, void* out)
{
  if (!r || !out) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (format < OCC_READBACK_RGBA8 || format > OCC_READBACK_PACKED_U16) return fail(OCC_ERR_INVALID_ARG, "unknown format");
  OCC_CHECK(flush_raster(r, nullptr));
  occ_ctx_s* ctx = r->ctx;
  const size_t bytes = (size_t)r->width * r->height * (format == OCC_READBACK_PACKED_U16 ? 2 : 4);
  DevBuf<uint8_t> dev;
  OCC_CHECK(dev.reserve(bytes));
  OCC_CUDA(launch_read_back(r->depth.p, r->hiz.p, r->width, r->height, format, dev.p, ctx->stream));
  OCC_CUDA(cudaMemcpyAsync(out, dev.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  return OCC_OK;
}

int occ_raster_read_back_depth(occ_raster r, void* rgba) { return occ_raster_read_back(r, OCC_READBACK_RGBA8, rgba); }

int occ_raster_read_depth_raw(occ_raster r, uint16_t* out)
{
  if (!r || !out) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CHECK(flush_raster(r, nullptr));
  OCC_CUDA(cudaMemcpyAsync(out, r->depth.p, (size_t)r->width * r->height * 2, cudaMemcpyDeviceToHost, r->ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(r->ctx->stream));
  return OCC_OK;
}

int occ_raster_read_hiz(occ_raster r, uint16_t* out, uint32_t* count)
{
  if (!r) return fail(OCC_ERR_INVALID_ARG, "null argument");
  const uint32_t n = r->blocksX * r->blocksY + 8;
  if (count) *count = n;
  if (!out) return OCC_OK;
  OCC_CHECK(flush_raster(r, nullptr));
  OCC_CUDA(cudaMemcpyAsync(out, r->hiz.p, (size_t)n * 2, cudaMemcpyDeviceToHost, r->ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(r->ctx->stream));
  return OCC_OK;
}

int occ_raster_write_depth_raw(occ_raster r, const uint16_t* in)
{
  if (!r || !in) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CHECK(flush_raster(r, nullptr));
  OCC_CUDA(cudaMemcpyAsync(r->depth.p, in, (size_t)r->width * r->height * 2, cudaMemcpyHostToDevice, r->ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(r->ctx->stream));
  return OCC_OK;
}

int occ_raster_write_hiz(occ_raster r, const uint16_t* in)
{
  if (!r || !in) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CHECK(flush_raster(r, nullptr));
  const uint32_t n = r->blocksX * r->blocksY + 8;
  OCC_CUDA(cudaMemcpyAsync(r->hiz.p, in, (size_t)n * 2, cudaMemcpyHostToDevice, r->ctx->stream));
  OCC_CUDA(launch_tile_hiz(r->hiz.p, r->tileHiz.p, r->blocksX, r->blocksY, r->ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(r->ctx->stream));
  return OCC_OK;
}

int occ_raster_size(occ_raster r, uint32_t* width, uint32_t* height)
{
  if (!r) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (width) *width = r->width;
  if (height) *height = r->height;
  return OCC_OK;
}

int occ_batch_execute(occ_ctx ctx, uint32_t numViews, const occ_view_work* views)
{
  if (!ctx || (numViews && !views)) return fail(OCC_ERR_INVALID_ARG, "null argument");
  std::vector<std::vector<PendingCmd>> cmds(numViews);
  std::vector<ViewJob> jobs(numViews);
  for (uint32_t v = 0; v < numViews; ++v) {
    const occ_view_work& W = views[v];
    occ_raster_s* r = W.raster;
    if (!r || r->ctx != ctx) return fail(OCC_ERR_INVALID_ARG, "view raster missing or from another context");
    if (W.numQueries && (!W.queryMins || !W.queryMaxs)) return fail(OCC_ERR_INVALID_ARG, "null query boxes");
    for (uint32_t u = 0; u < v; ++u)
      if (views[u].raster == r) return fail(OCC_ERR_INVALID_ARG, "a rasterizer appears twice in one batch");
    if (!r->pending.empty()) OCC_CHECK(flush_raster(r, nullptr));
    if (W.mvp) bake_mvp(W.mvp, r->width, r->height, r->cols, r->rows);
    auto& c = cmds[v];
    c.reserve(W.numOccluders);
    for (uint32_t i = 0; i < W.numOccluders; ++i) {
      if (W.occluders[i] >= ctx->occluders.size()) return fail(OCC_ERR_INVALID_ARG, "unknown occluder id");
      c.push_back(PendingCmd{W.occluders[i], W.flags ? (uint32_t)(W.flags[i] & 3u) : 0u});
    }
    ViewJob& J = jobs[v];
    J.r = r;
    J.cmds = c.data();
    J.ncmds = (uint32_t)c.size();
    J.clear = W.clear != 0 || r->clearPending;
    J.nq = W.numQueries;
    J.hmin = W.queryMins;
    J.hmax = W.queryMaxs;
    J.hvis = W.visibleBits;
    J.hnc = W.needsClippingBits;
  }
  OCC_CHECK(run_batch(ctx, ctx->scratch, jobs, true));
  for (uint32_t v = 0; v < numViews; ++v) views[v].raster->clearPending = false;
  return OCC_OK;
}

}  // extern "C"

// ==== prepared batches (CUDA graph) ======================================================

namespace {
constexpr int kRing = 4;
}

struct occ_mlp_s {
  occ_ctx_s* ctx = nullptr;
  DevBuf<float> params, m, v, grad;  // fp32 master weights, Adam moments, gradient (+ loss)
  DevBuf<MlpDevice> dev;             // the kernels' copy (bf16 matrices)
  DevBuf<float> feat, target, score, xb, h1, h2, ds, dh1, dh2, err2;  // training batch
  DevBuf<float> partial;  // per row block partial gradients
  DevBuf<uint32_t> groups;  // listwise loss: first row of each group, then the row count
  uint32_t step = 0;
};

static const MlpDevice* mlp_device(const occ_mlp_s* m) { return m->dev.p; }

struct occ_batch_s {
  occ_ctx_s* ctx = nullptr;
  std::vector<std::vector<PendingCmd>> cmds;
  std::vector<ViewJob> jobs;
  BatchLayout L;
  FrameScratch S;
  DevBuf<float4> qmin, qmax;
  DevBuf<uint32_t> vis, nc;
  PinBuf<uint8_t> ring[kRing];
  cudaEvent_t ringEv[kRing] = {};
  int cur = 0;
  bool dirty = false;
  size_t offCmds = 0, offChunks = 0, tablesBytes = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t copyNode = nullptr;
  FrameParams params{};
  bool anyRaster = false;
  // learned selection / win counts
  const struct occ_mlp_s* mlp = nullptr;
  float selectFrac = 1.0f;
  bool trackWins = false, features = false;
  bool zeroDepth = false;  // cleared views start each launch with zero depth (kViewZeroDepth)
  bool secondPass = false; // after the top-K pass, draw the other candidates still visible
  bool cullLabels = false; // per-pixel owners and per-command cull counts (training labels)
  LaunchTuning tune{};     // launch shapes (occ_batch_autotune)
  DevBuf<uint32_t> cullCount;
  DevBuf<float> feat, score;
  DevBuf<uint8_t> cand, select;
  DevBuf<uint32_t> wins;
  ~occ_batch_s()
  {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : ringEv)
      if (e) cudaEventDestroy(e);
  }
};

namespace {

void write_tables(occ_batch_s* b, uint8_t* dst)
{
  std::memcpy(dst, b->L.views.data(), b->L.views.size() * sizeof(ViewDesc));
  if (!b->L.cmds.empty()) std::memcpy(dst + b->offCmds, b->L.cmds.data(), b->L.cmds.size() * sizeof(Cmd));
  if (!b->L.chunks.empty()) std::memcpy(dst + b->offChunks, b->L.chunks.data(), b->L.chunks.size() * sizeof(Chunk));
}

// Between launches only the view table changes (matrices, owner buffers): the
// command and chunk tables are uploaded when the graph is captured, and each
// launch copies the view table alone (its first offCmds bytes).
void write_views(occ_batch_s* b, uint8_t* dst)
{
  std::memcpy(dst, b->L.views.data(), b->L.views.size() * sizeof(ViewDesc));
}

// (Re)captures the per-frame sequence: table upload from the current ring slot,
// then the five kernels.
int capture(occ_batch_s* b)
{
  occ_ctx_s* ctx = b->ctx;
  FrameScratch& S = b->S;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  OCC_CHECK(S.stList.reserve(S.capSt));
  OCC_CHECK(S.ck.reserve((size_t)S.capCks * kCkFloats));
  OCC_CHECK(S.rowOwner.reserve(S.capCks));
  // capacities into the header (synchronously, outside the graph)
  uint32_t hs[3] = {0, S.capCks, S.capSt};
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  OCC_CUDA(cudaMemcpy(&S.header.p->overflow, hs, 12, cudaMemcpyHostToDevice));

  FrameParams P{};
  P.views = reinterpret_cast<const ViewDesc*>(S.tables.p);
  P.numViews = (uint32_t)b->L.views.size();
  P.numCmds = (uint32_t)b->L.cmds.size();
  for (const auto& Vd : b->L.views) P.maxViewCmds = std::max(P.maxViewCmds, Vd.cmdCount);
  P.matSize = b->L.matSize;
  P.activeChunkList = S.activeChunks.p;
    P.chunkRank = S.viewActive.p;
    P.viewActiveCount = S.viewActiveCount.p;
  P.activeTileList = S.activeTiles.p;
  P.cmds = reinterpret_cast<const Cmd*>(S.tables.p + b->offCmds);
  P.chunks = reinterpret_cast<const Chunk*>(S.tables.p + b->offChunks);
  P.numChunks = (uint32_t)b->L.chunks.size();
  P.numTiles = b->L.numTiles;
  P.numQuerySlots = b->L.querySlots;
  P.pool = ctx->pool.p;
  P.rec = S.rec.p;
  P.walk = S.walk.p;
  P.ckBase = S.ckBase.p;
  P.chunkTot = S.chunkTot.p;
  P.chunkBase = S.chunkBase.p;
  P.mat = S.mat.p;
  P.stStart = S.stStart.p;
  P.stLen = S.stLen.p;
  P.viewTot = S.viewTot.p;
  P.viewBase = S.viewBase.p;
  P.stList = S.stList.p;
  P.ck = S.ck.p;
  P.rowOwner = S.rowOwner.p;
  P.header = S.header.p;
  P.cmdDraw = S.cmdDraw.p;
  P.qmin = b->qmin.p;
  P.qmax = b->qmax.p;
  P.visBits = b->vis.p;
  P.ncBits = b->nc.p;
  bool anyRaster = false;
  for (auto& J : b->jobs) anyRaster |= J.ncmds || J.clear;
  const uint32_t numCmds = (uint32_t)b->L.cmds.size();
  if (b->features) {
    P.feat = b->feat.p;
    P.cand = b->cand.p;
    P.wins = b->trackWins ? b->wins.p : nullptr;
    if (b->mlp) {
      P.score = b->score.p;
      P.select = b->select.p;
      P.mlp = mlp_device(b->mlp);
      P.selectFrac = b->selectFrac;
      uint32_t maxCmds = 0;
      for (const auto& V : b->L.views) maxCmds = std::max(maxCmds, V.cmdCount);
      P.fusedSelect = maxCmds <= kFusedSelectMaxCmds ? 1u : 0u;
    }
  }
  P.tune = b->tune;
  const bool labels = b->cullLabels && b->features && b->trackWins;
  if (labels) P.cullCount = b->cullCount.p;
  b->params = P;
  b->anyRaster = anyRaster;

  // every table once (every ring slot holds the command and chunk tables),
  // then the graph copies the view table at each launch
  OCC_CUDA(cudaMemcpyAsync(S.tables.p, b->ring[b->cur].p, b->tablesBytes, cudaMemcpyHostToDevice, ctx->stream));
  OCC_CUDA(cudaEventRecord(b->ringEv[b->cur], ctx->stream));
  OCC_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e1 = cudaMemcpyAsync(S.tables.p, b->ring[b->cur].p, b->offCmds, cudaMemcpyHostToDevice, ctx->stream);
  if (labels) {
    for (auto& J : b->jobs)
      if (e1 == cudaSuccess)
        e1 = cudaMemsetAsync(J.r->owner.p, 0, (size_t)J.r->width * J.r->height * sizeof(uint32_t), ctx->stream);
    if (e1 == cudaSuccess && numCmds) e1 = cudaMemsetAsync(b->cullCount.p, 0, (size_t)numCmds * 4, ctx->stream);
  }
  cudaError_t e2 = b->features ? launch_selection(P, numCmds, b->mlp != nullptr, ctx->stream) : cudaSuccess;
  const bool two = b->secondPass && b->mlp != nullptr;
  if (e2 == cudaSuccess)
    e2 = launch_flush(P, b->L.numSt, b->L.maxStPerView, anyRaster, !two && b->L.querySlots > 0, ctx->stream);
  if (e2 == cudaSuccess && two) {
    FrameParams P2 = P;
    P2.phase = 1;
    e2 = launch_flush(P2, b->L.numSt, b->L.maxStPerView, anyRaster, b->L.querySlots > 0, ctx->stream);
  }
  if (e2 == cudaSuccess && labels) e2 = launch_cull_labels(P, ctx->stream);
  cudaGraph_t g = nullptr;
  cudaError_t e3 = cudaStreamEndCapture(ctx->stream, &g);
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(OCC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e1 ? e1 : (e2 ? e2 : e3)));
  }
  b->graph = g;
  size_t n = 0;
  OCC_CUDA(cudaGraphGetNodes(g, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  OCC_CUDA(cudaGraphGetNodes(g, nodes.data(), &n));
  b->copyNode = nullptr;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    OCC_CUDA(cudaGraphNodeGetType(nd, &t));
    if (t == cudaGraphNodeTypeMemcpy) b->copyNode = nd;
  }
  if (!b->copyNode) return fail(OCC_ERR_CUDA, "graph capture lost the table upload");
  OCC_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
  return OCC_OK;
}

}  // namespace

namespace {

// Lays a prepared batch out again with super-tiles of 1 << shift blocks: the
// view table (super-tile grids and count-matrix ranges) changes, the count
// matrix and list heads are reserved for it, every ring slot is rewritten and
// the graph captured again.  Matrices, view flags and owner buffers carry over.
int relayout(occ_batch_s* b, uint32_t shift)
{
  BatchLayout L;
  OCC_CHECK(build_layout(b->ctx, b->jobs, L, shift));
  for (size_t v = 0; v < L.views.size(); ++v) {
    L.views[v].flags = b->L.views[v].flags;
    L.views[v].owner = b->L.views[v].owner;
  }
  b->L = std::move(L);
  FrameScratch& S = b->S;
  OCC_CHECK(S.mat.reserve(b->L.matSize));
  OCC_CHECK(S.stStart.reserve(b->L.numSt));
  OCC_CHECK(S.stLen.reserve(b->L.numSt));
  for (int k = 0; k < kRing; ++k) {
    OCC_CUDA(cudaEventSynchronize(b->ringEv[k]));
    write_tables(b, b->ring[k].p);
  }
  b->tune.superTile = 1u << shift;
  b->dirty = false;
  return capture(b);
}

// Launches until a launch fits the scratch (each overflow grows it), at most
// a few times; the frames are re-run by the caller's own timing afterwards.
int settle(occ_batch_s* b)
{
  for (int i = 0; i < 4; ++i) {
    OCC_CHECK(occ_batch_launch(b));
    const int st = occ_batch_check(b);
    if (st == OCC_OK) return OCC_OK;
    if (st != OCC_ERR_CAPACITY) return st;
  }
  return fail(OCC_ERR_CAPACITY, "the batch's scratch did not settle");
}

}  // namespace

extern "C" {

int occ_batch_prepare(occ_ctx ctx, uint32_t numViews, const occ_view_work* views, occ_batch* out)
{
  if (!ctx || !out || !numViews || !views) return fail(OCC_ERR_INVALID_ARG, "null argument");
  auto b = std::make_unique<occ_batch_s>();
  b->ctx = ctx;
  b->cmds.resize(numViews);
  b->jobs.resize(numViews);
  for (uint32_t v = 0; v < numViews; ++v) {
    const occ_view_work& W = views[v];
    occ_raster_s* r = W.raster;
    if (!r || r->ctx != ctx) return fail(OCC_ERR_INVALID_ARG, "view raster missing or from another context");
    if (W.numQueries && (!W.queryMins || !W.queryMaxs)) return fail(OCC_ERR_INVALID_ARG, "null query boxes");
    for (uint32_t u = 0; u < v; ++u)
      if (views[u].raster == r) return fail(OCC_ERR_INVALID_ARG, "a rasterizer appears twice in one batch");
    if (!r->pending.empty()) OCC_CHECK(flush_raster(r, nullptr));
    if (W.mvp) bake_mvp(W.mvp, r->width, r->height, r->cols, r->rows);
    for (uint32_t i = 0; i < W.numOccluders; ++i) {
      if (W.occluders[i] >= ctx->occluders.size()) return fail(OCC_ERR_INVALID_ARG, "unknown occluder id");
      b->cmds[v].push_back(PendingCmd{W.occluders[i], W.flags ? (uint32_t)(W.flags[i] & 3u) : 0u});
    }
    ViewJob& J = b->jobs[v];
    J.r = r;
    J.cmds = b->cmds[v].data();
    J.ncmds = (uint32_t)b->cmds[v].size();
    J.clear = W.clear != 0;
    J.nq = W.numQueries;
    J.hmin = W.queryMins;
    J.hmax = W.queryMaxs;
  }
  // one synchronous run sizes the scratch (and renders one frame)
  OCC_CHECK(run_batch(ctx, b->S, b->jobs, true));
  FrameScratch& S = b->S;
  S.capCks = std::max(S.capCks, 2 * S.capCks + 65536);
  S.capSt = std::max(S.capSt, 2 * S.capSt + 65536);
  OCC_CHECK(build_layout(ctx, b->jobs, b->L, 4));
  const uint32_t nv = (uint32_t)b->L.views.size();
  b->offCmds = align_up(nv * sizeof(ViewDesc), 256);
  b->offChunks = align_up(b->offCmds + b->L.cmds.size() * sizeof(Cmd), 256);
  b->tablesBytes = align_up(b->offChunks + b->L.chunks.size() * sizeof(Chunk), 256);
  for (int k = 0; k < kRing; ++k) {
    OCC_CHECK(b->ring[k].reserve(b->tablesBytes));
    OCC_CUDA(cudaEventCreateWithFlags(&b->ringEv[k], cudaEventDisableTiming));
    OCC_CUDA(cudaEventRecord(b->ringEv[k], ctx->stream));
  }
  for (int k = 0; k < kRing; ++k) write_tables(b.get(), b->ring[k].p);
  // query boxes, uploaded once
  const uint32_t slots = b->L.querySlots;
  if (slots) {
    OCC_CHECK(b->qmin.reserve(slots));
    OCC_CHECK(b->qmax.reserve(slots));
    OCC_CHECK(b->vis.reserve(slots / 32));
    OCC_CHECK(b->nc.reserve(slots / 32));
    std::vector<float4> hmin(slots, make_float4(0, 0, 0, 0)), hmax(slots, make_float4(0, 0, 0, 0));
    for (uint32_t v = 0; v < nv; ++v)
      if (b->jobs[v].nq) {
        std::memcpy(&hmin[b->L.views[v].queryStart], b->jobs[v].hmin, (size_t)b->jobs[v].nq * 16);
        std::memcpy(&hmax[b->L.views[v].queryStart], b->jobs[v].hmax, (size_t)b->jobs[v].nq * 16);
        b->jobs[v].hmin = b->jobs[v].hmax = nullptr;
      }
    OCC_CUDA(cudaMemcpy(b->qmin.p, hmin.data(), (size_t)slots * 16, cudaMemcpyHostToDevice));
    OCC_CUDA(cudaMemcpy(b->qmax.p, hmax.data(), (size_t)slots * 16, cudaMemcpyHostToDevice));
  }
  OCC_CHECK(S.tables.reserve(b->tablesBytes));
  OCC_CHECK(capture(b.get()));
  *out = b.release();
  return OCC_OK;
}

int occ_batch_set_mvp(occ_batch b, uint32_t view, const float matrix[16])
{
  if (!b || !matrix || view >= b->L.views.size()) return fail(OCC_ERR_INVALID_ARG, "bad argument");
  occ_raster_s* r = b->jobs[view].r;
  bake_mvp(matrix, r->width, r->height, r->cols, r->rows);
  std::memcpy(b->L.views[view].cols, r->cols, sizeof(r->cols));
  std::memcpy(b->L.views[view].rows, r->rows, sizeof(r->rows));
  b->dirty = true;
  return OCC_OK;
}

int occ_batch_set_mvps(occ_batch b, uint32_t first, uint32_t count, const float* matrices)
{
  if (!b || (count && !matrices) || first > b->L.views.size() || count > b->L.views.size() - first)
    return fail(OCC_ERR_INVALID_ARG, "bad argument");
  for (uint32_t i = 0; i < count; ++i) {
    occ_raster_s* r = b->jobs[first + i].r;
    bake_mvp(matrices + 16 * (size_t)i, r->width, r->height, r->cols, r->rows);
    std::memcpy(b->L.views[first + i].cols, r->cols, sizeof(r->cols));
    std::memcpy(b->L.views[first + i].rows, r->rows, sizeof(r->rows));
  }
  b->dirty = true;
  return OCC_OK;
}

int occ_batch_results_all(occ_batch b, uint32_t* visibleBits, uint32_t* needsClippingBits, uint32_t* firstWord)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  const size_t nw = b->L.querySlots / 32;  // every view's range starts on a word
  if (firstWord)
    for (size_t v = 0; v < b->L.views.size(); ++v) firstWord[v] = b->L.views[v].queryStart / 32;
  if (nw) {
    if (visibleBits)
      OCC_CUDA(cudaMemcpyAsync(visibleBits, b->vis.p, nw * 4, cudaMemcpyDeviceToHost, b->ctx->stream));
    if (needsClippingBits)
      OCC_CUDA(cudaMemcpyAsync(needsClippingBits, b->nc.p, nw * 4, cudaMemcpyDeviceToHost, b->ctx->stream));
  }
  OCC_CUDA(cudaStreamSynchronize(b->ctx->stream));
  return OCC_OK;
}

int occ_batch_results_all_async(occ_batch b, uint32_t* visibleBits, uint32_t* needsClippingBits)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  const size_t nw = b->L.querySlots / 32;
  if (nw) {
    if (visibleBits)
      OCC_CUDA(cudaMemcpyAsync(visibleBits, b->vis.p, nw * 4, cudaMemcpyDeviceToHost, b->ctx->stream));
    if (needsClippingBits)
      OCC_CUDA(cudaMemcpyAsync(needsClippingBits, b->nc.p, nw * 4, cudaMemcpyDeviceToHost, b->ctx->stream));
  }
  return OCC_OK;
}

int occ_batch_set_queries(occ_batch b, uint32_t first, uint32_t count, const float* mins, const float* maxs)
{
  if (!b || first > b->L.views.size() || count > b->L.views.size() - first)
    return fail(OCC_ERR_INVALID_ARG, "bad argument");
  // views whose slot ranges follow one another without padding (box counts
  // that are multiples of 32) take one copy per array together
  size_t at = 0;                     // boxes consumed from the host arrays
  uint32_t runStart = 0, runLen = 0;  // device slots of the pending copy
  size_t runAt = 0;
  auto flush = [&]() -> int {
    if (!runLen) return OCC_OK;
    OCC_CUDA(cudaMemcpyAsync(b->qmin.p + runStart, mins + 4 * runAt, (size_t)runLen * 16, cudaMemcpyHostToDevice,
                             b->ctx->stream));
    OCC_CUDA(cudaMemcpyAsync(b->qmax.p + runStart, maxs + 4 * runAt, (size_t)runLen * 16, cudaMemcpyHostToDevice,
                             b->ctx->stream));
    runLen = 0;
    return OCC_OK;
  };
  for (uint32_t v = first; v < first + count; ++v) {
    const ViewDesc& V = b->L.views[v];
    if (!V.queryCount) continue;
    if (!mins || !maxs) return fail(OCC_ERR_INVALID_ARG, "null query boxes");
    if (runLen && runStart + runLen == V.queryStart) {
      runLen += V.queryCount;
    } else {
      OCC_CHECK(flush());
      runStart = V.queryStart;
      runLen = V.queryCount;
      runAt = at;
    }
    at += V.queryCount;
    if (V.queryCount % 32) OCC_CHECK(flush());  // the next view starts after padding
  }
  return flush();
}

int occ_batch_result_words(occ_batch b, uint32_t* words)
{
  if (!b || !words) return fail(OCC_ERR_INVALID_ARG, "null argument");
  *words = b->L.querySlots / 32;
  return OCC_OK;
}

int occ_batch_launch(occ_batch b)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  occ_ctx_s* ctx = b->ctx;
  if (b->dirty) {
    const int slot = (b->cur + 1) % kRing;
    OCC_CUDA(cudaEventSynchronize(b->ringEv[slot]));
    write_views(b, b->ring[slot].p);
    OCC_CUDA(cudaGraphExecMemcpyNodeSetParams1D(b->exec, b->copyNode, b->S.tables.p, b->ring[slot].p,
                                                b->offCmds, cudaMemcpyHostToDevice));
    b->cur = slot;
    b->dirty = false;
  }
  OCC_CUDA(cudaGraphLaunch(b->exec, ctx->stream));
  OCC_CUDA(cudaEventRecord(b->ringEv[b->cur], ctx->stream));
  return OCC_OK;
}

int occ_batch_results(occ_batch b, uint32_t view, uint32_t* visibleBits, uint32_t* needsClippingBits)
{
  if (!b || view >= b->L.views.size()) return fail(OCC_ERR_INVALID_ARG, "bad argument");
  const ViewDesc& V = b->L.views[view];
  const size_t nw = div_up(V.queryCount, 32);
  if (nw) {
    if (visibleBits)
      OCC_CUDA(cudaMemcpyAsync(visibleBits, b->vis.p + V.queryStart / 32, nw * 4, cudaMemcpyDeviceToHost, b->ctx->stream));
    if (needsClippingBits)
      OCC_CUDA(cudaMemcpyAsync(needsClippingBits, b->nc.p + V.queryStart / 32, nw * 4, cudaMemcpyDeviceToHost,
                               b->ctx->stream));
  }
  OCC_CUDA(cudaStreamSynchronize(b->ctx->stream));
  return OCC_OK;
}

int occ_batch_check(occ_batch b)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  occ_ctx_s* ctx = b->ctx;
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  FrameHeader H;
  OCC_CUDA(cudaMemcpy(&H, b->S.header.p, sizeof(H), cudaMemcpyDeviceToHost));
  if (!H.sticky) return OCC_OK;
  // grow to the largest totals seen and capture again; the caller re-runs its frames
  b->S.capCks = std::max(b->S.capCks, H.maxCks + H.maxCks / 2 + 4096);
  b->S.capSt = std::max(b->S.capSt, H.maxSt + H.maxSt / 2 + 4096);
  uint32_t zero[4] = {0, 0, 0, 0};
  OCC_CUDA(cudaMemcpy(&b->S.header.p->sticky, zero, 12, cudaMemcpyHostToDevice));
  OCC_CHECK(capture(b));
  return fail(OCC_ERR_CAPACITY, "a launch exceeded the scratch capacity; grown, re-run the frames");
}

int occ_batch_profile(occ_batch b, uint32_t iterations, float* msPerKernel)
{
  if (!b || !msPerKernel || !iterations) return fail(OCC_ERR_INVALID_ARG, "bad argument");
  occ_ctx_s* ctx = b->ctx;
  cudaEvent_t ev[8];
  for (auto& e : ev) OCC_CUDA(cudaEventCreate(&e));
  for (int k = 0; k < 7; ++k) msPerKernel[k] = 0.0f;
  int status = OCC_OK;
  for (uint32_t it = 0; it < iterations && status == OCC_OK; ++it) {
    if (b->dirty) {
      const int slot = (b->cur + 1) % kRing;
      cudaEventSynchronize(b->ringEv[slot]);
      write_views(b, b->ring[slot].p);
      b->cur = slot;
      b->dirty = false;
      OCC_CUDA(cudaGraphExecMemcpyNodeSetParams1D(b->exec, b->copyNode, b->S.tables.p, b->ring[slot].p,
                                                  b->offCmds, cudaMemcpyHostToDevice));
    }
    cudaMemcpyAsync(b->S.tables.p, b->ring[b->cur].p, b->offCmds, cudaMemcpyHostToDevice, ctx->stream);
    cudaEventRecord(ev[7], ctx->stream);
    cudaError_t e = b->features ? launch_selection(b->params, (uint32_t)b->L.cmds.size(), b->mlp != nullptr, ctx->stream)
                                : cudaSuccess;
    const bool two = b->secondPass && b->mlp != nullptr;
    if (e == cudaSuccess) e = launch_flush_timed(b->params, b->L.numSt, b->L.maxStPerView, b->anyRaster,
                                                 !two && b->L.querySlots > 0, ctx->stream, ev);
    if (e == cudaSuccess && cudaEventSynchronize(ev[6]) == cudaSuccess) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[7], ev[0]);
      msPerKernel[6] += ms / (float)iterations;
      if (two) {  // the second pass is timed into the same stages
        for (int k = 0; k < 6; ++k) {
          cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
          msPerKernel[k] += ms / (float)iterations;
        }
        FrameParams P2 = b->params;
        P2.phase = 1;
        e = launch_flush_timed(P2, b->L.numSt, b->L.maxStPerView, b->anyRaster, b->L.querySlots > 0, ctx->stream,
                               ev);
      }
    }
    cudaEventRecord(b->ringEv[b->cur], ctx->stream);
    if (e != cudaSuccess) status = fail(OCC_ERR_CUDA, std::string("profile launch: ") + cudaGetErrorString(e));
    if (cudaEventSynchronize(ev[6]) != cudaSuccess) status = fail(OCC_ERR_CUDA, "profile sync");
    for (int k = 0; k < 6 && status == OCC_OK; ++k) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
      msPerKernel[k] += ms / (float)iterations;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return status;
}

int occ_batch_set_selection(occ_batch b, occ_mlp mlp, float fraction, int trackWins)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  if (mlp && !(fraction > 0.0f && fraction <= 1.0f)) return fail(OCC_ERR_INVALID_ARG, "fraction must be in (0, 1]");
  if (mlp && mlp->ctx != b->ctx) return fail(OCC_ERR_INVALID_ARG, "network from another context");
  const size_t n = std::max<size_t>(b->L.cmds.size(), 1);
  if (trackWins)
    for (const auto& V : b->L.views)
      if (V.cmdCount > 65534u) return fail(OCC_ERR_INVALID_ARG, "win counting takes at most 65,534 occluders per view");
  b->features = mlp != nullptr || trackWins != 0;
  b->mlp = mlp;
  b->selectFrac = fraction;
  b->trackWins = trackWins != 0;
  if (b->features) {
    OCC_CHECK(b->feat.reserve(n * kFeatures));
    OCC_CHECK(b->score.reserve(n));
    OCC_CHECK(b->cand.reserve(n));
    OCC_CHECK(b->select.reserve(n));
    OCC_CHECK(b->wins.reserve(n));
    OCC_CUDA(cudaMemsetAsync(b->wins.p, 0, n * 4, b->ctx->stream));
    OCC_CUDA(cudaMemsetAsync(b->score.p, 0, n * 4, b->ctx->stream));
    if (!b->L.cmds.empty())  // no launch before: nothing drawn
      OCC_CUDA(cudaMemsetAsync(b->S.cmdDraw.p, 0, b->L.cmds.size() * 4, b->ctx->stream));
  }
  return capture(b);
}

int occ_batch_stats(occ_batch b, uint32_t out[7])
{
  if (!b || !out) return fail(OCC_ERR_INVALID_ARG, "null argument");
  FrameHeader H;
  OCC_CUDA(cudaStreamSynchronize(b->ctx->stream));
  OCC_CUDA(cudaMemcpy(&H, b->S.header.p, sizeof(H), cudaMemcpyDeviceToHost));
  out[0] = H.totalRows;
  out[1] = H.totalCks;
  out[2] = H.totalSt;
  out[3] = H.activeChunks;
  out[4] = H.activeTiles;
  out[5] = (uint32_t)b->L.chunks.size();
  out[6] = (uint32_t)b->offCmds;  // host->device bytes per launch (the view table)
  return OCC_OK;
}

// Mean per-stage milliseconds of `iterations` frames with launch shape `t`.
static int profile_with(occ_batch b, const LaunchTuning& t, uint32_t iterations, float ms[7])
{
  const LaunchTuning saved = b->params.tune;
  b->params.tune = t;
  const int st = occ_batch_profile(b, iterations, ms);
  b->params.tune = saved;
  return st;
}

int occ_batch_autotune(occ_batch b, uint32_t iterations, uint32_t tuned[9], float msBefore[7], float msAfter[7])
{
  if (!b || !iterations) return fail(OCC_ERR_INVALID_ARG, "bad argument");
  uint32_t lim[7];
  tuning_limits(lim);
  LaunchTuning best = b->tune;
  float ms[7], base[7];
  OCC_CHECK(profile_with(b, best, iterations, base));
  if (msBefore) std::memcpy(msBefore, base, sizeof(base));
  // each parameter moves one stage's time only: search them one at a time
  auto search = [&](uint32_t LaunchTuning::*field, int stage, std::vector<uint32_t> cands) -> int {
    float bestMs = 3.0e38f;
    uint32_t bestV = best.*field;
    for (uint32_t v : cands) {
      LaunchTuning t = best;
      t.*field = v;
      OCC_CHECK(profile_with(b, t, iterations, ms));
      if (ms[stage] < bestMs) {
        bestMs = ms[stage];
        bestV = v;
      }
    }
    best.*field = bestV;
    return OCC_OK;
  };
  auto upTo = [](uint32_t n) {
    std::vector<uint32_t> v;
    for (uint32_t i = 1; i <= n; ++i) v.push_back(i);
    return v;
  };
  // super-tile edge (binning granularity): changes the layout and every stage
  // from setup to raster, so whole frames decide
  {
    float bestMs = 3.0e38f;
    uint32_t bestShift = b->tune.superTile == 8 ? 3u : 4u;
    for (uint32_t shift : {4u, 3u}) {
      OCC_CHECK(relayout(b, shift));
      OCC_CHECK(settle(b));
      OCC_CHECK(profile_with(b, best, iterations, ms));
      const float frame = ms[0] + ms[1] + ms[2] + ms[3] + ms[4];
      if (frame < bestMs) {
        bestMs = frame;
        bestShift = shift;
      }
    }
    OCC_CHECK(relayout(b, bestShift));
    OCC_CHECK(settle(b));
    best.superTile = 1u << bestShift;
  }
  OCC_CHECK(search(&LaunchTuning::setupPerSm, 0, upTo(lim[0])));
  OCC_CHECK(search(&LaunchTuning::fillPerSm, 2, upTo(lim[1])));
  OCC_CHECK(search(&LaunchTuning::walkPerSm, 3, {2, 4, 8, 16}));
  // raster form: one warp per unit of 1, 2 or 4 block rows, or a CTA per unit
  // of 8x1 or 8x2 blocks (128 + rows)
  {
    float bestMs = 3.0e38f;
    LaunchTuning pick = best;
    for (uint32_t form : {1u, 2u, 4u, 129u, 130u}) {
      LaunchTuning t = best;
      t.rasterThreads = form > 128u ? 128u : 32u;
      t.rasterRows = form > 128u ? form - 128u : form;
      OCC_CHECK(profile_with(b, t, iterations, ms));
      if (ms[4] < bestMs) {
        bestMs = ms[4];
        pick = t;
      }
    }
    best = pick;
  }
  const uint32_t limIdx = best.rasterThreads == 128u ? 5 : (best.rasterRows == 1 ? 2 : (best.rasterRows == 2 ? 3 : 4));
  OCC_CHECK(search(&LaunchTuning::rasterPerSm, 4, upTo(lim[limIdx])));
  OCC_CHECK(search(&LaunchTuning::rasterChunk, 4, {1, 2, 4, 8, 16}));
  OCC_CHECK(search(&LaunchTuning::queryRounds, 5, {kQueryPerThread, 1, 2, 4, 8}));
  b->tune = best;
  OCC_CHECK(capture(b));
  if (msAfter) OCC_CHECK(occ_batch_profile(b, iterations, msAfter));
  if (tuned) {
    tuned[0] = best.setupPerSm;
    tuned[1] = best.fillPerSm;
    tuned[2] = best.walkPerSm;
    tuned[3] = best.rasterPerSm;
    tuned[4] = best.rasterChunk;
    tuned[5] = best.queryRounds;
    tuned[6] = best.rasterRows ? best.rasterRows : kDefaultRasterRows;
    tuned[7] = best.rasterThreads;
    tuned[8] = best.superTile;
  }
  return OCC_OK;
}

int occ_batch_set_cull_labels(occ_batch b, int enable)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  if (enable && !(b->features && b->trackWins))
    return fail(OCC_ERR_INVALID_ARG, "cull labels need win counting (occ_batch_set_selection with trackWins)");
  b->cullLabels = enable != 0;
  if (b->cullLabels) {
    OCC_CHECK(b->cullCount.reserve(std::max<size_t>(b->L.cmds.size(), 1)));
    for (size_t v = 0; v < b->jobs.size(); ++v) {
      occ_raster_s* r = b->jobs[v].r;
      OCC_CHECK(r->owner.reserve((size_t)r->width * r->height));
      b->L.views[v].owner = r->owner.p;
    }
  } else {
    for (auto& V : b->L.views) V.owner = nullptr;
  }
  b->dirty = true;  // the next launch uploads the view table with the owner buffers
  return capture(b);
}

int occ_batch_read_cull_labels(occ_batch b, uint32_t view, uint32_t* counts)
{
  if (!b || !counts || view >= b->L.views.size()) return fail(OCC_ERR_INVALID_ARG, "bad argument");
  if (!b->cullLabels) return fail(OCC_ERR_INVALID_ARG, "cull labels are not enabled on this batch");
  const ViewDesc& V = b->L.views[view];
  if (V.cmdCount)
    OCC_CUDA(cudaMemcpyAsync(counts, b->cullCount.p + V.cmdStart, (size_t)V.cmdCount * 4, cudaMemcpyDeviceToHost,
                             b->ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(b->ctx->stream));
  return OCC_OK;
}

int occ_batch_set_second_pass(occ_batch b, int enable)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  b->secondPass = enable != 0;
  return capture(b);
}

int occ_batch_set_tuning(occ_batch b, const uint32_t tune[9])
{
  if (!b || !tune) return fail(OCC_ERR_INVALID_ARG, "null argument");
  for (int i = 0; i < 5; ++i)
    if (tune[i] > 64) return fail(OCC_ERR_INVALID_ARG, "launch shape out of range (at most 64)");
  if (tune[5] > kQueryRounds && tune[5] != kQueryPerThread) return fail(OCC_ERR_INVALID_ARG, "unknown query form");
  if (tune[6] != 0 && tune[6] != 1 && tune[6] != 2 && tune[6] != 4)
    return fail(OCC_ERR_INVALID_ARG, "raster unit rows must be 1, 2 or 4 (0: the default)");
  if (tune[7] != 0 && tune[7] != 32 && tune[7] != 128)
    return fail(OCC_ERR_INVALID_ARG, "raster threads per unit must be 32 or 128 (0: chosen per launch)");
  if (tune[7] == 128 && tune[6] == 4)
    return fail(OCC_ERR_INVALID_ARG, "the 128-thread raster form takes units of 1 or 2 block rows");
  if (tune[8] != 0 && tune[8] != 8 && tune[8] != 16)
    return fail(OCC_ERR_INVALID_ARG, "super-tile edge must be 8 or 16 blocks (0: 16)");
  LaunchTuning t{};
  t.setupPerSm = tune[0];
  t.fillPerSm = tune[1];
  t.walkPerSm = tune[2];
  t.rasterPerSm = tune[3];
  t.rasterChunk = tune[4];
  t.queryRounds = tune[5];
  t.rasterRows = tune[6];
  t.rasterThreads = tune[7];
  const uint32_t shift = tune[8] == 8 ? 3u : 4u;
  const bool newLayout = (b->tune.superTile == 8 ? 3u : 4u) != shift;
  t.superTile = 1u << shift;
  b->tune = t;
  if (newLayout) return relayout(b, shift);
  return capture(b);
}

int occ_batch_set_zero_depth(occ_batch b, int enable)
{
  if (!b) return fail(OCC_ERR_INVALID_ARG, "null batch");
  b->zeroDepth = enable != 0;
  // the kernels zero the depth of every block of a cleared view that no
  // fragment reaches; the flag travels in the view table of the next launch
  for (size_t v = 0; v < b->L.views.size(); ++v) {
    uint32_t& f = b->L.views[v].flags;
    f = (b->zeroDepth && b->jobs[v].clear) ? (f | kViewZeroDepth) : (f & ~kViewZeroDepth);
  }
  b->dirty = true;
  return OCC_OK;
}

int occ_batch_read_selection(occ_batch b, uint32_t view, float* features, uint32_t* wins, uint8_t* candidate,
                             uint8_t* selected, float* scores)
{
  if (!b || view >= b->L.views.size()) return fail(OCC_ERR_INVALID_ARG, "bad argument");
  if (!b->features) return fail(OCC_ERR_INVALID_ARG, "selection / win counting is not enabled on this batch");
  const ViewDesc& V = b->L.views[view];
  cudaStream_t st = b->ctx->stream;
  const size_t c0 = V.cmdStart, n = V.cmdCount;
  if (n) {
    if (features) OCC_CUDA(cudaMemcpyAsync(features, b->feat.p + c0 * kFeatures, n * kFeatures * 4, cudaMemcpyDeviceToHost, st));
    if (wins) OCC_CUDA(cudaMemcpyAsync(wins, b->wins.p + c0, n * 4, cudaMemcpyDeviceToHost, st));
    if (candidate) OCC_CUDA(cudaMemcpyAsync(candidate, b->cand.p + c0, n, cudaMemcpyDeviceToHost, st));
    if (selected) {
      if (b->mlp) OCC_CUDA(cudaMemcpyAsync(selected, b->select.p + c0, n, cudaMemcpyDeviceToHost, st));
      else OCC_CUDA(cudaMemcpyAsync(selected, b->cand.p + c0, n, cudaMemcpyDeviceToHost, st));
      if (b->mlp && b->secondPass) {
        std::vector<uint32_t> draw(n);
        OCC_CUDA(cudaMemcpyAsync(draw.data(), b->S.cmdDraw.p + c0, n * 4, cudaMemcpyDeviceToHost, st));
        OCC_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < n; ++i)
          if (!selected[i] && (draw[i] & 1u)) selected[i] = 2;  // drawn by the second pass
      }
    }
    if (scores) OCC_CUDA(cudaMemcpyAsync(scores, b->score.p + c0, n * 4, cudaMemcpyDeviceToHost, st));
  }
  OCC_CUDA(cudaStreamSynchronize(st));
  return OCC_OK;
}

int occ_batch_destroy(occ_batch b)
{
  if (!b) return OCC_OK;
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return OCC_OK;
}

int occ_build_coverage_table(int64_t* out4096)
{
  if (!out4096) return fail(OCC_ERR_INVALID_ARG, "null argument");
  occ_table::build_coverage_table(out4096);
  return OCC_OK;
}

int occ_coverage_table(int64_t* out4096)
{
  if (!out4096) return fail(OCC_ERR_INVALID_ARG, "null argument");
  static const unsigned long long t[4096] = {OCC_COVERAGE_TABLE_VALUES};
  std::memcpy(out4096, t, sizeof(t));
  return OCC_OK;
}


int occ_mlp_param_count(void) { return mlp_param_count(); }

int occ_mlp_create(occ_ctx ctx, uint32_t seed, occ_mlp* out)
{
  if (!ctx || !out) return fail(OCC_ERR_INVALID_ARG, "null argument");
  auto m = std::make_unique<occ_mlp_s>();
  m->ctx = ctx;
  const int np = mlp_param_count();
  OCC_CHECK(m->params.reserve(np));
  OCC_CHECK(m->m.reserve(np));
  OCC_CHECK(m->v.reserve(np));
  OCC_CHECK(m->grad.reserve(np + 1));
  OCC_CHECK(m->dev.reserve(1));
  // He-normal initialisation (fixed seed, host RNG), zero biases
  std::vector<float> p(np, 0.0f);
  uint64_t st = 0x9E3779B97F4A7C15ull ^ seed;
  auto next = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
  };
  auto normal = [&]() {
    double u1 = next(), u2 = next();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  };
  const int nW1 = kHidden * kFeatures, nW2 = kHidden * kHidden;
  for (int i = 0; i < nW1; ++i) p[i] = (float)(normal() * std::sqrt(2.0 / kFeatures));
  for (int i = 0; i < nW2; ++i) p[nW1 + kHidden + i] = (float)(normal() * std::sqrt(2.0 / kHidden));
  for (int i = 0; i < kHidden; ++i) p[nW1 + kHidden + nW2 + kHidden + i] = (float)(normal() * std::sqrt(1.0 / kHidden));
  OCC_CUDA(cudaMemcpyAsync(m->params.p, p.data(), (size_t)np * 4, cudaMemcpyHostToDevice, ctx->stream));
  OCC_CUDA(cudaMemsetAsync(m->m.p, 0, (size_t)np * 4, ctx->stream));
  OCC_CUDA(cudaMemsetAsync(m->v.p, 0, (size_t)np * 4, ctx->stream));
  OCC_CUDA(cudaMemsetAsync(m->dev.p, 0, sizeof(MlpDevice), ctx->stream));
  OCC_CUDA(launch_mlp_publish(m->params.p, m->dev.p, ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = m.release();
  return OCC_OK;
}

int occ_mlp_destroy(occ_mlp m)
{
  if (!m) return OCC_OK;
  cudaStreamSynchronize(m->ctx->stream);
  delete m;
  return OCC_OK;
}

int occ_mlp_get_params(occ_mlp m, float* out)
{
  if (!m || !out) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CUDA(cudaMemcpyAsync(out, m->params.p, (size_t)mlp_param_count() * 4, cudaMemcpyDeviceToHost, m->ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return OCC_OK;
}

int occ_mlp_set_params(occ_mlp m, const float* in)
{
  if (!m || !in) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CUDA(cudaMemcpyAsync(m->params.p, in, (size_t)mlp_param_count() * 4, cudaMemcpyHostToDevice, m->ctx->stream));
  OCC_CUDA(launch_mlp_publish(m->params.p, m->dev.p, m->ctx->stream));
  OCC_CUDA(cudaStreamSynchronize(m->ctx->stream));
  return OCC_OK;
}

int occ_mlp_get_state(occ_mlp m, float* params, float* adamM, float* adamV, uint32_t* step)
{
  if (!m) return fail(OCC_ERR_INVALID_ARG, "null network");
  const size_t bytes = (size_t)mlp_param_count() * 4;
  cudaStream_t st = m->ctx->stream;
  if (params) OCC_CUDA(cudaMemcpyAsync(params, m->params.p, bytes, cudaMemcpyDeviceToHost, st));
  if (adamM) OCC_CUDA(cudaMemcpyAsync(adamM, m->m.p, bytes, cudaMemcpyDeviceToHost, st));
  if (adamV) OCC_CUDA(cudaMemcpyAsync(adamV, m->v.p, bytes, cudaMemcpyDeviceToHost, st));
  if (step) *step = m->step;
  OCC_CUDA(cudaStreamSynchronize(st));
  return OCC_OK;
}

int occ_mlp_set_state(occ_mlp m, const float* params, const float* adamM, const float* adamV, uint32_t step)
{
  if (!m || !params || !adamM || !adamV) return fail(OCC_ERR_INVALID_ARG, "null argument");
  const size_t bytes = (size_t)mlp_param_count() * 4;
  cudaStream_t st = m->ctx->stream;
  OCC_CUDA(cudaMemcpyAsync(m->params.p, params, bytes, cudaMemcpyHostToDevice, st));
  OCC_CUDA(cudaMemcpyAsync(m->m.p, adamM, bytes, cudaMemcpyHostToDevice, st));
  OCC_CUDA(cudaMemcpyAsync(m->v.p, adamV, bytes, cudaMemcpyHostToDevice, st));
  OCC_CUDA(launch_mlp_publish(m->params.p, m->dev.p, st));
  OCC_CUDA(cudaStreamSynchronize(st));
  m->step = step;
  return OCC_OK;
}

static int mlp_batch(occ_mlp m, uint32_t n, const float* features, const float* targets)
{
  OCC_CHECK(m->feat.reserve((size_t)n * kFeatures));
  OCC_CHECK(m->score.reserve(n));
  OCC_CHECK(m->target.reserve(n));
  OCC_CHECK(m->xb.reserve((size_t)n * kFeatures));
  OCC_CHECK(m->h1.reserve((size_t)n * kHidden));
  OCC_CHECK(m->h2.reserve((size_t)n * kHidden));
  OCC_CHECK(m->ds.reserve(n));
  OCC_CHECK(m->dh1.reserve((size_t)n * kHidden));
  OCC_CHECK(m->dh2.reserve((size_t)n * kHidden));
  OCC_CHECK(m->err2.reserve(n));
  OCC_CHECK(m->partial.reserve((size_t)mlp_grad_blocks(n) * (mlp_param_count() + 1)));
  cudaStream_t st = m->ctx->stream;
  OCC_CUDA(cudaMemcpyAsync(m->feat.p, features, (size_t)n * kFeatures * 4, cudaMemcpyHostToDevice, st));
  if (targets) OCC_CUDA(cudaMemcpyAsync(m->target.p, targets, (size_t)n * 4, cudaMemcpyHostToDevice, st));
  return OCC_OK;
}

int occ_mlp_forward(occ_mlp m, uint32_t n, const float* features, float* scores)
{
  if (!m || (n && (!features || !scores))) return fail(OCC_ERR_INVALID_ARG, "null argument");
  if (!n) return OCC_OK;
  OCC_CHECK(mlp_batch(m, n, features, nullptr));
  cudaStream_t st = m->ctx->stream;
  OCC_CUDA(launch_mlp_forward(m->feat.p, n, m->dev.p, m->score.p, nullptr, nullptr, nullptr, st));
  OCC_CUDA(cudaMemcpyAsync(scores, m->score.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
  OCC_CUDA(cudaStreamSynchronize(st));
  return OCC_OK;
}

int occ_mlp_gradients(occ_mlp m, uint32_t n, const float* features, const float* targets, float* loss, float* grads)
{
  if (!m || !n || !features || !targets) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CHECK(mlp_batch(m, n, features, targets));
  cudaStream_t st = m->ctx->stream;
  OCC_CUDA(launch_mlp_forward(m->feat.p, n, m->dev.p, m->score.p, m->h1.p, m->h2.p, m->xb.p, st));
  OCC_CUDA(launch_mlp_backward(m->score.p, m->target.p, n, m->dev.p, m->xb.p, m->h1.p, m->h2.p, m->ds.p, m->dh1.p,
                               m->dh2.p, m->err2.p, m->partial.p, m->grad.p, st));
  const int np = mlp_param_count();
  if (grads) OCC_CUDA(cudaMemcpyAsync(grads, m->grad.p, (size_t)np * 4, cudaMemcpyDeviceToHost, st));
  if (loss) OCC_CUDA(cudaMemcpyAsync(loss, m->grad.p + np, 4, cudaMemcpyDeviceToHost, st));
  OCC_CUDA(cudaStreamSynchronize(st));
  return OCC_OK;
}

static int mlp_groups(occ_mlp m, uint32_t n, uint32_t numGroups, const uint32_t* groupStart)
{
  if (!groupStart || !numGroups || groupStart[0] != 0 || groupStart[numGroups] != n)
    return fail(OCC_ERR_INVALID_ARG, "group starts must run from 0 to n");
  for (uint32_t g = 0; g < numGroups; ++g)
    if (groupStart[g + 1] < groupStart[g]) return fail(OCC_ERR_INVALID_ARG, "group starts must not decrease");
  OCC_CHECK(m->groups.reserve(numGroups + 1));
  OCC_CUDA(cudaMemcpyAsync(m->groups.p, groupStart, (size_t)(numGroups + 1) * 4, cudaMemcpyHostToDevice,
                           m->ctx->stream));
  return OCC_OK;
}

int occ_mlp_gradients_listwise(occ_mlp m, uint32_t n, const float* features, const float* targets,
                               uint32_t numGroups, const uint32_t* groupStart, float* loss, float* grads)
{
  if (!m || !n || !features || !targets) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CHECK(mlp_groups(m, n, numGroups, groupStart));
  OCC_CHECK(mlp_batch(m, n, features, targets));
  cudaStream_t st = m->ctx->stream;
  OCC_CUDA(launch_mlp_forward(m->feat.p, n, m->dev.p, m->score.p, m->h1.p, m->h2.p, m->xb.p, st));
  OCC_CUDA(launch_mlp_backward(m->score.p, m->target.p, n, m->dev.p, m->xb.p, m->h1.p, m->h2.p, m->ds.p, m->dh1.p,
                               m->dh2.p, m->err2.p, m->partial.p, m->grad.p, st, m->groups.p, numGroups));
  const int np = mlp_param_count();
  if (grads) OCC_CUDA(cudaMemcpyAsync(grads, m->grad.p, (size_t)np * 4, cudaMemcpyDeviceToHost, st));
  if (loss) OCC_CUDA(cudaMemcpyAsync(loss, m->grad.p + np, 4, cudaMemcpyDeviceToHost, st));
  OCC_CUDA(cudaStreamSynchronize(st));
  return OCC_OK;
}

int occ_mlp_train_step_listwise(occ_mlp m, uint32_t n, const float* features, const float* targets,
                                uint32_t numGroups, const uint32_t* groupStart, float lr, float* loss)
{
  if (!m || !n || !features || !targets) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CHECK(mlp_groups(m, n, numGroups, groupStart));
  OCC_CHECK(mlp_batch(m, n, features, targets));
  cudaStream_t st = m->ctx->stream;
  OCC_CUDA(launch_mlp_forward(m->feat.p, n, m->dev.p, m->score.p, m->h1.p, m->h2.p, m->xb.p, st));
  OCC_CUDA(launch_mlp_backward(m->score.p, m->target.p, n, m->dev.p, m->xb.p, m->h1.p, m->h2.p, m->ds.p, m->dh1.p,
                               m->dh2.p, m->err2.p, m->partial.p, m->grad.p, st, m->groups.p, numGroups));
  OCC_CUDA(launch_adam(m->params.p, m->grad.p, m->m.p, m->v.p, lr, ++m->step, st));
  OCC_CUDA(launch_mlp_publish(m->params.p, m->dev.p, st));
  if (loss) OCC_CUDA(cudaMemcpyAsync(loss, m->grad.p + mlp_param_count(), 4, cudaMemcpyDeviceToHost, st));
  OCC_CUDA(cudaStreamSynchronize(st));
  return OCC_OK;
}

int occ_mlp_train_step(occ_mlp m, uint32_t n, const float* features, const float* targets, float lr, float* loss)
{
  if (!m || !n || !features || !targets) return fail(OCC_ERR_INVALID_ARG, "null argument");
  OCC_CHECK(mlp_batch(m, n, features, targets));
  cudaStream_t st = m->ctx->stream;
  OCC_CUDA(launch_mlp_forward(m->feat.p, n, m->dev.p, m->score.p, m->h1.p, m->h2.p, m->xb.p, st));
  OCC_CUDA(launch_mlp_backward(m->score.p, m->target.p, n, m->dev.p, m->xb.p, m->h1.p, m->h2.p, m->ds.p, m->dh1.p,
                               m->dh2.p, m->err2.p, m->partial.p, m->grad.p, st));
  OCC_CUDA(launch_adam(m->params.p, m->grad.p, m->m.p, m->v.p, lr, ++m->step, st));
  OCC_CUDA(launch_mlp_publish(m->params.p, m->dev.p, st));
  if (loss) OCC_CUDA(cudaMemcpyAsync(loss, m->grad.p + mlp_param_count(), 4, cudaMemcpyDeviceToHost, st));
  OCC_CUDA(cudaStreamSynchronize(st));
  return OCC_OK;
}

}  // extern "C"
