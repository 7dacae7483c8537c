/*
 * rasterizer_gb300 -- C ABI of the GB300 occluder rasteriser.
 *
 * Drop-in GPU replacement for the hot path of rawrunprotected/rasterizer
 * (SoftwareRasterizer/Rasterizer.h:10-61, Occluder.h:7-21): occluder
 * rasterisation into a hierarchical 16-bit depth buffer and bounding-box
 * visibility queries against it, bit-exact with the reference's AVX2 path.
 * Plain C types only; every call returns OCC_OK (0) or a negative status and
 * occ_last_error() gives a message for the calling thread.
 *
 * Execution model: one CUDA stream per context.  Rasterisation is deferred:
 * occ_raster_rasterize() appends to the rasterizer's command list and the
 * next query, read-back or flush runs all pending work in one batch of
 * kernels.  A context and its rasterizers are not thread-safe (nor is the
 * reference's Rasterizer); several contexts may be used from several threads.
 */
#ifndef RASTERIZER_GB300_H
#define RASTERIZER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCC_OK 0
#define OCC_ERR_INVALID_ARG (-1)
#define OCC_ERR_OUT_OF_MEMORY (-2)
#define OCC_ERR_CUDA (-3)
#define OCC_ERR_CAPACITY (-4)
#define OCC_ERR_UNSUPPORTED (-5)
#define OCC_ERR_IO (-6)          /* a file could not be read or written, or is not valid */

typedef struct occ_ctx_s* occ_ctx;
typedef struct occ_raster_s* occ_raster;
typedef uint32_t occ_occluder; /* context-scoped occluder id */

/* Per-occluder flags for occ_raster_rasterize_many / batches. */
#define OCC_NEAR_CLIP 1u /* rasterize<true> (Rasterizer.cpp:713-728, :973-982) */
#define OCC_GATED 2u     /* decide visibility and near-clip variant on the GPU from the
                            occluder bounds, as queryVisibility on an empty buffer would
                            (Rasterizer.cpp:123-281); replaces the caller's query */

const char* occ_last_error(void);
int occ_version(void);

/* ---- context ---------------------------------------------------------------- */
int occ_ctx_create(int device, occ_ctx* out);
/* Destroy a context after every rasterizer, batch and selector made on it:
 * they refer to its stream and occluder pool. */
int occ_ctx_destroy(occ_ctx ctx);
int occ_ctx_synchronize(occ_ctx ctx);
void* occ_ctx_stream(occ_ctx ctx); /* the context's cudaStream_t */

/* ---- occluders (Occluder.h:7-21) --------------------------------------------
 * Uploads the reference's packed occluder data unchanged: packetCount 32-byte
 * vectors (Occluder::m_vertexData, m_packetCount; Occluder.cpp:153-156), with
 * the quantisation box (m_refMin/m_refMax) and bounds (m_boundsMin/m_boundsMax). */
int occ_occluder_upload(occ_ctx ctx, const uint32_t* packed, uint32_t packetCount, const float refMin[4],
                        const float refMax[4], const float boundsMin[4], const float boundsMax[4],
                        occ_occluder* out);
/* Occluder::bake (Occluder.cpp:7-181) on the GPU for `count` occluders in one
 * launch, asynchronous on the context's stream; the bytes equal
 * occ_occluder_bake's.  Device pointers: vertices (float4, vertexStart[count]
 * of them), packed (out, one word per vertex, occluder k's words at
 * vertexStart[k]), bounds (out, 20 floats per occluder: refMin, refMax,
 * boundsMin, boundsMax, center).  Host arrays: vertexStart (count + 1,
 * vertexStart[0] = 0, each occluder a positive multiple of 32 vertices),
 * refBoxes (8 floats per occluder: refMin, refMax). */
int occ_occluders_bake_device(occ_ctx ctx, uint32_t count, const float* vertices, const uint32_t* vertexStart,
                              const float* refBoxes, uint32_t* packed, float* bounds);
/* occ_occluder_upload from device memory (e.g. occ_occluders_bake_device's
 * output): packed is a device pointer, bounds a host copy of the 20 floats
 * (refMin, refMax, boundsMin, boundsMax, center).  The copy into the
 * context's occluder pool is queued on the context's stream: packed must stay
 * valid (and unchanged) until the stream has run it (occ_ctx_synchronize). */
int occ_occluder_upload_device(occ_ctx ctx, const uint32_t* packed, uint32_t packetCount, const float bounds[20],
                               occ_occluder* out);
int occ_occluder_count(occ_ctx ctx, uint32_t* count);

/* ---- rasterizer (Rasterizer.h:13-26) ----------------------------------------- */
/* Rasterizer::Rasterizer (Rasterizer.cpp:66-74): width, height multiples of 8. */
int occ_raster_create(occ_ctx ctx, uint32_t width, uint32_t height, occ_raster* out);
int occ_raster_destroy(occ_raster r);
/* Rasterizer::setModelViewProjection (Rasterizer.cpp:76-105): row-vector float[16]. */
int occ_raster_set_mvp(occ_raster r, const float matrix[16]);
/* Rasterizer::clear (Rasterizer.cpp:107-121): hiZ := 1, depth keeps stale values. */
int occ_raster_clear(occ_raster r);
/* Rasterizer::rasterize<possiblyNearClipped> (Rasterizer.cpp:606-1295), deferred. */
int occ_raster_rasterize(occ_raster r, occ_occluder occ, int possiblyNearClipped);
/* Many rasterize calls at once; flags[i] = OCC_NEAR_CLIP | OCC_GATED (NULL = all 0). */
int occ_raster_rasterize_many(occ_raster r, uint32_t n, const occ_occluder* occ, const uint8_t* flags);
/* Runs pending work; gatedFlags (optional, n of the last OCC_GATED call) receives
 * per command: bit0 drawn, bit1 near-clipped. */
int occ_raster_flush(occ_raster r);
int occ_raster_command_flags(occ_raster r, uint32_t n, uint8_t* out);
/* Rasterizer::queryVisibility (Rasterizer.cpp:123-281). */
int occ_raster_query_visibility(occ_raster r, const float boundsMin[4], const float boundsMax[4], int* visible,
                                int* needsClipping);
/* Batch of queries from host memory: mins/maxs n float4 each; results one bit per
 * query in ceil(n/32) words (bit i%32 of word i/32). */
int occ_raster_query_batch(occ_raster r, uint32_t n, const float* mins, const float* maxs, uint32_t* visibleBits,
                           uint32_t* needsClippingBits);
/* Same, all pointers in device memory, asynchronous on the context stream. */
int occ_raster_query_batch_device(occ_raster r, uint32_t n, const void* dMins, const void* dMaxs,
                                  void* dVisibleBits, void* dNeedsClippingBits);
/* No counterpart in the reference (its queries never allocate).  The same
 * queries as occ_raster_query_batch for callers that must not allocate device
 * memory: frame loops with a fixed memory budget reserved at start-up, and
 * engines that forbid cudaMalloc/cudaFree on their frame thread because both
 * can synchronise and stall the whole device.  Boxes and result bits are
 * staged in one fixed device array of OCC_NOALLOC_MAX_QUERIES boxes (about
 * 2 MiB, held on every GPU that loads the library until exit); larger n is
 * rejected.  Call it from an ordinary host thread, never from a host function
 * enqueued with cudaLaunchHostFunc: it makes CUDA calls and blocks until the
 * bits are in the host buffers.  The first call on a device looks up the
 * array's device address (a one-time set-up), so make that first call before
 * any stream capture.  "Allocates nothing" holds once the library's device
 * code is loaded on the device: with lazy module loading the first kernel
 * launch or symbol lookup loads it, and loading allocates, so flush a
 * rasterizer or make one no-allocation call during set-up.  All calls on a
 * device share the array and it keeps the last call's contents: calls whose
 * work overlaps on the GPU race and must be serialised.  Pending
 * rasterisation is not run here (running it may allocate): flush first. */
#define OCC_NOALLOC_MAX_QUERIES 65536u
int occ_raster_query_batch_noalloc(occ_raster r, uint32_t n, const float* mins, const float* maxs,
                                   uint32_t* visibleBits, uint32_t* needsClippingBits);
/* Rasterizer::query2D (Rasterizer.cpp:283-349). */
int occ_raster_query2d(occ_raster r, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY, uint32_t maxZ,
                       int* visible);
/* Rasterizer::readBackDepth (Rasterizer.cpp:351-399): width*height RGBA8. */
int occ_raster_read_back_depth(occ_raster r, void* rgba);
/* readBackDepth and the values it computes on the way to its bytes, for
 * debugging and visualisation: width*height row-major elements; blocks with
 * hiZ == 1 (cleared) give 0 in every format, as the reference's bytes do. */
enum {
  OCC_READBACK_RGBA8 = 0,      /* the reference's bytes, as occ_raster_read_back_depth */
  OCC_READBACK_LINEAR_F32 = 1, /* float linDepth = 0.5 / (1000.25 - (1 - depth) * 999.75) (:381) */
  OCC_READBACK_DEPTH_F32 = 2,  /* float depth = float bits (u16 << 12) * 3.9623753e28 (:378-379) */
  OCC_READBACK_PACKED_U16 = 3  /* the packed 16-bit depth itself, block layout undone */
};
int occ_raster_read_back(occ_raster r, int format, void* out);
/* Raw buffers in the reference's layout: depth width*height u16 (8x8 blocks,
 * block-major, 8 rows of 8 pixels), hiZ blocks+8 u16. */
int occ_raster_read_depth_raw(occ_raster r, uint16_t* out);
int occ_raster_read_hiz(occ_raster r, uint16_t* out, uint32_t* count);
int occ_raster_write_depth_raw(occ_raster r, const uint16_t* in);
int occ_raster_write_hiz(occ_raster r, const uint16_t* in);
int occ_raster_size(occ_raster r, uint32_t* width, uint32_t* height);

/* ---- batched multi-view ------------------------------------------------------
 * Sets up, bins, rasterises and queries many views in one batch of kernels. */
typedef struct {
  occ_raster raster;
  const float* mvp;            /* float[16] or NULL (keep the rasterizer's matrix) */
  int clear;                   /* clear before drawing */
  uint32_t numOccluders;
  const occ_occluder* occluders;
  const uint8_t* flags;        /* per occluder OCC_NEAR_CLIP | OCC_GATED, NULL = all 0 */
  uint32_t numQueries;
  const float* queryMins;      /* host, numQueries float4 */
  const float* queryMaxs;
  uint32_t* visibleBits;       /* host, ceil(numQueries/32) words, may be NULL */
  uint32_t* needsClippingBits;
} occ_view_work;
int occ_batch_execute(occ_ctx ctx, uint32_t numViews, const occ_view_work* views);

/* Prepared batch: tables and query boxes uploaded once, the per-frame kernel
 * sequence captured in a CUDA graph.  occ_batch_launch is asynchronous. */
typedef struct occ_batch_s* occ_batch;
int occ_batch_prepare(occ_ctx ctx, uint32_t numViews, const occ_view_work* views, occ_batch* out);
int occ_batch_set_mvp(occ_batch b, uint32_t view, const float matrix[16]);
int occ_batch_launch(occ_batch b);
/* Matrices of views first .. first+count-1 in one call (count float[16]). */
int occ_batch_set_mvps(occ_batch b, uint32_t first, uint32_t count, const float* matrices);
/* All views' result bits in one copy (syncs): `words` = occ_batch_result_words
 * words per array; view v's bits start at word firstWord[v] (numViews entries). */
int occ_batch_result_words(occ_batch b, uint32_t* words);
int occ_batch_results_all(occ_batch b, uint32_t* visibleBits, uint32_t* needsClippingBits, uint32_t* firstWord);
/* occ_batch_results_all without waiting: the copies are queued on the
 * context's stream behind the launches queued so far, and the buffers hold
 * the bits once the stream has run them (occ_ctx_synchronize).  Page-locked
 * host buffers keep the copies asynchronous.  No reference counterpart. */
int occ_batch_results_all_async(occ_batch b, uint32_t* visibleBits, uint32_t* needsClippingBits);
/* Replaces the query boxes of views first .. first+count-1: each view's
 * numQueries boxes, the views back to back in mins / maxs (float4 per box),
 * e.g. the boxes of moving objects every frame, as the reference takes every
 * query's box from the caller (Rasterizer.cpp:123-281).  The copies are
 * queued on the context's stream ahead of the next launch; page-locked host
 * arrays must stay unchanged until the stream has run them. */
int occ_batch_set_queries(occ_batch b, uint32_t first, uint32_t count, const float* mins, const float* maxs);
int occ_batch_results(occ_batch b, uint32_t view, uint32_t* visibleBits, uint32_t* needsClippingBits);
int occ_batch_check(occ_batch b); /* syncs; OCC_ERR_CAPACITY if a launch overflowed */
/* Runs the frame `iterations` times kernel by kernel with CUDA events between
 * them on the context stream; msPerKernel[7] receives the mean duration of
 * setup, scan, list fill, row walk, raster, query and (when selection is on,
 * see occ_batch_set_selection) the selection kernels before them. */
int occ_batch_profile(occ_batch b, uint32_t iterations, float* msPerKernel);
int occ_batch_destroy(occ_batch b);

/* ---- learned occluder selection (replaces Main.cpp:184-206's distance-sorted
 *      loop) ------------------------------------------------------------------
 * An MLP 16 -> 64 -> 64 -> 1 (bf16 tensor-core inference, fp32 master weights)
 * scores each occluder of a view from features of its bounds (screen rect,
 * depth bounds, distance, size, quads) and the pixels it won in the previous
 * launch; only the top fraction of each view's candidates is rasterised. */
typedef struct occ_mlp_s* occ_mlp;
#define OCC_MLP_FEATURES 16
int occ_mlp_param_count(void); /* 5313 floats: W1t[64][16] b1[64] W2t[64][64] b2[64] w3[64] b3 */
int occ_mlp_create(occ_ctx ctx, uint32_t seed, occ_mlp* out);
int occ_mlp_destroy(occ_mlp m);
int occ_mlp_get_params(occ_mlp m, float* out);
int occ_mlp_set_params(occ_mlp m, const float* in);
/* host arrays: features n x 16, scores n */
int occ_mlp_forward(occ_mlp m, uint32_t n, const float* features, float* scores);
/* mean-squared-error loss and its gradient (param_count floats) without an update */
int occ_mlp_gradients(occ_mlp m, uint32_t n, const float* features, const float* targets, float* loss, float* grads);
/* Training state for checkpoints: fp32 weights, Adam moments (param_count
 * floats each; any pointer may be NULL on get) and the Adam step count. */
int occ_mlp_get_state(occ_mlp m, float* params, float* adamM, float* adamV, uint32_t* step);
int occ_mlp_set_state(occ_mlp m, const float* params, const float* adamM, const float* adamV, uint32_t step);
/* Listwise loss: rows form numGroups groups (one view in one frame each),
 * group g = rows [groupStart[g], groupStart[g+1]), groupStart[numGroups] = n;
 * targets are a distribution over each group's rows; loss = mean over groups
 * of the cross-entropy between it and the softmax of the group's scores. */
int occ_mlp_gradients_listwise(occ_mlp m, uint32_t n, const float* features, const float* targets,
                               uint32_t numGroups, const uint32_t* groupStart, float* loss, float* grads);
int occ_mlp_train_step_listwise(occ_mlp m, uint32_t n, const float* features, const float* targets,
                                uint32_t numGroups, const uint32_t* groupStart, float lr, float* loss);
/* one Adam step (beta 0.9 / 0.999) on one batch */
int occ_mlp_train_step(occ_mlp m, uint32_t n, const float* features, const float* targets, float lr, float* loss);
/* On a prepared batch: mlp != NULL keeps ceil(fraction * candidates) occluders
 * per view (top scores); trackWins counts per occluder the pixels whose final
 * depth it produced (labels, and the next launch's previous-frame feature). */
int occ_batch_set_selection(occ_batch b, occ_mlp mlp, float fraction, int trackWins);
/* With enable != 0, every view the batch clears also starts each launch with
 * zero depth, the state of a freshly created rasterizer: the kernels write
 * zeros to the blocks no fragment reaches (no separate pass over the buffer).
 * The reference's clear only marks blocks (hiZ := 1) and its
 * queryVisibility still reads the old depth of a cleared block that a query
 * box covers partially (Rasterizer.cpp:305-344), so a frame's results depend
 * on the frames before it; zeroed depth makes each frame stand alone (used to
 * compare a selected subset against the full frame).  No reference counterpart. */
int occ_batch_set_zero_depth(occ_batch b, int enable);
/* Autotuner: times the batch's frame stage by stage (occ_batch_profile) over
 * launch shapes -- resident CTAs per SM of the persistent setup, list-fill and
 * raster kernels, row-walk CTAs per SM, tiles per raster queue fetch, the
 * query kernel's form -- and keeps, per stage, the fastest; the graph is
 * captured again with them.  tuned[OCC_TUNING_FIELDS] = {setup, fill, walk,
 * raster CTAs per SM, raster units per queue fetch, query form: 255 = one box
 * per thread in place, 1..8 = frustum survivors listed per warp over that many
 * rounds of 32 boxes, raster unit rows: 1, 2 or 4 block rows of 8 blocks,
 * raster threads per unit: 32 (one warp per unit) or 128 (a CTA per unit of
 * 1 or 2 rows; 0 in set_tuning: chosen per launch by its unit count), binning
 * super-tile edge: 8 or 16 blocks (quads are listed per super-tile; smaller
 * ones give shorter lists and more entries)};
 * msBefore/msAfter[7] as occ_batch_profile (either may be NULL).  No
 * reference counterpart (the reference has no launch shapes). */
#define OCC_TUNING_FIELDS 9
int occ_batch_autotune(occ_batch b, uint32_t iterations, uint32_t tuned[OCC_TUNING_FIELDS], float msBefore[7],
                       float msAfter[7]);
/* Sets the launch shapes directly, in occ_batch_autotune's layout (0 in any
 * entry: the default), e.g. to reuse a tuned choice for a batch of the same
 * shape without timing it again.  CTAs per SM and units per fetch up to 64;
 * query form 0, 1..8 or 255; unit rows 0, 1, 2 or 4; threads per unit 0, 32
 * or 128 (with rows 0, 1 or 2; 0: 1); super-tile edge 0, 8 or 16 (a new edge lays the
 * batch out again).  No reference counterpart. */
int occ_batch_set_tuning(occ_batch b, const uint32_t tune[OCC_TUNING_FIELDS]);
/* Work counts of the last launch (syncs): block rows walked, row-walk
 * checkpoints, super-tile list entries, chunks with a drawn occluder, warp-tiles
 * rasterised (the others only cleared), the batch's chunk count, and the
 * bytes of tables each launch copies from the host. */
int occ_batch_stats(occ_batch b, uint32_t out[7]);
/* With enable != 0 (and a network set), each launch runs a second pass after
 * the top-K one: every other candidate whose bounds are still visible against
 * the first pass's buffer (queryVisibility, as Main.cpp:192-206 runs it before
 * each rasterize) is drawn too, without a clear; the queries follow the second
 * pass.  The frame then differs from the full frame only by drawing order.
 * A pixel whose value the second pass replaces counts as a win of both
 * occluders. */
int occ_batch_set_second_pass(occ_batch b, int enable);
/* Training labels of the selector (needs trackWins): each launch records the
 * owner of every pixel's final value and, for every query box culled by
 * depth (inside the frustum), credits the owners of a 4x4 grid of sample
 * pixels in its screen rectangle.  Per occluder of the view: its credits. */
int occ_batch_set_cull_labels(occ_batch b, int enable);
int occ_batch_read_cull_labels(occ_batch b, uint32_t view, uint32_t* counts);
/* Per occluder of the view, after the last launch: its features, pixel wins,
 * candidate flag (passes the visibility test), selected flag (1 = top-K,
 * 2 = drawn by the second pass) and score. */
int occ_batch_read_selection(occ_batch b, uint32_t view, float* features, uint32_t* wins, uint8_t* candidate,
                             uint8_t* selected, float* scores);

/* ---- host-side occluder preparation (QuadDecomposition.h:5-10,
 *      SurfaceAreaHeuristic.h:5-12, Occluder.h:9) -------------------------------
 * Byte-identical to the reference's output. */
/* QuadDecomposition::decompose: indices 3 per triangle -> 4 per quad; out has room
 * for 4*(nIndices/3) entries; *outCount receives the number written. */
int occ_quad_decompose(const uint32_t* indices, uint32_t nIndices, const float* vertices, uint32_t nVertices,
                       uint32_t* out, uint32_t* outCount);
/* SurfaceAreaHeuristic::generateBatches: aabbs n x (min4, max4); flat receives the
 * batched quad indices (n entries), offsets numBatches+1 entries (room for n+1). */
int occ_sah_generate_batches(const float* aabbs, uint32_t n, uint32_t targetSize, uint32_t splitGranularity,
                             uint32_t* flat, uint32_t* offsets, uint32_t* numBatches);
/* SurfaceAreaHeuristic::generateBatches (SurfaceAreaHeuristic.cpp:96-104) on
 * the GPU, the same batches as occ_sah_generate_batches: aabbs and flat are
 * device pointers (n x (min4, max4) floats; n indices), offsets and
 * numBatches host memory (room for n+1 offsets).  Runs on the context's
 * stream and returns when the batches are known.  Boxes with a NaN centre
 * coordinate (min + max) give OCC_ERR_UNSUPPORTED: the reference's order for
 * them comes from its library's merge sort under a comparison that is no
 * strict order; the host form handles them. */
int occ_sah_generate_batches_device(occ_ctx ctx, const float* aabbs, uint32_t n, uint32_t targetSize,
                                    uint32_t splitGranularity, uint32_t* flat, uint32_t* offsets,
                                    uint32_t* numBatches);
/* Occluder::bake: vertices nVertices float4 (quads of 4, a multiple of 32: whole
 * packets of 8 quads; the reference asserts 16 but reads 32 at a time);
 * packedOut nVertices words; returns the packet count (32-byte vectors). */
int occ_occluder_bake(const float* vertices, uint32_t nVertices, const float refMin[4], const float refMax[4],
                      uint32_t* packedOut, uint32_t* packetCount, float boundsMin[4], float boundsMax[4],
                      float center[4]);

/* ---- files (host) ----------------------------------------------------------------
 * The reference demo's mesh files (Main.cpp:56-84): VertexBuffer.bin, raw
 * float4 vertices; IndexBuffer.bin, raw u32 triangle indices.  With vertices
 * and indices NULL only the counts are returned; otherwise *numVertices and
 * *numIndices give the buffers' capacities on input and the counts on output. */
int occ_mesh_load_bin(const char* vertexPath, const char* indexPath, float* vertices, uint32_t* numVertices,
                      uint32_t* indices, uint32_t* numIndices);
/* Baked occluders of a scene in one file (versioned, hashed; no reference
 * counterpart: the demo bakes at every start, Main.cpp:86-128).  Occluder k:
 * packetCounts[k] 32-byte vectors at packed[k] (Occluder.h:19-20) and
 * bounds[20k..20k+19] = refMin, refMax, boundsMin, boundsMax, center (4 floats
 * each, Occluder.h:12-16).  Written to path + ".part", then renamed. */
int occ_occluders_save(const char* path, uint32_t count, const uint32_t* packetCounts, const uint32_t* const* packed,
                       const float* bounds);
/* Occluder count and packed words (sum of 8 * packetCount) of a baked file. */
int occ_occluders_file_info(const char* path, uint32_t* count, uint64_t* words);
/* Loads a baked file into caller buffers sized by occ_occluders_file_info:
 * packetCounts[count], packed[words] (occluders back to back), bounds[20 * count]. */
int occ_occluders_load(const char* path, uint32_t capacityCount, uint64_t capacityWords, uint32_t* packetCounts,
                       uint32_t* packed, float* bounds);

/* The demo's whole scene preparation in one call (Main.cpp:86-128):
 * decompose, pad to whole packets with the first quad, per-quad boxes, SAH
 * batches (targetSize, splitGranularity: the demo uses 512, 8), the reference
 * box of all vertices, Occluder::bake per batch; the same bytes as those steps
 * one by one.  *count and *words receive the occluder count and the packed
 * words over all occluders; with packetCounts, packed and bounds all NULL
 * only those sizes are computed.  Otherwise packetCounts[count], packed[words]
 * (occluders back to back, in batch order) and bounds[20 * count] (refMin,
 * refMax, boundsMin, boundsMax, center per occluder) receive the occluders;
 * OCC_ERR_CAPACITY if capacityCount / capacityWords are too small (at most
 * (nIndices/3 + 7)/8 + 1 occluders and 4 * (nIndices/3 + 7) words). */
int occ_scene_bake(const float* vertices, uint32_t nVertices, const uint32_t* indices, uint32_t nIndices,
                   uint32_t targetSize, uint32_t splitGranularity, uint32_t capacityCount, uint64_t capacityWords,
                   uint32_t* count, uint64_t* words, uint32_t* packetCounts, uint32_t* packed, float* bounds);

/* The coverage-mask table as the reference builds it on this host
 * (Rasterizer.cpp:547-604) and the table the GPU uses (generated on x86-64). */
int occ_build_coverage_table(int64_t* out4096);
int occ_coverage_table(int64_t* out4096);

#ifdef __cplusplus
}
#endif

#endif /* RASTERIZER_GB300_H */
