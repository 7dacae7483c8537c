// Data layout shared by the host launcher (capi.cu) and the kernels (kernels.cu).
//
// One flush rasterises the pending commands of one or more views ("rasterizer
// targets") and then answers their queries.  Everything below is laid out for
// a batch of views; a single view is a batch of one.
//
// Global quad numbering: the commands of a view are concatenated in
// submission order (each command = one occluder = packets*2 quads); every view
// starts at a multiple of kChunk so that setup chunk c = quad >> kChunkShift
// belongs to exactly one view.  Padding quads are invalid.
#pragma once
#include <stdint.h>

namespace occ {

constexpr int kChunkShift = 8;
constexpr int kChunk = 1 << kChunkShift;  // quads per setup CTA
constexpr int kSuperTile = 16;            // default binning super-tile edge, in 8x8 blocks (8 or 16: whole warp-tiles)
constexpr int kTileW = 8;                 // warp-tile: 8 x 4 blocks, one lane per block
constexpr int kTileH = 4;
constexpr int kCkSpan = 8;                // row-walk checkpoint every 8 block columns (== kTileW)
constexpr uint32_t kDefaultRasterRows = 2;  // raster unit: 8 x R blocks of a warp-tile, R = 1, 2 or 4
constexpr uint32_t kDefaultCtaRows = 1;     // the 128-thread form's unit: 8 x 1 blocks (or 8 x 2)
constexpr int kMaxUnitsPerTile = kTileH;    // raster units per warp-tile at R = 1
constexpr int kMaxCmdPerChunk = 40;       // commands are >= 8 quads, so <= 33 per chunk
constexpr int kCkFloats = 12;             // 4 edge offsets + 8 depth lanes
constexpr int kMaxStPerView = 3072;       // super-tiles per view (e.g. 12288 x 6144 pixels)
constexpr uint32_t kNoAllocMaxQueries = 65536;  // boxes per occ_raster_query_batch_noalloc call

enum : uint32_t {
  kViewClear = 1u << 0,      // hiZ := 1 before rasterising (Rasterizer::clear)
  kViewZeroDepth = 1u << 1,  // with kViewClear: depth := 0 as well (a freshly created rasterizer's state)
};

enum : uint32_t {
  kCmdNearClip = 1u << 0,  // rasterize<true>
  kCmdGated = 1u << 1,     // decide draw / near-clip on the GPU from the occluder bounds
};

enum : uint8_t {
  kQuadNearClip = 1u << 0,
  kQuadSafe = 1u << 1,     // depth interpolation cannot overflow: plain IEEE adds are x86-exact
};

enum : int {
  kModeCulled = 0, kModeTriangle0, kModeTriangle1, kModeConcaveRight, kModeConcaveLeft,
  kModeConcaveCenter, kModeConvex
};

struct ViewDesc {
  uint16_t* depth;   // width*height u16, 8x8 blocks of 8 rows x 8 pixels, block-major
  uint16_t* hiz;     // blocks + 8
  uint16_t* tileHiz; // per warp-tile (8x4 blocks, row-major), 4 entries: the minimum hiZ of
                     // each of its block rows (0xFFFF for rows outside the view)
  uint32_t width, height, blocksX, blocksY;
  float cols[16];    // prebaked matrix columns (Rasterizer.cpp:91-104)
  float rows[16];    // rows of the transposed input matrix (frustum planes)
  uint32_t cmdStart, cmdCount;
  uint32_t chunkStart, chunkCount;      // setup chunks of this view (global indices)
  uint32_t tileStart, tilesX, tilesY;   // warp-tiles of this view (global indices)
  uint32_t stBase, stX, stY;            // super-tiles (global index base) and grid
  uint32_t matBase;                     // count matrix base: stX*stY*chunkCount entries
  uint32_t queryStart, queryCount;      // query slots; queryStart is a multiple of 32
  uint32_t flags;
  uint32_t stShift;                     // super-tile edge = 1 << stShift blocks (3 or 4)
  uint32_t* owner;   // optional, width*height (depth layout): command + 1 that produced each
                     // pixel's final value this launch, 0 if none (cull labels of the selector)
};

struct alignas(16) Cmd {
  uint32_t view;
  uint32_t wordOffset;   // first packed word of the occluder in the occluder pool
  uint32_t quadStart;    // first global quad index
  uint32_t quadCount;    // 2 * packet vectors
  uint32_t flags;        // kCmdNearClip / kCmdGated
  uint32_t pad[3];
  float refMin[4], refMax[4];
  float boundsMin[4], boundsMax[4];
};

struct alignas(16) Chunk {
  uint32_t view;
  uint32_t localIndex;   // chunk index within its view
  uint32_t quadCount;    // real quads in this chunk (the rest is padding)
  uint32_t cmdFirst;     // first command overlapping the chunk
  uint32_t cmdCount;     // commands overlapping the chunk
  uint32_t pad[3];
};

// Per-quad setup output read by the rasteriser (48 bytes, moved as three
// 16-byte words).
struct alignas(16) QuadRaster {
  uint16_t minX, minY, maxX, maxY;  // block bbox [min, max); minX == maxX marks an invalid quad
  uint16_t maxZ;                    // packed 16-bit nearest depth bound
  uint8_t mode, flags;
  uint32_t ckLocal;                 // checkpoint offset within the chunk
  float Dx, Dy;                     // depth plane gradient per block
  uint16_t slope[4];                // slope part of the table index, per edge
  float nx[4];                      // normalised edge x coefficients
};

// Per-quad setup output read by the row walk (48 bytes, moved as three
// 16-byte words).
struct alignas(16) QuadWalk {
  float plane0;     // depth at the bbox origin
  float off[4];     // edge offsets at the bbox origin (quantisation units)
  float ny[4];      // normalised edge y coefficients
  uint32_t rowLocal; // first row of this quad within the chunk's row numbering
  uint32_t pad[2];
};

constexpr int kFeatures = 16;  // per-occluder features of the learned selector
constexpr int kHidden = 64;    // MLP 16 -> 64 -> 64 -> 1

// MLP weights as the kernels read them: bf16 matrices stored output-major
// (w1t[n][k], w2t[n][k]), fp32 biases and output layer.
struct MlpDevice {
  uint16_t w1t[kHidden * kFeatures];
  uint16_t w2t[kHidden * kHidden];
  float b1[kHidden];
  float b2[kHidden];
  float w3[kHidden];
  float b3;
  float pad[3];
};

struct Totals {
  uint32_t rows, cks, st, pad;
};

// Device-side frame header: totals, capacities and status.
struct FrameHeader {
  uint32_t totalRows, totalCks, totalSt, overflow;
  uint32_t capCks, capSt, viewsDone, sticky;  // sticky: overflow seen since the last check
  uint32_t maxCks, maxSt, pad[2];              // largest totals seen since the last check
  // reset at the start of every launch
  uint32_t activeChunks;  // chunks with a drawn command (k_chunk_gate)
  uint32_t activeTiles;   // queued raster units (tile preparation in k_walk_prep)
  uint32_t tileCursor;    // next entry of the active tile list (k_raster)
  uint32_t pad2;
};
constexpr uint32_t kHeaderResetWords = 3;  // activeChunks, activeTiles, tileCursor

// One occluder of a GPU bake: vertexCount float4 (a multiple of 32) from
// vertexStart in the launch's vertex array, quantised in [refMin, refMax].
struct BakeJob {
  uint32_t vertexStart, vertexCount, pad[2];
  float refMin[4], refMax[4];
};

// readBack formats (the OCC_READBACK_* values of the C ABI).
constexpr int kReadBackRgba8 = 0, kReadBackLinearF32 = 1, kReadBackDepthF32 = 2, kReadBackPackedU16 = 3;

// k_query forms: kQueryPerThread runs one box per thread in place; 1..kQueryRounds
// are the compacting warps with that many rounds of 32 slots each.
constexpr uint32_t kQueryRounds = 8;
constexpr uint32_t kQueryPerThread = 255;

// Launch shape of one flush (0 = the default: as many resident CTAs per SM
// as the kernel's registers and shared memory allow; one tile per fetch).
// Chosen per batch by occ_batch_autotune.
struct LaunchTuning {
  uint32_t setupPerSm, fillPerSm, walkPerSm, rasterPerSm, rasterChunk;
  uint32_t queryRounds;  // 0: chosen by slot count; else a k_query form (above)
  uint32_t rasterRows;   // block rows per raster unit: 1, 2 or 4 (0: kDefaultRasterRows, or
                         // kDefaultCtaRows for the 128-thread form, which takes 1 or 2)
  uint32_t rasterThreads;  // threads per raster unit: 32 (one warp) or 128 (a CTA, units of 2 rows);
                           // 0: chosen by the launch's unit count
  uint32_t superTile;      // binning super-tile edge in blocks: 8 or 16 (0: kSuperTile); set by the host layout
};

struct FrameParams {
  const ViewDesc* views;
  uint32_t numViews;
  uint32_t numCmds;
  uint32_t maxViewCmds;  // commands of the view with the most
  uint32_t matSize;      // entries of `mat` over all views
  LaunchTuning tune;
  uint32_t phase;        // 0: the frame (or the top-K pass); 1: the second pass of a
                         // selection (no clear; draws the remaining candidates still visible)
  const Cmd* cmds;
  const Chunk* chunks;
  uint32_t numChunks;
  uint32_t numTiles;     // warp-tiles over all views
  uint32_t numQuerySlots;
  const uint32_t* pool;  // packed occluder words
  QuadRaster* rec;
  QuadWalk* walk;
  Totals* chunkTot;      // per active chunk, at chunkStart + rank: totals (rows, cks)
  Totals* chunkBase;     // per active chunk, at chunkStart + rank: exclusive prefix within the view
  uint32_t* mat;         // super-tile x active chunk (by rank) counts -> exclusive prefixes (per view,
                         // st-major, chunkCount columns)
  uint32_t* stStart;     // per global super-tile: list start (global)
  uint32_t* stLen;
  Totals* viewTot;
  Totals* viewBase;
  uint32_t* viewChunksDone;
  uint4* stList;         // per super-tile, submission order: {quad, minX | minY << 16, maxX | maxY << 16, maxZ}
  uint32_t* ckBase;      // per quad: global index of its first row-walk checkpoint
  uint2* rowOwner;       // per block row of the batch: {quad, row within the quad}
  float* ck;             // row-walk checkpoints, kCkFloats floats each
  FrameHeader* header;
  const float4* qmin;    // query boxes per slot
  const float4* qmax;
  uint32_t* visBits;     // one bit per query slot
  uint32_t* ncBits;
  uint32_t* cmdDraw;     // per command: bit0 drawn (this pass), bit1 near-clipped, bit2 drawn by
                         // the first pass of this launch (second pass only)
  uint32_t* activeChunkList;  // chunks with a drawn command (header->activeChunks of them)
  uint32_t* chunkRank;        // per active chunk: its rank among its view's active chunks (chunk order)
  uint32_t* viewActiveCount;  // per view: how many
  uint4* activeTileList;      // queued raster units (header->activeTiles): {warp-tile * 4 + first block
                              // row, view, first entry and length of the unit's super-tile list}
  // learned occluder selection and win counts (all optional)
  float* feat;           // per command: kFeatures features
  float* score;          // per command: MLP score
  uint8_t* cand;         // per command: passes the gating test (selection candidate)
  uint8_t* select;       // per command: 1 = rasterise; null = every command
  uint32_t* wins;        // per command: pixels whose final depth it produced (read as the
                         // previous frame's wins by the feature kernel, then reset)
  const MlpDevice* mlp;
  float selectFrac;      // fraction of each view's candidates kept
  uint32_t* cullCount;   // per command: samples of occlusion-culled boxes it owns (labels; optional)
  uint32_t fusedSelect;  // 1: one CTA per view scores, selects and gates (k_select_view; no k_gate)
};

// Views of at most this many commands are selected by one CTA each; larger
// ones spread the network over many CTAs (k_mlp_forward, k_topk, k_gate).
constexpr uint32_t kFusedSelectMaxCmds = 1024;

}  // namespace occ

namespace occ {
static_assert(sizeof(QuadRaster) == 48 && sizeof(QuadWalk) == 48 && sizeof(Cmd) % 16 == 0 && sizeof(Chunk) == 32,
              "record sizes");
}  // namespace occ
