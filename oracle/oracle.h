/*
 * CPU oracle for the occluder rasteriser's hot path: a portable scalar-C
 * restatement of the reference's Rasterizer (SoftwareRasterizer/Rasterizer.cpp).
 *
 * TEST INFRASTRUCTURE ONLY.  Only the tests, the smoke check and the CPU
 * baseline leg of the benchmark load this library, and only as the checker or
 * as the timed CPU baseline.  The GPU library never links or calls it.
 *
 * It reproduces the x86 AVX2 build bit for bit on any IEEE-754 host: the
 * RCPPS approximation comes from the measured table in x86_tables.h, fused
 * multiply-adds happen exactly where the reference writes _mm*_fmadd/fmsub/
 * fnmadd, and NaN results follow x86 rules (first NaN operand propagated
 * quiet, the "default NaN" 0xFFC00000 for invalid operations).  Pinned
 * against the reference compiled here (oracle/_ref) and against the golden
 * fixtures in tests/golden.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_raster orc_raster;

/* width, height: multiples of 8 (Rasterizer.cpp:68).  table: 4096 coverage
 * masks, or NULL to build them as Rasterizer.cpp:547-604 does. */
orc_raster* orc_create(uint32_t width, uint32_t height, const int64_t* table);
void orc_destroy(orc_raster* r);

/* 1 (default): reproduce the reference's 16-bit block-index product
 * (Rasterizer.cpp:1054); 0: use the full 32-bit product. */
void orc_set_block_index_wrap(orc_raster* r, int wrap16);

void orc_set_mvp(orc_raster* r, const float* m16);          /* Rasterizer.cpp:76-105 */
void orc_clear(orc_raster* r);                              /* Rasterizer.cpp:107-121 */

/* packed: packetCount 32-byte vectors of 8 uint32 words (Occluder.cpp:153-156).
 * nearClip selects rasterize<true> / rasterize<false> (Rasterizer.cpp:606-1295). */
void orc_rasterize(orc_raster* r, const uint32_t* packed, uint32_t packetCount,
                   const float* refMin, const float* refMax, int nearClip);

uint32_t orc_setup_dump(orc_raster* r, const uint32_t* packed, uint32_t packetCount, const float* refMin,
                        const float* refMax, int nearClip, int32_t* out6);

int orc_query(orc_raster* r, const float* bmin, const float* bmax, int* needsClipping); /* :123-281 */
int orc_query2d(const orc_raster* r, uint32_t minX, uint32_t maxX, uint32_t minY, uint32_t maxY,
                uint32_t maxZ);                                                         /* :283-349 */
void orc_query_batch(orc_raster* r, uint32_t n, const float* mins, const float* maxs,
                     uint8_t* visible, uint8_t* needsClipping);

void orc_read_back(const orc_raster* r, uint8_t* rgba);     /* :351-399 */
void orc_read_back_values(const orc_raster* r, int format, void* out); /* :378-381 */
void orc_read_depth(const orc_raster* r, uint16_t* out);    /* width*height u16, block-major */
uint32_t orc_read_hiz(const orc_raster* r, uint16_t* out);  /* blocks+8 u16; returns count */
void orc_read_table(const orc_raster* r, int64_t* out);     /* 4096 masks */
void orc_write_depth(orc_raster* r, const uint16_t* in);    /* seed the (stale) depth buffer */
void orc_write_hiz(orc_raster* r, const uint16_t* in);

/* Per-frame counters of the last orc_rasterize calls (reset by orc_clear):
 * [0] quads set up, [1] valid quads, [2] block visits, [3] hiZ skips,
 * [4] blocks written. */
void orc_read_counters(const orc_raster* r, uint64_t* out5);

/* One plain frame (the parity-mode loop): clear, set MVP; for each occluder k,
 * queryVisibility of its bounds against an empty buffer decides whether it is
 * drawn and with which near-clip variant.  occ_packed[k] etc. describe occluder
 * k.  flags[k] = visible | needsClipping << 1 (may be NULL). */
void orc_frame_plain(orc_raster* r, uint32_t n, const uint32_t* const* occ_packed,
                     const uint32_t* occ_packets, const float* occ_ref /* n x 8: min4,max4 */,
                     const float* occ_bounds /* n x 8 */, const float* mvp, uint8_t* flags);

/* Main.cpp's own frame loop (Main.cpp:181-206): clear, set MVP, occluders
 * sorted front to back by the squared distance of their centre (occ_centers,
 * n x 4) to `eye` (DPPS sum of the x, y, z products), each queried against
 * the live buffer and rasterised with the near-clip variant the query gives.
 * Equal distances keep submission order (the reference's std::sort leaves
 * their order unspecified).  order_out (may be NULL) receives the drawing
 * order, flags (may be NULL) per occluder visible | needsClipping << 1. */
void orc_frame_gated(orc_raster* r, uint32_t n, const uint32_t* const* occ_packed, const uint32_t* occ_packets,
                     const float* occ_ref, const float* occ_bounds, const float* occ_centers, const float* eye,
                     const float* mvp, uint32_t* order_out, uint8_t* flags);

#ifdef __cplusplus
}
#endif
