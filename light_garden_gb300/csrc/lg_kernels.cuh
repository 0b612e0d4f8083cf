// lg_kernels.cuh — kernel entry points shared between the .cu translation units.
#pragma once
#include "lg_device.cuh"

namespace lgd {

struct Unit {              // one raster work unit: a chunk of one tile's segment list
  uint32_t tile;
  uint32_t n;              // refs in this unit
  uint64_t begin;          // first ref
};

struct BlendDev {
  int32_t src[4];          // source factor per channel (lg_blend_factor)
  int32_t op[4];           // op per channel (lg_blend_op)
  float constant[4];
  float clear[4];
};

// One scene's canvas in a multi-scene accumulation: its bins (2 per tile) start at
// bin_base and its pixels at px_base of the shared accumulation buffer.
struct SceneCanvas {
  uint32_t W, H, ntx, nty;
  uint64_t bin_base, px_base;
};

struct RasterArgs {
  const lg_segment* segs;
  const uint16_t* seg_scene;      // multi-scene: scene of each segment (nullptr: one scene)
  const SceneCanvas* canvases;    // multi-scene: per-scene canvas, in bin order
  uint32_t n_scenes;
  uint64_t seg_cap;
  uint32_t W, H, ntx, nty;
  uint32_t n_tiles;
  uint32_t unit_refs;      // refs per work unit
  BlendDev blend;
  uint32_t* tile_count;    // refs per tile
  uint64_t* tile_off;      // exclusive prefix of tile_count
  unsigned long long* tile_cursor;
  uint64_t* unit_off;      // exclusive prefix of units per tile
  uint32_t* refs;          // segment index per (tile, segment) pair, grouped by tile
  uint64_t refs_cap;
  Unit* units;
  uint64_t units_cap;
  // shared-memory binning with the scatter's launch shape: k_bin_count leaves each CTA's bin
  // counts here ([CTA][bin]) and k_bin_scatter reserves its ranges from them instead of
  // counting its segments again (nullptr: the scatter counts)
  uint32_t* cta_hist;
  void* accum;             // H * W * 4 of int64 (FIXED64) or float (F32)
  Counters* ctr;
};

template <bool MULTI>
__global__ void k_light_setup(SceneDev S);
// CULL: the culling-grid walk is compiled in (scenes whose grid has nx == 0 still take
// the full scan); without it the kernels scan every object.
// EXACT: the rays hold FP64 coordinates (exact mode); no FP32 canvas exits.
// CHUNK: pair slots per lane between classifications (8 or 16).
template <bool MULTI, bool CULL, bool EXACT, int CHUNK>
__global__ void k_scan(SceneDev S, TraceBufs B, uint32_t gen, int smem_fits);
int scan_smem_bytes(int pairs);  // dynamic shared memory of k_scan<.., pairs> before the object table
constexpr int SCAN_THREADS = 128;
template <bool MULTI>
__global__ void k_refine(SceneDev S, TraceBufs B, uint32_t gen);
template <bool MULTI>
__global__ void k_full(SceneDev S, TraceBufs B, uint32_t gen, int smem_fits);
template <bool MULTI, bool CULL>
__global__ void k_bounce(SceneDev S, TraceBufs B, uint32_t gen, int smem_fits);
// exact FP64 mode (lg_exact.cu)
template <bool MULTI>
__global__ void k_light_setup_x(SceneDev S);
template <bool MULTI>
__global__ void k_solve_x(SceneDev S, TraceBufs B, uint32_t gen);
template <bool MULTI, bool CULL>
__global__ void k_bounce_x(SceneDev S, TraceBufs B, uint32_t gen);
// The string-mod lines' table and the modulo-colour table on the device (sm.colors is the
// caller's host pointer and is never read on the device).
struct ChordArgs {
  lg_chord* out;
  const lg_mod_color* colors;
  uint32_t n_colors;
  const double2* pts;  // nested mod: its points (the outer mod's line crossings), else null
  uint64_t n_pts;
};
// Crossings of a string mod's lines (lg_string_mod.nested): the lines' endpoints, then the
// (diff, line) pairs in blocks of CROSS_PAIRS_PER_BLOCK: counts per block, their exclusive
// scan (one CTA), and the crossing points written in pair order.
constexpr int CROSS_THREADS = 256;
constexpr int CROSS_PER_THREAD = 16;
constexpr uint64_t CROSS_PAIRS_PER_BLOCK = (uint64_t)CROSS_THREADS * CROSS_PER_THREAD;
__global__ void k_sm_lines(lg_string_mod sm, double2* lines);
__global__ void k_cross_count(const double2* lines, uint64_t m, uint32_t* blk);
__global__ void k_cross_scan(uint32_t* blk, uint32_t n_blk, unsigned long long* total);
__global__ void k_cross_write(const double2* lines, uint64_t m, const uint32_t* blk_off, double2* pts);
__global__ void k_overlay(SceneDev S, TraceBufs B, const uint32_t* cubic_objs, const uint16_t* cubic_scene,
                          uint32_t n_cubic, lg_string_mod sm, ChordArgs CA);
__global__ void k_scene_hist(SceneDev S, TraceBufs B, uint32_t gen, unsigned* count);
__global__ void k_scene_offsets(unsigned* count, unsigned* off, uint32_t n_scenes);
__global__ void k_scene_scatter(SceneDev S, TraceBufs B, uint32_t gen, unsigned* off, uint32_t* order);

__global__ void k_clear_accum(RasterArgs A, int fixed);
__global__ void k_bin_count(RasterArgs A, int smem_tiles);
__global__ void k_scan_tiles(RasterArgs A);
__global__ void k_build_units(RasterArgs A);
__global__ void k_bin_scatter(RasterArgs A, int smem_tiles);
// One CTA of 1024 threads per SM: each CTA fills its own range of every tile list, so the
// partially written 32 B sectors still open are CTAs x tiles; with one CTA per SM they stay
// in L2 and are written back whole (8 CTAs per SM overflowed L2 and turned every 4 B
// reference into a DRAM read-modify-write).
constexpr int SCATTER_THREADS = 1024;
inline int scatter_grid(int n_sm, int smem_tiles) { return smem_tiles ? n_sm : 2 * n_sm; }
template <int MODE>
__global__ void k_raster(RasterArgs A);
int raster_smem_bytes(int mode);
template <int MODE>
__global__ void k_raster_warp(RasterArgs A);
// String-mod lines straight into the image (one warp per line, global atomics), colour
// interpolated along the major axis; FIXED: int64 Q31.32, else f32.
template <bool FIXED>
__global__ void k_raster_chords(RasterArgs A, const lg_chord* chords, uint64_t n);
int raster_warp_smem_bytes();
constexpr int RM_FIXED_SPLIT_ = 0, RM_FIXED_MINMAX_ = 1, RM_F32_ = 2;
// Segments per work unit of the shared-atomic raster: bounds the split-plane sums.
constexpr uint32_t SPLIT_UNIT_REFS = 16384;
constexpr uint32_t MAX_SMEM_TILES = 32768;  // tile bins (2 per tile) with 32-bit counters in 128 KB
// multi-scene streaming accumulation
__global__ void k_stream_rotate(Counters* ctr, uint64_t seg_cap);
__global__ void k_stream_decide(Counters* ctr, uint32_t gen, uint64_t seg_cap, uint64_t queue_cap, int last);
__global__ void k_clear_counts(RasterArgs A);
constexpr int TILE_SCAN_CHUNK = 4096;  // bins per CTA of the multi-block tile scan
__global__ void k_tiles_partial(RasterArgs A, unsigned long long* part);
__global__ void k_tiles_scan_partials(RasterArgs A, unsigned long long* part, uint32_t n_part);
__global__ void k_tiles_apply(RasterArgs A, const unsigned long long* part);
__global__ void k_resolve_f16(const void* accum, int fixed, uint32_t W, uint32_t H, uint16_t* dst, size_t pitch);
__global__ void k_resolve_rgba8(const void* accum, int fixed, uint32_t W, uint32_t H, uint8_t* dst, size_t pitch);

}  // namespace lgd
