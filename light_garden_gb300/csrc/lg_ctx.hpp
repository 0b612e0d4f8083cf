// lg_ctx.hpp — the context behind lg_ctx* and the host helpers shared by lg_api.cu
// (single scene) and lg_batch.cu (multi-scene batches and serving).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lg_host.hpp"

namespace lgh {
struct ServeState;  // lg_serve.cu

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

constexpr uint32_t UNIT_REFS = SPLIT_UNIT_REFS;  // shared-atomic raster: keeps the split sums within 2^31
constexpr uint32_t UNIT_REFS_WARP = 8192;  // warp-private raster: no bound, bigger units flush less
// the smaller of the two: the unit table is sized for whichever raster the context runs
constexpr uint32_t MIN_UNIT_REFS = UNIT_REFS < UNIT_REFS_WARP ? UNIT_REFS : UNIT_REFS_WARP;
constexpr size_t OBJ_SMEM_MAX = 96 * 1024;

}  // namespace lgh

using namespace lgh;

struct lg_ctx {
  int device = 0;
  int n_sm = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // scene
  DevBuf d_scan, d_info, d_leaves, d_prog, d_lights, d_cubics;
  DevBuf d_xgeo, d_xnode;  // exact mode: geometry nodes and per-object preorder trees
  DevBuf d_mod_colors;     // string mod: the modulo-colour table of the mod drawn (the nested one if any)
  DevBuf d_chords;         // string mod: the frame's lines (lg_string_mod.modulo of them)
  uint64_t chords_ready = 0;  // lines the last trace left in d_chords (0: none to draw)
  // nested string mod: its parameters (pointers cleared), the crossing points of the outer
  // mod's lines (double2, computed at upload) and their count
  bool has_nested = false;
  lg_string_mod nested{};
  DevBuf d_sm_lines, d_cross_blk, d_cross;
  uint64_t n_cross = 0;
  uint32_t n_obj = 0, n_leaves = 0, n_prog = 0, n_lights = 0, n_cubic = 0;
  uint64_t n_primary = 0;
  lg_params prm{};
  bool has_scene = false;
  double aspect = 1.0;
  // trace
  DevBuf d_queue[2], d_scanrec, d_hitrec, d_list[N_LISTS];
  uint64_t queue_cap = 0;
  DevBuf d_segs, d_paths;
  uint64_t seg_cap = 0;
  DevBuf d_ctr;
  Counters* h_ctr = nullptr;
  uint64_t seg_cap_hint = 0, queue_cap_hint = 0;
  // raster
  DevBuf d_tile_count, d_tile_off, d_tile_cursor, d_unit_off, d_refs, d_units, d_accum, d_stage;
  DevBuf d_cta_hist;  // per-CTA bin counts of the shared-memory binning (scatter launch shape)
  uint64_t refs_cap = 0, units_cap = 0;
  uint32_t n_tiles = 0, ntx = 0, nty = 0;
  // launch shapes
  // scan, refine, full, bounce (fast mode), solve, bounce (exact mode)
  int trace_grid[6] = {0, 0, 0, 0, 0, 0}, raster_grid = 0, bin_grid = 0;
  int raster_warp_grid = 0;
  int raster_variant = 0;  // 1 shared-atomic tile raster, 2 warp-private tile raster; 0 = not tuned yet
  int scan_pairs = 0;      // pair slots per lane of the scan (8 / 16; 0: by the culling grid)
  int scan_pairs_opt = 0;  // lg_device_opts.scan_pairs (0: tune on a scene's first render)
  bool scan_tune = false;  // armed by a new scene: its second lg_render (lg_batch_render) times
                           // both sizes first; a scene rendered once is never tuned
  uint32_t renders = 0;    // lg_render / lg_batch_render calls since the scene or batch changed
  size_t obj_smem = 0;
  int smem_fits = 0;
  // graph
  cudaGraphExec_t gexec = nullptr;
  bool graph_valid = false;
  bool streaming = false;  // lg_render accumulates while tracing (the frame's segments exceed one pass)
  uint64_t stream_ring = 256ull << 20;  // ... with a ring of this many segments
  cudaEvent_t ev[6] = {};
  // multi-scene mode (lg_batch_upload): the concatenated scenes replace the single scene
  bool multi = false;
  uint32_t n_scenes = 0;
  std::vector<SceneRec> h_scenes;
  std::vector<SceneCanvas> h_canvases;
  std::vector<uint64_t> h_px_base;       // first pixel of each scene's image
  DevBuf d_scenes, d_canvases, d_seg_scene, d_cubic_scene, d_part;
  DevBuf d_bounds, d_order, d_scene_count, d_scene_off;
  // culling grids (one record per scene; a single scene uses record 0)
  DevBuf d_grids, d_cell_start, d_cell_obj;
  int culling = LG_CULL_AUTO;
  float grid_density = 0.0f;
  int32_t wait_polls = 1 << 22;  // bounded device waits (lg_device_opts.wait_polls)
  bool culled = false;  // the uploaded scene (or some scene of the batch) has a grid
  bool scan_walk = false;  // the nearest-hit scan walks the grid (else it scans the object table)
  uint64_t total_px = 0;
  uint32_t total_bins = 0;
  uint32_t max_bounce_all = 0;
  uint64_t n_overlay = 0;
  int batch_grid_scan = 0;
  std::vector<cudaEvent_t> bev;          // batch stage events (start, per generation x 2, resolved)
  // lg_render: events around the trace kernels of every generation (before the scan, after
  // the scan, after the solve, after the bounce), recorded while kev_on
  std::vector<cudaEvent_t> kev;
  bool kev_on = false;
  ServeState* serve = nullptr;           // serving mode (lg_serve_begin .. lg_serve_end)
};


namespace lgh {

lg_status fail(lg_ctx* c, lg_status st, const std::string& msg);
lg_status cuda_fail(lg_ctx* c, cudaError_t e, const char* what);
lg_status ensure(lg_ctx* c, DevBuf& b, size_t bytes, const char* what);
void release(DevBuf& b);
lg_status sync_counters(lg_ctx* c);
float elapsed(cudaEvent_t a, cudaEvent_t b);
lg_status ensure_trace_buffers(lg_ctx* c);
// Copies concatenated culling grids to the device (asynchronous: the caller synchronizes
// the stream before the host tables go away).
lg_status upload_grids(lg_ctx* c, const lgh::GridTables& G);
// Per-CTA bin counts for `bins` bins when they fit shared memory (else nothing to do), and
// the pointer RasterArgs should carry for them (nullptr when absent).
lg_status ensure_cta_hist(lg_ctx* c, size_t bins);
uint32_t* cta_hist_for(const lg_ctx* c, size_t bins);
// k_bin_count with the scatter's launch shape when the per-CTA counts are kept.
void launch_bin_count(lg_ctx* c, const RasterArgs& A, int smem_tiles, size_t bsm);
// The scan and bounce kernels for the context's mode (single scene or multi-scene, with or
// without the culling walk).
using TraceKernel = void (*)(SceneDev, TraceBufs, uint32_t, int);
using TraceKernel3 = void (*)(SceneDev, TraceBufs, uint32_t);
TraceKernel scan_kernel(bool multi, bool culled, bool exact, int pairs);
// The scan's pair slots per lane for the context, its occupancy-sized grid (trace_grid[0], or
// batch_grid_scan when multi), and a switch to another size (new grid, graph invalidated).
int scan_pairs_of(const lg_ctx* c);
lg_status scan_grid(lg_ctx* c, bool multi);
lg_status set_scan_pairs(lg_ctx* c, int pairs, bool multi);
TraceKernel bounce_kernel(bool multi, bool culled);
TraceKernel3 bounce_x_kernel(bool multi, bool culled);
// Occupancy-sized grids of the trace kernels for the context's mode (trace_grid[1..5]).
lg_status trace_grids(lg_ctx* c, bool multi, size_t tsm);
// The light setup and one generation's chain for the context's precision: the FP32 scan,
// then k_refine + k_full + k_bounce (fast) or k_solve_x + k_bounce_x (exact).
void launch_light_setup(lg_ctx* c, const SceneDev& S, bool multi, int blocks);
void launch_generation(lg_ctx* c, const SceneDev& S, const TraceBufs& B, uint32_t g, bool multi, int scan_grid,
                       size_t scan_smem, size_t tsm, int smem_fits);
// Uploads a flattened scene's exact-mode tables (geometry nodes, preorder trees).
lg_status upload_exact(lg_ctx* c, const Flat& F);
SceneDev scene_dev(lg_ctx* c);
TraceBufs trace_bufs(lg_ctx* c);
RasterArgs raster_args(lg_ctx* c);
void fill_stats(lg_ctx* c, lg_trace_stats* s);
void serve_free(lg_ctx* c);

#define CK(call, what)                                      \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what);   \
  } while (0)

}  // namespace lgh
