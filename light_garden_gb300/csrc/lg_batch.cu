// lg_batch.cu — many scenes in one multi-scene trace (lg_batch_upload / lg_batch_render).
//
// The reference traces one scene per Tracer (src/light_garden/tracer.rs:276-358).  A batch
// concatenates the object, leaf, program and light tables of k scenes; every ray carries its
// scene, and each generation of all trees of all scenes is one wavefront, so small scenes
// share the GPU instead of each leaving most of it idle.  The segment ring holds one
// generation: after each generation its segments are binned into the scenes' tiles (the
// bins of all canvases are numbered consecutively) and rasterised into the scenes' images,
// which live one after another in one accumulation buffer.  Fixed-point sums make every
// scene's image bit-identical to rendering that scene alone.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "lg_ctx.hpp"

using namespace lgd;

namespace lgh {
namespace {

constexpr uint32_t SMALL_BINS = 32768;          // up to this many bins the single-CTA tile scan is used
constexpr uint64_t RING_SEGMENTS = 256ull << 20;  // segment ring of a batch (8.5 GB with scene ids)

lg_status batch_buffers(lg_ctx* c) {
  lg_status st;
  if ((st = ensure_trace_buffers(c))) return st;
  if ((st = ensure(c, c->d_seg_scene, c->seg_cap * sizeof(uint16_t), "segment scenes"))) return st;
  const size_t elem = c->prm.accum == LG_ACCUM_F32 ? 4 : 8;
  if ((st = ensure(c, c->d_accum, c->total_px * 4 * elem, "accumulation images"))) return st;
  if ((st = ensure(c, c->d_stage, c->total_px * 8, "resolved images"))) return st;
  const size_t bins = c->total_bins;
  if ((st = ensure(c, c->d_tile_count, bins * 4, "tile counts"))) return st;
  if ((st = ensure(c, c->d_tile_off, bins * 8, "tile offsets"))) return st;
  if ((st = ensure(c, c->d_tile_cursor, bins * 8, "tile cursors"))) return st;
  if ((st = ensure(c, c->d_unit_off, bins * 8, "unit offsets"))) return st;
  if ((st = ensure(c, c->d_refs, c->refs_cap * 4, "tile refs"))) return st;
  c->units_cap = bins + c->refs_cap / MIN_UNIT_REFS + 1;
  if ((st = ensure(c, c->d_units, c->units_cap * sizeof(Unit), "raster units"))) return st;
  if ((st = ensure_cta_hist(c, bins))) return st;
  const size_t parts = (bins + TILE_SCAN_CHUNK - 1) / TILE_SCAN_CHUNK;
  if ((st = ensure(c, c->d_part, std::max<size_t>(parts, 1) * 16, "tile scan partials"))) return st;
  if ((st = ensure(c, c->d_order, c->queue_cap * 4, "scene order"))) return st;
  return LG_OK;
}

SceneDev batch_scene_dev(lg_ctx* c) {
  SceneDev S = scene_dev(c);
  S.n_obj = c->n_obj;
  S.max_bounce = c->max_bounce_all;
  S.scenes = (const SceneRec*)c->d_scenes.p;
  S.bounds = (const float4*)c->d_bounds.p;
  S.n_scenes = c->n_scenes;
  return S;
}

RasterArgs batch_raster_args(lg_ctx* c) {
  RasterArgs A = raster_args(c);
  A.seg_scene = (const uint16_t*)c->d_seg_scene.p;
  A.canvases = (const SceneCanvas*)c->d_canvases.p;
  A.n_scenes = c->n_scenes;
  A.W = (uint32_t)std::min<uint64_t>(c->total_px, 0xffffffffu);  // the clear covers all images
  A.H = 1;
  A.ntx = 0;
  A.nty = 0;
  A.n_tiles = c->total_bins;
  A.cta_hist = cta_hist_for(c, A.n_tiles);
  return A;
}

// The whole batch: clear, light setup, then per generation the trace chain followed by the
// accumulation of that generation's segments; finally the resolve of all images.
// ev: 2 * max_bounce + 2 events (start, per generation traced / accumulated, resolved).
lg_status enqueue_batch(lg_ctx* c, cudaEvent_t* ev) {
  const SceneDev S = batch_scene_dev(c);
  TraceBufs B = trace_bufs(c);
  B.seg_scene = (uint16_t*)c->d_seg_scene.p;
  B.order = (const uint32_t*)c->d_order.p;
  const RasterArgs A = batch_raster_args(c);
  const int fixed = c->prm.accum == LG_ACCUM_FIXED64;
  CK(cudaEventRecordWithFlags(ev[0], c->stream, cudaEventRecordExternal), "stage event");
  CK(cudaMemsetAsync(c->d_ctr.p, 0, sizeof(Counters), c->stream), "memset counters");
  CK(cudaMemsetAsync(c->d_scene_count.p, 0, (size_t)c->n_scenes * 4, c->stream), "memset scene counts");
  k_clear_accum<<<c->n_sm * 8, 256, 0, c->stream>>>(A, fixed);
  if (c->n_lights) launch_light_setup(c, S, true, (int)((c->n_lights + 255) / 256));
  const uint32_t bins = c->total_bins;
  const int smem_tiles = bins <= MAX_SMEM_TILES ? 1 : 0;
  const size_t bsm = smem_tiles ? (size_t)bins * 4 : 0;
  const uint32_t n_part = (bins + TILE_SCAN_CHUNK - 1) / TILE_SCAN_CHUNK;
  const int mode = raster_mode(c->prm);
  const size_t rsm = (size_t)raster_smem_bytes(mode);
  lg_string_mod no_sm;
  std::memset(&no_sm, 0, sizeof no_sm);
  for (uint32_t g = 0; g < c->max_bounce_all; ++g) {
    if (g > 0) {  // visit this generation's queue in scene order
      k_scene_hist<<<c->n_sm * 8, 256, 0, c->stream>>>(S, B, g, (unsigned*)c->d_scene_count.p);
      k_scene_offsets<<<1, 1024, 0, c->stream>>>((unsigned*)c->d_scene_count.p, (unsigned*)c->d_scene_off.p,
                                                  c->n_scenes);
      k_scene_scatter<<<c->n_sm * 8, 256, 0, c->stream>>>(S, B, g, (unsigned*)c->d_scene_off.p,
                                                          (uint32_t*)c->d_order.p);
    }
    launch_generation(c, S, B, g, true, c->batch_grid_scan, (size_t)scan_smem_bytes(scan_pairs_of(c)), 0, 0);
    if (g == 0 && c->n_cubic) {
      const int blocks = (int)std::min<uint64_t>((3ull * c->n_cubic + 255) / 256, 4096);
      k_overlay<<<blocks, 256, 0, c->stream>>>(S, B, (const uint32_t*)c->d_cubics.p,
                                               (const uint16_t*)c->d_cubic_scene.p, c->n_cubic, no_sm, ChordArgs{});
    }
    CK(cudaEventRecordWithFlags(ev[1 + 2 * g], c->stream, cudaEventRecordExternal), "stage event");
    // accumulate when the ring is full enough (every kernel below returns at once otherwise)
    k_stream_decide<<<1, 1, 0, c->stream>>>((Counters*)c->d_ctr.p, g, c->seg_cap, c->queue_cap,
                                             g + 1 == c->max_bounce_all ? 1 : 0);
    k_clear_counts<<<c->n_sm * 4, 256, 0, c->stream>>>(A);
    launch_bin_count(c, A, smem_tiles, bsm);
    if (bins <= SMALL_BINS) {
      k_scan_tiles<<<1, 1024, 0, c->stream>>>(A);
    } else {
      k_tiles_partial<<<n_part, 1024, 0, c->stream>>>(A, (unsigned long long*)c->d_part.p);
      k_tiles_scan_partials<<<1, 1024, 0, c->stream>>>(A, (unsigned long long*)c->d_part.p, n_part);
      k_tiles_apply<<<n_part, 1024, 0, c->stream>>>(A, (const unsigned long long*)c->d_part.p);
    }
    k_build_units<<<std::max(1u, (bins + 255) / 256), 256, 0, c->stream>>>(A);
    k_bin_scatter<<<scatter_grid(c->n_sm, smem_tiles), SCATTER_THREADS, bsm, c->stream>>>(A, smem_tiles);
    if (c->raster_variant == 2) {
      if (mode == RM_F32_)
        k_raster_warp<RM_F32_><<<c->raster_warp_grid, 32, raster_warp_smem_bytes(), c->stream>>>(A);
      else
        k_raster_warp<RM_FIXED_SPLIT_><<<c->raster_warp_grid, 32, raster_warp_smem_bytes(), c->stream>>>(A);
    } else if (mode == RM_FIXED_SPLIT_) {
      k_raster<RM_FIXED_SPLIT_><<<c->raster_grid, 256, rsm, c->stream>>>(A);
    } else if (mode == RM_FIXED_MINMAX_) {
      k_raster<RM_FIXED_MINMAX_><<<c->raster_grid, 256, rsm, c->stream>>>(A);
    } else {
      k_raster<RM_F32_><<<c->raster_grid, 256, rsm, c->stream>>>(A);
    }
    k_stream_rotate<<<1, 1, 0, c->stream>>>((Counters*)c->d_ctr.p, c->seg_cap);
    CK(cudaEventRecordWithFlags(ev[2 + 2 * g], c->stream, cudaEventRecordExternal), "stage event");
  }
  // all images at once: they are consecutive in both buffers
  k_resolve_f16<<<c->n_sm * 8, 256, 0, c->stream>>>(c->d_accum.p, fixed, (uint32_t)c->total_px, 1,
                                                    (uint16_t*)c->d_stage.p, c->total_px * 8);
  CK(cudaEventRecordWithFlags(ev[1 + 2 * c->max_bounce_all], c->stream, cudaEventRecordExternal), "stage event");
  CK(cudaGetLastError(), "batch launch");
  return LG_OK;
}

// true (with the capacities to grow to) if a queue, the ring or the tile lists overflowed
bool batch_overflowed(lg_ctx* c, uint64_t& need_seg, uint64_t& need_q, uint64_t& need_refs) {
  const Counters& k = *c->h_ctr;
  need_seg = k.seg_max;
  need_q = 0;
  for (int g = 0; g <= MAX_GEN; ++g) need_q = std::max<uint64_t>(need_q, k.queue_count[g]);
  need_refs = k.refs_max;
  return need_seg > c->seg_cap || need_q > c->queue_cap || need_refs > c->refs_cap;
}

lg_status run_batch(lg_ctx* c, std::vector<cudaEvent_t>& ev, uint32_t& retries) {
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (!c->graph_valid) {
      if (c->gexec) cudaGraphExecDestroy(c->gexec);
      c->gexec = nullptr;
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      lg_status s1 = enqueue_batch(c, ev.data());
      cudaError_t e = cudaMemcpyAsync(c->h_ctr, c->d_ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream);
      cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
      if (s1) { if (g) cudaGraphDestroy(g); return s1; }
      if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(c, e, "capture counters"); }
      if (e2 != cudaSuccess) return cuda_fail(c, e2, "end capture");
      e = cudaGraphInstantiate(&c->gexec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(c, e, "graph instantiate");
      c->graph_valid = true;
    }
    CK(cudaGraphLaunch(c->gexec, c->stream), "graph launch");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (c->h_ctr->error_flags & ERR_TMA_TIMEOUT)
      return fail(c, LG_ERR_TIMEOUT, "object-table bulk copy did not complete within its wait limit");
    uint64_t ns, nq, nr;
    if (!batch_overflowed(c, ns, nq, nr)) return LG_OK;
    ++retries;
    c->graph_valid = false;
    if (nq > c->queue_cap) c->queue_cap = nq + nq / 2 + 1024;
    c->seg_cap = std::max(c->seg_cap, std::max(ns, c->queue_cap + c->n_overlay));
    if (nr > c->refs_cap) c->refs_cap = nr + nr / 4 + 4096;
    if (c->refs_cap >= 0xffffffffull) return fail(c, LG_ERR_UNSUPPORTED, "more than 2^32 (segment, tile) pairs in one generation");
    lg_status st = batch_buffers(c);
    if (st) return st;
  }
  return fail(c, LG_ERR_OUT_OF_MEMORY, "batch buffers kept overflowing");
}

}  // namespace
}  // namespace lgh

extern "C" {

lg_status lg_batch_upload(lg_ctx* c, const lg_scene_desc* scenes, uint32_t k) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (!scenes || k == 0) return fail(c, LG_ERR_INVALID_ARGUMENT, "no scenes");
  if (c->serve) return fail(c, LG_ERR_INVALID_ARGUMENT, "serving in progress: lg_serve_end first");
  if (k > 65535) return fail(c, LG_ERR_INVALID_ARGUMENT, "at most 65535 scenes per batch");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const lg_params* p0 = scenes[0].params;
  if (!p0) return fail(c, LG_ERR_INVALID_ARGUMENT, "scene 0: null params");
  Flat F;
  GridTables grids;
  std::vector<SceneRec> recs(k);
  std::vector<SceneCanvas> canv(k);
  std::vector<uint64_t> px_base(k);
  std::vector<uint16_t> cubic_scene;
  uint64_t n_primary = 0, total_px = 0, total_bins = 0;
  uint32_t max_b = 0;
  for (uint32_t s = 0; s < k; ++s) {
    const lg_scene_desc& d = scenes[s];
    const std::string where = "scene " + std::to_string(s) + ": ";
    if (!d.params || (d.n_geo && !d.geos) || (d.n_objects && !d.objects) || (d.n_lights && !d.lights))
      return fail(c, LG_ERR_INVALID_ARGUMENT, where + "null pointer");
    const lg_params& p = *d.params;
    lg_status st = validate_params(c->err, p);
    if (st) { c->err = where + c->err; return st; }
    if (p.accum != p0->accum || std::memcmp(&p.color_blend, &p0->color_blend, sizeof p.color_blend) ||
        std::memcmp(&p.alpha_blend, &p0->alpha_blend, sizeof p.alpha_blend) ||
        std::memcmp(p.clear_color, p0->clear_color, sizeof p.clear_color) ||
        std::memcmp(p.blend_constant, p0->blend_constant, sizeof p.blend_constant) || p.precision != p0->precision)
      return fail(c, LG_ERR_UNSUPPORTED,
                  where + "the scenes of a batch must share accum mode, precision, blend state and clear colour");
    if (p.string_mod.modulo) return fail(c, LG_ERR_UNSUPPORTED, where + "the string-mod overlay is not supported in batches");
    if (p.ray_stride > 1) return fail(c, LG_ERR_UNSUPPORTED, where + "sampled frames (ray_stride) are one-scene only");
    if (d.n_objects > 65535) return fail(c, LG_ERR_UNSUPPORTED, where + "at most 65535 objects");
    Flat Fs;
    st = flatten_scene(c->err, d.geos, d.n_geo, d.objects, d.n_objects, d.lights, d.n_lights, Fs);
    if (!st) st = validate_exact(c->err, p, Fs);
    if (st) { c->err = where + c->err; return st; }
    const uint32_t obj0 = (uint32_t)F.scan.size(), leaf0 = (uint32_t)F.leaves.size(), prog0 = (uint32_t)F.prog.size();
    const uint32_t xnode0 = F.append_exact(Fs);
    for (ObjInfo oi : Fs.info) {
      oi.leaf_begin += leaf0;
      oi.prog_begin += prog0;
      oi.xnode_begin += xnode0;
      F.info.push_back(oi);
    }
    F.scan.insert(F.scan.end(), Fs.scan.begin(), Fs.scan.end());
    F.leaves.insert(F.leaves.end(), Fs.leaves.begin(), Fs.leaves.end());
    F.prog.insert(F.prog.end(), Fs.prog.begin(), Fs.prog.end());
    build_grid(Fs.scan, c->culling, c->grid_density, Fs.grid);
    grids.append(Fs.grid);
    if (p.emit_control_lines)
      for (uint32_t cu : Fs.cubics) {
        F.cubics.push_back(obj0 + cu);
        cubic_scene.push_back((uint16_t)s);
      }
    const uint32_t light0 = (uint32_t)F.lights.size();
    for (LightDev L : Fs.lights) {
      L.first += n_primary;
      L.scene = s;
      F.lights.push_back(L);
    }
    for (uint32_t l = 0; l < d.n_lights; ++l) n_primary += d.lights[l].num_rays;
    SceneRec& R = recs[s];
    std::memset(&R, 0, sizeof R);
    R.obj_base = obj0;
    R.n_obj = d.n_objects;
    R.aspect = DF((double)((float)p.width / (float)p.height));
    R.aspect64 = (double)((float)p.width / (float)p.height);
    for (int i = 0; i < 4; ++i) R.cutoff[i] = p.cutoff_color[i];
    R.max_bounce = p.max_bounce;
    R.light_base = light0;
    max_b = std::max(max_b, p.max_bounce);
    SceneCanvas& C = canv[s];
    C.W = p.width;
    C.H = p.height;
    C.ntx = (p.width + TILE - 1) / TILE;
    C.nty = (p.height + TILE - 1) / TILE;
    C.bin_base = total_bins;
    C.px_base = total_px;
    px_base[s] = total_px;
    total_bins += 2ull * C.ntx * C.nty;
    total_px += (uint64_t)p.width * p.height;
  }
  if (F.lights.size() > 65535) return fail(c, LG_ERR_UNSUPPORTED, "at most 65535 lights per batch");
  if (total_bins >= 0xffffffffull || total_px >= 0xffffffffull)
    return fail(c, LG_ERR_UNSUPPORTED, "more than 2^32 pixels in one batch");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  // from here on the previous scene or batch is being overwritten
  c->has_scene = false;
  c->multi = false;
  c->graph_valid = false;
  lg_status st;
  std::vector<Leaf64> dleaves;
  to_device_leaves(F.leaves, dleaves);
  auto up = [&](DevBuf& b, const void* src, size_t bytes, const char* what) -> lg_status {
    lg_status s2 = ensure(c, b, bytes + 16, what);
    if (s2) return s2;
    if (bytes) CK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c->stream), what);
    return LG_OK;
  };
  if ((st = up(c->d_scan, F.scan.data(), F.scan.size() * sizeof(ObjScan), "scene"))) return st;
  if ((st = up(c->d_info, F.info.data(), F.info.size() * sizeof(ObjInfo), "scene"))) return st;
  if ((st = up(c->d_leaves, dleaves.data(), dleaves.size() * sizeof(Leaf64), "scene"))) return st;
  if ((st = up(c->d_prog, F.prog.data(), F.prog.size(), "scene"))) return st;
  if ((st = up(c->d_lights, F.lights.data(), F.lights.size() * sizeof(LightDev), "scene"))) return st;
  if ((st = up(c->d_cubics, F.cubics.data(), F.cubics.size() * 4, "scene"))) return st;
  if ((st = upload_exact(c, F))) return st;
  if ((st = up(c->d_cubic_scene, cubic_scene.data(), cubic_scene.size() * 2, "scene"))) return st;
  if ((st = up(c->d_scenes, recs.data(), recs.size() * sizeof(SceneRec), "scene table"))) return st;
  if ((st = up(c->d_canvases, canv.data(), canv.size() * sizeof(SceneCanvas), "canvas table"))) return st;
  std::vector<float4> bounds(F.scan.size());
  for (size_t i = 0; i < F.scan.size(); ++i) std::memcpy(&bounds[i], &F.scan[i], sizeof(float4));
  if ((st = up(c->d_bounds, bounds.data(), bounds.size() * sizeof(float4), "object bounds"))) return st;
  if ((st = upload_grids(c, grids))) return st;
  c->culled = false;
  for (const GridRec& g : grids.recs) c->culled = c->culled || g.nx > 0;
  c->scan_walk = c->culled;  // scenes without a grid take the table scan inside the walking kernel
  if ((st = ensure(c, c->d_scene_count, (size_t)k * 4, "scene counts"))) return st;
  if ((st = ensure(c, c->d_scene_off, (size_t)k * 4, "scene offsets"))) return st;
  CK(cudaStreamSynchronize(c->stream), "upload");
  c->n_scenes = k;
  c->h_scenes = recs;
  c->h_canvases = canv;
  c->h_px_base = px_base;
  c->n_obj = (uint32_t)F.scan.size();
  c->n_leaves = (uint32_t)F.leaves.size();
  c->n_prog = (uint32_t)F.prog.size();
  c->n_lights = (uint32_t)F.lights.size();
  c->n_cubic = (uint32_t)F.cubics.size();
  c->n_overlay = 3ull * c->n_cubic;
  c->n_primary = n_primary;
  c->prm = *p0;
  c->prm.width = 0;
  c->prm.height = 0;
  c->prm.string_mod.modulo = 0;
  c->prm.string_mod.n_colors = 0;
  c->prm.string_mod.colors = nullptr;
  c->prm.string_mod.nested = nullptr;
  c->has_nested = false;
  c->n_cross = 0;
  c->chords_ready = 0;
  c->total_px = total_px;
  c->total_bins = (uint32_t)total_bins;
  c->max_bounce_all = max_b;
  // The ring holds at least the widest generation (one segment per ray); beyond that it is
  // sized so that several generations are accumulated in one pass (RING_SEGMENTS, or an
  // eighth of free device memory).
  const uint64_t want_q = std::max<uint64_t>(c->queue_cap_hint, n_primary + n_primary / 2 + 1024);
  c->queue_cap = std::max(c->queue_cap, want_q);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const uint64_t ring = std::min<uint64_t>(RING_SEGMENTS, free_b / 8 / (sizeof(lg_segment) + 2));
  c->seg_cap = std::max(c->seg_cap, std::max(c->queue_cap + c->n_overlay, std::max<uint64_t>(ring, c->seg_cap_hint)));
  c->refs_cap = std::max<uint64_t>(c->refs_cap, std::min<uint64_t>(4 * c->seg_cap + 4096, 0xfffffff0ull));
  if ((st = batch_buffers(c))) return st;
  // launch shapes: the multi-scene kernels read the object tables from global memory
  int occ = 0;
  c->scan_pairs = c->scan_pairs_opt;  // a new batch: its second lg_batch_render times both scan sizes
  c->scan_tune = c->scan_pairs_opt == 0;
  c->renders = 0;
  if ((st = scan_grid(c, true))) return st;
  if ((st = trace_grids(c, true, 0))) return st;
  const int mode = raster_mode(c->prm);
  const int rsm = raster_smem_bytes(mode);
  if (mode == RM_FIXED_SPLIT_) {
    CK(cudaFuncSetAttribute(k_raster<RM_FIXED_SPLIT_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm), "smem attr");
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_FIXED_SPLIT_>, 256, rsm), "occupancy");
  } else if (mode == RM_FIXED_MINMAX_) {
    CK(cudaFuncSetAttribute(k_raster<RM_FIXED_MINMAX_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm), "smem attr");
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_FIXED_MINMAX_>, 256, rsm), "occupancy");
  } else {
    CK(cudaFuncSetAttribute(k_raster<RM_F32_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm), "smem attr");
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_F32_>, 256, rsm), "occupancy");
  }
  c->raster_grid = c->n_sm * std::max(1, occ);
  CK(cudaFuncSetAttribute(k_raster_warp<RM_FIXED_SPLIT_>, cudaFuncAttributeMaxDynamicSharedMemorySize, raster_warp_smem_bytes()), "smem attr");
  CK(cudaFuncSetAttribute(k_raster_warp<RM_F32_>, cudaFuncAttributeMaxDynamicSharedMemorySize, raster_warp_smem_bytes()), "smem attr");
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster_warp<RM_FIXED_SPLIT_>, 32, raster_warp_smem_bytes()), "occupancy");
  c->raster_warp_grid = c->n_sm * std::max(1, occ);
  c->bin_grid = c->n_sm * 8;
  c->multi = true;  // the single-scene entry points need lg_scene_upload again
  return LG_OK;
}

lg_status lg_batch_image_offset(const lg_ctx* c, uint32_t scene, uint64_t* px_offset) {
  if (!c || !px_offset) return LG_ERR_INVALID_ARGUMENT;
  if (!c->multi) return LG_ERR_NO_SCENE;
  if (scene >= c->n_scenes) return LG_ERR_INVALID_ARGUMENT;
  *px_offset = c->h_px_base[scene];
  return LG_OK;
}

lg_status lg_batch_render(lg_ctx* c, uint16_t* dst, uint64_t dst_bytes, int32_t dst_is_device, lg_trace_stats* stats) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (!c->multi) return fail(c, LG_ERR_NO_SCENE, "no batch uploaded");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const uint64_t bytes = c->total_px * 8;
  if (!dst || dst_bytes < bytes) return fail(c, LG_ERR_INVALID_ARGUMENT, "destination null or smaller than 8 bytes per pixel of all scenes");
  // stage events, recorded as nodes of the captured graph: created once per context
  if (c->bev.empty()) {
    c->bev.assign(2 * MAX_GEN + 2, nullptr);
    for (auto& e : c->bev) CK(cudaEventCreate(&e), "event");
  }
  std::vector<cudaEvent_t>& ev = c->bev;
  uint32_t retries = 0;
  lg_status st;
  if (c->renders < 0xffffffffu) ++c->renders;
  if (c->scan_tune && c->renders >= 2) {
    // autotune of the scan's pair slots per lane on the batch's second render: the whole
    // batch with each size (identical images), keep the one whose generations trace faster
    c->scan_tune = false;
    float best = INFINITY;
    int pick = scan_pairs_of(c);
    for (int pairs : {8, 16}) {
      if ((st = set_scan_pairs(c, pairs, true))) return st;
      if ((st = run_batch(c, ev, retries))) return st;
      float ms = 0.f;
      for (uint32_t g = 0; g < c->max_bounce_all; ++g) ms += elapsed(g == 0 ? ev[0] : ev[2 * g], ev[1 + 2 * g]);
      if (ms < best) { best = ms; pick = pairs; }
    }
    if ((st = set_scan_pairs(c, pick, true))) return st;
  }
  if (c->raster_variant == 0) {
    // autotune: the whole batch with each tile-raster kernel (identical images), keep the faster
    float best = INFINITY;
    int pick = 1;
    for (int v = 1; v <= 2; ++v) {
      c->raster_variant = v;
      c->graph_valid = false;
      if ((st = run_batch(c, ev, retries))) { c->raster_variant = 0; return st; }
      float ms = 0.f;
      for (uint32_t g = 0; g < c->max_bounce_all; ++g) ms += elapsed(ev[1 + 2 * g], ev[2 + 2 * g]);
      if (ms < best) { best = ms; pick = v; }
    }
    if (pick != c->raster_variant) {
      c->raster_variant = pick;
      c->graph_valid = false;
      if ((st = run_batch(c, ev, retries))) return st;
    }
  } else if ((st = run_batch(c, ev, retries))) {
    return st;
  }
  CK(cudaMemcpyAsync(dst, c->d_stage.p, bytes, dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                     c->stream), "copy images");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    const Counters& k = *c->h_ctr;
    stats->primary_rays = c->n_primary;
    stats->ray_visits = k.visits;
    stats->segments = k.seg_total;
    stats->fp64_solves = k.fp64_solves;
    stats->fp64_fallbacks = k.fallbacks;
    stats->near_degenerate = k.near;
    stats->pixels = k.pixels;
    stats->tile_refs = k.refs_total;
    stats->bound_tests = k.bound_tests;
    stats->object_tests = k.object_tests;
    stats->retries = retries;
    float tr = 0.f, ac = 0.f;
    for (uint32_t g = 0; g < c->max_bounce_all; ++g) {
      tr += elapsed(g == 0 ? ev[0] : ev[2 * g], ev[1 + 2 * g]);
      ac += elapsed(ev[1 + 2 * g], ev[2 + 2 * g]);
    }
    stats->trace_ms = tr;
    stats->accumulate_ms = ac;
    stats->raster_ms = ac;
    stats->resolve_ms = elapsed(ev[2 * c->max_bounce_all], ev[1 + 2 * c->max_bounce_all]);
    stats->total_ms = elapsed(ev[0], ev[1 + 2 * c->max_bounce_all]);
  }
  return LG_OK;
}

}  // extern "C"
