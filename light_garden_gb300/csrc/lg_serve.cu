// lg_serve.cu — a render server with continuous batching (lg_serve_*).
//
// No counterpart in the reference (one interactive scene per process).  Requests are
// scenes; each lg_serve_step runs one generation of the multi-scene wavefront over every
// scene in flight, and admits waiting requests at every step: their primary rays join the
// same launch as the older scenes' deeper generations, so work from requests that arrived at
// different times overlaps on the device.  Admission is bounded by an HBM budget fixed at
// lg_serve_begin (ray queues, segment ring and a pool for the scenes' accumulation and
// result images).  A scene whose rays have all finished is accumulated, resolved to
// RGBA16F into the result pool and retired; lg_serve_poll copies the image out.  Every
// image is bit-identical to rendering the scene alone (fixed-point accumulation).
//
// The ray queue is sized from the budget; admission keeps twice the rays of a step within
// it (a ray has at most two children).  If a step still overflows the queue, every scene in
// flight is restarted from its primaries with a larger queue (results stay exact).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <unordered_map>

#include "lg_ctx.hpp"

using namespace lgd;

namespace lgh {

namespace {

// first-fit allocator over [0, capacity) in pixels
struct Pool {
  uint64_t capacity = 0;
  std::map<uint64_t, uint64_t> free_;  // offset -> size
  void reset(uint64_t cap) {
    capacity = cap;
    free_.clear();
    if (cap) free_[0] = cap;
  }
  bool alloc(uint64_t n, uint64_t& off) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      off = it->first;
      const uint64_t rest = it->second - n;
      free_.erase(it);
      if (rest) free_[off + n] = rest;
      return true;
    }
    return false;
  }
  void release(uint64_t off, uint64_t n) {
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

struct Request {
  uint64_t id = 0;
  Flat F;
  lg_params prm{};
  uint64_t primaries = 0;
  uint64_t px() const { return (uint64_t)prm.width * prm.height; }
};

struct Slot {
  bool active = false;
  Request req;
  uint64_t acc_off = 0, res_off = 0;  // pool offsets in pixels
  uint32_t obj_base = 0, light_base = 0, steps = 0;
};

struct Done {
  uint64_t res_off, px;
  uint32_t width, height;
};

}  // namespace

struct ServeState {
  uint32_t max_slots = 0;
  uint64_t budget = 0;
  lg_params common{};
  bool have_common = false;
  uint64_t next_id = 1;
  uint64_t step = 0;
  uint64_t live = 0;  // queued rays for the next step
  std::deque<Request> pending;
  std::vector<Slot> slots;
  std::unordered_map<uint64_t, Done> done;
  Pool acc_pool, res_pool;
  DevBuf d_acc, d_res, d_live;
  std::vector<unsigned> h_live;
  uint32_t restarts = 0;
};

void serve_free(lg_ctx* c) {
  if (!c || !c->serve) return;
  release(c->serve->d_acc);
  release(c->serve->d_res);
  release(c->serve->d_live);
  delete c->serve;
  c->serve = nullptr;
}

namespace {

constexpr size_t RAY_BYTES = 2 * sizeof(RayRec) + sizeof(ScanRec) + sizeof(HitRec) + 4 * N_LISTS + 4;
constexpr size_t SEG_BYTES = sizeof(lg_segment) + 2 + 4 * 4;  // + scene id + about 4 tile refs
constexpr size_t PX_BYTES = 32 + 8;                           // int64 RGBA accumulation + RGBA16F result

// Rebuild the concatenated tables of the scenes in flight: old scenes first, then the ones
// admitted now (whose lights must form one range).  Scene records are indexed by slot.
lg_status upload_tables(lg_ctx* c, ServeState& V, const std::vector<uint32_t>& admitted, uint32_t& light_lo,
                        uint32_t& light_hi, std::vector<uint32_t>& cubic_obj, std::vector<uint16_t>& cubic_slot) {
  Flat F;
  std::vector<SceneRec> recs(V.max_slots);
  std::memset(recs.data(), 0, recs.size() * sizeof(SceneRec));
  GridTables grids;  // records indexed by slot, like the scene records
  grids.recs.resize(V.max_slots);
  std::memset(grids.recs.data(), 0, grids.recs.size() * sizeof(GridRec));
  std::vector<uint32_t> order;
  for (uint32_t s = 0; s < V.max_slots; ++s)
    if (V.slots[s].active && std::find(admitted.begin(), admitted.end(), s) == admitted.end()) order.push_back(s);
  const size_t n_old = order.size();
  order.insert(order.end(), admitted.begin(), admitted.end());
  uint64_t first = 0;
  for (size_t oi = 0; oi < order.size(); ++oi) {
    const uint32_t s = order[oi];
    Slot& sl = V.slots[s];
    const Flat& Fs = sl.req.F;
    const uint32_t obj0 = (uint32_t)F.scan.size(), leaf0 = (uint32_t)F.leaves.size(), prog0 = (uint32_t)F.prog.size();
    if (oi == n_old) light_lo = (uint32_t)F.lights.size();
    const uint32_t xnode0 = F.append_exact(Fs);
    for (ObjInfo o : Fs.info) {
      o.leaf_begin += leaf0;
      o.prog_begin += prog0;
      o.xnode_begin += xnode0;
      F.info.push_back(o);
    }
    F.scan.insert(F.scan.end(), Fs.scan.begin(), Fs.scan.end());
    F.leaves.insert(F.leaves.end(), Fs.leaves.begin(), Fs.leaves.end());
    F.prog.insert(F.prog.end(), Fs.prog.begin(), Fs.prog.end());
    grids.recs[s] = grids.add(Fs.grid);
    const uint32_t light0 = (uint32_t)F.lights.size();
    for (LightDev L : Fs.lights) {
      L.scene = s;
      if (oi >= n_old) {  // new lights: primaries numbered from 0 at this step
        L.first = first;
        first += L.num_rays;
      }
      F.lights.push_back(L);
    }
    if (oi >= n_old && sl.req.prm.emit_control_lines)
      for (uint32_t cu : Fs.cubics) {
        cubic_obj.push_back(obj0 + cu);
        cubic_slot.push_back((uint16_t)s);
      }
    sl.obj_base = obj0;
    sl.light_base = light0;
    SceneRec& R = recs[s];
    R.obj_base = obj0;
    R.n_obj = (uint32_t)Fs.scan.size();
    R.aspect = DF((double)((float)sl.req.prm.width / (float)sl.req.prm.height));
    R.aspect64 = (double)((float)sl.req.prm.width / (float)sl.req.prm.height);
    for (int i = 0; i < 4; ++i) R.cutoff[i] = sl.req.prm.cutoff_color[i];
    R.max_bounce = sl.req.prm.max_bounce;
    R.light_base = light0;
  }
  if (n_old == order.size()) light_lo = (uint32_t)F.lights.size();
  light_hi = (uint32_t)F.lights.size();
  if (F.lights.size() > 0xffffffffu) return fail(c, LG_ERR_UNSUPPORTED, "too many lights in flight");
  std::vector<Leaf64> dleaves;
  to_device_leaves(F.leaves, dleaves);
  std::vector<float4> bounds(F.scan.size());
  for (size_t i = 0; i < F.scan.size(); ++i) std::memcpy(&bounds[i], &F.scan[i], sizeof(float4));
  auto up = [&](DevBuf& b, const void* src, size_t bytes, const char* what) -> lg_status {
    lg_status s2 = ensure(c, b, bytes + 16, what);
    if (s2) return s2;
    if (bytes) CK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c->stream), what);
    return LG_OK;
  };
  lg_status st;
  if ((st = up(c->d_scan, F.scan.data(), F.scan.size() * sizeof(ObjScan), "scene"))) return st;
  if ((st = up(c->d_info, F.info.data(), F.info.size() * sizeof(ObjInfo), "scene"))) return st;
  if ((st = up(c->d_leaves, dleaves.data(), dleaves.size() * sizeof(Leaf64), "scene"))) return st;
  if ((st = up(c->d_prog, F.prog.data(), F.prog.size(), "scene"))) return st;
  if ((st = up(c->d_lights, F.lights.data(), F.lights.size() * sizeof(LightDev), "scene"))) return st;
  if ((st = upload_exact(c, F))) return st;
  if ((st = up(c->d_bounds, bounds.data(), bounds.size() * sizeof(float4), "object bounds"))) return st;
  if ((st = upload_grids(c, grids))) return st;
  if ((st = up(c->d_scenes, recs.data(), recs.size() * sizeof(SceneRec), "scene table"))) return st;
  if ((st = up(c->d_cubics, cubic_obj.data(), cubic_obj.size() * 4, "scene"))) return st;
  if ((st = up(c->d_cubic_scene, cubic_slot.data(), cubic_slot.size() * 2, "scene"))) return st;
  c->n_obj = (uint32_t)F.scan.size();
  c->n_lights = (uint32_t)F.lights.size();
  // the host tables must outlive the asynchronous copies
  CK(cudaStreamSynchronize(c->stream), "upload tables");
  return LG_OK;
}

SceneDev serve_scene_dev(lg_ctx* c, ServeState& V, uint64_t n_new, uint32_t light_lo, uint32_t light_hi) {
  SceneDev S = scene_dev(c);
  S.n_obj = c->n_obj;
  S.n_lights = c->n_lights;
  S.n_primary = 0;
  S.max_bounce = MAX_GEN;
  S.record_paths = 0;
  S.scenes = (const SceneRec*)c->d_scenes.p;
  S.bounds = (const float4*)c->d_bounds.p;
  S.n_scenes = V.max_slots;
  S.serve = 1;
  S.n_new = n_new;
  S.light_lo = light_lo;
  S.light_hi = light_hi;
  return S;
}

TraceBufs serve_trace_bufs(lg_ctx* c) {
  TraceBufs B = trace_bufs(c);
  B.paths = nullptr;
  B.seg_scene = (uint16_t*)c->d_seg_scene.p;
  B.order = (const uint32_t*)c->d_order.p;
  return B;
}

// Canvases of the scenes in flight (bins numbered in slot order) and the raster arguments.
lg_status serve_raster_args(lg_ctx* c, ServeState& V, RasterArgs& A) {
  std::vector<SceneCanvas> canv(V.max_slots);
  uint64_t bins = 0;
  for (uint32_t s = 0; s < V.max_slots; ++s) {
    SceneCanvas& K = canv[s];
    std::memset(&K, 0, sizeof K);
    K.bin_base = bins;
    const Slot& sl = V.slots[s];
    if (!sl.active) continue;
    K.W = sl.req.prm.width;
    K.H = sl.req.prm.height;
    K.ntx = (K.W + TILE - 1) / TILE;
    K.nty = (K.H + TILE - 1) / TILE;
    K.px_base = sl.acc_off;
    bins += 2ull * K.ntx * K.nty;
  }
  if (bins >= 0xffffffffull) return fail(c, LG_ERR_UNSUPPORTED, "too many tiles in flight");
  c->total_bins = (uint32_t)bins;
  lg_status st;
  if ((st = ensure(c, c->d_canvases, canv.size() * sizeof(SceneCanvas), "canvas table"))) return st;
  CK(cudaMemcpyAsync(c->d_canvases.p, canv.data(), canv.size() * sizeof(SceneCanvas), cudaMemcpyHostToDevice, c->stream),
     "canvas table");
  if ((st = ensure(c, c->d_tile_count, std::max<size_t>(bins, 1) * 4, "tile counts"))) return st;
  if ((st = ensure(c, c->d_tile_off, std::max<size_t>(bins, 1) * 8, "tile offsets"))) return st;
  if ((st = ensure(c, c->d_tile_cursor, std::max<size_t>(bins, 1) * 8, "tile cursors"))) return st;
  if ((st = ensure(c, c->d_unit_off, std::max<size_t>(bins, 1) * 8, "unit offsets"))) return st;
  if ((st = ensure(c, c->d_refs, c->refs_cap * 4, "tile refs"))) return st;
  c->units_cap = bins + c->refs_cap / MIN_UNIT_REFS + 1;
  if ((st = ensure(c, c->d_units, c->units_cap * sizeof(Unit), "raster units"))) return st;
  const size_t parts = (bins + TILE_SCAN_CHUNK - 1) / TILE_SCAN_CHUNK;
  if ((st = ensure(c, c->d_part, std::max<size_t>(parts, 1) * 16, "tile scan partials"))) return st;
  c->raster_variant = 1;
  A = raster_args(c);
  A.seg_scene = (const uint16_t*)c->d_seg_scene.p;
  A.canvases = (const SceneCanvas*)c->d_canvases.p;
  A.n_scenes = V.max_slots;
  A.accum = V.d_acc.p;
  A.W = 0;
  A.H = 0;
  A.n_tiles = c->total_bins;
  A.cta_hist = nullptr;  // serving bins in global memory (its scatter counts for itself)
  // the stream-ordered canvas copy above reads the host vector: finish it here
  CK(cudaStreamSynchronize(c->stream), "canvas table");
  return LG_OK;
}

// Accumulates every segment in the ring into the scenes' images (two phases, so that a
// reference list too small for the pass is grown before anything is accumulated).
lg_status serve_raster(lg_ctx* c, ServeState& V) {
  Counters* dctr = (Counters*)c->d_ctr.p;
  for (int attempt = 0; attempt < 4; ++attempt) {
    RasterArgs A;
    lg_status st = serve_raster_args(c, V, A);
    if (st) return st;
    const uint32_t bins = c->total_bins;
    CK(cudaMemsetAsync(&dctr->skip_raster, 0, sizeof(unsigned), c->stream), "raster flag");
    k_clear_counts<<<c->n_sm * 4, 256, 0, c->stream>>>(A);
    k_bin_count<<<c->n_sm * 8, 256, 0, c->stream>>>(A, 0);
    const uint32_t n_part = (bins + TILE_SCAN_CHUNK - 1) / TILE_SCAN_CHUNK;
    if (bins) {
      k_tiles_partial<<<n_part, 1024, 0, c->stream>>>(A, (unsigned long long*)c->d_part.p);
      k_tiles_scan_partials<<<1, 1024, 0, c->stream>>>(A, (unsigned long long*)c->d_part.p, n_part);
      k_tiles_apply<<<n_part, 1024, 0, c->stream>>>(A, (const unsigned long long*)c->d_part.p);
    }
    CK(cudaGetLastError(), "bin launch");
    unsigned long long refs = 0;
    CK(cudaMemcpyAsync(&refs, &dctr->tile_refs, sizeof refs, cudaMemcpyDeviceToHost, c->stream), "read refs");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (bins && refs > c->refs_cap) {
      c->refs_cap = refs + refs / 4 + 4096;
      if (c->refs_cap >= 0xffffffffull) return fail(c, LG_ERR_UNSUPPORTED, "more than 2^32 (segment, tile) pairs in one pass");
      continue;
    }
    if (bins) {
      k_build_units<<<std::max(1u, (bins + 255) / 256), 256, 0, c->stream>>>(A);
      k_bin_scatter<<<scatter_grid(c->n_sm, 0), SCATTER_THREADS, 0, c->stream>>>(A, 0);
      k_raster<RM_FIXED_SPLIT_><<<c->raster_grid, 256, (size_t)raster_smem_bytes(RM_FIXED_SPLIT_), c->stream>>>(A);
    }
    k_stream_rotate<<<1, 1, 0, c->stream>>>(dctr, c->seg_cap);
    CK(cudaGetLastError(), "raster launch");
    return LG_OK;
  }
  return fail(c, LG_ERR_OUT_OF_MEMORY, "tile reference list kept overflowing");
}

lg_status serve_buffers(lg_ctx* c) {
  lg_status st;
  if ((st = ensure_trace_buffers(c))) return st;
  if ((st = ensure(c, c->d_seg_scene, c->seg_cap * sizeof(uint16_t), "segment scenes"))) return st;
  if ((st = ensure(c, c->d_order, c->queue_cap * 4, "scene order"))) return st;
  return LG_OK;
}

// Every scene in flight goes back to the front of the queue; the rays are dropped.
lg_status serve_restart(lg_ctx* c, ServeState& V) {
  std::vector<Request> back;
  for (Slot& sl : V.slots) {
    if (!sl.active) continue;
    V.acc_pool.release(sl.acc_off, sl.req.px());
    V.res_pool.release(sl.res_off, sl.req.px());
    back.push_back(std::move(sl.req));
    sl = Slot();
  }
  std::sort(back.begin(), back.end(), [](const Request& a, const Request& b) { return a.id < b.id; });
  for (auto it = back.rbegin(); it != back.rend(); ++it) V.pending.push_front(std::move(*it));
  V.live = 0;
  V.step = 0;
  ++V.restarts;
  CK(cudaMemsetAsync(c->d_ctr.p, 0, sizeof(Counters), c->stream), "reset counters");
  CK(cudaMemsetAsync(c->d_scene_count.p, 0, (size_t)V.max_slots * 4, c->stream), "reset scene counts");
  std::memset(c->h_ctr, 0, sizeof(Counters));
  return LG_OK;
}

}  // namespace
}  // namespace lgh

extern "C" {

lg_status lg_serve_begin(lg_ctx* c, const lg_serve_opts* opts) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (!opts || opts->max_slots == 0 || opts->max_slots > 65535)
    return fail(c, LG_ERR_INVALID_ARGUMENT, "max_slots must be 1..65535");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  serve_free(c);
  c->has_scene = false;
  c->multi = false;
  c->graph_valid = false;
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b), "memory info");
  const uint64_t budget = opts->hbm_budget_bytes ? opts->hbm_budget_bytes : (uint64_t)(free_b * 0.8);
  if (budget > free_b) return fail(c, LG_ERR_BUDGET, "HBM budget larger than the free device memory");
  ServeState* V = new (std::nothrow) ServeState();
  if (!V) return LG_ERR_OUT_OF_MEMORY;
  c->serve = V;
  c->culled = true;  // requests come and go: the scan takes each scene's grid or full scan as it finds it
  c->scan_walk = true;
  V->max_slots = opts->max_slots;
  V->budget = budget;
  V->slots.assign(V->max_slots, Slot());
  V->h_live.assign(V->max_slots, 0u);
  // budget split: 30 % ray queues, 10 % segment ring + tile lists, the rest image pools
  c->queue_cap = std::max<uint64_t>(1024, (uint64_t)(budget * 0.30) / RAY_BYTES);
  // the ring takes a whole step (at most one segment per queued ray) plus the admitted
  // scenes' control lines, which admission keeps within seg_cap - queue_cap
  c->seg_cap = std::max<uint64_t>(c->queue_cap + c->queue_cap / 4 + 4096, (uint64_t)(budget * 0.10) / SEG_BYTES);
  c->refs_cap = std::min<uint64_t>(4 * c->seg_cap, 0xfffffff0ull);
  c->prm.record_paths = 0;
  const uint64_t px = (uint64_t)(budget * 0.60) / PX_BYTES;
  V->acc_pool.reset(px);
  V->res_pool.reset(px);
  lg_status st;
  if ((st = serve_buffers(c))) { serve_free(c); return st; }
  if ((st = ensure(c, V->d_acc, px * 32, "accumulation pool"))) { serve_free(c); return st; }
  if ((st = ensure(c, V->d_res, px * 8, "result pool"))) { serve_free(c); return st; }
  if ((st = ensure(c, V->d_live, (size_t)V->max_slots * 4, "live counts"))) { serve_free(c); return st; }
  if ((st = ensure(c, c->d_scene_count, (size_t)V->max_slots * 4, "scene counts"))) { serve_free(c); return st; }
  if ((st = ensure(c, c->d_scene_off, (size_t)V->max_slots * 4, "scene offsets"))) { serve_free(c); return st; }
  CK(cudaMemsetAsync(c->d_ctr.p, 0, sizeof(Counters), c->stream), "reset counters");
  CK(cudaMemsetAsync(c->d_scene_count.p, 0, (size_t)V->max_slots * 4, c->stream), "reset scene counts");
  std::memset(c->h_ctr, 0, sizeof(Counters));
  // launch shapes of the multi-scene kernels
  int occ = 0;
  c->scan_pairs = c->scan_pairs_opt;  // served requests keep the untuned rule (or the requested size)
  c->scan_tune = false;
  if ((st = scan_grid(c, true))) { serve_free(c); return st; }
  if ((st = trace_grids(c, true, 0))) { serve_free(c); return st; }
  const int rsm = raster_smem_bytes(RM_FIXED_SPLIT_);
  CK(cudaFuncSetAttribute(k_raster<RM_FIXED_SPLIT_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm), "smem attr");
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_FIXED_SPLIT_>, 256, rsm), "occupancy");
  c->raster_grid = c->n_sm * std::max(1, occ);
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return LG_OK;
}

lg_status lg_serve_submit(lg_ctx* c, const lg_scene_desc* d, uint64_t* id_out) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (!c->serve) return fail(c, LG_ERR_NO_SCENE, "lg_serve_begin first");
  ServeState& V = *c->serve;
  if (!d || !id_out || !d->params || (d->n_geo && !d->geos) || (d->n_objects && !d->objects) ||
      (d->n_lights && !d->lights))
    return fail(c, LG_ERR_INVALID_ARGUMENT, "null pointer");
  const lg_params& p = *d->params;
  lg_status st = validate_params(c->err, p);
  if (st) return st;
  if (p.accum != LG_ACCUM_FIXED64 || raster_mode(p) != RM_FIXED_SPLIT_)
    return fail(c, LG_ERR_UNSUPPORTED, "serving accumulates in int64 fixed point with additive blends");
  if (V.have_common && (std::memcmp(&p.color_blend, &V.common.color_blend, sizeof p.color_blend) ||
                        std::memcmp(&p.alpha_blend, &V.common.alpha_blend, sizeof p.alpha_blend) ||
                        std::memcmp(p.clear_color, V.common.clear_color, sizeof p.clear_color) ||
                        std::memcmp(p.blend_constant, V.common.blend_constant, sizeof p.blend_constant) ||
                        p.precision != V.common.precision))
    return fail(c, LG_ERR_UNSUPPORTED, "all requests of a server share precision, blend state and clear colour");
  if (p.string_mod.modulo) return fail(c, LG_ERR_UNSUPPORTED, "the string-mod overlay is not served");
  if (p.ray_stride > 1) return fail(c, LG_ERR_UNSUPPORTED, "sampled frames (ray_stride) are one-scene only");
  if (d->n_objects > 65535 || d->n_lights > 65535) return fail(c, LG_ERR_UNSUPPORTED, "at most 65535 objects and lights");
  Request R;
  st = flatten_scene(c->err, d->geos, d->n_geo, d->objects, d->n_objects, d->lights, d->n_lights, R.F);
  if (!st) st = validate_exact(c->err, p, R.F);
  if (st) return st;
  build_grid(R.F.scan, c->culling, c->grid_density, R.F.grid);
  R.prm = p;
  for (uint32_t l = 0; l < d->n_lights; ++l) R.primaries += d->lights[l].num_rays;
  if (2 * R.primaries > c->queue_cap) return fail(c, LG_ERR_BUDGET, "scene has more primary rays than the budget's ray queue admits");
  if (R.px() > V.acc_pool.capacity) return fail(c, LG_ERR_BUDGET, "canvas larger than the budget's image pool");
  if (!V.have_common) {
    V.common = p;
    V.have_common = true;
    c->prm = p;  // blend state for the raster
    c->prm.string_mod.colors = nullptr;
    c->prm.string_mod.nested = nullptr;
    c->has_nested = false;
    c->n_cross = 0;
    c->chords_ready = 0;
  }
  R.id = V.next_id++;
  *id_out = R.id;
  V.pending.push_back(std::move(R));
  return LG_OK;
}

lg_status lg_serve_step(lg_ctx* c, lg_serve_step_stats* stats) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (!c->serve) return fail(c, LG_ERR_NO_SCENE, "lg_serve_begin first");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  ServeState& V = *c->serve;
  const auto t0 = std::chrono::steady_clock::now();
  lg_serve_step_stats S0;
  std::memset(&S0, 0, sizeof S0);
  // ---- admission: free slot, image pools, and room for this step's children
  std::vector<uint32_t> admitted;
  uint64_t n_new = 0;
  uint32_t free_slot = 0;
  uint64_t n_overlay = 0;
  const uint64_t overlay_room = c->seg_cap - c->queue_cap;
  while (!V.pending.empty()) {
    Request& R = V.pending.front();
    const uint64_t rays = V.live + n_new + R.primaries;
    if (2 * rays > c->queue_cap && V.live + n_new > 0) break;
    const uint64_t ov = R.prm.emit_control_lines ? 3ull * R.F.cubics.size() : 0;
    if (n_overlay + ov > overlay_room) break;
    while (free_slot < V.max_slots && V.slots[free_slot].active) ++free_slot;
    if (free_slot == V.max_slots) break;
    uint64_t acc = 0, res = 0;
    if (!V.acc_pool.alloc(R.px(), acc)) break;
    if (!V.res_pool.alloc(R.px(), res)) {
      V.acc_pool.release(acc, R.px());
      break;
    }
    Slot& sl = V.slots[free_slot];
    sl.active = true;
    sl.acc_off = acc;
    sl.res_off = res;
    sl.steps = 0;
    sl.req = std::move(R);
    V.pending.pop_front();
    admitted.push_back(free_slot);
    n_new += sl.req.primaries;
    n_overlay += ov;
  }
  uint32_t n_active = 0;
  for (const Slot& sl : V.slots) n_active += sl.active ? 1u : 0u;
  S0.admitted = (uint32_t)admitted.size();
  S0.pending = (uint32_t)V.pending.size();
  if (n_active == 0) {
    if (stats) *stats = S0;
    return LG_OK;
  }
  lg_status st;
  // the ring must take this step's segments: accumulate what it holds first if it could not
  if (c->h_ctr->seg_count && c->h_ctr->seg_count + std::min<uint64_t>(V.live + n_new, c->queue_cap) + n_overlay > c->seg_cap) {
    if ((st = serve_raster(c, V))) return st;
    c->h_ctr->seg_count = 0;
    S0.rasterised = 1;
  }
  uint32_t light_lo = 0, light_hi = 0;
  std::vector<uint32_t> cubic_obj;
  std::vector<uint16_t> cubic_slot;
  if (!admitted.empty()) {
    if ((st = upload_tables(c, V, admitted, light_lo, light_hi, cubic_obj, cubic_slot))) return st;
    // clear the new scenes' images to the clear colour
    for (uint32_t s : admitted) {
      RasterArgs A;
      std::memset(&A, 0, sizeof A);
      const Slot& sl = V.slots[s];
      A.W = (uint32_t)sl.req.px();
      A.H = 1;
      A.accum = (char*)V.d_acc.p + sl.acc_off * 32;
      for (int ch = 0; ch < 4; ++ch) A.blend.clear[ch] = V.common.clear_color[ch];
      k_clear_accum<<<c->n_sm * 4, 256, 0, c->stream>>>(A, 1);
    }
  } else {
    light_lo = light_hi = c->n_lights;
  }
  const SceneDev SD = serve_scene_dev(c, V, n_new, light_lo, light_hi);
  const TraceBufs B = serve_trace_bufs(c);
  Counters* dctr = (Counters*)c->d_ctr.p;
  const uint32_t g = (uint32_t)(V.step % MAX_GEN);
  if (g == 0 && V.step > 0)  // the previous step counted its children in the last slot
    CK(cudaMemcpyAsync(&dctr->queue_count[0], &dctr->queue_count[MAX_GEN], 8, cudaMemcpyDeviceToDevice, c->stream), "carry count");
  CK(cudaMemsetAsync(&dctr->list_count[g][0], 0, sizeof(dctr->list_count[g]), c->stream), "list counts");
  CK(cudaMemsetAsync(&dctr->queue_count[g + 1], 0, 8, c->stream), "queue count");
  if (!admitted.empty() && c->n_lights) {
    // the rebuilt light table holds every scene in flight: their start media again
    SceneDev SL = SD;
    SL.light_lo = 0;
    SL.light_hi = c->n_lights;
    launch_light_setup(c, SL, true, (int)((c->n_lights + 255) / 256));
  }
  if (V.live > 0) {  // queued rays in scene order
    k_scene_hist<<<c->n_sm * 8, 256, 0, c->stream>>>(SD, B, g, (unsigned*)c->d_scene_count.p);
    k_scene_offsets<<<1, 1024, 0, c->stream>>>((unsigned*)c->d_scene_count.p, (unsigned*)c->d_scene_off.p, V.max_slots);
    k_scene_scatter<<<c->n_sm * 8, 256, 0, c->stream>>>(SD, B, g, (unsigned*)c->d_scene_off.p, (uint32_t*)c->d_order.p);
  }
  launch_generation(c, SD, B, g, true, c->batch_grid_scan, (size_t)scan_smem_bytes(scan_pairs_of(c)), 0, 0);
  if (!cubic_obj.empty()) {
    lg_string_mod no_sm;
    std::memset(&no_sm, 0, sizeof no_sm);
    const int blocks = (int)std::min<uint64_t>((3ull * cubic_obj.size() + 255) / 256, 4096);
    k_overlay<<<blocks, 256, 0, c->stream>>>(SD, B, (const uint32_t*)c->d_cubics.p, (const uint16_t*)c->d_cubic_scene.p,
                                             (uint32_t)cubic_obj.size(), no_sm, ChordArgs{});
  }
  // rays left per scene after this step
  CK(cudaMemsetAsync(V.d_live.p, 0, (size_t)V.max_slots * 4, c->stream), "live counts");
  {
    SceneDev SN = SD;  // the children: queue entries of the next generation slot
    SN.n_new = 0;
    k_scene_hist<<<c->n_sm * 8, 256, 0, c->stream>>>(SN, B, g + 1, (unsigned*)V.d_live.p);
  }
  CK(cudaGetLastError(), "step launch");
  CK(cudaMemcpyAsync(c->h_ctr, c->d_ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "read counters");
  CK(cudaMemcpyAsync(V.h_live.data(), V.d_live.p, (size_t)V.max_slots * 4, cudaMemcpyDeviceToHost, c->stream), "read live");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  if (c->h_ctr->error_flags & ERR_TMA_TIMEOUT)
    return fail(c, LG_ERR_TIMEOUT, "object-table bulk copy did not complete within its wait limit");
  const uint64_t next = c->h_ctr->queue_count[g + 1];
  if (next > c->queue_cap || c->h_ctr->seg_count > c->seg_cap) {
    // overflow: grow within the budget and start every scene in flight again
    const uint64_t want = std::max<uint64_t>(2 * c->queue_cap, next + next / 2);
    const uint64_t images = (uint64_t)V.d_acc.bytes + V.d_res.bytes;
    if (want * RAY_BYTES + c->seg_cap * SEG_BYTES + images > V.budget + V.budget / 2)
      return fail(c, LG_ERR_BUDGET, "a step needs more ray queue than the HBM budget allows");
    c->queue_cap = want;
    c->seg_cap = std::max(c->seg_cap, c->queue_cap + c->queue_cap / 4 + 4096);
    if ((st = serve_buffers(c))) return st;
    if ((st = serve_restart(c, V))) return st;
    S0.restarted = 1;
    if (stats) *stats = S0;
    return LG_OK;
  }
  V.live = next;
  ++V.step;
  for (uint32_t s : admitted) V.slots[s].steps = 0;
  std::vector<uint32_t> finished;
  for (uint32_t s = 0; s < V.max_slots; ++s) {
    Slot& sl = V.slots[s];
    if (!sl.active) continue;
    ++sl.steps;
    if (V.h_live[s] == 0) finished.push_back(s);
  }
  // accumulate when a scene finished, the ring could not take the next step, or all is done
  const uint64_t nxt = std::min<uint64_t>(next, c->queue_cap);
  const bool raster = !finished.empty() || c->h_ctr->seg_count + nxt > c->queue_cap || next == 0;
  if (raster && c->h_ctr->seg_count > 0) {
    if ((st = serve_raster(c, V))) return st;
    c->h_ctr->seg_count = 0;
    S0.rasterised = 1;
  } else if (raster) {
    CK(cudaMemsetAsync(&dctr->seg_count, 0, 8, c->stream), "ring");
  }
  for (uint32_t s : finished) {
    Slot& sl = V.slots[s];
    k_resolve_f16<<<c->n_sm * 4, 256, 0, c->stream>>>((const char*)V.d_acc.p + sl.acc_off * 32, 1,
                                                      (uint32_t)sl.req.px(), 1,
                                                      (uint16_t*)((char*)V.d_res.p + sl.res_off * 8), sl.req.px() * 8);
    Done d;
    d.res_off = sl.res_off;
    d.px = sl.req.px();
    d.width = sl.req.prm.width;
    d.height = sl.req.prm.height;
    V.done[sl.req.id] = d;
    V.acc_pool.release(sl.acc_off, sl.req.px());
    sl = Slot();
  }
  CK(cudaGetLastError(), "resolve launch");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  S0.finished = (uint32_t)finished.size();
  S0.in_flight = n_active - (uint32_t)finished.size();
  S0.live_rays = next;
  S0.segments = c->h_ctr->seg_total;
  S0.step_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = S0;
  return LG_OK;
}

lg_status lg_serve_poll(lg_ctx* c, uint64_t id, uint16_t* dst, uint64_t dst_bytes, int32_t dst_is_device) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (!c->serve) return fail(c, LG_ERR_NO_SCENE, "lg_serve_begin first");
  ServeState& V = *c->serve;
  auto it = V.done.find(id);
  if (it == V.done.end()) {
    for (const Request& r : V.pending)
      if (r.id == id) return LG_ERR_NOT_READY;
    for (const Slot& s : V.slots)
      if (s.active && s.req.id == id) return LG_ERR_NOT_READY;
    return fail(c, LG_ERR_NOT_FOUND, "unknown request id");
  }
  const Done d = it->second;
  if (!dst || dst_bytes < d.px * 8) return fail(c, LG_ERR_INVALID_ARGUMENT, "destination null or smaller than width * height * 8");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  CK(cudaMemcpyAsync(dst, (const char*)V.d_res.p + d.res_off * 8, d.px * 8,
                     dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream), "copy image");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  V.res_pool.release(d.res_off, d.px);
  V.done.erase(it);
  return LG_OK;
}

lg_status lg_serve_end(lg_ctx* c) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (c->stream) cudaStreamSynchronize(c->stream);
  serve_free(c);
  return LG_OK;
}

}  // extern "C"
