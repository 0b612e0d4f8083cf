// lg_trace.cu — ray generation and the per-generation trace kernels (sm_103a).
//
// Tracer::trace (src/light_garden/tracer.rs:360-493) walks a breadth-first ray tree per
// primary ray.  Here each generation of all trees of all lights is one device queue (a
// wavefront), processed by a short chain of kernels so that warps stay full no matter how
// the trees branch:
//   gen 0 reads a virtual queue (light, ray index) and generates the primary ray
//   (light.rs:103-115, 163-174, 225-249); gen g > 0 reads the queue written by gen g-1.
//   For each ray: cutoff (tracer.rs:378-384), nearest hit (412-424), medium (428-442),
//   refract / reflect with colour split (444-481) or canvas exit (482-488).
//   Segments are appended to the segment ring and children to the next queue with one
//   atomic per warp (ballot + popc compaction).
// The chain per generation (k_scan, k_refine over 4 leaf-kind lists, k_full, k_bounce) is
// described above k_scan below.
#include "lg_kernels.cuh"
#include "lg_trace_common.cuh"

namespace lgd {

// ------------------------------------------------------------- bulk copy to shared memory
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  unsigned ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(d),
      "l"(src), "r"(bytes), "r"(b)
      : "memory");
}

// Stages the ObjScan table into shared memory.  Returns the table to scan: shared memory
// on success, the global table if it does not fit or the bounded wait expired (in which
// case ERR_TMA_TIMEOUT is raised and the caller returns).
__device__ const ObjScan* stage_objects(const SceneDev& S, ObjScan* sobj, uint64_t* bar, bool fits,
                                        Counters* ctr, bool& failed) {
  failed = false;
  if (!fits || S.n_obj == 0) return S.scan;
  const unsigned bytes = S.n_obj * (unsigned)sizeof(ObjScan);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_expect_tx(bar, bytes);
    const unsigned chunk = 32768u;
    for (unsigned off = 0; off < bytes; off += chunk) {
      const unsigned n = bytes - off < chunk ? bytes - off : chunk;
      bulk_g2s(reinterpret_cast<char*>(sobj) + off, reinterpret_cast<const char*>(S.scan) + off, n, bar);
    }
  }
  __syncthreads();  // barrier initialised before anyone waits on it
  bool done = false;
  const int polls = S.wait_polls;
  for (int it = 0; it < polls && !done; ++it) {
    done = mbar_try_wait(bar, 0);
    if (!done && it > 64) __nanosleep(64);
  }
  if (!done) {
    atomicOr(&ctr->error_flags, ERR_TMA_TIMEOUT);
    // give the copy a last bounded chance to land before this CTA's shared memory is released
    for (int it = 0; it < (1 << 20) && !mbar_try_wait(bar, 0); ++it) __nanosleep(256);
    failed = true;
  }
  __syncthreads();
  return sobj;
}

// ------------------------------------------------------------------- primary rays
// native FP64 (only here): the reference's f64 sin_cos / atan per primary ray
__device__ inline void primary_ray(const LightDev& L, uint64_t i, double& ox, double& oy, double& dx, double& dy) {
  const double n = (double)L.num_rays;
  if (L.kind == LG_LIGHT_POINT) {  // light.rs:168-172
    const double f = (double)i * 3.141592653589793 * 2.0 / n;
    double s, c;
    sincos(f, &s, &c);
    ox = L.ox; oy = L.oy; dx = c; dy = s;
  } else if (L.kind == LG_LIGHT_SPOT) {  // light.rs:230-247
    const double sx = L.vx, sy = L.vy;
    const double dir_angle =
        fabs(sx) < SPOT_EPSILON ? (sy >= 0.0 ? 3.141592653589793 * 0.5 : -3.141592653589793 * 0.5) : atan(sy / sx);
    const double min_angle = dir_angle - 0.5 * L.spot_angle;
    const double ang = min_angle + ((double)(i + 1) / n) * L.spot_angle;
    double s, c;
    sincos(ang, &s, &c);
    const double sign = signbit(sx) ? -1.0 : 1.0;
    ox = L.ox; oy = L.oy; dx = sign * c; dy = sign * s;
  } else {  // directional: origins along a -> b, unit left normal
    const double ex = L.vx - L.ox, ey = L.vy - L.oy;
    const double r = (double)i / n;
    ox = L.ox + ex * r;
    oy = L.oy + ey * r;
    const double l = sqrt(ey * ey + ex * ex);
    dx = l > 0.0 ? -ey / l : -ey;
    dy = l > 0.0 ? ex / l : ex;
  }
}

template <bool MULTI>
__global__ void k_light_setup(SceneDev S) {
  const uint32_t l0 = S.serve ? S.light_lo : 0u, l1 = S.serve ? S.light_hi : S.n_lights;
  for (uint32_t l = l0 + blockIdx.x * blockDim.x + threadIdx.x; l < l1; l += gridDim.x * blockDim.x) {
    LightDev& L = S.lights[l];
    const SceneLoc sl = scene_of<MULTI>(S, L.scene);
    df n = DF_ONE;  // tracer.rs:280-287: the last containing object wins
    const df px = df_from_double(L.ox), py = df_from_double(L.oy);
    for (uint32_t k = sl.base; k < sl.base + sl.n; ++k) {
      bool near = false;
      if ((S.info[k].flags & INFO_MATERIAL) && obj_contains64(S, k, px, py, near, 0.0f)) n = S.info[k].n;
    }
    L.n0 = n;
  }
}
template __global__ void k_light_setup<false>(SceneDev);
template __global__ void k_light_setup<true>(SceneDev);

// ------------------------------------------------------------------- one generation
// Each generation runs as four kernels over the generation's queue (a wavefront), so that
// every kernel executes one compact code path on coherent work:
//   k_scan     FP32: nearest-hit search bound and candidate list per ray; sorts the rays
//              into work lists (refine circle / rect / segment, full solve)
//   k_refine   double-float refinement of a winner the FP32 scan proved (the leaf-kind
//              lists one after the other)
//   k_full     double-float solve of every candidate (near ties, uncertain roots, cubic
//              and deep CSG objects), grouped by solve class
//   k_bounce   medium (tracer.rs:428-442), refract / reflect with colour split
//              (444-481) or canvas exit (482-488); appends segments and children
__device__ __forceinline__ int leaf_kind_of(uint32_t info, int leaf) {
  return (int)(leaf == 0 ? info_leaf_a(info) : info_leaf_b(info));
}

// appends idx to work list `list` (-1: none) with one atomic per (warp, list)
__device__ __forceinline__ void list_append(const TraceBufs& B, uint32_t gen, int list, uint32_t idx) {
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, list);
  if (list < 0) return;
  const int leader = __ffs(grp) - 1;
  unsigned long long base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(&B.ctr->list_count[gen][list], (unsigned long long)__popc(grp));
  base = __shfl_sync(grp, base, leader);
  const unsigned long long slot = base + __popc(grp & lanemask_lt());
  if (slot < B.queue_cap) B.list[list][slot] = idx;
}

// Canvas exit of a ray that hits no object, when its origin is clearly inside the canvas
// and the exit is clearly not at a corner: the exit face is found in FP32, the exit point
// computed in double-float.  Anything else takes the precise path in k_bounce.
__device__ __forceinline__ bool fast_canvas_exit(const df aspect, const RayRec& r, float& x1, float& y1, float& L) {
  const float ax = aspect.hi, ox = r.ox.hi, oy = r.oy.hi, dx = r.dx.hi, dy = r.dy.hi;
  if (!(fabsf(ox) < ax - 1e-4f && fabsf(oy) < 1.0f - 1e-4f)) return false;
  const float tx = dx > 0.0f ? (ax - ox) / dx : dx < 0.0f ? (-ax - ox) / dx : INFINITY;
  const float ty = dy > 0.0f ? (1.0f - oy) / dy : dy < 0.0f ? (-1.0f - oy) / dy : INFINITY;
  if (!(fabsf(tx - ty) > 1e-4f * (fminf(tx, ty) + 1.0f))) return false;
  df t;
  if (tx < ty) {
    const df bound = dx > 0.0f ? aspect : -aspect;
    t = (bound - r.ox) / r.dx;
  } else {
    const df bound = dy > 0.0f ? DF_ONE : -DF_ONE;
    t = (bound - r.oy) / r.dy;
  }
  x1 = (r.ox + r.dx * t).hi;
  y1 = (r.oy + r.dy * t).hi;
  L = r.ex + t.hi * r.ea;
  return true;
}

// appends one segment per emitting lane with one atomic per warp (all lanes call)
__device__ __forceinline__ void emit_segments(const SceneDev& S, const TraceBufs& B, bool emit, const RayRec& r,
                                              float x1, float y1, uint8_t flags, int hit,
                                              unsigned long long& my_near, unsigned long long& my_ill) {
  const unsigned lane = lane_id();
  const unsigned emask = __ballot_sync(0xffffffffu, emit);
  if (!emask) return;
  unsigned long long sbase = 0;
  const int leader = __ffs(emask) - 1;
  if ((int)lane == leader) sbase = atomicAdd(&B.ctr->seg_count, (unsigned long long)__popc(emask));
  sbase = __shfl_sync(0xffffffffu, sbase, leader);
  if (!emit) return;
  const unsigned long long slot = sbase + __popc(emask & lanemask_lt());
  if (flags & LG_PATH_NEAR_DEGENERATE) ++my_near;
  if (flags & LG_PATH_ILL_CONDITIONED) ++my_ill;
  if (slot >= B.seg_cap) return;
  float4* dst = reinterpret_cast<float4*>(B.segs + slot);
  dst[0] = make_float4(r.ox.hi, r.oy.hi, x1, y1);
  dst[1] = make_float4(r.c[0], r.c[1], r.c[2], r.c[3]);
  if (B.seg_scene) B.seg_scene[slot] = r.scene;
  if (S.record_paths) {
    lg_path_record pr;
    pr.path = r.path; pr.primary = r.prim; pr.light = r.light; pr.gen = r.gen;
    pr.flags = flags; pr.hit = hit; pr.source = LG_SRC_TRACE;
    B.paths[slot] = pr;
  }
}

// Warp-cooperative FP32 scan.  Every lane bounding-tests its own ray against a run of
// objects (pruned by its running bound thr) and writes the passing (ray, object) pairs to
// the warp's shared buffer; then all 32 lanes classify the warp's pairs side by side, so
// the exact FP32 tests run at full SIMD width instead of only in the lanes whose ray
// happens to cross a given object.  Each lane then folds its own results: thr shrinks
// with every certain hit and the candidates (key <= thr) go to the precise solve, which
// applies the first-in-object-order tie rule of tracer.rs:404,417 itself.  The runs are
// either the object table in chunks of SCAN_CHUNK, or (culling grid) the objects listed
// in the grid cells the lane's ray crosses, nearest cell first.
// Launch shape.  The pair slots per lane between classifications (CHUNK, 8 or 16) are a
// template parameter that each context tunes on its first frame (lg_device_opts.scan_pairs):
// the culled walk tends to do best with 8 (a smaller shared-memory buffer leaves more of the
// SM's L1 to the grid and queue loads), the table scan with 16 (CSG frame: 8 slots 1217 ms of
// scan, 16 slots 1469; mid frame: 16 slots 68 ms, 8 slots 73).  CTAs per SM of the culled scan
// and its walk steps between classifications are build-time (-DLG_SCAN_CULL_BLOCKS=...,
// -DLG_SCAN_WALK_STEPS=..., for sweeps).
#ifndef LG_SCAN_CULL_BLOCKS
#define LG_SCAN_CULL_BLOCKS 4
#endif
#ifndef LG_SCAN_WALK_STEPS
#define LG_SCAN_WALK_STEPS 32
#endif
constexpr int SCAN_WARPS = 4;
constexpr int WALK_STEPS = LG_SCAN_WALK_STEPS;  // culled scan: cell steps and object tests between classifications
constexpr int SCAN_CULL_BLOCKS = LG_SCAN_CULL_BLOCKS;  // culled scan: CTAs per SM the registers are sized for

struct __align__(16) PairSlot {
  float key, ub, s;
  uint32_t m;  // object | (leaf + 1) << 16 | (face + 1) << 24; before classification key holds lb
};

template <int CHUNK>
struct ScanSmemT {  // [slot][lane]: a warp's 32 lanes touch 32 consecutive slots
  PairSlot pairs[SCAN_WARPS][CHUNK][32];
  PairSlot cand[SCAN_WARPS][CAND][32];
  float4 ray[SCAN_WARPS][32];
  uint32_t src[SCAN_WARPS][32];
  uint32_t base[SCAN_WARPS][32];
  int off[SCAN_WARPS][33];
};

int scan_smem_bytes(int pairs) { return pairs <= 8 ? (int)sizeof(ScanSmemT<8>) : (int)sizeof(ScanSmemT<16>); }

template <bool MULTI, bool CULL, bool EXACT, int CHUNK>
__global__ void __launch_bounds__(SCAN_WARPS * 32, CULL ? SCAN_CULL_BLOCKS : 4)
    k_scan(SceneDev S, TraceBufs B, uint32_t gen, int smem_fits) {
  constexpr int SCAN_CHUNK = CHUNK;
  using ScanSmem = ScanSmemT<SCAN_CHUNK>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  ScanSmem& W = *reinterpret_cast<ScanSmem*>(smem_raw);
  ObjScan* sobj = reinterpret_cast<ObjScan*>(smem_raw + sizeof(ScanSmem));
  __shared__ unsigned long long blk_visits, blk_near, blk_ill, blk_tests, blk_cls;
  if (threadIdx.x == 0) { blk_visits = 0; blk_near = 0; blk_ill = 0; blk_tests = 0; blk_cls = 0; }
  unsigned long long my_visits = 0, my_near = 0, my_ill = 0;
  uint32_t my_tests = 0;
  bool failed;
  const ObjScan* objs = stage_objects(S, sobj, &bar, !MULTI && smem_fits != 0, B.ctr, failed);
  if (failed) return;
  const uint64_t n_real = n_real_of(S, B, gen);
  const uint64_t n_in = n_in_of(S, B, gen);
  RayRec* q = B.queue[gen & 1];
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t base = warp * 32; base < n_in; base += nwarps * 32) {
    // multi-scene launches visit the queued rays in scene order, so that a warp's rays (and
    // a CTA's warps) share one scene; new primaries follow, ordered by light
    uint64_t idx = base + lane;
    bool valid = idx < n_in;
    if (MULTI && valid && idx < n_real) {
      idx = B.order[idx];
      valid = idx < n_real;
    }
    bool live = valid;
    RayRec r;
    if (live) {
      if (idx >= n_real) {
        const uint64_t v = idx - n_real;  // primary number among this launch's new lights
        uint32_t l = S.serve ? S.light_lo : 0u, lhi = S.serve ? S.light_hi : S.n_lights;
        while (lhi - l > 1) {  // the last light whose first primary is <= v
          const uint32_t mid = (l + lhi) >> 1;
          if (S.lights[mid].first <= v) l = mid; else lhi = mid;
        }
        const LightDev& L = S.lights[l];
        const uint64_t i = S.ray_offset + (uint64_t)S.ray_stride * (v - L.first);
        double pox, poy, pdx, pdy;
        if (EXACT) {  // exact mode: the FP64 coordinates themselves, in the df slots
          lgx::primary_ray_x(L.kind, L.ox, L.oy, L.vx, L.vy, L.spot_angle, L.dir_angle, (double)L.num_rays, i, pox,
                             poy, pdx, pdy);
          r.ox = xdf(pox); r.oy = xdf(poy); r.dx = xdf(pdx); r.dy = xdf(pdy);
        } else {
          primary_ray(L, i, pox, poy, pdx, pdy);
          r.ox = df_from_double(pox); r.oy = df_from_double(poy);
          r.dx = df_from_double(pdx); r.dy = df_from_double(pdy);
        }
        r.medium = MEDIUM_LIGHT;
        r.src_obj = SRC_NONE;
        r.src_leaf = 0;
        r.c[0] = L.color[0]; r.c[1] = L.color[1]; r.c[2] = L.color[2]; r.c[3] = L.color[3];
        r.path = 0;
        r.prim = (uint32_t)i;
        r.light = (uint16_t)(MULTI ? l - S.scenes[L.scene].light_base : l);
        r.gen = 0;
        r.flags = 0;
        r._pad = 0;
        r.scene = MULTI ? (uint16_t)L.scene : (uint16_t)0;
        // rounding of the light's ray generator (sin/cos/atan) and the double-float split
        r.ex = EXACT ? 0.0f : DF_ROUND * (1.0f + fabsf(r.ox.hi) + fabsf(r.oy.hi));
        r.ea = EXACT ? 0.0f : DF_ROUND;
        if (idx < B.queue_cap) q[idx] = r;
      } else {
        r = q[idx];
      }
    }
    const SceneLoc sl = scene_of<MULTI>(S, live ? r.scene : 0u);
    const bool dead = live && below_cutoff(r.c, sl.cutoff);
    live = live && !dead;
    const float ox = EXACT ? (float)xd(r.ox) : r.ox.hi, oy = EXACT ? (float)xd(r.oy) : r.oy.hi;
    const float dx = EXACT ? (float)xd(r.dx) : r.dx.hi, dy = EXACT ? (float)xd(r.dy) : r.dy.hi;
    W.ray[w][lane] = make_float4(ox, oy, dx, dy);
    W.src[w][lane] = live ? ((uint32_t)r.src_obj << 8 | r.src_leaf) : 0xffffffffu;
    W.base[w][lane] = sl.base;
    float thr = INFINITY;
    int nc = 0;
    bool overflow = false;
    // The warp scans one scene at a time: a multi-scene warp (rays of several scenes, at
    // the seams of the queue) runs one pass per distinct scene with that scene's lanes;
    // a single-scene warp runs exactly one pass.
    const unsigned live_mask = __ballot_sync(0xffffffffu, live);
    const uint32_t my_scene = live ? (uint32_t)r.scene : 0xffffffffu;
    unsigned pending = MULTI ? live_mask : (live_mask ? 1u : 0u);
    while (pending) {
      bool mine;
      uint32_t g_lo, g_hi, pass_scene = 0;
      if (MULTI) {
        const int leader = __ffs(pending) - 1;
        pass_scene = __shfl_sync(0xffffffffu, my_scene, leader);
        const unsigned grp = __ballot_sync(0xffffffffu, my_scene == pass_scene);
        pending &= ~grp;
        mine = (grp >> lane) & 1u;
        g_lo = __shfl_sync(0xffffffffu, sl.base, leader);
        g_hi = g_lo + __shfl_sync(0xffffffffu, sl.n, leader);
      } else {
        pending = 0;
        mine = live;
        g_lo = 0;
        g_hi = S.n_obj;
      }
      // Classifies the warp's cnt-per-lane pairs side by side, then folds each lane's own
      // results: thr shrinks with every certain hit, candidates (key <= thr) are kept.
      auto classify_fold = [&](int cnt) {
        // flatten the warp's pairs: exclusive scan of the per-lane counts
        int incl = cnt;
  #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if ((int)lane >= o) incl += y;
        }
        W.off[w][lane] = incl - cnt;
        if (lane == 31) {
          W.off[w][32] = incl;
          if (incl) atomicAdd(&blk_cls, (unsigned long long)incl);
        }
        __syncwarp();
        const int total = W.off[w][32];
        for (int p = (int)lane; p < total; p += 32) {
          int lo = 0, hi = 32;  // owner: the last lane whose offset is <= p
          while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (W.off[w][mid] <= p) lo = mid; else hi = mid;
          }
          const int k = p - W.off[w][lo];
          PairSlot& ps = W.pairs[w][k][lo];
          const uint32_t j = ps.m;
          const float4 rr = W.ray[w][lo];
          const uint32_t src = W.src[w][lo];
          const Class32 c = classify32(objs[W.base[w][lo] + j], rr.x, rr.y, rr.z, rr.w, ps.key,
                                       (src >> 8) == j ? (int)(src & 0xffu) : -1);
          PairSlot o;
          o.key = c.key;
          o.ub = c.ub;
          o.s = c.s;
          o.m = j | ((uint32_t)(c.leaf + 1) << 16) | ((uint32_t)(c.face + 1) << 24);
          ps = o;
        }
        __syncwarp();
        for (int k = 0; k < cnt; ++k) {
          const PairSlot ps = W.pairs[w][k][lane];
          if (ps.ub < INFINITY) thr = fminf(thr, ps.ub * (1.0f + 1e-4f) + 1e-4f);
          if (!(ps.key <= thr)) continue;
          if (nc == CAND) {  // full: drop candidates the bound has since excluded
            int wr = 0;
            for (int q2 = 0; q2 < CAND; ++q2)
              if (W.cand[w][q2][lane].key <= thr) W.cand[w][wr++][lane] = W.cand[w][q2][lane];
            nc = wr;
          }
          if (nc < CAND) W.cand[w][nc++][lane] = ps;
          else overflow = true;
        }
        __syncwarp();
      };
      const GridRec& G = grid_of<MULTI>(S, pass_scene);
      const uint32_t gnx = CULL ? G.nx : 0u;
      if (gnx == 0) {
        // every object in table order
        for (uint32_t j0 = g_lo; j0 < g_hi; j0 += SCAN_CHUNK) {
          const uint32_t jn = min((uint32_t)SCAN_CHUNK, g_hi - j0);
          int cnt = 0;
          if (mine) my_tests += jn;
          for (uint32_t jj = 0; jj < jn; ++jj) {
            const uint32_t j = j0 + jj;
            const float4 h = MULTI ? __ldg(&S.bounds[j]) : *reinterpret_cast<const float4*>(&objs[j]);
            float lb;
            if (mine && bound_test(h, ox, oy, dx, dy, thr, lb)) {
              PairSlot ps;
              ps.key = lb;
              ps.ub = 0.0f;
              ps.s = 0.0f;
              ps.m = j - g_lo;  // scene-local object index
              W.pairs[w][cnt++][lane] = ps;
            }
          }
          classify_fold(cnt);
        }
      } else {
        // Culled: every lane walks the cells its own ray crosses, nearest first, and stops
        // at the first cell entered beyond its bound thr.  The walk moves one cell in x or
        // in y at a time, so the cells of an object's range that it visits are consecutive:
        // an object whose range holds the previous cell was tested there and is skipped,
        // and each object is tested at most once per ray.  Only the range's edge on the
        // side the walk came from needs checking (step in +x: does it start left of ix?).
        const uint32_t gny = G.ny;
        const float gx0 = G.x0, gy0 = G.y0, cw = G.cw, ch = G.ch, margin = G.margin;
        const uint32_t* cstart = S.cell_start + G.cell_base;
        const uint16_t* cobj = S.cell_obj + G.list_base;
        const float idx = fabsf(dx) > 1e-30f ? 1.0f / dx : 0.0f;
        const float idy = fabsf(dy) > 1e-30f ? 1.0f / dy : 0.0f;
        const int sx = dx > 0.0f ? 1 : -1, sy = dy > 0.0f ? 1 : -1;
        int ix = 0, iy = 0;
        int came = 0;  // 0: first cell; 1: entered by an x step; 2: by a y step
        float tx = INFINITY, ty = INFINITY;
        uint32_t p = 0, pe = 0, steps = 0;
        bool act = mine, linear = false;
        if (act) {
          if (!(fabsf(ox) + fabsf(oy) <= G.reach)) {
            // an origin this far out carries FP32 errors above the margin: every object
            linear = true;
            pe = g_hi - g_lo;
          } else {
            const float bx1 = gx0 + (float)gnx * cw, by1 = gy0 + (float)gny * ch;
            float t0 = 0.0f, t1 = INFINITY;
            if (idx != 0.0f) {
              const float a = (gx0 - ox) * idx, b = (bx1 - ox) * idx;
              t0 = fmaxf(t0, fminf(a, b));
              t1 = fminf(t1, fmaxf(a, b));
            } else if (!(ox >= gx0 && ox <= bx1)) {
              t1 = -1.0f;
            }
            if (idy != 0.0f) {
              const float a = (gy0 - oy) * idy, b = (by1 - oy) * idy;
              t0 = fmaxf(t0, fminf(a, b));
              t1 = fminf(t1, fmaxf(a, b));
            } else if (!(oy >= gy0 && oy <= by1)) {
              t1 = -1.0f;
            }
            act = t0 <= t1 && t0 <= thr + margin;
            if (act) {
              const float fx = fminf(fmaxf(floorf((ox + dx * t0 - gx0) * G.iw), 0.0f), (float)(gnx - 1));
              const float fy = fminf(fmaxf(floorf((oy + dy * t0 - gy0) * G.ih), 0.0f), (float)(gny - 1));
              ix = (int)fx;
              iy = (int)fy;
              tx = idx != 0.0f ? (gx0 + (float)(ix + (dx > 0.0f ? 1 : 0)) * cw - ox) * idx : INFINITY;
              ty = idy != 0.0f ? (gy0 + (float)(iy + (dy > 0.0f ? 1 : 0)) * ch - oy) * idy : INFINITY;
              const uint32_t c = (uint32_t)iy * gnx + (uint32_t)ix;
              p = __ldg(cstart + c);
              pe = __ldg(cstart + c + 1);
            }
          }
        }
        // tests object j (scene-local) with bound h, unless met in the previous cell
        auto test = [&](uint32_t j, const float4& h, int& cnt) {
          if (came == 1) {
            if (sx > 0 ? cell_lo(h.x, h.z, margin, gx0, G.iw) < (float)ix : cell_hi(h.x, h.z, margin, gx0, G.iw) > (float)ix)
              return;
          } else if (came == 2) {
            if (sy > 0 ? cell_lo(h.y, h.z, margin, gy0, G.ih) < (float)iy : cell_hi(h.y, h.z, margin, gy0, G.ih) > (float)iy)
              return;
          }
          ++my_tests;
          float lb;
          if (bound_test(h, ox, oy, dx, dy, thr, lb)) {
            PairSlot ps;
            ps.key = lb;
            ps.ub = 0.0f;
            ps.s = 0.0f;
            ps.m = j;
            W.pairs[w][cnt++][lane] = ps;
          }
        };
        while (__any_sync(0xffffffffu, act)) {
          int cnt = 0;
          bool yield = false;  // a lane that finished a cell with pairs waits for the fold
          for (int st = 0; st < WALK_STEPS; ++st) {
            const bool can = act && !yield && cnt + 2 <= SCAN_CHUNK;
            if (!__any_sync(0xffffffffu, can)) break;
            if (!can) continue;
            if (p < pe) {
              // two objects of the cell per step: their loads overlap
              const bool two = p + 1 < pe;
              const uint32_t j0 = linear ? p : (uint32_t)__ldg(cobj + p);
              const uint32_t j1 = two ? (linear ? p + 1 : (uint32_t)__ldg(cobj + p + 1)) : j0;
              p += two ? 2u : 1u;
              const float4 h0 = MULTI ? __ldg(&S.bounds[g_lo + j0]) : *reinterpret_cast<const float4*>(&objs[j0]);
              const float4 h1 = MULTI ? __ldg(&S.bounds[g_lo + j1]) : *reinterpret_cast<const float4*>(&objs[j1]);
              test(j0, h0, cnt);
              if (two) test(j1, h1, cnt);
            } else if (cnt > 0 && !linear) {
              // fold before the next cell: a hit in this one may end the walk here
              yield = true;
            } else if (linear || ++steps > gnx + gny + 2) {
              act = false;
            } else {  // the next cell along the ray
              float te;
              if (tx <= ty) {
                ix += sx;
                te = tx;
                tx = (gx0 + (float)(ix + (sx > 0 ? 1 : 0)) * cw - ox) * idx;
                came = 1;
              } else {
                iy += sy;
                te = ty;
                ty = (gy0 + (float)(iy + (sy > 0 ? 1 : 0)) * ch - oy) * idy;
                came = 2;
              }
              if (ix < 0 || iy < 0 || ix >= (int)gnx || iy >= (int)gny || !(te <= thr + margin) || te == INFINITY) {
                act = false;
              } else {
                const uint32_t c = (uint32_t)iy * gnx + (uint32_t)ix;
                p = __ldg(cstart + c);
                pe = __ldg(cstart + c + 1);
              }
            }
          }
          classify_fold(cnt);
        }
      }
    }
    // the ray record again (primaries were stored above): the scan does not keep it live
    if (valid) r = q[idx];
    const SceneLoc slp = scene_of<MULTI>(S, valid ? r.scene : 0u);
    bool emit = false;
    float x1 = 0.0f, y1 = 0.0f;
    uint8_t eflags = 0;
    if (valid) {
      ScanRec sc;
      sc.nc = 0;
      sc.overflow = overflow ? 1 : 0;
      sc.leaf = -1;
      sc.face = -1;
      sc.t32 = 0.0f;
      sc.s32 = 0.0f;
      sc.thr = thr;
      int list = -1;
      if (dead) {
        sc.nc = NC_DEAD;
      } else {
        int m = 0;
        PairSlot first;
        first.key = INFINITY;
        for (int k = 0; k < nc; ++k) {
          const PairSlot ps = W.cand[w][k][lane];
          if (!(ps.key <= thr)) continue;
          if (m == 0) first = ps;
          sc.cand[m++] = (uint16_t)(ps.m & 0xffffu);
        }
        sc.nc = (uint8_t)m;
        const int leaf = (int)((first.m >> 16) & 0xffu) - 1, face = (int)(first.m >> 24) - 1;
        if (!overflow && m == 1 && first.key == first.ub && leaf >= 0) {
          // a single candidate whose nearest root is certain: only that root is refined
          const uint32_t oinfo = reinterpret_cast<const uint32_t*>(&objs[slp.base + sc.cand[0]])[3];
          const int kind = leaf_kind_of(oinfo, leaf);
          sc.leaf = (int8_t)leaf;
          sc.face = (int8_t)face;
          sc.t32 = first.ub;
          sc.s32 = first.s;
          list = kind == LEAF_CIRCLE ? LIST_REFINE_CIRCLE : kind == LEAF_RECT ? LIST_REFINE_RECT
               : kind == LEAF_SEGMENT ? LIST_REFINE_SEGMENT : LIST_REFINE_CUBIC;
        } else if (m > 0 || overflow) {
          list = LIST_FULL;
        } else {
          // no object can be hit: leave through the canvas (tracer.rs:482-488)
          float L;
          if (!EXACT && fast_canvas_exit(slp.aspect, r, x1, y1, L)) {
            emit = true;
            ++my_visits;
            eflags = r.flags | (near_cutoff(r.c, slp.cutoff) ? LG_PATH_NEAR_DEGENERATE : 0) |
                     (L > ILL_COND ? LG_PATH_ILL_CONDITIONED : 0);
          } else {
            list = LIST_EXIT;
          }
        }
      }
      B.scan[idx] = sc;
      list_append(B, gen, list, (uint32_t)idx);
    }
    emit_segments(S, B, emit, r, x1, y1, eflags, -1, my_near, my_ill);
  }
  atomicAdd(&blk_visits, my_visits);
  atomicAdd(&blk_near, my_near);
  atomicAdd(&blk_ill, my_ill);
  atomicAdd(&blk_tests, (unsigned long long)my_tests);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&B.ctr->visits, blk_visits);
    atomicAdd(&B.ctr->near, blk_near);
    atomicAdd(&B.ctr->ill, blk_ill);
    atomicAdd(&B.ctr->bound_tests, blk_tests);
    atomicAdd(&B.ctr->object_tests, blk_cls);
  }
}

template __global__ void k_scan<false, false, false, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<false, false, true, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<false, true, false, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<false, true, true, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, false, false, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, false, true, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, true, false, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, true, true, 8>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<false, false, false, 16>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<false, false, true, 16>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<false, true, false, 16>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<false, true, true, 16>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, false, false, 16>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, false, true, 16>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, true, false, 16>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_scan<true, true, true, 16>(SceneDev, TraceBufs, uint32_t, int);

__device__ __forceinline__ void store_hit(HitRec& o, int obj, const Hit64& h, float ev, uint8_t flags) {
  o.obj = obj < 0 ? HIT_NONE : (uint16_t)obj;
  o.t = h.t; o.px = h.px; o.py = h.py; o.nx = h.nx; o.ny = h.ny;
  o.k = h.k;
  o.leaf = h.leaf;
  o.ev = ev;
  o.flags = flags;
}

// One launch refines the four leaf-kind lists one after the other (a warp's rays come from
// one list except at the seams, so the kinds stay apart as in four launches).
template <bool MULTI>
__global__ void __launch_bounds__(256) k_refine(SceneDev S, TraceBufs B, uint32_t gen) {
  auto count = [&](int l) -> uint64_t {
    const unsigned long long c = B.ctr->list_count[gen][l];
    return c < B.queue_cap ? c : B.queue_cap;
  };
  const uint64_t o1 = count(LIST_REFINE_CIRCLE), o2 = o1 + count(LIST_REFINE_RECT);
  const uint64_t o3 = o2 + count(LIST_REFINE_SEGMENT), n = o3 + count(LIST_REFINE_CUBIC);
  const RayRec* q = B.queue[gen & 1];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t idx = i < o1 ? B.list[LIST_REFINE_CIRCLE][i]
                       : i < o2 ? B.list[LIST_REFINE_RECT][i - o1]
                       : i < o3 ? B.list[LIST_REFINE_SEGMENT][i - o2] : B.list[LIST_REFINE_CUBIC][i - o3];
    const RayRec r = q[idx];
    const ScanRec sc = B.scan[idx];
    Hit64 h;
    if (refine_root(S, obj_base_of<MULTI>(S, r.scene) + sc.cand[0], sc.leaf, sc.face, sc.t32, sc.s32, r.ox, r.oy,
                    r.dx, r.dy, h)) {
      store_hit(B.hit[idx], sc.cand[0], h, INFINITY, 0);
    } else {  // cannot refine (degenerate): solve it fully after this kernel
      B.scan[idx].leaf = LEAF_REFINE_FAILED;
      const unsigned long long slot = atomicAdd(&B.ctr->list_count[gen][LIST_FULL], 1ull);
      if (slot < B.queue_cap) B.list[LIST_FULL][slot] = idx;
    }
  }
}

template __global__ void k_refine<false>(SceneDev, TraceBufs, uint32_t);
template __global__ void k_refine<true>(SceneDev, TraceBufs, uint32_t);

template <bool MULTI>
__global__ void __launch_bounds__(256, 2) k_full(SceneDev S, TraceBufs B, uint32_t gen, int smem_fits) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ unsigned long long blk_solves;
  if (threadIdx.x == 0) blk_solves = 0;
  bool failed;
  const ObjScan* objs = stage_objects(S, reinterpret_cast<ObjScan*>(smem_raw), &bar, !MULTI && smem_fits != 0, B.ctr,
                                      failed);
  if (failed) return;
  unsigned long long n = B.ctr->list_count[gen][LIST_FULL];
  if (n > B.queue_cap) n = B.queue_cap;
  const RayRec* q = B.queue[gen & 1];
  unsigned long long my_solves = 0;
  // block-uniform loop: the CTA's warps solve one class at a time together (a barrier
  // between classes), so that one solver's code is in flight per CTA
  for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const bool valid = i < n;
    const uint32_t idx = B.list[LIST_FULL][valid ? i : base];  // idle lanes read a real entry, store nothing
    const RayRec r = q[idx];
    const ScanRec sc = B.scan[idx];
    const SceneLoc sl = scene_of<MULTI>(S, r.scene);
    const ObjScan* sobjs = objs + sl.base;
    df best_d2 = DF_INF, second = DF_INF;
    Near ev{INFINITY, ray_tol(r.ex, r.ea)};
    int best = -1;
    Hit64 bh;
    bh.leaf = 0;
    // the nearest hit is the minimum of (d2, object index): candidates may be solved in
    // any order, so the warp runs one solve class at a time
    auto consider = [&](uint32_t j) {
      Hit64 hh;
      df d2;
      ++my_solves;
      if (obj_solve64(S, sl.base + j, r.ox, r.oy, r.dx, r.dy, hh, d2, ev)) {
        if (d2 < best_d2 || (d2 == best_d2 && (int)j < best)) {
          second = best_d2;
          best_d2 = d2;
          best = (int)j;
          bh = hh;
        } else if (d2 < second) {
          second = d2;
        }
      }
    };
    {
      uint32_t pending = valid && !sc.overflow ? (1u << sc.nc) - 1u : 0u;
      uint32_t cls[CAND];
      for (int k = 0; k < CAND; ++k)
        cls[k] = k < sc.nc ? solve_class(reinterpret_cast<const uint32_t*>(&sobjs[sc.cand[k]])[3]) : 7u;
      for (uint32_t c = 0; c < N_SOLVE_CLASSES; ++c) {
        for (;;) {
          int k = -1;
          for (int kk = 0; kk < CAND; ++kk)
            if (k < 0 && ((pending >> kk) & 1u) && cls[kk] == c) k = kk;
          if (!__any_sync(0xffffffffu, k >= 0)) break;
          if (k >= 0) {
            pending &= ~(1u << k);
            consider(sc.cand[k]);
          }
        }
        __syncthreads();
      }
    }
    if (!valid) continue;
    if (sc.overflow) {  // list overflow (rare): every object that passes the FP32 filters, in order
      const float ox = r.ox.hi, oy = r.oy.hi, dx = r.dx.hi, dy = r.dy.hi;
      for (uint32_t j = 0; j < sl.n; ++j) {
        const float4 h = *reinterpret_cast<const float4*>(&sobjs[j]);
        float lb;
        if (!bound_test(h, ox, oy, dx, dy, sc.thr, lb)) continue;
        if (!(classify32(sobjs[j], ox, oy, dx, dy, lb, j == r.src_obj ? (int)r.src_leaf : -1).key <= sc.thr)) continue;
        consider(j);
      }
    }
    uint8_t fl = sc.overflow ? LG_PATH_FALLBACK : 0;
    // a tie between two objects, within the band or within what the ray's error bound moves d2
    if (best >= 0 && second.hi < INFINITY &&
        (second - best_d2).hi <= fmaxf(1e-10f * best_d2.hi, 4.0f * sqrtf(best_d2.hi) * ev.tol))
      fl |= LG_PATH_NEAR_DEGENERATE;
    store_hit(B.hit[idx], best, bh, ev.ev, fl);
  }
  atomicAdd(&blk_solves, my_solves);
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(&B.ctr->fp64_solves, blk_solves);
}
template __global__ void k_full<false>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_full<true>(SceneDev, TraceBufs, uint32_t, int);

struct Bounce {
  bool emit;
  float x1, y1;
  int hit;
  uint8_t flags;
  int nchild;
  RayRec child[2];
};

template <bool MULTI, bool CULL>
__device__ __forceinline__ void bounce(const SceneDev& S, const ObjScan* objs, const RayRec& r, const ScanRec& sc,
                                       const HitRec* hrec, Bounce& v) {
  v.emit = false;
  v.nchild = 0;
  const SceneLoc sl = scene_of<MULTI>(S, r.scene);
  uint8_t fl = r.flags;
  if (near_cutoff(r.c, sl.cutoff)) fl |= LG_PATH_NEAR_DEGENERATE;
  const df ox = r.ox, oy = r.oy, dx = r.dx, dy = r.dy;
  HitRec bh;
  bh.obj = HIT_NONE;
  bh.flags = 0;
  bh.ev = INFINITY;
  if (sc.nc > 0) bh = *hrec;
  fl |= bh.flags;
  const int best = bh.obj == HIT_NONE ? -1 : (int)bh.obj;
  if (best >= 0 ? bh.ev <= bh.t.hi * (1.0f + 1e-6f) + 1e-12f : bh.ev < INFINITY) fl |= LG_PATH_NEAR_DEGENERATE;

  if (best >= 0) {
    const ObjInfo oi = S.info[sl.base + best];
    v.emit = true;
    v.x1 = bh.px.hi; v.y1 = bh.py.hi;
    v.hit = best;
    // first-order error at the hit: lateral offset L, offset along the surface ds
    const df ddn = dx * bh.nx + dy * bh.ny;
    const float ci_abs = fabsf(ddn.hi);
    const float kap = fminf(bh.k, 1e30f);
    // The FP64 quadratic of a curved surface (b^2 - a c with |b| ~ |o - c|) moves the
    // reference's own hit by about eps64 |o - c|^2 / (r cos) along the ray: an origin far
    // from a small circle makes the reference's result itself uncertain, and the path is
    // flagged once that, carried through the bounces, passes ILL_COND.
    const float oc = bh.t.hi + (kap > 0.0f ? 1.0f / kap : 0.0f);
    const float ref_solve = kap > 0.0f ? FP64_SOLVE_EPS * oc * oc * kap / fmaxf(ci_abs, 1e-6f) : 0.0f;
    const float L = r.ex + bh.t.hi * r.ea + DF_ROUND * (1.0f + fabsf(bh.px.hi) + fabsf(bh.py.hi)) + ref_solve;
    const float ds = L / fmaxf(ci_abs, 1e-6f);
    if (L > ILL_COND) fl |= LG_PATH_ILL_CONDITIONED;
    if (oi.flags & INFO_MATERIAL) {
      // medium on the far side (tracer.rs:428-442); "origin inside obj" at the midpoint
      df n2 = DF_ONE;
      uint16_t m2 = MEDIUM_AIR;
      bool near = false;
      if (obj_contains64(S, sl.base + (uint32_t)best, DF_HALF * (ox + bh.px), DF_HALF * (oy + bh.py), near, L)) {
        const float px32 = bh.px.hi, py32 = bh.py.hi;
        // the first other material object, in table order, that contains the hit point
        auto far_side = [&](uint32_t k) -> bool {
          if ((int)k == best) return false;
          const float4 h = MULTI ? __ldg(&S.bounds[sl.base + k]) : *reinterpret_cast<const float4*>(&objs[sl.base + k]);
          if (!(__float_as_uint(h.w) & INFO_MATERIAL)) return false;
          const float ex = px32 - h.x, ey = py32 - h.y;
          const float tol = 2e-6f * (fabsf(px32) + fabsf(py32) + fabsf(h.x) + fabsf(h.y) + h.z) + 1e-6f;
          if (ex * ex + ey * ey > (h.z + tol) * (h.z + tol)) return false;
          if (!obj_contains64(S, sl.base + k, bh.px, bh.py, near, L)) return false;
          n2 = S.info[sl.base + k].n;
          m2 = (uint16_t)k;
          return true;
        };
        const GridRec& G = grid_of<MULTI>(S, r.scene);
        if (!CULL || G.nx == 0) {
          for (uint32_t k = 0; k < sl.n; ++k)
            if (far_side(k)) break;
        } else {
          // the hit point's cell lists, in table order, every object whose box holds it
          const float fx = fminf(fmaxf(floorf((px32 - G.x0) * G.iw), 0.0f), (float)(G.nx - 1));
          const float fy = fminf(fmaxf(floorf((py32 - G.y0) * G.ih), 0.0f), (float)(G.ny - 1));
          const uint32_t c = (uint32_t)fy * G.nx + (uint32_t)fx;
          const uint32_t* cs = S.cell_start + G.cell_base;
          const uint16_t* co = S.cell_obj + G.list_base;
          for (uint32_t q = __ldg(cs + c), qe = __ldg(cs + c + 1); q < qe; ++q)
            if (far_side(__ldg(co + q))) break;
        }
      } else {
        n2 = oi.n;
        m2 = (uint16_t)best;
      }
      if (near) fl |= LG_PATH_NEAR_DEGENERATE;
      // Ray::refract: Snell + unpolarised Fresnel, TIR -> reflectance 1
      df nx = bh.nx, ny = bh.ny;
      df ci = -ddn;
      if (df_neg(ci)) { ci = -ci; nx = -nx; ny = -ny; }
      const df n1 = r.medium == MEDIUM_AIR ? DF_ONE
                    : r.medium == MEDIUM_LIGHT ? S.lights[sl.light_base + r.light].n0 : S.info[sl.base + r.medium].n;
      const df eta = n1 / n2;
      const df k = DF_ONE - eta * eta * (DF_ONE - ci * ci);
      if (fabsf(k.hi) <= 1e-10f) fl |= LG_PATH_NEAR_DEGENERATE;
      float R = 1.0f;
      bool refr = false;
      df tx = DF_ZERO, ty = DF_ZERO, ct = DF_ZERO;
      if (!df_neg(k)) {
        ct = dsqrt(k);
        const df m = eta * ci - ct;
        tx = eta * dx + m * nx;
        ty = eta * dy + m * ny;
        refr = true;
        const df dsn = n1 * ci + n2 * ct, dp = n1 * ct + n2 * ci;
        if (dsn.hi != 0.0f && dp.hi != 0.0f) {
          const df rs = (n1 * ci - n2 * ct) / dsn, rp = (n1 * ct - n2 * ci) / dp;
          R = (DF_HALF * (rs * rs + rp * rp)).hi;
        }
      }
      v.flags = fl | (refr ? 0 : LG_PATH_TIR);
      const float refl = R;
      const float om = 1.0f - refl;
      RayRec& a = v.child[0];
      const df ci2 = ci * 2.0f;
      a.ox = bh.px; a.oy = bh.py; a.dx = dx + ci2 * nx; a.dy = dy + ci2 * ny;
      a.medium = r.medium;
      a.src_obj = (uint16_t)best;
      a.src_leaf = bh.leaf;
      a.c[0] = __fmul_rn(r.c[0], refl); a.c[1] = __fmul_rn(r.c[1], refl); a.c[2] = __fmul_rn(r.c[2], refl);
      a.c[3] = r.c[3];
      a.path = r.path;
      a.flags = fl;
      a.ex = L;
      a.ea = r.ea + 2.0f * kap * ds;
      v.nchild = 1;
      if (refr) {
        RayRec& t = v.child[1];
        t.ox = bh.px; t.oy = bh.py; t.dx = tx; t.dy = ty;
        t.medium = m2;
        t.src_obj = (uint16_t)best;
        t.src_leaf = bh.leaf;
        t.c[0] = __fmul_rn(r.c[0], om); t.c[1] = __fmul_rn(r.c[1], om); t.c[2] = __fmul_rn(r.c[2], om);
        t.c[3] = r.c[3];
        t.path = r.path | (1ull << r.gen);
        t.flags = fl;
        const float gain = eta.hi * ci.hi / fmaxf(ct.hi, 1e-6f);
        t.ex = ds * ct.hi + L;
        t.ea = gain * (r.ea + kap * ds) + kap * ds;
        v.nchild = 2;
      }
    } else {
      v.flags = fl;
      const df dn2 = ddn * 2.0f;  // Ray::reflect
      RayRec& a = v.child[0];
      a.ox = bh.px; a.oy = bh.py; a.dx = dx - dn2 * bh.nx; a.dy = dy - dn2 * bh.ny;
      a.medium = r.medium;
      a.src_obj = (uint16_t)best;
      a.src_leaf = bh.leaf;
      a.c[0] = r.c[0]; a.c[1] = r.c[1]; a.c[2] = r.c[2]; a.c[3] = r.c[3];
      a.path = r.path;
      a.flags = fl;
      a.ex = L;
      a.ea = r.ea + 2.0f * kap * ds;
      v.nchild = 1;
    }
  } else {
    // canvas exit: nearest hit with the canvas rectangle (tracer.rs:482-488)
    Leaf64 canvas;
    canvas.kind = LEAF_RECT;
    canvas.p[0] = DF_ZERO; canvas.p[1] = DF_ZERO; canvas.p[2] = DF_ONE; canvas.p[3] = DF_ZERO;
    canvas.p[4] = sl.aspect; canvas.p[5] = DF_ONE;
    Hit64 ch[3];
    Near cev{INFINITY, ray_tol(r.ex, r.ea)};
    const int nh = leaf_hits64(canvas, ox, oy, dx, dy, ch, cev);
    if (nh > 0) {
      int bi = 0;
      for (int q = 1; q < nh; ++q)
        if (ch[q].t < ch[bi].t) bi = q;
      v.emit = true;
      v.x1 = ch[bi].px.hi; v.y1 = ch[bi].py.hi;
      v.hit = -1;
      const float L = r.ex + ch[bi].t.hi * r.ea;
      v.flags = fl | (cev.ev < INFINITY ? LG_PATH_NEAR_DEGENERATE : 0) | (L > ILL_COND ? LG_PATH_ILL_CONDITIONED : 0);
    }
  }
  // children: the next generation skips colours below the cutoff (tracer.rs:378-384)
  int w = 0;
  for (int q = 0; q < v.nchild; ++q) {
    RayRec c = v.child[q];
    if ((uint32_t)r.gen + 1 >= sl.max_bounce || below_cutoff(c.c, sl.cutoff)) continue;
    c.gen = (uint8_t)(r.gen + 1);
    c.prim = r.prim;
    c.light = r.light;
    c._pad = 0;
    c.scene = r.scene;
    if (near_cutoff(c.c, sl.cutoff)) c.flags |= LG_PATH_NEAR_DEGENERATE;
    if (!(c.ex <= ILL_COND && c.ea <= ILL_COND)) c.flags |= LG_PATH_ILL_CONDITIONED;
    v.child[w++] = c;
  }
  v.nchild = w;
}

template <bool MULTI, bool CULL>
__global__ void __launch_bounds__(256, 3) k_bounce(SceneDev S, TraceBufs B, uint32_t gen, int smem_fits) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ unsigned long long blk_visits, blk_near, blk_ill;
  if (threadIdx.x == 0) { blk_visits = 0; blk_near = 0; blk_ill = 0; }
  bool failed;
  const ObjScan* objs = stage_objects(S, reinterpret_cast<ObjScan*>(smem_raw), &bar, !MULTI && smem_fits != 0, B.ctr,
                                      failed);
  if (failed) return;
  // the rays with work: every work list of this generation, one after the other
  uint64_t off[N_LISTS + 1];
  off[0] = 0;
  for (int l = 0; l < N_LISTS; ++l) {
    const unsigned long long c = B.ctr->list_count[gen][l];
    off[l + 1] = off[l] + (c < B.queue_cap ? c : B.queue_cap);
  }
  const uint64_t total = off[N_LISTS];
  const RayRec* qin = B.queue[gen & 1];
  RayRec* qout = B.queue[(gen + 1) & 1];
  const unsigned lane = lane_id();
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  unsigned long long my_visits = 0, my_near = 0, my_ill = 0;
  for (uint64_t base = warp * 32; base < total; base += nwarps * 32) {
    const uint64_t i = base + lane;
    Bounce v;
    v.emit = false;
    v.nchild = 0;
    v.flags = 0;
    v.hit = -1;
    RayRec r;
    if (i < total) {
      int l = 0;
      while (i >= off[l + 1]) ++l;
      const uint32_t idx = B.list[l][i - off[l]];
      const ScanRec sc = B.scan[idx];
      if (!(l < LIST_FULL && sc.leaf == LEAF_REFINE_FAILED)) {  // those are in the full list too
        r = qin[idx];
        ++my_visits;
        bounce<MULTI, CULL>(S, objs, r, sc, &B.hit[idx], v);
      }
    }
    emit_segments(S, B, v.emit, r, v.x1, v.y1, v.flags, v.hit, my_near, my_ill);
    // children: warp prefix sum of 0..2 per lane, one atomic per warp
    int incl = v.nchild;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += y;
    }
    const int tot = __shfl_sync(0xffffffffu, incl, 31);
    if (tot > 0 && (MULTI || gen + 1 < S.max_bounce)) {  // multi-scene: bounce() checks each ray's scene
      unsigned long long qbase = 0;
      if (lane == 31) qbase = atomicAdd(&B.ctr->queue_count[gen + 1], (unsigned long long)tot);
      qbase = __shfl_sync(0xffffffffu, qbase, 31);
      const unsigned long long first = qbase + (unsigned long long)(incl - v.nchild);
      for (int q = 0; q < v.nchild; ++q)
        if (first + q < B.queue_cap) qout[first + q] = v.child[q];
    }
  }
  atomicAdd(&blk_visits, my_visits);
  atomicAdd(&blk_near, my_near);
  atomicAdd(&blk_ill, my_ill);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&B.ctr->visits, blk_visits);
    atomicAdd(&B.ctr->near, blk_near);
    atomicAdd(&B.ctr->ill, blk_ill);
  }
}
template __global__ void k_bounce<false, false>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_bounce<false, true>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_bounce<true, false>(SceneDev, TraceBufs, uint32_t, int);
template __global__ void k_bounce<true, true>(SceneDev, TraceBufs, uint32_t, int);

// ------------------------------------------------------------------- scene order
// Multi-scene generations > 0: a counting sort of the queue entries by scene (histogram,
// exclusive scan, scatter of entry indices), so that k_scan's warps each see one scene.
__device__ __forceinline__ unsigned long long warp_scene_atomic(unsigned* slot_base, uint32_t s, bool on) {
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, on ? s : 0xffffffffu);
  if (!on) return 0;
  const int leader = __ffs(grp) - 1;
  unsigned base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(&slot_base[s], (unsigned)__popc(grp));
  base = __shfl_sync(grp, base, leader);
  return base + __popc(grp & lanemask_lt());
}

__global__ void k_scene_hist(SceneDev S, TraceBufs B, uint32_t gen, unsigned* count) {
  const uint64_t n = n_real_of(S, B, gen);
  const RayRec* q = B.queue[gen & 1];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t s = q[i].scene;
    warp_scene_atomic(count, s, s < S.n_scenes);
  }
}

// single CTA: off = exclusive scan of count; count is cleared for the next generation
__global__ void __launch_bounds__(1024) k_scene_offsets(unsigned* count, unsigned* off, uint32_t n_scenes) {
  __shared__ unsigned wsum[32];
  __shared__ unsigned carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
  for (uint32_t base = 0; base < n_scenes; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const unsigned c = i < n_scenes ? count[i] : 0u;
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += y;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      unsigned sw = lane < (blockDim.x >> 5) ? wsum[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, sw, o);
        if ((int)lane >= o) sw += y;
      }
      wsum[lane] = sw;
    }
    __syncthreads();
    const unsigned cr = carry;
    const unsigned excl = cr + (wid ? wsum[wid - 1] : 0u) + incl - c;
    if (i < n_scenes) {
      off[i] = excl;
      count[i] = 0u;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + c;
    __syncthreads();
  }
}

__global__ void k_scene_scatter(SceneDev S, TraceBufs B, uint32_t gen, unsigned* off, uint32_t* order) {
  const uint64_t n = n_real_of(S, B, gen);
  const RayRec* q = B.queue[gen & 1];
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t s = q[i].scene;
    const bool on = s < S.n_scenes;
    const unsigned long long pos = warp_scene_atomic(off, s, on);
    if (on && pos < n) order[pos] = (uint32_t)i;
  }
}

// ------------------------------------------------------------------- overlays
// A point of the string-mod curve (string_mod.rs:33-85), the same FP64 operations as the
// oracle: angle (turns * n) * 2 pi / m, the library's own sine and cosine.
__device__ void string_mod_point(const lg_string_mod& sm, uint64_t n, double& x, double& y) {
  using namespace lgx;
  const uint64_t k = sm.turns * n;
  if (sm.curve == LG_CURVE_COMPLEX_EXP) {
    // (re + i im)^(u32)k by binary powering (num-complex 0.4.6, Pow<u32> for &Complex)
    uint32_t e = (uint32_t)k;
    if (e == 0) { x = 1.0; y = 0.0; return; }
    double br = sm.curve_f[0], bi = sm.curve_f[1];
    while ((e & 1u) == 0) {
      const double r = sub(mul(br, br), mul(bi, bi)), i = add(mul(br, bi), mul(bi, br));
      br = r; bi = i; e >>= 1;
    }
    double ar = br, ai = bi;
    while (e > 1) {
      e >>= 1;
      const double r = sub(mul(br, br), mul(bi, bi)), i = add(mul(br, bi), mul(bi, br));
      br = r; bi = i;
      if (e & 1u) {
        const double r2 = sub(mul(ar, br), mul(ai, bi)), i2 = add(mul(ar, bi), mul(ai, br));
        ar = r2; ai = i2;
      }
    }
    x = ar; y = ai;
    return;
  }
  const double angle = dvd(mul((double)k, 2.0 * 3.141592653589793), (double)sm.modulo);
  double s, c;
  if (sm.curve == LG_CURVE_HYPOTROCHOID) {
    const double r = (double)sm.curve_u[0], big = (double)sm.curve_u[1], d = (double)sm.curve_u[2];
    const double smr = sub(big, r), ratio = add(smr, d);
    double s2, c2;
    sincos_x(angle, s, c);
    sincos_x(dvd(mul(angle, smr), r), s2, c2);
    x = dvd(add(mul(smr, c), mul(d, c2)), ratio);
    y = dvd(sub(mul(smr, s), mul(d, s2)), ratio);
  } else if (sm.curve == LG_CURVE_LISSAJOUS) {
    double s2, c2;
    sincos_x(add(mul((double)sm.curve_u[0], angle), sm.curve_f[0]), s, c);
    sincos_x(mul((double)sm.curve_u[1], angle), s2, c2);
    x = s;
    y = s2;
  } else {
    sincos_x(angle, s, c);
    x = c;
    y = s;
  }
}

// The point that line iix of a string mod joins to point iix, by the mod's mode
// (string_mod.rs:112-117; u64 arithmetic wrapping like Rust's release build).
__device__ __forceinline__ uint64_t string_mod_target(const lg_string_mod& sm, uint64_t iix) {
  const uint64_t m = sm.modulo;
  if (sm.mode == LG_SM_ADD) return (iix + sm.num) % m;
  if (sm.mode == LG_SM_MUL) return (iix * sm.num) % m;
  uint64_t b = sm.mode == LG_SM_POW ? iix : sm.num, e = sm.mode == LG_SM_POW ? (uint32_t)sm.num : (uint32_t)iix, p = 1;
  while (e) {
    if (e & 1) p *= b;
    b *= b;
    e >>= 1;
  }
  return p % m;
}

// StringMod::get_color (string_mod.rs:124-150): the f32 mean of the matching modulo colours,
// summed in table order, else the base colour.
__device__ void string_mod_color(const lg_string_mod& sm, const lg_mod_color* colors, uint32_t n_colors,
                                 uint64_t ix, float* out) {
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  uint32_t cnt = 0;
  for (uint32_t k = 0; k < n_colors; ++k) {
    const lg_mod_color& e = colors[k];
    if (ix % e.modulo == e.rem) {
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) acc[ch] = __fadd_rn(acc[ch], e.color[ch]);
      ++cnt;
    }
  }
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) out[ch] = cnt ? __fdiv_rn(acc[ch], (float)cnt) : sm.color[ch];
}

// Overlays drawn after the trace: the control polygons of curved mirrors (tracer.rs:341-346)
// appended to the segment ring, and the string-mod lines (string_mod.rs:104-122) written to
// their own table, one per point: chord iix joins point iix and point ix(iix) of the mode,
// each vertex with its own colour.
__global__ void k_overlay(SceneDev S, TraceBufs B, const uint32_t* cubic_objs, const uint16_t* cubic_scene,
                          uint32_t n_cubic, lg_string_mod sm, ChordArgs CA) {
  const uint64_t n_ctrl = 3ull * n_cubic;
  const uint64_t total = n_ctrl + sm.modulo;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    if (i < n_ctrl) {
      lg_segment s;
      lg_path_record pr;
      pr.path = 0; pr.light = 0xffff; pr.flags = 0; pr.hit = -1;
      uint16_t scene = 0;
      if (cubic_scene) scene = cubic_scene[i / 3];
      const uint32_t k = cubic_objs[i / 3];
      const int q = (int)(i % 3);
      const Leaf64& L = S.leaves[S.info[k].leaf_begin];
      s.x0 = L.p[2 * q].hi; s.y0 = L.p[2 * q + 1].hi;
      s.x1 = L.p[2 * q + 2].hi; s.y1 = L.p[2 * q + 3].hi;
      s.color[0] = 1.f; s.color[1] = 0.f; s.color[2] = 0.f; s.color[3] = 1.f;
      pr.primary = k; pr.gen = (uint8_t)q; pr.source = LG_SRC_CONTROL_LINE;
      const unsigned long long slot = atomicAdd(&B.ctr->seg_count, 1ull);
      if (slot < B.seg_cap) {
        B.segs[slot] = s;
        if (B.seg_scene) B.seg_scene[slot] = scene;
        if (S.record_paths) B.paths[slot] = pr;
      }
    } else {
      const uint64_t m = sm.modulo, iix = i - n_ctrl;
      const uint64_t ix = string_mod_target(sm, iix);
      double xa, ya, xb, yb;
      if (CA.pts) {  // nested: points iix and ix of the outer mod's crossings (string_mod.rs:118-119)
        const double2 pa = CA.pts[iix % CA.n_pts], pb = CA.pts[ix % CA.n_pts];
        xa = pa.x; ya = pa.y; xb = pb.x; yb = pb.y;
      } else {
        string_mod_point(sm, iix % m, xa, ya);
        string_mod_point(sm, ix % m, xb, yb);
      }
      lg_chord c;
      c.x0 = (float)xa; c.y0 = (float)ya; c.x1 = (float)xb; c.y1 = (float)yb;
      string_mod_color(sm, CA.colors, CA.n_colors, iix, c.color0);
      string_mod_color(sm, CA.colors, CA.n_colors, ix, c.color1);
      if (CA.out) CA.out[iix] = c;
    }
  }
}

// ---------------------------------------------------------- nested string mods
// StringMod::line_crossings_as_points (string_mod.rs:87-102): line k of the outer mod joins
// point k and point ix(k) of its curve, in FP64 (lines[2k], lines[2k + 1]).
__global__ void k_sm_lines(lg_string_mod sm, double2* lines) {
  const uint64_t m = sm.modulo;
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < m; k += (uint64_t)gridDim.x * blockDim.x) {
    double x, y;
    string_mod_point(sm, k % m, x, y);
    lines[2 * k] = make_double2(x, y);
    string_mod_point(sm, string_mod_target(sm, k) % m, x, y);
    lines[2 * k + 1] = make_double2(x, y);
  }
}

// Crossing of segments ab and cd (collision2d's LineSegment::intersect is not vendored; this
// is the definition include/lg.h states): the 2x2 parametric solve a + t (b - a) =
// c + u (d - c), each FP64 operation rounded on its own, a crossing when the determinant is
// not zero and t, u lie in [0, 1]; the point is a + t (b - a).
__device__ __forceinline__ bool seg_cross_x(double2 a, double2 b, double2 c, double2 d, double2& p) {
  using namespace lgx;
  const double rx = sub(b.x, a.x), ry = sub(b.y, a.y), sx = sub(d.x, c.x), sy = sub(d.y, c.y);
  const double den = sub(mul(rx, sy), mul(ry, sx));
  if (den == 0.0) return false;
  const double wx = sub(c.x, a.x), wy = sub(c.y, a.y);
  const double t = dvd(sub(mul(wx, sy), mul(wy, sx)), den);
  const double u = dvd(sub(mul(wx, ry), mul(wy, rx)), den);
  if (!(t >= 0.0 && t <= 1.0 && u >= 0.0 && u <= 1.0)) return false;
  p.x = add(a.x, mul(rx, t));
  p.y = add(a.y, mul(ry, t));
  return true;
}

// pair q of m (m - 1), in the reference's order: diff = q / m + 1 (outer loop), line a = q % m
__device__ __forceinline__ bool pair_cross(const double2* lines, uint64_t m, uint64_t q, double2& p) {
  const uint64_t diff = q / m + 1, a = q % m, b = (a + diff) % m;
  return seg_cross_x(lines[2 * a], lines[2 * a + 1], lines[2 * b], lines[2 * b + 1], p);
}

// A thread's run of CROSS_PER_THREAD consecutive pairs: how many of them cross.
__device__ __forceinline__ uint32_t run_crossings(const double2* lines, uint64_t m, uint64_t q0, uint64_t n_pairs) {
  uint32_t c = 0;
  for (int k = 0; k < CROSS_PER_THREAD; ++k) {
    double2 p;
    if (q0 + k < n_pairs && pair_cross(lines, m, q0 + k, p)) ++c;
  }
  return c;
}

// exclusive sum over the CTA's threads (CROSS_THREADS of them); *total receives the sum
__device__ __forceinline__ uint32_t cta_exclusive(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if ((int)lane >= o) incl += y;
  }
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (unsigned k = 0; k < CROSS_THREADS / 32; ++k) {
    if (k < w) before += warp_sums[k];
    all += warp_sums[k];
  }
  if (total) *total = all;
  return before + incl - v;
}

__global__ void __launch_bounds__(CROSS_THREADS) k_cross_count(const double2* lines, uint64_t m, uint32_t* blk) {
  __shared__ uint32_t warp_sums[CROSS_THREADS / 32];
  const uint64_t n_pairs = m * (m - 1);
  const uint64_t q0 = blockIdx.x * CROSS_PAIRS_PER_BLOCK + (uint64_t)threadIdx.x * CROSS_PER_THREAD;
  const uint32_t c = run_crossings(lines, m, q0, n_pairs);
  uint32_t total = 0;
  cta_exclusive(c, warp_sums, &total);
  if (threadIdx.x == 0) blk[blockIdx.x] = total;
}

// one CTA of 1024 threads: exclusive scan of the per-block counts in place
__global__ void __launch_bounds__(1024) k_cross_scan(uint32_t* blk, uint32_t n_blk, unsigned long long* total) {
  __shared__ unsigned long long carry;
  __shared__ uint32_t warp_sums[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  for (uint32_t base = 0; base < n_blk; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < n_blk ? blk[i] : 0u;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[w] = incl;
    __syncthreads();
    uint32_t before = 0, all = 0;
    for (unsigned k = 0; k < blockDim.x / 32; ++k) {
      if (k < w) before += warp_sums[k];
      all += warp_sums[k];
    }
    const unsigned long long c0 = carry;
    if (i < n_blk) blk[i] = (uint32_t)(c0 + before + incl - v);
    __syncthreads();
    if (threadIdx.x == 0) carry = c0 + all;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// the crossing points in pair order: block offset + the thread's place in the block + its run
__global__ void __launch_bounds__(CROSS_THREADS) k_cross_write(const double2* lines, uint64_t m,
                                                                const uint32_t* blk_off, double2* pts) {
  __shared__ uint32_t warp_sums[CROSS_THREADS / 32];
  const uint64_t n_pairs = m * (m - 1);
  const uint64_t q0 = blockIdx.x * CROSS_PAIRS_PER_BLOCK + (uint64_t)threadIdx.x * CROSS_PER_THREAD;
  const uint32_t c = run_crossings(lines, m, q0, n_pairs);
  uint64_t slot = (uint64_t)blk_off[blockIdx.x] + cta_exclusive(c, warp_sums, nullptr);
  for (int k = 0; k < CROSS_PER_THREAD; ++k) {
    double2 p;
    if (q0 + k < n_pairs && pair_cross(lines, m, q0 + k, p)) pts[slot++] = p;
  }
}

}  // namespace lgd
