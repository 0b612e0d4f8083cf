// lg_device.cuh — device-side scene tables, geometry and raster rule of the GB300 path.
//
// Scene layout in HBM (built by lg_api.cu from the lg.h tables):
//   ObjScan[n_obj]   64 B per object, FP32: inflated bounding circle + up to two leaves
//                    inline.  This is the table every ray scans; each CTA stages it in
//                    shared memory with one cp.async.bulk copy.
//   ObjInfo[n_obj]   48 B per object: leaf range, membership program, material, FP64 tree range.
//   Leaf64[n_leaf]   72 B per leaf, double-float world-space primitive (CSG trees flattened).
//   prog[]           membership programs (postfix over leaf membership bits).
//
// Precision split (tracer.rs:395-424 does one FP64 intersection per object per ray):
//   * the O(objects) scan runs in FP32 and classifies each object as a certain miss, a
//     certain hit at t32 (margins well above FP32 error), or uncertain;
//   * every object that could be the nearest hit (certain hits within the FP32 error of
//     the best, and every uncertain object in front of it) is re-solved in double-float
//     (lg_df.cuh, ~48-bit significand on the FP32 pipe), as are the bounce
//     (reflect / refract), the medium test and the canvas exit.
//   That work is O(1) per ray visit; the FP32 scan carries the object count.  Native
//   FP64 (1/64 of the FP32 rate on GB300) is used only to generate primary rays.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lg.h"
#include "lg_df.cuh"
#include "lg_x64.cuh"

namespace lgd {

constexpr double T_MIN = 1e-9;        // hits at t <= T_MIN are the surface the ray leaves
constexpr double SPOT_EPSILON = 1e-9; // SpotLight::set_num_rays |dir.x| < EPSILON
constexpr double BAND = 1e-10;        // FP64 near-degenerate band (relative)
constexpr float TAU32 = 1e-4f;        // FP32: |t| below this cannot decide t > T_MIN
constexpr int MAX_LEAVES = 64;
constexpr int MAX_GEN = 64;
constexpr int CAND = 8;               // FP64 candidate list per ray visit
constexpr int TILE = 32;              // raster tile edge in pixels
constexpr int TILE_PAD = 33;          // smem row stride (int64 words): no bank conflicts for y-major

// scan kinds (ObjScan::info bits 0..3)
enum : uint32_t { SCAN_BOUND = 0, SCAN_ONE = 1, SCAN_TWO = 2 };
// leaf kinds (Leaf64::kind and ObjScan leaf kinds)
enum : uint32_t { LEAF_CIRCLE = 0, LEAF_RECT = 1, LEAF_SEGMENT = 2, LEAF_CUBIC = 3,
                  // leaves the FP32 scan only bounds (their objects take the precise solve)
                  LEAF_ELLIPSE = 4, LEAF_HALFPLANE = 5 };
// ObjScan::info layout
__host__ __device__ inline uint32_t info_scan(uint32_t i) { return i & 0xfu; }
__host__ __device__ inline uint32_t info_leaf_a(uint32_t i) { return (i >> 4) & 0x3u; }
__host__ __device__ inline uint32_t info_leaf_b(uint32_t i) { return (i >> 6) & 0x3u; }
__host__ __device__ inline uint32_t info_op(uint32_t i) { return (i >> 8) & 0x3u; }
// solve class of an object (which precise-solve code path it takes): 0 circle, 1 rect,
// 2 segment (single-leaf objects), 3 cubic or deep CSG (bounding circle only), 4 two-leaf CSG
constexpr uint32_t N_SOLVE_CLASSES = 5;
__host__ __device__ inline uint32_t solve_class(uint32_t info) {
  const uint32_t sk = info & 0xfu;
  if (sk == 1u) return (info >> 4) & 0x3u;
  return sk == 2u ? 4u : 3u;
}
constexpr uint32_t INFO_MATERIAL = 1u << 10;
constexpr uint32_t INFO_NO_CONTAINS = 1u << 11; // mirror objects enclose nothing (object.rs:243-244)

struct __align__(16) ObjScan {
  float cx, cy, R;  // bounding circle, inflated for FP32 rounding
  uint32_t info;
  float a[6];       // leaf A: circle (cx,cy,r) | rect (cx,cy,cos,sin,hw,hh) | segment (ax,ay,ex,ey)
  float b[6];       // leaf B (SCAN_TWO)
};
static_assert(sizeof(ObjScan) == 64, "ObjScan is 64 B");

struct __align__(16) ObjInfo {
  uint32_t leaf_begin;
  uint16_t n_leaves;
  uint16_t prog_len;
  uint32_t prog_begin;
  uint32_t flags;     // INFO_MATERIAL | INFO_NO_CONTAINS
  df n;               // refractive index
  double n64;         // the same in FP64 (exact mode)
  uint32_t xnode_begin, xnode_count;  // exact mode: the object's geometry tree in preorder (lgx::XNode)
  uint64_t _pad;
};
static_assert(sizeof(ObjInfo) == 48, "ObjInfo is 48 B");

struct __align__(8) Leaf64 {
  uint32_t kind;
  uint32_t _pad;
  df p[8];  // circle cx,cy,r,1/r | rect cx,cy,cos,sin,hw,hh | segment ax,ay,bx,by,nx,ny (unit
            // left normal) | cubic P0..P3 | ellipse cx,cy,cos,sin,a,b,1/a,1/b | half-plane
            // px,py,nx,ny: a point of the boundary line and the unit outward normal (a convex
            // polygon is the And of its edges' half-planes)
};
static_assert(sizeof(Leaf64) == 72, "Leaf64 is 72 B");

enum : uint8_t { PROG_AND = 0x80, PROG_OR = 0x81, PROG_AND_NOT = 0x82 };  // < 0x40: push leaf k

struct __align__(16) LightDev {
  double ox, oy, vx, vy;
  double spot_angle;
  df n0;               // start medium (tracer.rs:280-287), filled on the device
  float color[4];
  uint32_t kind, num_rays;
  uint64_t first;      // index of this light's first primary in the virtual gen-0 queue
  uint32_t scene;      // scene of this light (multi-scene traces)
  uint32_t _pad;
  double dir_angle;    // exact mode: spot base angle (light.rs:230-234), filled on the device
  double n0x;          // exact mode: start medium in FP64, filled on the device
};

// Medium a ray travels in: an object index (its refractive index), or
constexpr uint16_t MEDIUM_AIR = 0xffff;    // 1.0
constexpr uint16_t MEDIUM_LIGHT = 0xfffe;  // the light's start medium (tracer.rs:280-287)
constexpr uint16_t SRC_NONE = 0xffff;

struct __align__(16) RayRec {
  df ox, oy, dx, dy;
  uint64_t path;
  float c[4];
  uint32_t prim;
  uint16_t light;
  uint8_t gen, flags;
  // first-order bound of how far rounding may have moved this ray: lateral offset of the
  // origin (world units) and direction (radians).  A path whose bound grows past
  // ILL_COND is flagged near-degenerate; below it the bound widens the decision bands.
  float ex, ea;
  uint16_t medium;   // see MEDIUM_*
  uint16_t src_obj;  // object whose surface the ray starts on (SRC_NONE for primaries)
  uint8_t src_leaf;  // leaf of src_obj that holds the start point
  uint8_t _pad;
  uint16_t scene;    // scene of the ray (multi-scene traces); object indices are scene-local
};
static_assert(sizeof(RayRec) == 80, "RayRec is 80 B");
// A path whose error bound exceeds ILL_COND (world units / radians) is flagged: its
// endpoints may then differ from an FP64 trace by more than a tenth of the 1e-5 endpoint
// tolerance.  Below it, decisions are checked against the bound itself (Near).
constexpr float ILL_COND = 1e-6f;
constexpr float FP64_SOLVE_EPS = 8.9e-16f;  // 4 ulp(1) of FP64: rounding of an FP64 discriminant
constexpr float TOL_REACH = 5.0f;  // longest ray parameter inside a canvas (16:9 diagonal ~ 4.1)
__device__ __forceinline__ float ray_tol(float ex, float ea) { return ex + TOL_REACH * ea; }
constexpr float DF_ROUND = 2e-14f;  // double-float rounding per bounce, relative to the coordinates

// work lists of one generation (k_scan appends, k_refine / k_full consume)
enum : int {
  LIST_REFINE_CIRCLE = 0, LIST_REFINE_RECT = 1, LIST_REFINE_SEGMENT = 2, LIST_REFINE_CUBIC = 3, LIST_FULL = 4,
  LIST_EXIT = 5,  // no object hit and the canvas exit needs the precise path (origin outside, corner)
  N_LISTS = 6
};
constexpr int8_t LEAF_REFINE_FAILED = -2;  // ScanRec::leaf after k_refine handed the ray to k_full

struct Counters {
  unsigned long long seg_count;               // ring cursor (= segments demanded)
  unsigned long long queue_count[MAX_GEN + 1]; // entries demanded per generation
  unsigned long long list_count[MAX_GEN][N_LISTS];
  unsigned long long visits, fp64_solves, fallbacks, near, ill;
  unsigned long long pixels, tile_refs, units;
  unsigned long long unit_cursor;
  // multi-scene streaming accumulation: the ring and the tile lists are reused every
  // generation; these keep the totals and the largest per-generation demands
  unsigned long long seg_total, seg_max, refs_total, refs_max;
  unsigned long long bound_tests, object_tests;  // nearest-hit search: bounding tests, classifications
  unsigned int error_flags;
  unsigned int skip_raster;  // streaming accumulation: this generation's accumulation is deferred
};
constexpr unsigned ERR_TMA_TIMEOUT = 1u;

// One scene of a multi-scene trace: its objects are [obj_base, obj_base + n_obj) of the
// concatenated tables (ray, scan and hit records hold indices relative to obj_base).
struct __align__(16) SceneRec {
  uint32_t obj_base, n_obj;
  df aspect;              // canvas half width (height is 1)
  float cutoff[4];
  uint32_t max_bounce;
  uint32_t light_base;    // the scene's first light (rays hold scene-local light indices)
  double aspect64;        // exact mode: the canvas half width in FP64
};
static_assert(sizeof(SceneRec) == 48, "SceneRec is 48 B");

// Uniform culling grid of one scene (built on the host).  The box is the union of the
// objects' FP32 bounding circles, each inflated by `margin` (above the FP32 error of the
// traversal: a cell the walk reports at ray parameter t is within far less than margin of
// the exact ray).  Cell c = iy * nx + ix lists, in ascending object order, every object
// whose inflated box overlaps it: cell_start[cell_base + c] .. cell_start[cell_base + c + 1]
// index cell_obj[list_base + ...] (scene-local object numbers).  An object's cell range
// comes from grid_cell_range, the same FP32 operations on host and device, so a walk that
// enters a cell knows whether it already met the object in the cell before.  nx == 0: no
// grid, the scan is brute force.
// Rays whose origin lies farther out than `reach` (|ox| + |oy|) carry FP32 errors above
// the margin and test every object instead.
struct __align__(16) GridRec {
  float x0, y0;           // lower-left corner
  float cw, ch;           // cell size
  float iw, ih;           // 1 / cell size
  float margin;           // world units: box inflation and traversal slack
  uint32_t nx, ny;
  uint32_t cell_base;     // first of the scene's nx * ny + 1 cell offsets
  uint32_t list_base;     // first of the scene's object-list entries
  float reach;
};
static_assert(sizeof(GridRec) == 48, "GridRec is 48 B");

struct SceneDev {
  const ObjScan* scan;
  const ObjInfo* info;
  const Leaf64* leaves;
  const uint8_t* prog;
  LightDev* lights;
  uint32_t n_obj, n_lights;
  uint64_t n_primary;
  df aspect;              // canvas half width (height is 1)
  float cutoff[4];
  uint32_t max_bounce;    // multi-scene: the largest of the scenes
  uint32_t record_paths;
  const SceneRec* scenes; // multi-scene traces only
  const float4* bounds;   // multi-scene: bounding circle + info word of every object (ObjScan's first 16 B)
  uint32_t n_scenes;
  // Serving (continuous batching): every launch takes the queued rays of the previous
  // step plus the primaries of the lights admitted now, [light_lo, light_hi), whose
  // `first` indices count from 0 at this step.
  uint32_t serve;
  uint64_t n_new;
  uint32_t light_lo, light_hi;
  // culling grids: one per scene (index 0 for a single-scene trace)
  const GridRec* grids;
  const uint32_t* cell_start;
  const uint16_t* cell_obj;
  // polls of a bounded device wait before it gives up (lg_device_opts.wait_polls; < 0: at once)
  int32_t wait_polls;
  // exact mode (LG_PRECISION_EXACT): the geometry nodes as uploaded, every object's tree in
  // preorder (ObjInfo::xnode_begin / xnode_count), the canvas half width in FP64
  const lg_geo* xgeo;
  const lgx::XNode* xnode;
  double aspect64;
  // sampled frame (one scene): queue entry v of a light is its primary ray_offset + ray_stride * v
  uint32_t ray_stride, ray_offset;
};

// First / last cell (unclamped, as a float) of [c - R - margin, c + R + margin] on one
// axis: round-to-nearest FP32 steps that no compiler may fuse, so the host that fills the
// cells and the device that walks them get the same integers.
__host__ __device__ inline float cell_lo(float c, float R, float margin, float org, float inv) {
#ifdef __CUDA_ARCH__
  return floorf(__fmul_rn(__fsub_rn(__fsub_rn(__fsub_rn(c, R), margin), org), inv));
#else
  volatile float t = c - R;
  t = t - margin;
  t = t - org;
  t = t * inv;
  return floorf(t);
#endif
}
__host__ __device__ inline float cell_hi(float c, float R, float margin, float org, float inv) {
#ifdef __CUDA_ARCH__
  return floorf(__fmul_rn(__fsub_rn(__fadd_rn(__fadd_rn(c, R), margin), org), inv));
#else
  volatile float t = c + R;
  t = t + margin;
  t = t - org;
  t = t * inv;
  return floorf(t);
#endif
}
// Cell range [x0, x1] x [y0, y1] of the box of a bounding circle (cx, cy, R) inflated by the
// grid's margin.
__host__ __device__ inline void grid_cell_range(const GridRec& G, float cx, float cy, float R, int& x0, int& y0,
                                                int& x1, int& y1) {
  const float fx0 = cell_lo(cx, R, G.margin, G.x0, G.iw), fx1 = cell_hi(cx, R, G.margin, G.x0, G.iw);
  const float fy0 = cell_lo(cy, R, G.margin, G.y0, G.ih), fy1 = cell_hi(cy, R, G.margin, G.y0, G.ih);
  const float mx = (float)(G.nx - 1), my = (float)(G.ny - 1);
  x0 = (int)fminf(fmaxf(fx0, 0.0f), mx); x1 = (int)fminf(fmaxf(fx1, 0.0f), mx);
  y0 = (int)fminf(fmaxf(fy0, 0.0f), my); y1 = (int)fminf(fmaxf(fy1, 0.0f), my);
}

template <bool MULTI>
__device__ __forceinline__ const GridRec& grid_of(const SceneDev& S, uint32_t sid) {
  return S.grids[MULTI ? sid : 0u];
}

// The scene a ray belongs to, as the kernels use it.  Single-scene kernels (MULTI false)
// take everything from the kernel parameters; multi-scene kernels read the scene table.
struct SceneLoc {
  uint32_t base, n;
  df aspect;
  float cutoff[4];
  uint32_t max_bounce;
  uint32_t light_base;
};
template <bool MULTI>
__device__ __forceinline__ SceneLoc scene_of(const SceneDev& S, uint32_t sid) {
  SceneLoc L;
  if (!MULTI) {
    L.base = 0; L.n = S.n_obj; L.aspect = S.aspect; L.max_bounce = S.max_bounce; L.light_base = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) L.cutoff[i] = S.cutoff[i];
  } else {
    const SceneRec& R = S.scenes[sid];
    L.base = R.obj_base; L.n = R.n_obj; L.aspect = R.aspect; L.max_bounce = R.max_bounce; L.light_base = R.light_base;
#pragma unroll
    for (int i = 0; i < 4; ++i) L.cutoff[i] = R.cutoff[i];
  }
  return L;
}
template <bool MULTI>
__device__ __forceinline__ uint32_t obj_base_of(const SceneDev& S, uint32_t sid) {
  return MULTI ? S.scenes[sid].obj_base : 0u;
}

// per-ray result of the FP32 scan
struct __align__(16) ScanRec {
  uint16_t cand[8];  // candidate objects, in object order
  uint8_t nc;        // number of candidates; NC_DEAD: the ray is below the colour cutoff
  uint8_t overflow;  // more than CAND candidates: the full solve re-scans every object
  int8_t leaf, face; // refine path: the winner's leaf and rect face
  float t32;         // refine path: the winner's FP32 root
  float thr;         // FP32 bound on the nearest hit distance
  float s32;         // refine path, cubic: the winner's FP32 curve parameter
};
static_assert(sizeof(ScanRec) == 32, "ScanRec is 32 B");
constexpr uint8_t NC_DEAD = 0xff;

// per-ray nearest hit (k_refine / k_full), consumed by k_bounce
struct __align__(16) HitRec {
  df t, px, py, nx, ny;
  float k;           // curvature at the hit
  float ev;          // nearest near-degenerate decision event (full solve)
  uint16_t obj;      // HIT_NONE: no object hit
  uint8_t leaf, flags;
  uint32_t _pad;
};
static_assert(sizeof(HitRec) == 64, "HitRec is 64 B");
constexpr uint16_t HIT_NONE = 0xffff;

struct TraceBufs {
  RayRec* queue[2];
  uint64_t queue_cap;
  ScanRec* scan;       // [queue_cap]
  HitRec* hit;         // [queue_cap]
  uint32_t* list[N_LISTS];  // [queue_cap] each
  lg_segment* segs;
  lg_path_record* paths;
  uint16_t* seg_scene;      // multi-scene traces: the scene of every segment
  const uint32_t* order;    // multi-scene traces, generations > 0: queue entries sorted by scene
  uint64_t seg_cap;
  Counters* ctr;
};

// ------------------------------------------------------------------------------ helpers
// Exact mode keeps FP64 values in the 8-byte df slots of the ray and hit records (the same
// bytes a double would occupy); these move the bits, no arithmetic.
__device__ __forceinline__ double xd(df v) { return __hiloint2double(__float_as_int(v.lo), __float_as_int(v.hi)); }
__device__ __forceinline__ df xdf(double x) { return df{__int_as_float(__double2loint(x)), __int_as_float(__double2hiint(x))}; }
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// ------------------------------------------------------------------- double-float geometry
struct Hit64 {
  df t, px, py, nx, ny;
  float k;       // curvature of the surface at the hit (1/r for circles, 0 for flat faces)
  uint8_t leaf;  // leaf of the object that was hit
};

// Near-degenerate decision events.  ev keeps the smallest ray parameter at which a
// decision (hit or no hit, which side of a boundary) fell inside its band: the relative
// band BAND of the arithmetic, widened to the ray's own error bound tol (world units: how
// far rounding in earlier bounces may have moved the ray), since a decision whose margin is
// below tol may come out either way in any finite precision.
struct Near {
  float ev;   // earliest near decision (ray parameter), INFINITY: none
  float tol;  // position error bound of the ray
};
__device__ __forceinline__ void near_event(Near& n, float t) {
  if (t < 0.0f) t = 0.0f;
  if (t < n.ev) n.ev = t;
}
__device__ __forceinline__ void tmin_band(df t, Near& n) {
  if (t.hi > 1e-11f && t.hi < fmaxf(1e-7f, 4.0f * n.tol)) near_event(n, t.hi);
}
__device__ __forceinline__ bool past_tmin(df t) { return t.hi > 1e-9f || (t.hi == 1e-9f && t.lo > 0.0f); }

// Roots of one leaf: up to 3 hits with t > T_MIN, in ascending order of the leaf's own
// parametrisation (circle: t; rect: entry, exit; cubic: curve parameter).  Each kind is
// one out-of-line function so the kernel keeps a single copy of it in the instruction
// cache however many call sites a ray visit has.
// Discriminant b^2 - a (|f|^2 - r^2) of the ray o + t d against the circle |p - c| = r
// (f = o - c, a = d.d, b = f.d), computed as a (r^2 - |l|^2) with l = f - (b / a) d the
// centre's perpendicular offset from the ray.  For an origin far from a small circle,
// b^2 and a |f|^2 are large and nearly equal and their difference keeps only the
// rounding of |f|^2; l is formed from f directly, so the error stays at the rounding of f.
__device__ __forceinline__ df perp_disc(df fx, df fy, df dx, df dy, df a, df b, df r2) {
  const df s = b / a;
  const df lx = fx - dx * s, ly = fy - dy * s;
  return a * (r2 - (lx * lx + ly * ly));
}

static __device__ __noinline__ int hits_circle(const Leaf64& L, df ox, df oy, df dx, df dy, Hit64* h, Near& ev) {
  int n = 0;
  (void)n;
  const df cx = L.p[0], cy = L.p[1], r = L.p[2];
  const df ocx = ox - cx, ocy = oy - cy;
  const df a = dx * dx + dy * dy, b = ocx * dx + ocy * dy, cc = ocx * ocx + ocy * ocy - r * r;
  const df disc = perp_disc(ocx, ocy, dx, dy, a, b, r * r);
  const float tc = -b.hi / a.hi;
  // a lateral shift tol of the ray moves disc / a = r^2 - perp^2 by at most 2 r tol
  if (fabsf(disc.hi) <= fmaxf(1e-10f * (b.hi * b.hi + fabsf(a.hi * cc.hi)), 2.0f * fabsf(r.hi) * ev.tol * a.hi) &&
      tc > -1e-9f - ev.tol)
    near_event(ev, tc);
  if (df_neg(disc)) return 0;
  const df sq = dsqrt(disc);
  const df q = -(b + (df_neg(b) ? -sq : sq));
  df t1 = DF_ZERO, t2 = DF_ZERO;
  if (q.hi != 0.0f) {
    t1 = q / a;
    t2 = cc / q;
  }
  if (t2 < t1) { const df x = t1; t1 = t2; t2 = x; }
  const df ts[2] = {t1, t2};
  const float rabs = fabsf(r.hi);
  for (int k = 0; k < 2; ++k) {
    tmin_band(ts[k], ev);
    if (past_tmin(ts[k])) {
      const df px = ox + dx * ts[k], py = oy + dy * ts[k];
      const df rinv = DF_ONE / r;
      h[n].t = ts[k]; h[n].px = px; h[n].py = py;
      h[n].nx = (px - cx) * rinv; h[n].ny = (py - cy) * rinv;
      h[n].k = 1.0f / rabs;
      ++n;
    }
  }
  return n;

}

static __device__ __noinline__ int hits_segment(const Leaf64& L, df ox, df oy, df dx, df dy, Hit64* h, Near& ev) {
  const df ax = L.p[0], ay = L.p[1], ex = L.p[2] - ax, ey = L.p[3] - ay;
  const df den = dx * ey - dy * ex;
  const float le = sqrtf(ex.hi * ex.hi + ey.hi * ey.hi), ld = sqrtf(dx.hi * dx.hi + dy.hi * dy.hi);
  const df wx = ax - ox, wy = ay - oy;
  const df cwe = wx * ey - wy * ex;
  if (fabsf(den.hi) <= 1e-10f * le * ld) near_event(ev, den.hi != 0.0f ? cwe.hi / den.hi : 0.0f);
  if (den.hi == 0.0f) return 0;
  const df inv = DF_ONE / den;
  const df t = cwe * inv;
  const df u = (wx * dy - wy * dx) * inv;
  // a lateral shift tol moves the crossing along the segment by tol / sin(angle): du = tol ld / |den|
  const float ub = fmaxf(1e-10f, ev.tol * ld / fabsf(den.hi));
  if (fabsf(u.hi) <= ub || fabsf(u.hi - 1.0f) <= ub) near_event(ev, t.hi);
  if (df_neg(u) || DF_ONE < u) return 0;
  tmin_band(t, ev);
  if (!past_tmin(t)) return 0;
  h[0].t = t; h[0].px = ox + dx * t; h[0].py = oy + dy * t;
  h[0].nx = L.p[4]; h[0].ny = L.p[5];
  h[0].k = 0.0f;
  return 1;

}

static __device__ __noinline__ int hits_rect(const Leaf64& L, df ox, df oy, df dx, df dy, Hit64* h, Near& ev) {
  int n = 0;
  (void)n;
  const df c = L.p[2], s = L.p[3];
  const df rx = ox - L.p[0], ry = oy - L.p[1];
  const df O[2] = {c * rx + s * ry, c * ry - s * rx};
  const df D[2] = {c * dx + s * dy, c * dy - s * dx};
  const df hh[2] = {L.p[4], L.p[5]};
  df tn = -DF_INF, tf = DF_INF, tn_other = -DF_INF;
  float sn = 0.0f, sf = 0.0f;
  int an = -1, af = -1;
  for (int ax = 0; ax < 2; ++ax) {
    if (D[ax].hi == 0.0f) {
      if (fabsf(fabsf(O[ax].hi) - hh[ax].hi) <= fmaxf(1e-10f * hh[ax].hi, ev.tol)) near_event(ev, 0.0f);
      if (hh[ax] < dabs(O[ax])) return 0;
      continue;
    }
    const df inv = DF_ONE / D[ax];
    df t1 = (-hh[ax] - O[ax]) * inv, t2 = (hh[ax] - O[ax]) * inv;
    float s1 = -1.0f, s2 = 1.0f;
    if (t2 < t1) { const df x = t1; t1 = t2; t2 = x; s1 = 1.0f; s2 = -1.0f; }
    if (tn < t1) { tn_other = tn; tn = t1; an = ax; sn = s1; } else if (tn_other < t1) tn_other = t1;
    if (t2 < tf) { tf = t2; af = ax; sf = s2; }
  }
  if (an < 0 || af < 0) return 0;
  const float scale = fabsf(tn.hi) + fabsf(tf.hi) + 1.0f;
  // slab crossings: a lateral shift tol moves each crossing by up to tol / |D| along the ray
  const float dmin = fmaxf(fminf(fabsf(D[0].hi), fabsf(D[1].hi)), 1e-3f);
  const float tb = fmaxf(1e-10f * scale, 2.0f * ev.tol / dmin);
  if (fabsf(tf.hi - tn.hi) <= tb) near_event(ev, tn.hi);
  if (tn_other.hi > -INFINITY && fabsf(tn.hi - tn_other.hi) <= tb) near_event(ev, tn.hi);
  if (tf < tn) return 0;
  tmin_band(tn, ev);
  if (past_tmin(tn)) {
    const float lx = an == 0 ? sn : 0.0f, ly = an == 0 ? 0.0f : sn;
    h[n].t = tn; h[n].px = ox + dx * tn; h[n].py = oy + dy * tn;
    h[n].nx = c * lx - s * ly; h[n].ny = s * lx + c * ly;
    h[n].k = 0.0f;
    ++n;
  }
  tmin_band(tf, ev);
  if (past_tmin(tf)) {
    const float lx = af == 0 ? sf : 0.0f, ly = af == 0 ? 0.0f : sf;
    h[n].t = tf; h[n].px = ox + dx * tf; h[n].py = oy + dy * tf;
    h[n].nx = c * lx - s * ly; h[n].ny = s * lx + c * ly;
    h[n].k = 0.0f;
    ++n;
  }
  return n;

}

static __device__ __noinline__ int hits_cubic(const Leaf64& L, df ox, df oy, df dx, df dy, Hit64* h, Near& ev) {
  int n = 0;
  (void)n;
  const df* v = L.p;
  // power basis B(s) = C3 s^3 + C2 s^2 + C1 s + C0
  const df c0x = v[0], c0y = v[1];
  const df c1x = 3.0f * (v[2] - v[0]), c1y = 3.0f * (v[3] - v[1]);
  const df c2x = 3.0f * (v[4] - 2.0f * v[2]) + 3.0f * v[0], c2y = 3.0f * (v[5] - 2.0f * v[3]) + 3.0f * v[1];
  const df c3x = v[6] + 3.0f * (v[2] - v[4]) - v[0], c3y = v[7] + 3.0f * (v[3] - v[5]) - v[1];
  const df a0 = dx * (c0y - oy) - dy * (c0x - ox);
  const df a1 = dx * c1y - dy * c1x, a2 = dx * c2y - dy * c2x, a3 = dx * c3y - dy * c3x;
  const float scale = fabsf(a0.hi) + fabsf(a1.hi) + fabsf(a2.hi) + fabsf(a3.hi) + 1e-30f;
  const df dd = dx * dx + dy * dy;
  // f(s) = cross(d, B(s) - o) is |d| times a signed distance: a lateral shift tol moves it by tol |d|
  const float fb = fmaxf(1e-10f * scale, ev.tol * sqrtf(dd.hi));
  auto f = [&](df s) { return ((a3 * s + a2) * s + a1) * s + a0; };
  auto tof = [&](df s) {
    const df bx = ((c3x * s + c2x) * s + c1x) * s + c0x, by = ((c3y * s + c2y) * s + c1y) * s + c0y;
    return ((bx - ox) * dx + (by - oy) * dy) / dd;
  };
  df knots[4];
  int nk = 0;
  knots[nk++] = DF_ZERO;
  const df qa = 3.0f * a3, qb = 2.0f * a2, qc = a1;
  if (qa.hi != 0.0f) {
    const df disc = qb * qb - 4.0f * qa * qc;
    if (!df_neg(disc)) {
      const df sq = dsqrt(disc);
      const df q = -0.5f * (qb + (df_neg(qb) ? -sq : sq));
      df r1 = q / qa, r2 = q.hi != 0.0f ? qc / q : r1;
      if (r2 < r1) { const df x = r1; r1 = r2; r2 = x; }
      if (DF_ZERO < r1 && r1 < DF_ONE) knots[nk++] = r1;
      if (DF_ZERO < r2 && r2 < DF_ONE && (nk == 1 || r2 != knots[nk - 1])) knots[nk++] = r2;
    }
  } else if (qb.hi != 0.0f) {
    const df r = -qc / qb;
    if (DF_ZERO < r && r < DF_ONE) knots[nk++] = r;
  }
  knots[nk++] = DF_ONE;
  df roots[3];
  int nr = 0;
  for (int i = 0; i + 1 < nk; ++i) {
    const df lo0 = knots[i], hi0 = knots[i + 1];
    df flo = f(lo0);
    const df fhi = f(hi0);
    if (i > 0 && fabsf(flo.hi) <= fb) near_event(ev, tof(lo0).hi);
    if (flo.hi == 0.0f) {
      if (nr == 0 || roots[nr - 1] != lo0) roots[nr++] = lo0;
      continue;
    }
    if (fhi.hi == 0.0f) {
      if (i + 2 == nk) roots[nr++] = hi0;
      continue;
    }
    if (df_neg(flo) == df_neg(fhi)) continue;
    // safeguarded Newton on the monotone bracket
    df lo = lo0, hi = hi0, sv = DF_HALF * (lo0 + hi0);
    for (int it = 0; it < 64; ++it) {
      const df fs = f(sv);
      if (fs.hi == 0.0f) break;
      if (df_neg(fs) == df_neg(flo)) { lo = sv; flo = fs; } else { hi = sv; }
      const df dfs = (3.0f * a3 * sv + 2.0f * a2) * sv + a1;
      df sn = dfs.hi != 0.0f ? sv - fs / dfs : DF_HALF * (lo + hi);
      if (!(lo < sn && sn < hi)) sn = DF_HALF * (lo + hi);
      // converged: a step at the double-float resolution (the next one would be below it),
      // or a bracket that narrow; a root approached from one side never closes the bracket
      const float tiny = 1e-14f * (1.0f + fabsf(sv.hi));
      if (sn == sv || fabsf((sn - sv).hi) <= 2.0f * tiny || (hi - lo).hi <= tiny) { sv = sn; break; }
      sv = sn;
    }
    roots[nr++] = sv;
  }
  if (fabsf(a0.hi) <= fb) near_event(ev, tof(DF_ZERO).hi);
  if (fabsf(f(DF_ONE).hi) <= fb) near_event(ev, tof(DF_ONE).hi);
  for (int i = 0; i < nr; ++i) {
    const df sv = roots[i];
    const df t = tof(sv);
    tmin_band(t, ev);
    if (!past_tmin(t)) continue;
    const df bx = (3.0f * c3x * sv + 2.0f * c2x) * sv + c1x, by = (3.0f * c3y * sv + 2.0f * c2y) * sv + c1y;
    const df l = dsqrt(bx * bx + by * by);
    h[n].t = t; h[n].px = ox + dx * t; h[n].py = oy + dy * t;
    if (l.hi > 0.0f) {
      const df li = DF_ONE / l;
      h[n].nx = -(by * li); h[n].ny = bx * li;
    } else {
      near_event(ev, t.hi);
      const df li = DF_ONE / dsqrt(dd);
      h[n].nx = -(dy * li); h[n].ny = dx * li;
    }
    // curvature |B' x B''| / |B'|^3
    const float bbx = 6.0f * c3x.hi * sv.hi + 2.0f * c2x.hi, bby = 6.0f * c3y.hi * sv.hi + 2.0f * c2y.hi;
    const float lf = l.hi;
    h[n].k = lf > 0.0f ? fabsf(bx.hi * bby - by.hi * bbx) / (lf * lf * lf) : 1e30f;
    ++n;
  }
  return n;

}

// Ellipse: the ray in the ellipse's frame scaled by (1/a, 1/b) meets the unit circle at the
// same ray parameter; the normal is the normalised gradient (x/a^2, y/b^2).
static __device__ __noinline__ int hits_ellipse(const Leaf64& L, df ox, df oy, df dx, df dy, Hit64* h, Near& ev) {
  int n = 0;
  const df c = L.p[2], s = L.p[3], ia = L.p[6], ib = L.p[7];
  const df rx = ox - L.p[0], ry = oy - L.p[1];
  const df lox = c * rx + s * ry, loy = c * ry - s * rx, ldx = c * dx + s * dy, ldy = c * dy - s * dx;
  const df sox = lox * ia, soy = loy * ib, sdx = ldx * ia, sdy = ldy * ib;
  const df a = sdx * sdx + sdy * sdy, b = sox * sdx + soy * sdy, cc = sox * sox + soy * soy - DF_ONE;
  const df disc = perp_disc(sox, soy, sdx, sdy, a, b, DF_ONE);
  const float tc = -b.hi / a.hi;
  const float mn = fminf(L.p[4].hi, L.p[5].hi), mx = fmaxf(L.p[4].hi, L.p[5].hi);
  // a lateral shift tol is at most tol / min(a, b) in the scaled frame
  if (fabsf(disc.hi) <= fmaxf(1e-10f * (b.hi * b.hi + fabsf(a.hi * cc.hi)), 2.0f * ev.tol / mn * a.hi) &&
      tc > -1e-9f - ev.tol)
    near_event(ev, tc);
  if (df_neg(disc)) return 0;
  const df sq = dsqrt(disc);
  const df q = -(b + (df_neg(b) ? -sq : sq));
  df t1 = DF_ZERO, t2 = DF_ZERO;
  if (q.hi != 0.0f) {
    t1 = q / a;
    t2 = cc / q;
  }
  if (t2 < t1) { const df x = t1; t1 = t2; t2 = x; }
  const df ts[2] = {t1, t2};
  for (int k = 0; k < 2; ++k) {
    tmin_band(ts[k], ev);
    if (!past_tmin(ts[k])) continue;
    const df plx = lox + ldx * ts[k], ply = loy + ldy * ts[k];
    const df gx = plx * ia * ia, gy = ply * ib * ib;
    const df gl = dsqrt(gx * gx + gy * gy);
    const df gi = gl.hi > 0.0f ? DF_ONE / gl : DF_ZERO;
    const df nlx = gx * gi, nly = gy * gi;
    h[n].t = ts[k];
    h[n].px = ox + dx * ts[k];
    h[n].py = oy + dy * ts[k];
    h[n].nx = c * nlx - s * nly;
    h[n].ny = s * nlx + c * nly;
    h[n].k = mx / (mn * mn);  // the largest curvature of the ellipse
    ++n;
  }
  return n;
}

// Half-plane (one edge of a convex polygon): the ray crossing its boundary line.
static __device__ __noinline__ int hits_halfplane(const Leaf64& L, df ox, df oy, df dx, df dy, Hit64* h, Near& ev) {
  const df nx = L.p[2], ny = L.p[3];
  const df den = dx * nx + dy * ny;
  const df dist = (L.p[0] - ox) * nx + (L.p[1] - oy) * ny;
  const float ld = sqrtf(dx.hi * dx.hi + dy.hi * dy.hi);
  const float scale = fabsf(L.p[0].hi) + fabsf(L.p[1].hi) + 1.0f;
  if (fabsf(den.hi) <= 1e-10f * ld && fabsf(dist.hi) <= fmaxf(1e-10f * scale, ev.tol)) near_event(ev, 0.0f);
  if (den.hi == 0.0f) return 0;
  const df t = dist / den;
  tmin_band(t, ev);
  if (!past_tmin(t)) return 0;
  h[0].t = t;
  h[0].px = ox + dx * t;
  h[0].py = oy + dy * t;
  h[0].nx = nx;
  h[0].ny = ny;
  h[0].k = 0.0f;
  return 1;
}

__device__ __forceinline__ int leaf_hits64(const Leaf64& L, df ox, df oy, df dx, df dy, Hit64* h, Near& ev) {
  switch (L.kind) {
    case LEAF_CIRCLE: return hits_circle(L, ox, oy, dx, dy, h, ev);
    case LEAF_SEGMENT: return hits_segment(L, ox, oy, dx, dy, h, ev);
    case LEAF_RECT: return hits_rect(L, ox, oy, dx, dy, h, ev);
    case LEAF_ELLIPSE: return hits_ellipse(L, ox, oy, dx, dy, h, ev);
    case LEAF_HALFPLANE: return hits_halfplane(L, ox, oy, dx, dy, h, ev);
    default: return hits_cubic(L, ox, oy, dx, dy, h, ev);
  }
}

// closed-set membership of a leaf, with a near-boundary flag (within the relative band or
// within tol, the point's own error bound, of the boundary)
__device__ __forceinline__ bool leaf_contains64(const Leaf64& L, df px, df py, bool& near, float tol) {
  if (L.kind == LEAF_CIRCLE) {
    const df dx = px - L.p[0], dy = py - L.p[1], r = L.p[2];
    const df m = dx * dx + dy * dy - r * r;
    if (fabsf(m.hi) <= fmaxf(1e-10f * r.hi * r.hi, 2.0f * fabsf(r.hi) * tol)) near = true;
    return !(DF_ZERO < m);
  }
  if (L.kind == LEAF_RECT) {
    const df c = L.p[2], s = L.p[3], rx = px - L.p[0], ry = py - L.p[1];
    const df lx = c * rx + s * ry, ly = c * ry - s * rx;
    const df ex = dabs(lx) - L.p[4], ey = dabs(ly) - L.p[5];
    const df sd = dmax(ex, ey);
    if (fabsf(sd.hi) <= fmaxf(1e-10f * (L.p[4].hi + L.p[5].hi), tol)) near = true;
    return !(DF_ZERO < sd);
  }
  if (L.kind == LEAF_ELLIPSE) {
    const df c = L.p[2], s = L.p[3], rx = px - L.p[0], ry = py - L.p[1];
    const df u = (c * rx + s * ry) * L.p[6], w = (c * ry - s * rx) * L.p[7];
    const df m = u * u + w * w - DF_ONE;
    if (fabsf(m.hi) <= fmaxf(1e-10f, 2.0f * tol / fminf(L.p[4].hi, L.p[5].hi))) near = true;
    return !(DF_ZERO < m);
  }
  if (L.kind == LEAF_HALFPLANE) {
    const df sd = (px - L.p[0]) * L.p[2] + (py - L.p[1]) * L.p[3];  // > 0: outside
    if (fabsf(sd.hi) <= fmaxf(1e-10f * (fabsf(L.p[0].hi) + fabsf(L.p[1].hi) + 1.0f), tol)) near = true;
    return !(DF_ZERO < sd);
  }
  return false;
}

__device__ __forceinline__ bool prog_eval(const uint8_t* prog, int len, uint64_t mask) {
  uint64_t st = 0;
  int sp = 0;
  for (int i = 0; i < len; ++i) {
    const uint8_t op = prog[i];
    if (op < 0x40) {
      st = (st & ~(1ull << sp)) | (((mask >> op) & 1ull) << sp);
      ++sp;
    } else {
      const bool b = (st >> (sp - 1)) & 1ull, a = (st >> (sp - 2)) & 1ull;
      const bool r = op == PROG_AND ? (a && b) : op == PROG_OR ? (a || b) : (a && !b);
      sp -= 2;
      st = (st & ~(1ull << sp)) | ((uint64_t)r << sp);
      ++sp;
    }
  }
  return st & 1ull;
}

// Object::contains (object.rs:240-259)
static __device__ __noinline__ bool obj_contains64(const SceneDev& S, uint32_t k, df px, df py, bool& near,
                                                   float tol) {
  const ObjInfo oi = S.info[k];
  if (oi.flags & INFO_NO_CONTAINS) return false;
  uint64_t mask = 0;
  for (int i = 0; i < oi.n_leaves; ++i)
    if (leaf_contains64(S.leaves[oi.leaf_begin + i], px, py, near, tol)) mask |= 1ull << i;
  return prog_eval(S.prog + oi.prog_begin, oi.prog_len, mask);
}

// nearest valid hit of one object (geometry intersect + CSG filter)
static __device__ __noinline__ bool obj_solve64(const SceneDev& S, uint32_t k, df ox, df oy, df dx, df dy, Hit64& best,
                                   df& best_d2, Near& ev) {
  const ObjInfo oi = S.info[k];
  const uint8_t* prog = S.prog + oi.prog_begin;
  bool found = false;
  best_d2 = DF_INF;
  for (int li = 0; li < oi.n_leaves; ++li) {
    const Leaf64 L = S.leaves[oi.leaf_begin + li];
    Hit64 h[3];
    const int nh = leaf_hits64(L, ox, oy, dx, dy, h, ev);
    for (int j = 0; j < nh; ++j) {
      if (oi.n_leaves > 1) {
        // keep the hit if flipping this leaf's membership flips the combination
        bool near = false;
        uint64_t mask = 0;
        for (int i = 0; i < oi.n_leaves; ++i)
          if (i != li && leaf_contains64(S.leaves[oi.leaf_begin + i], h[j].px, h[j].py, near, ev.tol)) mask |= 1ull << i;
        if (near) near_event(ev, h[j].t.hi);
        const bool in1 = prog_eval(prog, oi.prog_len, mask | (1ull << li));
        const bool in0 = prog_eval(prog, oi.prog_len, mask & ~(1ull << li));
        if (in1 == in0) continue;
      }
      const df vx = h[j].px - ox, vy = h[j].py - oy;
      const df d2 = vx * vx + vy * vy;
      if (d2 < best_d2) {
        best_d2 = d2;
        best = h[j];
        best.leaf = (uint8_t)li;
        found = true;
      }
    }
  }
  return found;
}

// ------------------------------------------------------------------- FP32 classification
// Per object: key = lower bound of its nearest valid hit (INFINITY: certainly no hit),
// ub = a certainly valid hit distance (INFINITY if none is certain).
struct Class32 {
  float key, ub;
  int leaf, face;  // leaf and face (rect: 2 * axis + (outward sign > 0)) of the root at ub
  float s;         // cubic: curve parameter of the root at ub
};

__device__ __forceinline__ void root32(float t, float tol, Class32& c, bool certain, int leaf, int face, float sv) {
  if (t < -TAU32) return;                     // certainly behind the origin
  if (certain && t > TAU32) {
    if (t < c.ub) { c.ub = t; c.leaf = leaf; c.face = face; c.s = sv; }
    c.key = fminf(c.key, t);
  } else {
    c.key = fminf(c.key, fmaxf(t - tol, 0.0f));
  }
}

// membership of a leaf in FP32 at a point known to within `delta`:
// 1 inside, 0 outside, -1 too close to call
__device__ __forceinline__ int leaf_member32(uint32_t kind, const float* L, float px, float py, float delta) {
  delta += 1e-6f * (fabsf(px) + fabsf(py) + 1.0f);
  if (kind == LEAF_CIRCLE) {
    const float dx = px - L[0], dy = py - L[1], r = L[2];
    const float m = dx * dx + dy * dy - r * r;
    const float band = 2.0f * r * delta + delta * delta + 4e-7f * (dx * dx + dy * dy + r * r);
    return m < -band ? 1 : (m > band ? 0 : -1);
  }
  if (kind == LEAF_RECT) {
    const float rx = px - L[0], ry = py - L[1];
    const float lx = L[2] * rx + L[3] * ry, ly = -L[3] * rx + L[2] * ry;
    const float sd = fmaxf(fabsf(lx) - L[4], fabsf(ly) - L[5]);
    const float band = delta + 1e-6f * (fabsf(rx) + fabsf(ry) + L[4] + L[5]);
    return sd < -band ? 1 : (sd > band ? 0 : -1);
  }
  return 0;  // segments enclose nothing
}

// Roots of a cubic Bezier leaf in FP32: f(s) = cross(d, B(s) - o) is monotone between the
// roots of f', so each sign change between consecutive knots is one root, found by
// bisection.  A knot where |f| is within the FP32 error (tangency, a curve end on the ray)
// or a root where f' is small makes the whole leaf "unknown" (precise solve).
__device__ __forceinline__ int cubic_roots32(const float* A, const float* Bp, float ox, float oy, float dx, float dy,
                                             float* t, bool* cert, float* sv, float& tol, bool& unknown) {
  const float c0x = A[0], c0y = A[1];
  const float c1x = 3.0f * (A[2] - A[0]), c1y = 3.0f * (A[3] - A[1]);
  const float c2x = 3.0f * (A[4] - 2.0f * A[2] + A[0]), c2y = 3.0f * (A[5] - 2.0f * A[3] + A[1]);
  const float c3x = Bp[0] + 3.0f * (A[2] - A[4]) - A[0], c3y = Bp[1] + 3.0f * (A[3] - A[5]) - A[1];
  const float a0 = dx * (c0y - oy) - dy * (c0x - ox);
  const float a1 = dx * c1y - dy * c1x, a2 = dx * c2y - dy * c2x, a3 = dx * c3y - dy * c3x;
  const float sc = fabsf(a0) + fabsf(a1) + fabsf(a2) + fabsf(a3) + 1e-30f;
  const float err = 1e-4f * sc + 2e-6f * (fabsf(c0x) + fabsf(c0y) + fabsf(ox) + fabsf(oy));
  auto f = [&](float u) { return ((a3 * u + a2) * u + a1) * u + a0; };
  float knots[4];
  int nk = 0;
  knots[nk++] = 0.0f;
  const float qa = 3.0f * a3, qb = 2.0f * a2, qc = a1;
  if (fabsf(qa) > 1e-7f * sc) {
    const float disc = qb * qb - 4.0f * qa * qc;
    if (disc >= 0.0f) {
      const float sq = sqrtf(disc);
      const float q = -0.5f * (qb + (qb >= 0.0f ? sq : -sq));
      float r1 = q / qa, r2 = q != 0.0f ? qc / q : r1;
      if (r1 > r2) { const float x = r1; r1 = r2; r2 = x; }
      if (r1 > 0.0f && r1 < 1.0f) knots[nk++] = r1;
      if (r2 > 0.0f && r2 < 1.0f && r2 != knots[nk - 1]) knots[nk++] = r2;
    }
  } else if (fabsf(qb) > 1e-7f * sc) {
    const float r = -qc / qb;
    if (r > 0.0f && r < 1.0f) knots[nk++] = r;
  }
  knots[nk++] = 1.0f;
  int n = 0;
  tol = 1e-6f;
  const float dd = dx * dx + dy * dy;
  for (int i = 0; i + 1 < nk; ++i) {
    float lo = knots[i], hi = knots[i + 1];
    float flo = f(lo);
    const float fhi = f(hi);
    if (fabsf(flo) <= err || fabsf(fhi) <= err) { unknown = true; return 0; }
    if ((flo < 0.0f) == (fhi < 0.0f)) continue;
    // f is monotone between knots: Newton from the secant point, kept inside the sign
    // bracket (a step that leaves it bisects instead), until the step is below 3e-8
    float u = (flo * hi - fhi * lo) / (flo - fhi);
    if (!(u > lo && u < hi)) u = 0.5f * (lo + hi);
    for (int it = 0; it < 40; ++it) {
      const float fu = f(u);
      if (fu == 0.0f) break;  // u is the root (the bracket update below would step off it)
      if ((fu < 0.0f) == (flo < 0.0f)) { lo = u; flo = fu; } else { hi = u; }
      const float fpu = (3.0f * a3 * u + 2.0f * a2) * u + a1;
      float un = u - fu / fpu;
      if (!(un > lo && un < hi)) un = 0.5f * (lo + hi);
      const bool done = fabsf(un - u) <= 3e-8f;
      u = un;
      if (done) break;
    }
    const float fp = (3.0f * a3 * u + 2.0f * a2) * u + a1;
    if (fabsf(fp) < 1e-3f * sc) { unknown = true; return 0; }
    const float bx = ((c3x * u + c2x) * u + c1x) * u + c0x, by = ((c3y * u + c2y) * u + c1y) * u + c0y;
    const float dbx = (3.0f * c3x * u + 2.0f * c2x) * u + c1x, dby = (3.0f * c3y * u + 2.0f * c2y) * u + c1y;
    // constant indices only, so that t, sv and cert stay in registers (n <= 2 here)
    const float tn = ((bx - ox) * dx + (by - oy) * dy) / dd;
    const bool cn = u > 1e-4f && u < 1.0f - 1e-4f;
    if (n == 0) { t[0] = tn; sv[0] = u; cert[0] = cn; }
    else if (n == 1) { t[1] = tn; sv[1] = u; cert[1] = cn; }
    else { t[2] = tn; sv[2] = u; cert[2] = cn; }
    const float tl = fabsf(dbx * dx + dby * dy) * (err / fabsf(fp) + 1e-6f) +
                     2e-6f * (fabsf(bx) + fabsf(by) + fabsf(ox) + fabsf(oy)) + 1e-6f;
    tol = fmaxf(tol, tl);
    ++n;
  }
  return n;
}

// roots of one FP32 leaf: t values with a certainty flag each
__device__ __forceinline__ int leaf_roots32(uint32_t kind, const float* L, const float* L2, float ox, float oy,
                                            float dx, float dy, float* t, bool* cert, int* face, float* sv, float& tol,
                                            bool& unknown) {
  unknown = false;
  face[0] = face[1] = face[2] = -1;
  sv[0] = sv[1] = sv[2] = 0.0f;
  if (kind == LEAF_CUBIC) return cubic_roots32(L, L2, ox, oy, dx, dy, t, cert, sv, tol, unknown);
  if (kind == LEAF_CIRCLE) {
    const float ocx = ox - L[0], ocy = oy - L[1], r = L[2];
    const float b = ocx * dx + ocy * dy, perp = ocx * dy - ocy * dx;
    const float disc = (r - perp) * (r + perp);
    const float scale = fabsf(b) + fabsf(perp) + r;
    tol = 4e-6f * scale + 1e-6f;
    const float band = 2e-5f * scale * scale + 1e-3f * r * r;
    if (disc < -band) return 0;
    if (disc <= band) {  // near-tangent: hit or miss is decided in FP64
      const float w = sqrtf(band) + tol;
      if (-b + w < -TAU32) return 0;  // the tangent point is behind the origin
      t[0] = fmaxf(-b - w, 0.0f);
      cert[0] = false;
      return 1;
    }
    const float sq = sqrtf(disc);
    t[0] = -b - sq; cert[0] = true;
    t[1] = -b + sq; cert[1] = true;
    return 2;
  }
  if (kind == LEAF_SEGMENT) {
    const float ex = L[2], ey = L[3], wx = L[0] - ox, wy = L[1] - oy;
    const float den = dx * ey - dy * ex;
    const float le = fabsf(ex) + fabsf(ey);
    const float wn = fabsf(wx) + fabsf(wy);
    if (fabsf(den) <= 1e-4f * le) { unknown = true; return 0; }
    // one approximate reciprocal (2 ulp) for both quotients: far inside the 4e-6 tolerance
    const float inv = __fdividef(1.0f, den);
    const float t0 = (wx * ey - wy * ex) * inv, u = (wx * dy - wy * dx) * inv;
    tol = 4e-6f * (wn + le) * (1.0f + le * fabsf(inv)) + 1e-6f;
    const float ub = 1e-5f * (1.0f + (wn + le) / le) * (1.0f + le * fabsf(inv));
    if (u < -ub || u > 1.0f + ub) return 0;
    t[0] = t0;
    cert[0] = !(u < ub || u > 1.0f - ub);
    return 1;
  }
  // rect: slab in the local frame
  const float rx = ox - L[0], ry = oy - L[1];
  const float O[2] = {L[2] * rx + L[3] * ry, -L[3] * rx + L[2] * ry};
  const float D[2] = {L[2] * dx + L[3] * dy, -L[3] * dx + L[2] * dy};
  const float H[2] = {L[4], L[5]};
  const float scale = fabsf(rx) + fabsf(ry) + H[0] + H[1];
  float tn = -INFINITY, tf = INFINITY, tn2 = -INFINITY, tf2 = INFINITY;
  int fn = -1, ff = -1;
  for (int ax = 0; ax < 2; ++ax) {
    const float band = 2e-6f * scale + 1e-6f;
    if (fabsf(D[ax]) < 1e-6f) {
      if (fabsf(O[ax]) > H[ax] + band) return 0;
      if (fabsf(O[ax]) >= H[ax] - band) { unknown = true; return 0; }
      continue;
    }
    const float inv = __fdividef(1.0f, D[ax]);  // approximate reciprocal (2 ulp): far inside tol
    float t1 = (-H[ax] - O[ax]) * inv, t2 = (H[ax] - O[ax]) * inv;
    // entering through the -H face when D > 0 (outward normal -1), else the +H face
    int f1 = 2 * ax + (D[ax] > 0.0f ? 0 : 1), f2 = 2 * ax + (D[ax] > 0.0f ? 1 : 0);
    if (t1 > t2) { const float x = t1; t1 = t2; t2 = x; }
    if (t1 > tn) { tn2 = tn; tn = t1; fn = f1; } else { tn2 = fmaxf(tn2, t1); }
    if (t2 < tf) { tf2 = tf; tf = t2; ff = f2; } else { tf2 = fminf(tf2, t2); }
  }
  tol = 4e-6f * (scale + fabsf(tn) + fabsf(tf)) + 1e-6f;
  if (tn > tf + tol) return 0;
  if (tn >= tf - tol) {  // corner graze
    t[0] = tn;
    cert[0] = false;
    return 1;
  }
  // a root whose face is ambiguous (the ray meets a corner) stays uncertain
  t[0] = tn; cert[0] = !(tn - tn2 <= tol); face[0] = fn;
  t[1] = tf; cert[1] = !(tf2 - tf <= tol); face[1] = ff;
  return 2;
}

__device__ __forceinline__ bool op_keep(uint32_t op, bool side_a, bool in_other) {
  if (op == LG_OP_AND) return in_other;
  if (op == LG_OP_OR) return !in_other;
  return side_a ? !in_other : in_other;
}

static // src_leaf: leaf of this object that holds the ray origin (-1: none).  On that leaf the
// root nearest t = 0 is the surface the ray leaves; it is excluded as certain unless the
// leaf's other root is also near 0 (grazing ray or a corner), which stays uncertain.
__device__ __noinline__ Class32 classify32(const ObjScan& r, float ox, float oy, float dx, float dy, float lb,
                                           int src_leaf) {
  Class32 c;
  c.key = INFINITY;
  c.ub = INFINITY;
  c.leaf = -1;
  c.face = -1;
  c.s = 0.0f;
  const uint32_t sk = info_scan(r.info);
  if (sk == SCAN_BOUND) {
    c.key = fmaxf(lb, 0.0f);
    return c;
  }
  const int nleaf = sk == SCAN_TWO ? 2 : 1;
  for (int side = 0; side < nleaf; ++side) {
    const float* L = side == 0 ? r.a : r.b;
    const uint32_t kind = side == 0 ? info_leaf_a(r.info) : info_leaf_b(r.info);
    float t[3] = {0.0f, 0.0f, 0.0f};
    bool cert[3] = {false, false, false};
    int face[3];
    float sv[3];
    float tol = 1e-5f;
    bool unknown = false;
    int n = leaf_roots32(kind, L, r.b, ox, oy, dx, dy, t, cert, face, sv, tol, unknown);
    if (unknown) {  // near-parallel: defer the whole object to the precise solve
      c.key = fminf(c.key, fmaxf(lb, 0.0f));
      continue;
    }
    // the root at the surface the ray leaves (source leaf) is skipped; the arrays are only
    // read at constant indices, so they stay in registers
    int skip = -1;
    if (side == src_leaf && n > 0) {
      int ks = 0;
      float tks = t[0];
      bool cks = cert[0];
#pragma unroll
      for (int k = 1; k < 3; ++k)
        if (k < n && fabsf(t[k]) < fabsf(tks)) { ks = k; tks = t[k]; cks = cert[k]; }
      bool other_near = false;
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (k < n && k != ks && fabsf(t[k]) < 4.0f * TAU32) other_near = true;
      if (fabsf(tks) < TAU32 && cks && !other_near) skip = ks;
    }
    // the roots move through three registers (no dynamically indexed array)
    float ta = t[0], tb = t[1], tc = t[2], sa = sv[0], sb = sv[1], sc2 = sv[2];
    bool ca = cert[0], cb = cert[1], cc = cert[2];
    int fa = face[0], fb = face[1], fc = face[2];
    for (int k = 0; k < n; ++k) {
      const float tk = ta, svk = sa;
      const bool ck = ca;
      const int fk = fa;
      ta = tb; tb = tc; sa = sb; sb = sc2; ca = cb; cb = cc; fa = fb; fb = fc;
      if (k == skip) continue;
      bool certain = ck;
      if (nleaf == 2 && certain) {
        // CSG filter at a well-located hit point; an uncertain root stays a candidate
        if (tk < -TAU32) continue;
        const float px = ox + dx * tk, py = oy + dy * tk;
        const float* Lo = side == 0 ? r.b : r.a;
        const uint32_t ko = side == 0 ? info_leaf_b(r.info) : info_leaf_a(r.info);
        const int m = leaf_member32(ko, Lo, px, py, 4.0f * tol);
        if (m < 0) certain = false;
        else if (!op_keep(info_op(r.info), side == 0, m == 1)) continue;
      }
      root32(tk, tol, c, certain, side, fk, svk);
    }
  }
  return c;
}

// ------------------------------------------------------------------- winner refinement
// The FP32 scan proved that the nearest hit is root `t32` of leaf `leaf` (rect: face
// `face`) with margins far above FP32 error; recompute that one root in double-float
// instead of solving the whole object: two Newton steps on |o + t d - c|^2 = r^2 for a
// circle, the face plane of a rect, the 2x2 solve of a mirror segment.
static __device__ __noinline__ bool refine_root(const SceneDev& S, uint32_t j, int leaf, int face, float t32, float s32,
                                                df ox, df oy, df dx, df dy, Hit64& h) {
  const ObjInfo oi = S.info[j];
  const Leaf64 L = S.leaves[oi.leaf_begin + leaf];
  df t;
  if (L.kind == LEAF_CIRCLE) {
    // Newton from the FP32 root until the step is below 1e-10 of t: the iterate's error is
    // then of the order of the step times the FP32 derivative's relative error.  An FP32
    // root far from the origin (|o - c| >> r) can be off by 1e-3 and takes several steps;
    // no convergence in 8 hands the ray to the full solve.
    t = df{t32, 0.0f};
    bool conv = false;
    for (int it = 0; it < 8 && !conv; ++it) {
      const df vx = ox + dx * t - L.p[0], vy = oy + dy * t - L.p[1];
      const df f = vx * vx + vy * vy - L.p[2] * L.p[2];
      const float fp = 2.0f * (vx.hi * dx.hi + vy.hi * dy.hi);
      if (fp == 0.0f) return false;
      const float step = __fdiv_rn(f.hi, fp);
      t = t - df{step, 0.0f};
      conv = fabsf(step) <= 1e-10f * (1.0f + fabsf(t.hi));
    }
    if (!conv) return false;
    h.px = ox + dx * t;
    h.py = oy + dy * t;
    h.nx = (h.px - L.p[0]) * L.p[3];
    h.ny = (h.py - L.p[1]) * L.p[3];
    h.k = 1.0f / fabsf(L.p[2].hi);
  } else if (L.kind == LEAF_SEGMENT) {
    const df ex = L.p[2] - L.p[0], ey = L.p[3] - L.p[1], wx = L.p[0] - ox, wy = L.p[1] - oy;
    const df den = dx * ey - dy * ex;
    if (den.hi == 0.0f) return false;
    t = (wx * ey - wy * ex) / den;
    h.px = ox + dx * t;
    h.py = oy + dy * t;
    h.nx = L.p[4];
    h.ny = L.p[5];
    h.k = 0.0f;
  } else if (L.kind == LEAF_RECT) {
    (void)s32;
    if (face < 0) return false;
    const int ax = face >> 1;
    const float sg = (face & 1) ? 1.0f : -1.0f;
    const df c = L.p[2], s = L.p[3];
    const df nx = ax == 0 ? c * sg : -(s * sg), ny = ax == 0 ? s * sg : c * sg;  // outward face normal
    const df den = nx * dx + ny * dy;
    if (den.hi == 0.0f) return false;
    const df off = nx * (ox - L.p[0]) + ny * (oy - L.p[1]);
    t = (L.p[4 + ax] - off) / den;
    h.px = ox + dx * t;
    h.py = oy + dy * t;
    h.nx = nx;
    h.ny = ny;
    h.k = 0.0f;
  } else {  // cubic: Newton on f(s) = cross(d, B(s) - o) from the FP32 root
    const df* v = L.p;
    const df c0x = v[0], c0y = v[1];
    const df c1x = 3.0f * (v[2] - v[0]), c1y = 3.0f * (v[3] - v[1]);
    const df c2x = 3.0f * (v[4] - 2.0f * v[2]) + 3.0f * v[0], c2y = 3.0f * (v[5] - 2.0f * v[3]) + 3.0f * v[1];
    const df c3x = v[6] + 3.0f * (v[2] - v[4]) - v[0], c3y = v[7] + 3.0f * (v[3] - v[5]) - v[1];
    const df a0 = dx * (c0y - oy) - dy * (c0x - ox);
    const df a1 = dx * c1y - dy * c1x, a2 = dx * c2y - dy * c2x, a3 = dx * c3y - dy * c3x;
    df u{s32, 0.0f};
    bool conv = false;  // as for the circle: step below 1e-10, at most 8
    for (int it = 0; it < 8 && !conv; ++it) {
      const df fu = ((a3 * u + a2) * u + a1) * u + a0;
      const float fp = (3.0f * a3.hi * u.hi + 2.0f * a2.hi) * u.hi + a1.hi;
      if (fp == 0.0f) return false;
      const float step = __fdiv_rn(fu.hi, fp);
      u = u - df{step, 0.0f};
      conv = fabsf(step) <= 1e-10f;
    }
    if (!conv) return false;
    const df bx = ((c3x * u + c2x) * u + c1x) * u + c0x, by = ((c3y * u + c2y) * u + c1y) * u + c0y;
    t = ((bx - ox) * dx + (by - oy) * dy) / (dx * dx + dy * dy);
    h.px = ox + dx * t;
    h.py = oy + dy * t;
    const df tx = (3.0f * c3x * u + 2.0f * c2x) * u + c1x, ty = (3.0f * c3y * u + 2.0f * c2y) * u + c1y;
    const df l = dsqrt(tx * tx + ty * ty);
    if (!(l.hi > 0.0f)) return false;
    const df li = DF_ONE / l;
    h.nx = -(ty * li);
    h.ny = tx * li;
    const float bbx = 6.0f * c3x.hi * u.hi + 2.0f * c2x.hi, bby = 6.0f * c3y.hi * u.hi + 2.0f * c2y.hi;
    h.k = fabsf(tx.hi * bby - ty.hi * bbx) / (l.hi * l.hi * l.hi);
  }
  h.t = t;
  h.leaf = (uint8_t)leaf;
  return true;
}

// ------------------------------------------------------------------- raster rule
// Pixel space: px = x * H/2 + W/2, py = H/2 - y * H/2 (row 0 at the top).  The major axis
// is the one with the larger extent; one sample per major-axis pixel centre in
// [ceil(a - 1/2), ceil(b - 1/2)), minor coordinate floor(v(i)).  Every operation is a
// single IEEE-rounded f32 op so a CPU restatement reproduces the pixel set exactly.
struct RSetup {
  int xmajor;
  float ua, va, slope;
  int lo, hi;
};

__device__ __forceinline__ bool raster_setup(const lg_segment& s, uint32_t W, uint32_t H, RSetup& R) {
  const float sc = (float)H * 0.5f, cx = (float)W * 0.5f, cy = sc;
  const float X0 = __fmaf_rn(s.x0, sc, cx), Y0 = __fmaf_rn(-s.y0, sc, cy);
  const float X1 = __fmaf_rn(s.x1, sc, cx), Y1 = __fmaf_rn(-s.y1, sc, cy);
  if (!isfinite(X0) || !isfinite(Y0) || !isfinite(X1) || !isfinite(Y1)) return false;
  const float adx = fabsf(__fsub_rn(X1, X0)), ady = fabsf(__fsub_rn(Y1, Y0));
  R.xmajor = adx >= ady;
  float ua, va, ub, vb;
  if (R.xmajor) { ua = X0; va = Y0; ub = X1; vb = Y1; } else { ua = Y0; va = X0; ub = Y1; vb = X1; }
  if (ub < ua) { float t = ua; ua = ub; ub = t; t = va; va = vb; vb = t; }
  const float du = __fsub_rn(ub, ua);
  if (!(du > 0.0f)) return false;
  R.slope = __fdiv_rn(__fsub_rn(vb, va), du);
  R.ua = ua;
  R.va = va;
  const float nmaj = (float)(R.xmajor ? W : H);
  float lo = ceilf(__fsub_rn(ua, 0.5f)), hi = ceilf(__fsub_rn(ub, 0.5f));
  lo = fmaxf(lo, 0.0f);
  hi = fminf(hi, nmaj);
  if (!(lo < hi)) return false;
  R.lo = (int)lo;
  R.hi = (int)hi;
  return true;
}

__device__ __forceinline__ int raster_minor(const RSetup& R, int i) {
  const float v = __fmaf_rn(__fsub_rn(__fadd_rn((float)i, 0.5f), R.ua), R.slope, R.va);
  const float fv = floorf(v);
  if (!(fv >= -1.0f)) return -1;
  if (fv > 2147483000.0f) return 2147483000;
  return (int)fv;
}

__device__ __forceinline__ long long to_fixed(float v) {
  if (v != v) return 0;
  v = fminf(fmaxf(v, -1048576.0f), 1048576.0f);
  return __float2ll_rn(__fmul_rn(v, 4294967296.0f));
}

}  // namespace lgd
