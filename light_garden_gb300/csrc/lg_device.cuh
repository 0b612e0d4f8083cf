// lg_device.cuh — device-side scene tables, geometry and raster rule of the GB300 path.
//
// Scene layout in HBM (built by lg_api.cu from the lg.h tables):
//   ObjScan[n_obj]   64 B per object, FP32: inflated bounding circle + up to two leaves
//                    inline.  This is the table every ray scans; each CTA stages it in
//                    shared memory with one cp.async.bulk copy.
//   ObjInfo[n_obj]   32 B per object: leaf range, membership program, material.
//   Leaf64[n_leaf]   72 B per leaf, FP64 world-space primitive (CSG trees flattened).
//   prog[]           membership programs (postfix over leaf membership bits).
//
// Precision split (tracer.rs:395-424 does one FP64 intersection per object per ray):
//   * the O(objects) scan runs in FP32 and classifies each object as a certain miss, a
//     certain hit at t32 (margins well above FP32 error), or uncertain;
//   * every object that could be the nearest hit (certain hits within the FP32 error of
//     the best, and every uncertain object in front of it) is re-solved in FP64, as are
//     the bounce (reflect / refract), the medium test and the canvas exit.
//   The FP64 work is O(1) per ray visit; the FP32 scan carries the object count.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lg.h"

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
enum : uint32_t { LEAF_CIRCLE = 0, LEAF_RECT = 1, LEAF_SEGMENT = 2, LEAF_CUBIC = 3 };
// ObjScan::info layout
__host__ __device__ inline uint32_t info_scan(uint32_t i) { return i & 0xfu; }
__host__ __device__ inline uint32_t info_leaf_a(uint32_t i) { return (i >> 4) & 0x3u; }
__host__ __device__ inline uint32_t info_leaf_b(uint32_t i) { return (i >> 6) & 0x3u; }
__host__ __device__ inline uint32_t info_op(uint32_t i) { return (i >> 8) & 0x3u; }
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
  double n;           // refractive index
  uint64_t _pad;
};
static_assert(sizeof(ObjInfo) == 32, "ObjInfo is 32 B");

struct __align__(8) Leaf64 {
  uint32_t kind;
  uint32_t _pad;
  double p[8];  // circle cx,cy,r | rect cx,cy,cos,sin,hw,hh | segment ax,ay,bx,by | cubic P0..P3
};
static_assert(sizeof(Leaf64) == 72, "Leaf64 is 72 B");

enum : uint8_t { PROG_AND = 0x80, PROG_OR = 0x81, PROG_AND_NOT = 0x82 };  // < 0x40: push leaf k

struct __align__(16) LightDev {
  double ox, oy, vx, vy;
  double spot_angle;
  double n0;           // start medium (tracer.rs:280-287), filled on the device
  float color[4];
  uint32_t kind, num_rays;
  uint64_t first;      // index of this light's first primary in the virtual gen-0 queue
};

struct __align__(16) RayRec {
  double ox, oy, dx, dy;
  double n;
  uint64_t path;
  float c[4];
  uint32_t prim;
  uint16_t light;
  uint8_t gen, flags;
  uint32_t _pad[2];
};
static_assert(sizeof(RayRec) == 80, "RayRec is 80 B");

struct Counters {
  unsigned long long seg_count;               // ring cursor (= segments demanded)
  unsigned long long queue_count[MAX_GEN + 1]; // entries demanded per generation
  unsigned long long visits, fp64_solves, fallbacks, near;
  unsigned long long pixels, tile_refs, units;
  unsigned long long unit_cursor;
  unsigned int error_flags;
  unsigned int _pad;
};
constexpr unsigned ERR_TMA_TIMEOUT = 1u;

struct SceneDev {
  const ObjScan* scan;
  const ObjInfo* info;
  const Leaf64* leaves;
  const uint8_t* prog;
  LightDev* lights;
  uint32_t n_obj, n_lights;
  uint64_t n_primary;
  double aspect;          // canvas half width (height is 1)
  float cutoff[4];
  uint32_t max_bounce;
  uint32_t record_paths;
};

struct TraceBufs {
  RayRec* queue[2];
  uint64_t queue_cap;
  lg_segment* segs;
  lg_path_record* paths;
  uint64_t seg_cap;
  Counters* ctr;
};

// ------------------------------------------------------------------------------ helpers
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// ------------------------------------------------------------------- FP64 geometry
struct Hit64 {
  double t, px, py, nx, ny;
};

__device__ __forceinline__ void near_event(double& ev, double t) {
  if (t < 0.0) t = 0.0;
  if (t < ev) ev = t;
}
__device__ __forceinline__ void tmin_band(double t, double& ev) {
  if (t > 1e-2 * T_MIN && t < 1e2 * T_MIN) near_event(ev, t);
}

// roots of a leaf: up to 3 hits with t > T_MIN, in ascending order of the leaf's own
// parametrisation (circle: t; rect: entry, exit; cubic: curve parameter)
__device__ inline int leaf_hits64(const Leaf64& L, double ox, double oy, double dx, double dy, Hit64* h,
                                  double& ev) {
  int n = 0;
  switch (L.kind) {
    case LEAF_CIRCLE: {
      const double cx = L.p[0], cy = L.p[1], r = L.p[2];
      const double ocx = ox - cx, ocy = oy - cy;
      const double a = dx * dx + dy * dy, b = ocx * dx + ocy * dy, cc = ocx * ocx + ocy * ocy - r * r;
      const double disc = b * b - a * cc;
      if (fabs(disc) <= BAND * (b * b + fabs(a * cc)) && -b / a > -T_MIN) near_event(ev, -b / a);
      if (disc < 0.0) return 0;
      const double sq = sqrt(disc);
      const double q = -(b + (b >= 0.0 ? sq : -sq));
      double t1 = 0.0, t2 = 0.0;
      if (q != 0.0) {
        t1 = q / a;
        t2 = cc / q;
      }
      if (t1 > t2) { const double x = t1; t1 = t2; t2 = x; }
      const double ts[2] = {t1, t2};
      for (int k = 0; k < 2; ++k) {
        tmin_band(ts[k], ev);
        if (ts[k] > T_MIN) {
          const double px = ox + dx * ts[k], py = oy + dy * ts[k];
          h[n].t = ts[k]; h[n].px = px; h[n].py = py;
          h[n].nx = (px - cx) / r; h[n].ny = (py - cy) / r;
          ++n;
        }
      }
      return n;
    }
    case LEAF_SEGMENT: {
      const double ax = L.p[0], ay = L.p[1], ex = L.p[2] - ax, ey = L.p[3] - ay;
      const double den = dx * ey - dy * ex;
      const double le = sqrt(ex * ex + ey * ey), ld = sqrt(dx * dx + dy * dy);
      const double wx = ax - ox, wy = ay - oy;
      if (fabs(den) <= BAND * le * ld) near_event(ev, den != 0.0 ? (wx * ey - wy * ex) / den : 0.0);
      if (den == 0.0) return 0;
      const double t = (wx * ey - wy * ex) / den;
      const double u = (wx * dy - wy * dx) / den;
      if (fabs(u) <= BAND || fabs(u - 1.0) <= BAND) near_event(ev, t);
      if (u < 0.0 || u > 1.0) return 0;
      tmin_band(t, ev);
      if (!(t > T_MIN)) return 0;
      h[0].t = t; h[0].px = ox + dx * t; h[0].py = oy + dy * t;
      if (le > 0.0) { h[0].nx = -ey / le; h[0].ny = ex / le; } else { h[0].nx = 0.0; h[0].ny = 0.0; }
      return 1;
    }
    case LEAF_RECT: {
      const double c = L.p[2], s = L.p[3];
      const double rx = ox - L.p[0], ry = oy - L.p[1];
      const double O[2] = {c * rx + s * ry, -s * rx + c * ry};
      const double D[2] = {c * dx + s * dy, -s * dx + c * dy};
      const double hh[2] = {L.p[4], L.p[5]};
      double tn = -INFINITY, tf = INFINITY, tn_other = -INFINITY, sn = 0.0, sf = 0.0;
      int an = -1, af = -1;
      for (int ax = 0; ax < 2; ++ax) {
        if (D[ax] == 0.0) {
          if (fabs(fabs(O[ax]) - hh[ax]) <= BAND * hh[ax]) near_event(ev, 0.0);
          if (fabs(O[ax]) > hh[ax]) return 0;
          continue;
        }
        double t1 = (-hh[ax] - O[ax]) / D[ax], t2 = (hh[ax] - O[ax]) / D[ax];
        double s1 = -1.0, s2 = 1.0;
        if (t1 > t2) { const double x = t1; t1 = t2; t2 = x; s1 = 1.0; s2 = -1.0; }
        if (t1 > tn) { tn_other = tn; tn = t1; an = ax; sn = s1; } else if (t1 > tn_other) tn_other = t1;
        if (t2 < tf) { tf = t2; af = ax; sf = s2; }
      }
      if (an < 0 || af < 0) return 0;
      const double scale = fabs(tn) + fabs(tf) + 1.0;
      if (fabs(tf - tn) <= BAND * scale) near_event(ev, tn);
      if (tn_other > -INFINITY && fabs(tn - tn_other) <= BAND * scale) near_event(ev, tn);
      if (tn > tf) return 0;
      tmin_band(tn, ev);
      if (tn > T_MIN) {
        const double lx = an == 0 ? sn : 0.0, ly = an == 0 ? 0.0 : sn;
        h[n].t = tn; h[n].px = ox + dx * tn; h[n].py = oy + dy * tn;
        h[n].nx = c * lx - s * ly; h[n].ny = s * lx + c * ly;
        ++n;
      }
      tmin_band(tf, ev);
      if (tf > T_MIN) {
        const double lx = af == 0 ? sf : 0.0, ly = af == 0 ? 0.0 : sf;
        h[n].t = tf; h[n].px = ox + dx * tf; h[n].py = oy + dy * tf;
        h[n].nx = c * lx - s * ly; h[n].ny = s * lx + c * ly;
        ++n;
      }
      return n;
    }
    default: {  // LEAF_CUBIC: f(s) = cross(d, B(s) - o), roots on [0, 1]
      const double* v = L.p;
      // power basis B(s) = C3 s^3 + C2 s^2 + C1 s + C0
      const double c0x = v[0], c0y = v[1];
      const double c1x = 3.0 * (v[2] - v[0]), c1y = 3.0 * (v[3] - v[1]);
      const double c2x = 3.0 * (v[4] - 2.0 * v[2]) + 3.0 * v[0], c2y = 3.0 * (v[5] - 2.0 * v[3]) + 3.0 * v[1];
      const double c3x = v[6] + 3.0 * (v[2] - v[4]) - v[0], c3y = v[7] + 3.0 * (v[3] - v[5]) - v[1];
      const double a0 = dx * (c0y - oy) - dy * (c0x - ox);
      const double a1 = dx * c1y - dy * c1x, a2 = dx * c2y - dy * c2x, a3 = dx * c3y - dy * c3x;
      const double scale = fabs(a0) + fabs(a1) + fabs(a2) + fabs(a3) + 1e-300;
      const double dd = dx * dx + dy * dy;
      auto f = [&](double s) { return ((a3 * s + a2) * s + a1) * s + a0; };
      auto tof = [&](double s) {
        const double bx = ((c3x * s + c2x) * s + c1x) * s + c0x, by = ((c3y * s + c2y) * s + c1y) * s + c0y;
        return ((bx - ox) * dx + (by - oy) * dy) / dd;
      };
      double knots[4];
      int nk = 0;
      knots[nk++] = 0.0;
      const double qa = 3.0 * a3, qb = 2.0 * a2, qc = a1;
      if (qa != 0.0) {
        const double disc = qb * qb - 4.0 * qa * qc;
        if (disc >= 0.0) {
          const double sq = sqrt(disc);
          const double q = -0.5 * (qb + (qb >= 0.0 ? sq : -sq));
          double r1 = q / qa, r2 = q != 0.0 ? qc / q : r1;
          if (r1 > r2) { const double x = r1; r1 = r2; r2 = x; }
          if (r1 > 0.0 && r1 < 1.0) knots[nk++] = r1;
          if (r2 > 0.0 && r2 < 1.0 && (nk == 1 || r2 != knots[nk - 1])) knots[nk++] = r2;
        }
      } else if (qb != 0.0) {
        const double r = -qc / qb;
        if (r > 0.0 && r < 1.0) knots[nk++] = r;
      }
      knots[nk++] = 1.0;
      double roots[3];
      int nr = 0;
      for (int i = 0; i + 1 < nk; ++i) {
        const double lo0 = knots[i], hi0 = knots[i + 1];
        double flo = f(lo0);
        const double fhi = f(hi0);
        if (i > 0 && fabs(flo) <= BAND * scale) near_event(ev, tof(lo0));
        if (flo == 0.0) {
          if (nr == 0 || roots[nr - 1] != lo0) roots[nr++] = lo0;
          continue;
        }
        if (fhi == 0.0) {
          if (i + 2 == nk) roots[nr++] = hi0;
          continue;
        }
        if ((flo < 0.0) == (fhi < 0.0)) continue;
        // safeguarded Newton on the monotone bracket
        double lo = lo0, hi = hi0, s = 0.5 * (lo0 + hi0);
        for (int it = 0; it < 64; ++it) {
          const double fs = f(s);
          if (fs == 0.0) break;
          if ((fs < 0.0) == (flo < 0.0)) { lo = s; flo = fs; } else { hi = s; }
          const double dfs = (3.0 * a3 * s + 2.0 * a2) * s + a1;
          double sn = dfs != 0.0 ? s - fs / dfs : 0.5 * (lo + hi);
          if (!(sn > lo && sn < hi)) sn = 0.5 * (lo + hi);
          if (sn == s || hi - lo <= 4e-16 * (1.0 + fabs(s))) { s = sn; break; }
          s = sn;
        }
        roots[nr++] = s;
      }
      if (fabs(a0) <= BAND * scale) near_event(ev, tof(0.0));
      if (fabs(f(1.0)) <= BAND * scale) near_event(ev, tof(1.0));
      for (int i = 0; i < nr; ++i) {
        const double s = roots[i];
        const double t = tof(s);
        tmin_band(t, ev);
        if (!(t > T_MIN)) continue;
        const double bx = (3.0 * c3x * s + 2.0 * c2x) * s + c1x, by = (3.0 * c3y * s + 2.0 * c2y) * s + c1y;
        const double l = sqrt(bx * bx + by * by);
        h[n].t = t; h[n].px = ox + dx * t; h[n].py = oy + dy * t;
        if (l > 0.0) { h[n].nx = -by / l; h[n].ny = bx / l; }
        else { near_event(ev, t); const double ld = sqrt(dd); h[n].nx = -dy / ld; h[n].ny = dx / ld; }
        ++n;
      }
      return n;
    }
  }
}

// closed-set membership of a leaf, with a near-boundary flag
__device__ __forceinline__ bool leaf_contains64(const Leaf64& L, double px, double py, bool& near) {
  if (L.kind == LEAF_CIRCLE) {
    const double dx = px - L.p[0], dy = py - L.p[1], r = L.p[2];
    const double m = dx * dx + dy * dy - r * r;
    if (fabs(m) <= BAND * r * r) near = true;
    return m <= 0.0;
  }
  if (L.kind == LEAF_RECT) {
    const double c = L.p[2], s = L.p[3], rx = px - L.p[0], ry = py - L.p[1];
    const double lx = c * rx + s * ry, ly = -s * rx + c * ry;
    const double ex = fabs(lx) - L.p[4], ey = fabs(ly) - L.p[5];
    const double sd = ex > ey ? ex : ey;
    if (fabs(sd) <= BAND * (L.p[4] + L.p[5])) near = true;
    return sd <= 0.0;
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

// Object::contains (object.rs:240-259) in FP64
__device__ inline bool obj_contains64(const SceneDev& S, uint32_t k, double px, double py, bool& near) {
  const ObjInfo oi = S.info[k];
  if (oi.flags & INFO_NO_CONTAINS) return false;
  uint64_t mask = 0;
  for (int i = 0; i < oi.n_leaves; ++i)
    if (leaf_contains64(S.leaves[oi.leaf_begin + i], px, py, near)) mask |= 1ull << i;
  return prog_eval(S.prog + oi.prog_begin, oi.prog_len, mask);
}

// nearest valid hit of one object (geometry intersect + CSG filter), FP64
__device__ inline bool obj_solve64(const SceneDev& S, uint32_t k, double ox, double oy, double dx, double dy,
                                   Hit64& best, double& best_d2, double& ev) {
  const ObjInfo oi = S.info[k];
  const uint8_t* prog = S.prog + oi.prog_begin;
  bool found = false;
  best_d2 = INFINITY;
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
          if (i != li && leaf_contains64(S.leaves[oi.leaf_begin + i], h[j].px, h[j].py, near)) mask |= 1ull << i;
        if (near) near_event(ev, h[j].t);
        const bool in1 = prog_eval(prog, oi.prog_len, mask | (1ull << li));
        const bool in0 = prog_eval(prog, oi.prog_len, mask & ~(1ull << li));
        if (in1 == in0) continue;
      }
      const double vx = h[j].px - ox, vy = h[j].py - oy;
      const double d2 = vx * vx + vy * vy;
      if (d2 < best_d2) {
        best_d2 = d2;
        best = h[j];
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
};

__device__ __forceinline__ void root32(float t, float tol, Class32& c, bool certain) {
  if (t < -TAU32) return;                     // certainly behind the origin
  if (certain && t > TAU32) {
    c.ub = fminf(c.ub, t);
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

// roots of one FP32 leaf: t values with a certainty flag each
__device__ __forceinline__ int leaf_roots32(uint32_t kind, const float* L, float ox, float oy, float dx, float dy,
                                            float* t, bool* cert, float& tol, bool& unknown) {
  unknown = false;
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
    const float t0 = (wx * ey - wy * ex) / den, u = (wx * dy - wy * dx) / den;
    tol = 4e-6f * (wn + le) * (1.0f + le / fabsf(den)) + 1e-6f;
    const float ub = 1e-5f * (1.0f + (wn + le) / le) * (1.0f + le / fabsf(den));
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
  float tn = -INFINITY, tf = INFINITY;
  for (int ax = 0; ax < 2; ++ax) {
    const float band = 2e-6f * scale + 1e-6f;
    if (fabsf(D[ax]) < 1e-6f) {
      if (fabsf(O[ax]) > H[ax] + band) return 0;
      if (fabsf(O[ax]) >= H[ax] - band) { unknown = true; return 0; }
      continue;
    }
    float t1 = (-H[ax] - O[ax]) / D[ax], t2 = (H[ax] - O[ax]) / D[ax];
    if (t1 > t2) { const float x = t1; t1 = t2; t2 = x; }
    tn = fmaxf(tn, t1);
    tf = fminf(tf, t2);
  }
  tol = 4e-6f * (scale + fabsf(tn) + fabsf(tf)) + 1e-6f;
  if (tn > tf + tol) return 0;
  if (tn >= tf - tol) {  // corner graze
    t[0] = tn;
    cert[0] = false;
    return 1;
  }
  t[0] = tn; cert[0] = true;
  t[1] = tf; cert[1] = true;
  return 2;
}

__device__ __forceinline__ bool op_keep(uint32_t op, bool side_a, bool in_other) {
  if (op == LG_OP_AND) return in_other;
  if (op == LG_OP_OR) return !in_other;
  return side_a ? !in_other : in_other;
}

__device__ inline Class32 classify32(const ObjScan& r, float ox, float oy, float dx, float dy, float lb) {
  Class32 c;
  c.key = INFINITY;
  c.ub = INFINITY;
  const uint32_t sk = info_scan(r.info);
  if (sk == SCAN_BOUND) {
    c.key = fmaxf(lb, 0.0f);
    return c;
  }
  const int nleaf = sk == SCAN_TWO ? 2 : 1;
  for (int side = 0; side < nleaf; ++side) {
    const float* L = side == 0 ? r.a : r.b;
    const uint32_t kind = side == 0 ? info_leaf_a(r.info) : info_leaf_b(r.info);
    float t[2];
    bool cert[2];
    float tol = 1e-5f;
    bool unknown = false;
    const int n = leaf_roots32(kind, L, ox, oy, dx, dy, t, cert, tol, unknown);
    if (unknown) {  // near-parallel: defer the whole object to FP64
      c.key = fminf(c.key, fmaxf(lb, 0.0f));
      continue;
    }
    for (int k = 0; k < n; ++k) {
      bool certain = cert[k];
      if (nleaf == 2 && certain) {
        // CSG filter at a well-located hit point; an uncertain root stays a candidate
        if (t[k] < -TAU32) continue;
        const float px = ox + dx * t[k], py = oy + dy * t[k];
        const float* Lo = side == 0 ? r.b : r.a;
        const uint32_t ko = side == 0 ? info_leaf_b(r.info) : info_leaf_a(r.info);
        const int m = leaf_member32(ko, Lo, px, py, 4.0f * tol);
        if (m < 0) certain = false;
        else if (!op_keep(info_op(r.info), side == 0, m == 1)) continue;
      }
      root32(t[k], tol, c, certain);
    }
  }
  return c;
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
