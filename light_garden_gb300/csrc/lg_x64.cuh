// lg_x64.cuh — the exact FP64 precision mode (LG_PRECISION_EXACT): geometry, membership,
// refraction and ray generation in IEEE-754 double with every operation rounded on its own.
//
// Every operation below goes through __dadd_rn / __dsub_rn / __dmul_rn / __ddiv_rn /
// __dsqrt_rn, which the compiler never fuses into a multiply-add, in the order the
// formulas are written.  A CPU program that evaluates the same formulas in the same order
// with plain IEEE doubles (no contraction) gets the same bits; the trace of this mode is
// therefore bit-for-bit the FP64 trace those formulas define.  The definitions follow
// collision2d's primitives as this project restates them (the geometry crate is not
// available): circle by the cancellation-free quadratic (Numerical Recipes 5.6), rect by
// the slab test in its frame, segment by the 2x2 parametric solve, cubic Bezier by the
// sign changes of cross(d, B(s) - o) between the roots of its derivative, each solved by
// safeguarded Newton, ellipse through the unit circle of its scaled frame, convex polygon as its edge
// segments, CSG (Logic) with the children in the node's local frame.
//
// Native FP64 issues at 1/64 of the FP32 rate on GB300, so this mode runs only where the
// trace needs the answer: the FP32 scan (lg_trace.cu) still prunes the object table and
// hands this code the candidates that can be nearest; only those are solved here.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lg.h"

namespace lgx {

constexpr double T_MIN = 1e-9;         // hits at t <= T_MIN are the surface the ray leaves
constexpr double BAND = 1e-10;         // near-degenerate decision band (relative)
constexpr double SPOT_EPSILON = 1e-9;  // SpotLight::set_num_rays |dir.x| < EPSILON
constexpr double PI = 3.141592653589793;
constexpr uint32_t NEAR = LG_PATH_NEAR_DEGENERATE;
constexpr int MAX_DEPTH = 8;    // LOGIC levels of one object's tree in this mode
constexpr int MAX_POLY = 63;

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double sqr(double a) { return __dsqrt_rn(a); }

struct V {
  double x, y;
};
__device__ __forceinline__ V mk(double x, double y) { return V{x, y}; }
__device__ __forceinline__ V vadd(V a, V b) { return mk(add(a.x, b.x), add(a.y, b.y)); }
__device__ __forceinline__ V vsub(V a, V b) { return mk(sub(a.x, b.x), sub(a.y, b.y)); }
__device__ __forceinline__ V vscl(V a, double s) { return mk(mul(a.x, s), mul(a.y, s)); }
__device__ __forceinline__ double dot(V a, V b) { return add(mul(a.x, b.x), mul(a.y, b.y)); }
__device__ __forceinline__ double cross(V a, V b) { return sub(mul(a.x, b.y), mul(a.y, b.x)); }
__device__ __forceinline__ V unit(V a) {
  const double l = sqr(dot(a, a));
  return l > 0.0 ? vscl(a, dvd(1.0, l)) : a;
}
// rotation by (c, s) and its inverse
__device__ __forceinline__ V rot(V a, double c, double s) {
  return mk(sub(mul(c, a.x), mul(s, a.y)), add(mul(s, a.x), mul(c, a.y)));
}
__device__ __forceinline__ V irot(V a, double c, double s) {
  return mk(add(mul(c, a.x), mul(s, a.y)), add(mul(-s, a.x), mul(c, a.y)));
}

// A hit as the object solve keeps it.  The normal is computed later, for the winning hit
// only (object_normal), from what the leaf leaves here, with the same operations the
// immediate computation would take.
struct Hit {
  double t;
  V p;       // the hit point, o + t d of the ray in the frame the caller passed (world after
             // object_hits lifts it through the Logic frames)
  V aux;     // circle: the point in the circle's frame; ellipse: the point in the ellipse's
             // own frame; cubic: (curve parameter, 0)
  int node;  // preorder index of the leaf within its object
  int sub;   // rect: face (axis + 2 if the outward normal points along +axis); polygon: edge
};

// Comparisons on the integer pipe (FP64 compares issue on the 1/64-rate FP64 pipe), each
// equal to the IEEE comparison for the values it is given.
__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
// a < b for a, b in [+0, +inf] (distances squared, curve parameters): the bit patterns of
// non-negative doubles order like the values
__device__ __forceinline__ bool plt(double a, double b) { return bits(a) < bits(b); }
// t > c for a constant 0 < c < inf: false for every negative t, -0 and NaN
__device__ __forceinline__ bool gt_pos(double t, double c) {
  const long long b = bits(t);
  return b > bits(c) && b <= 0x7ff0000000000000ll;
}
// lo < t < hi for constants 0 < lo < hi < inf
__device__ __forceinline__ bool in_pos(double t, double lo, double hi) {
  const long long b = bits(t);
  return b > bits(lo) && b < bits(hi);
}
// x < 0.0 and x == 0.0 for finite or infinite x (not NaN)
__device__ __forceinline__ bool is_neg(double x) { return bits(x) < 0 && (bits(x) << 1) != 0; }
__device__ __forceinline__ bool is_zero(double x) { return (bits(x) << 1) == 0; }

// Near-degenerate decision events: the smallest ray parameter at which a decision (hit or
// no hit, which side of a boundary) fell inside the band.
__device__ __forceinline__ void event(double& ev, double t) {
  if (t < 0.0) t = 0.0;
  if (t < ev) ev = t;
}
__device__ __forceinline__ void tmin_band(double t, double& ev) {
  if (in_pos(t, 1e-2 * T_MIN, 1e2 * T_MIN)) event(ev, t);
}
__device__ __forceinline__ Hit mkhit(double t, V o, V d, V aux, int sub) {
  return Hit{t, vadd(o, vscl(d, t)), aux, 0, sub};
}

// ------------------------------------------------------------------ ray generators
// sin / cos and atan from published methods in plain double operations (the same bits on
// every machine): Cody-Waite reduction by pi/2 (a 33 + 33 + 53-bit split of pi/2) and the
// Taylor series of sin and cos on [-pi/4, pi/4]; atan by the reductions atan(x) = pi/2 -
// atan(1/x) and atan(a) = pi/6 + atan((a sqrt3 - 1) / (a + sqrt3)) and its Taylor series on
// |a| <= tan(pi/12).  Each coefficient is 1/n! or 1/n rounded to double.
__device__ __forceinline__ void sincos_x(double x, double& s_out, double& c_out) {
  const double k = rint(mul(x, 0.6366197723675814));
  const double r = sub(sub(sub(x, mul(k, 1.5707963267341256)), mul(k, 6.077100506303966e-11)),
                       mul(k, 2.0222662487959506e-21));
  const double z = mul(r, r);
  double ps = -8.22063524662433e-18;
  ps = add(mul(ps, z), 2.8114572543455206e-15);
  ps = sub(mul(ps, z), 7.647163731819816e-13);
  ps = add(mul(ps, z), 1.6059043836821613e-10);
  ps = sub(mul(ps, z), 2.505210838544172e-08);
  ps = add(mul(ps, z), 2.7557319223985893e-06);
  ps = sub(mul(ps, z), 0.0001984126984126984);
  ps = add(mul(ps, z), 0.008333333333333333);
  ps = sub(mul(ps, z), 0.16666666666666666);
  const double sn = add(r, mul(mul(r, z), ps));
  double pc = 4.110317623312165e-19;
  pc = sub(mul(pc, z), 1.5619206968586225e-16);
  pc = add(mul(pc, z), 4.779477332387385e-14);
  pc = sub(mul(pc, z), 1.1470745597729725e-11);
  pc = add(mul(pc, z), 2.08767569878681e-09);
  pc = sub(mul(pc, z), 2.755731922398589e-07);
  pc = add(mul(pc, z), 2.48015873015873e-05);
  pc = sub(mul(pc, z), 0.001388888888888889);
  pc = add(mul(pc, z), 0.041666666666666664);
  const double cs = add(sub(1.0, mul(0.5, z)), mul(mul(z, z), pc));
  const long long q = ((long long)k % 4 + 4) % 4;
  s_out = q == 0 ? sn : q == 1 ? cs : q == 2 ? -sn : -cs;
  c_out = q == 0 ? cs : q == 1 ? -sn : q == 2 ? -cs : sn;
}

__device__ __forceinline__ double atan_x(double x) {
  if (x != x) return x;
  const bool neg = x < 0.0;
  double a = fabs(x);
  const bool inv = a > 1.0;
  if (inv) a = dvd(1.0, a);
  const bool off = a > 0.2679491924311227;
  if (off) a = dvd(sub(mul(a, 1.7320508075688772), 1.0), add(a, 1.7320508075688772));
  const double z = mul(a, a);
  double p = -0.034482758620689655;
  p = add(mul(p, z), 0.037037037037037035);
  p = sub(mul(p, z), 0.04);
  p = add(mul(p, z), 0.043478260869565216);
  p = sub(mul(p, z), 0.047619047619047616);
  p = add(mul(p, z), 0.05263157894736842);
  p = sub(mul(p, z), 0.058823529411764705);
  p = add(mul(p, z), 0.06666666666666667);
  p = sub(mul(p, z), 0.07692307692307693);
  p = add(mul(p, z), 0.09090909090909091);
  p = sub(mul(p, z), 0.1111111111111111);
  p = add(mul(p, z), 0.14285714285714285);
  p = sub(mul(p, z), 0.2);
  p = add(mul(p, z), 0.3333333333333333);
  double r = sub(a, mul(mul(a, z), p));
  if (off) r = add(0.5235987755982989, add(r, -5.360408832255455e-17));
  if (inv) r = sub(1.5707963267948966, sub(r, 6.123233995736766e-17));
  return neg ? -r : r;
}

// Primary ray i of a light (light.rs:103-115, 163-174, 225-249).  dir_angle: the spot
// light's base angle, atan_x(dy / dx) or +-pi/2 (filled once per light).
__device__ __forceinline__ void primary_ray_x(uint32_t kind, double lox, double loy, double lvx, double lvy,
                                              double spot_angle, double dir_angle, double n, uint64_t i,
                                              double& ox, double& oy, double& dx, double& dy) {
  if (kind == LG_LIGHT_POINT) {
    const double f = dvd(mul(mul((double)i, PI), 2.0), n);
    double s, c;
    sincos_x(f, s, c);
    ox = lox; oy = loy; dx = c; dy = s;
  } else if (kind == LG_LIGHT_SPOT) {
    const double min_angle = sub(dir_angle, mul(0.5, spot_angle));
    const double ang = add(min_angle, mul(dvd((double)(i + 1), n), spot_angle));
    const double sign = signbit(lvx) ? -1.0 : 1.0;
    double s, c;
    sincos_x(ang, s, c);
    ox = lox; oy = loy; dx = mul(sign, c); dy = mul(sign, s);
  } else {  // directional: origins a + (i / n)(b - a), unit left normal of b - a
    const V e = mk(sub(lvx, lox), sub(lvy, loy));
    const double r = dvd((double)i, n);
    ox = add(lox, mul(e.x, r));
    oy = add(loy, mul(e.y, r));
    const V nd = unit(mk(-e.y, e.x));
    dx = nd.x; dy = nd.y;
  }
}
__device__ __forceinline__ double spot_base_angle(double sx, double sy) {
  return fabs(sx) < SPOT_EPSILON ? (sy >= 0.0 ? mul(PI, 0.5) : mul(-PI, 0.5)) : atan_x(dvd(sy, sx));
}

// ------------------------------------------------------------------ leaves: membership
__device__ __forceinline__ int poly_vertices(const lg_geo* G, const lg_geo& g, V* out) {
  const int n = g.a;
  int k = 0;
  const lg_geo* cur = &g;
  while (k < n) {
    for (int i = 0; i < 4 && k < n; ++i, ++k) out[k] = mk(cur->v[2 * i], cur->v[2 * i + 1]);
    if (k < n) cur = &G[cur->b];
  }
  return n;
}
__device__ __forceinline__ double poly_orientation(const V* P, int n) {
  double a = 0.0;
  for (int i = 0; i < n; ++i) a = add(a, cross(P[i], P[(i + 1) % n]));
  return a >= 0.0 ? 1.0 : -1.0;
}

// closed membership of one leaf, p in the leaf's frame; fl (optional) receives NEAR when the
// point lies within the band of the boundary
static __device__ __noinline__ bool leaf_contains(const lg_geo* G, const lg_geo& g, V p, uint32_t* fl) {
  switch (g.kind) {
    case LG_GEO_CIRCLE: {
      const V d = vsub(p, mk(g.origin[0], g.origin[1]));
      const double r = g.v[0];
      const double m = sub(dot(d, d), mul(r, r));
      if (fl && fabs(m) <= mul(mul(BAND, r), r)) *fl |= NEAR;
      return m <= 0.0;
    }
    case LG_GEO_RECT: {
      const V l = irot(vsub(p, mk(g.origin[0], g.origin[1])), g.rot[0], g.rot[1]);
      const double hw = mul(0.5, g.v[0]), hh = mul(0.5, g.v[1]);
      const double ex = sub(fabs(l.x), hw), ey = sub(fabs(l.y), hh);
      const double sd = ex > ey ? ex : ey;
      if (fl && fabs(sd) <= mul(BAND, add(hw, hh))) *fl |= NEAR;
      return sd <= 0.0;
    }
    case LG_GEO_POLYGON: {
      V P[MAX_POLY];
      const int n = poly_vertices(G, g, P);
      const double sgn = poly_orientation(P, n);
      const V l = irot(vsub(p, mk(g.origin[0], g.origin[1])), g.rot[0], g.rot[1]);
      bool in = true;
      for (int i = 0; i < n; ++i) {
        const V e = vsub(P[(i + 1) % n], P[i]);
        const double le = sqr(dot(e, e));
        const double sd = dvd(mul(-sgn, cross(e, vsub(l, P[i]))), le > 0.0 ? le : 1.0);
        if (fl && fabs(sd) <= mul(BAND, add(le, 1e-300))) *fl |= NEAR;
        if (sd > 0.0) in = false;
      }
      return in;
    }
    case LG_GEO_ELLIPSE: {
      const V l = irot(vsub(p, mk(g.origin[0], g.origin[1])), g.rot[0], g.rot[1]);
      const double u = dvd(l.x, g.v[0]), w = dvd(l.y, g.v[1]);
      const double m = sub(add(mul(u, u), mul(w, w)), 1.0);
      if (fl && fabs(m) <= BAND) *fl |= NEAR;
      return m <= 0.0;
    }
    default:  // segments and cubics enclose nothing
      return false;
  }
}

// ------------------------------------------------------------------ leaves: hits
// Each calls emit(Hit) for every hit with t > T_MIN, in collision2d order; the normals are
// left to leaf_normal.
template <class F>
__device__ __forceinline__ void hits_circle(const lg_geo& g, V o, V d, double& ev, F&& emit) {
  const V c = mk(g.origin[0], g.origin[1]);
  const double r = g.v[0];
  const V oc = vsub(o, c);
  const double a = dot(d, d), b = dot(oc, d), cc = sub(dot(oc, oc), mul(r, r));
  const double disc = sub(mul(b, b), mul(a, cc));
  if (fabs(disc) <= mul(BAND, add(mul(b, b), fabs(mul(a, cc)))) && dvd(-b, a) > -T_MIN) event(ev, dvd(-b, a));
  if (is_neg(disc)) return;
  const double sq = sqr(disc);
  const double q = -add(b, b >= 0.0 ? sq : -sq);
  double t1, t2;
  if (!is_zero(q)) {
    t1 = dvd(q, a);
    t2 = dvd(cc, q);
  } else {
    t1 = t2 = 0.0;
  }
  if (t1 > t2) { const double x = t1; t1 = t2; t2 = x; }
  const double ts[2] = {t1, t2};
  for (int k = 0; k < 2; ++k) {
    tmin_band(ts[k], ev);
    if (gt_pos(ts[k], T_MIN)) {
      const V p = vadd(o, vscl(d, ts[k]));
      emit(Hit{ts[k], p, p, 0, 0});
    }
  }
}

template <class F>
__device__ __forceinline__ void hits_segment(V A, V Bp, V o, V d, double& ev, F&& emit) {
  const V e = vsub(Bp, A);
  const double den = cross(d, e);
  const V w = vsub(A, o);
  // |den| <= BAND |e| |d| needs both lengths (square roots) only when |den| is that small:
  // |e| <= |ex| + |ey| and |d| <= |dx| + |dy|, so a |den| above twice that bound settles it
  const float lb = 2e-10f * ((float)fabs(e.x) + (float)fabs(e.y)) * ((float)fabs(d.x) + (float)fabs(d.y));
  if (!(lb > 1e-30f) || !((float)fabs(den) > lb)) {
    const double le = sqr(dot(e, e)), ld = sqr(dot(d, d));
    if (fabs(den) <= mul(mul(BAND, le), ld)) event(ev, !is_zero(den) ? dvd(cross(w, e), den) : 0.0);
  }
  if (is_zero(den)) return;
  const double t = dvd(cross(w, e), den);
  const double u = dvd(cross(w, d), den);
  if (fabs(u) <= BAND || fabs(sub(u, 1.0)) <= BAND) event(ev, t);
  if (is_neg(u) || u > 1.0) return;
  tmin_band(t, ev);
  if (!gt_pos(t, T_MIN)) return;
  emit(mkhit(t, o, d, mk(0.0, 0.0), 0));
}

template <class F>
__device__ __forceinline__ void hits_rect(const lg_geo& g, V o, V d, double& ev, F&& emit) {
  const double c = g.rot[0], s = g.rot[1];
  const V ctr = mk(g.origin[0], g.origin[1]);
  const V lo = irot(vsub(o, ctr), c, s), ld = irot(d, c, s);
  const double h[2] = {mul(0.5, g.v[0]), mul(0.5, g.v[1])};
  const double O[2] = {lo.x, lo.y}, D[2] = {ld.x, ld.y};
  double tn = -INFINITY, tf = INFINITY;
  int an = -1, af = -1;
  double sn = 0.0, sf = 0.0;  // outward sign of the entry / exit face
  double tn_other = -INFINITY;
  for (int ax = 0; ax < 2; ++ax) {
    if (is_zero(D[ax])) {
      if (fabs(sub(fabs(O[ax]), h[ax])) <= mul(BAND, h[ax])) event(ev, 0.0);
      if (fabs(O[ax]) > h[ax]) return;
      continue;
    }
    double t1 = dvd(sub(-h[ax], O[ax]), D[ax]);
    double t2 = dvd(sub(h[ax], O[ax]), D[ax]);
    double s1 = -1.0, s2 = 1.0;
    if (t1 > t2) { const double x = t1; t1 = t2; t2 = x; s1 = 1.0; s2 = -1.0; }
    if (t1 > tn) { tn_other = tn; tn = t1; an = ax; sn = s1; } else if (t1 > tn_other) tn_other = t1;
    if (t2 < tf) { tf = t2; af = ax; sf = s2; }
  }
  if (an < 0 || af < 0) return;  // degenerate direction
  const double scale = add(add(fabs(tn), fabs(tf)), 1.0);
  if (fabs(sub(tf, tn)) <= mul(BAND, scale)) event(ev, tn);                          // corner graze
  if (tn_other > -INFINITY && fabs(sub(tn, tn_other)) <= mul(BAND, scale)) event(ev, tn);  // corner entry
  if (tn > tf) return;
  tmin_band(tn, ev);
  if (gt_pos(tn, T_MIN)) emit(mkhit(tn, o, d, mk(0.0, 0.0), an + (sn > 0.0 ? 2 : 0)));
  tmin_band(tf, ev);
  if (gt_pos(tf, T_MIN)) emit(mkhit(tf, o, d, mk(0.0, 0.0), af + (sf > 0.0 ? 2 : 0)));
}

// cubic in power basis: B(s) = c3 s^3 + c2 s^2 + c1 s + c0
struct Cubic {
  V c0, c1, c2, c3;
};
__device__ __forceinline__ Cubic cubic_of(const double* v) {
  const V P0 = mk(v[0], v[1]), P1 = mk(v[2], v[3]), P2 = mk(v[4], v[5]), P3 = mk(v[6], v[7]);
  Cubic k;
  k.c0 = P0;
  k.c1 = vscl(vsub(P1, P0), 3.0);
  k.c2 = vadd(vscl(vsub(P2, vscl(P1, 2.0)), 3.0), vscl(P0, 3.0));
  k.c3 = vsub(vadd(P3, vscl(vsub(P1, P2), 3.0)), P0);
  return k;
}
__device__ __forceinline__ double poly3(const double* a, double s) {
  return add(mul(add(mul(add(mul(a[3], s), a[2]), s), a[1]), s), a[0]);
}
__device__ __forceinline__ V cubic_point(const Cubic& k, double s) {
  return vadd(vadd(vadd(vscl(k.c3, mul(mul(s, s), s)), vscl(k.c2, mul(s, s))), vscl(k.c1, s)), k.c0);
}
__device__ __forceinline__ V cubic_tangent(const Cubic& k, double s) {
  return vadd(vadd(vscl(k.c3, mul(mul(3.0, s), s)), vscl(k.c2, mul(2.0, s))), k.c1);
}
__device__ __forceinline__ double cubic_t(const Cubic& k, double s, V o, V d) {
  return dvd(dot(vsub(cubic_point(k, s), o), d), dot(d, d));
}
// The root of f between knots lo < hi in [0, 1] (f(lo) = flo != 0, f(hi) of the other sign):
// ten bisection steps, then Newton steps from the bracket's midpoint kept inside the bracket
// (a step that leaves it bisects instead) until a step moves it by 1e-15 or less (Numerical
// Recipes 9.4, rtsafe); if twelve steps do not get there, bisection of the remaining bracket
// to full precision.  The bracket and the points tried are non-negative, so the comparisons
// run on the integer pipe with the FP64 comparisons' results.
static __device__ __noinline__ double cubic_root(const double* a, double lo, double hi, double flo) {
  const bool neg_lo = is_neg(flo);
  for (int it = 0; it < 10; ++it) {
    const double mid = mul(0.5, add(lo, hi));
    if (!plt(lo, mid) || !plt(mid, hi)) return mid;
    const double fm = poly3(a, mid);
    if (is_zero(fm)) return mid;
    if (is_neg(fm) == neg_lo) lo = mid; else hi = mid;
  }
  double s = mul(0.5, add(lo, hi));
  for (int it = 0; it < 12; ++it) {
    const double f = poly3(a, s);
    if (is_zero(f)) return s;
    if (is_neg(f) == neg_lo) lo = s; else hi = s;
    const double fp = add(mul(add(mul(mul(3.0, a[3]), s), mul(2.0, a[2])), s), a[1]);
    double sn = sub(s, dvd(f, fp));
    if (!(plt(lo, sn) && plt(sn, hi))) sn = mul(0.5, add(lo, hi));
    const double step = sub(sn, s);
    s = sn;
    if (fabs(step) <= 1e-15) return s;
  }
  for (int it = 0; it < 200; ++it) {
    const double mid = mul(0.5, add(lo, hi));
    if (!plt(lo, mid) || !plt(mid, hi)) return mid;
    const double fm = poly3(a, mid);
    if (is_zero(fm)) return mid;
    if (is_neg(fm) == neg_lo) lo = mid; else hi = mid;
  }
  return mul(0.5, add(lo, hi));
}

template <class F>
__device__ __forceinline__ void hits_cubic(const lg_geo& g, V o, V d, double& ev, F&& emit) {
  const Cubic k = cubic_of(g.v);
  const double a[4] = {cross(d, vsub(k.c0, o)), cross(d, k.c1), cross(d, k.c2), cross(d, k.c3)};
  const double scale = add(add(add(add(fabs(a[0]), fabs(a[1])), fabs(a[2])), fabs(a[3])), 1e-300);
  // critical points: 3 a3 s^2 + 2 a2 s + a1 = 0
  double cr[2];
  int ncr = 0;
  const double qa = mul(3.0, a[3]), qb = mul(2.0, a[2]), qc = a[1];
  if (qa != 0.0) {
    const double disc = sub(mul(qb, qb), mul(mul(4.0, qa), qc));
    if (disc >= 0.0) {
      const double sq = sqr(disc);
      const double q = mul(-0.5, add(qb, qb >= 0 ? sq : -sq));
      double r1 = dvd(q, qa), r2 = q != 0.0 ? dvd(qc, q) : r1;
      if (r1 > r2) { const double x = r1; r1 = r2; r2 = x; }
      if (r1 > 0.0 && r1 < 1.0) cr[ncr++] = r1;
      if (r2 > 0.0 && r2 < 1.0 && (ncr == 0 || r2 != cr[0])) cr[ncr++] = r2;
    }
  } else if (qb != 0.0) {
    const double r = dvd(-qc, qb);
    if (r > 0.0 && r < 1.0) cr[ncr++] = r;
  }
  double knots[4];
  int nk = 0;
  knots[nk++] = 0.0;
  for (int i = 0; i < ncr; ++i) knots[nk++] = cr[i];
  knots[nk++] = 1.0;
  double roots[4];
  int nr = 0;
  for (int i = 0; i + 1 < nk; ++i) {
    const double lo = knots[i], hi = knots[i + 1];
    const double flo = poly3(a, lo), fhi = poly3(a, hi);
    if (i > 0 && fabs(flo) <= mul(BAND, scale)) event(ev, cubic_t(k, lo, o, d));  // tangency
    if (is_zero(flo)) {
      if (nr == 0 || roots[nr - 1] != lo) roots[nr++] = lo;
      continue;
    }
    if (is_zero(fhi)) {
      if (i + 2 == nk) roots[nr++] = hi;
      continue;
    }
    if (is_neg(flo) != is_neg(fhi)) roots[nr++] = cubic_root(a, lo, hi, flo);
  }
  if (fabs(a[0]) <= mul(BAND, scale)) event(ev, cubic_t(k, 0.0, o, d));  // end points
  if (fabs(poly3(a, 1.0)) <= mul(BAND, scale)) event(ev, cubic_t(k, 1.0, o, d));
  const double dd = dot(d, d);
  for (int i = 0; i < nr; ++i) {
    const double s = roots[i];
    const V B = cubic_point(k, s);
    const double t = dvd(dot(vsub(B, o), d), dd);
    tmin_band(t, ev);
    if (!gt_pos(t, T_MIN)) continue;
    const V dB = cubic_tangent(k, s);
    if (is_zero(dot(dB, dB))) event(ev, t);  // |B'(s)| == 0: the normal falls back to the ray's
    emit(mkhit(t, o, d, mk(s, 0.0), 0));
  }
}

template <class F>
__device__ __forceinline__ void hits_polygon(const lg_geo* G, const lg_geo& g, V o, V d, double& ev, F&& emit) {
  V P[MAX_POLY];
  const int n = poly_vertices(G, g, P);
  const double c = g.rot[0], s = g.rot[1];
  const V org = mk(g.origin[0], g.origin[1]);
  const V lo = irot(vsub(o, org), c, s), ld = irot(d, c, s);
  for (int i = 0; i < n; ++i)
    hits_segment(P[i], P[(i + 1) % n], lo, ld, ev, [&](const Hit& h) { emit(mkhit(h.t, o, d, mk(0.0, 0.0), i)); });
}

template <class F>
__device__ __forceinline__ void hits_ellipse(const lg_geo& g, V o, V d, double& ev, F&& emit) {
  const double c = g.rot[0], s = g.rot[1], A = g.v[0], Bb = g.v[1];
  const V org = mk(g.origin[0], g.origin[1]);
  const V lo = irot(vsub(o, org), c, s), ld = irot(d, c, s);
  const V so = mk(dvd(lo.x, A), dvd(lo.y, Bb)), sd = mk(dvd(ld.x, A), dvd(ld.y, Bb));
  const double a = dot(sd, sd), b = dot(so, sd), cc = sub(dot(so, so), 1.0);
  const double disc = sub(mul(b, b), mul(a, cc));
  if (fabs(disc) <= mul(BAND, add(mul(b, b), fabs(mul(a, cc)))) && dvd(-b, a) > -T_MIN) event(ev, dvd(-b, a));
  if (is_neg(disc)) return;
  const double sq = sqr(disc);
  const double q = -add(b, b >= 0.0 ? sq : -sq);
  double t1 = 0.0, t2 = 0.0;
  if (!is_zero(q)) {
    t1 = dvd(q, a);
    t2 = dvd(cc, q);
  }
  if (t1 > t2) { const double x = t1; t1 = t2; t2 = x; }
  const double ts[2] = {t1, t2};
  for (int k = 0; k < 2; ++k) {
    tmin_band(ts[k], ev);
    if (gt_pos(ts[k], T_MIN)) emit(mkhit(ts[k], o, d, vadd(lo, vscl(ld, ts[k])), 0));
  }
}

template <class F>
__device__ __forceinline__ void leaf_hits(const lg_geo* G, const lg_geo& g, V o, V d, double& ev, F&& emit) {
  switch (g.kind) {
    case LG_GEO_CIRCLE: hits_circle(g, o, d, ev, emit); break;
    case LG_GEO_RECT: hits_rect(g, o, d, ev, emit); break;
    case LG_GEO_SEGMENT: hits_segment(mk(g.v[0], g.v[1]), mk(g.v[2], g.v[3]), o, d, ev, emit); break;
    case LG_GEO_CUBIC: hits_cubic(g, o, d, ev, emit); break;
    case LG_GEO_POLYGON: hits_polygon(G, g, o, d, ev, emit); break;
    case LG_GEO_ELLIPSE: hits_ellipse(g, o, d, ev, emit); break;
    default: break;
  }
}

// The normal of a leaf's hit (collision2d's formulas: (p - c) / r, the rect face, the unit
// left normal of a segment, the unit left normal of B'(s), a polygon edge's outward unit
// normal, the normalised gradient of an ellipse), in the leaf's parent frame.  d: the ray
// direction in that frame (the cubic's fallback when B'(s) = 0).
static __device__ __noinline__ V leaf_normal(const lg_geo* G, const lg_geo& g, const Hit& h, V d) {
  switch (g.kind) {
    case LG_GEO_CIRCLE:
      return vscl(vsub(h.aux, mk(g.origin[0], g.origin[1])), dvd(1.0, g.v[0]));
    case LG_GEO_RECT: {
      const double sg = (h.sub & 2) ? 1.0 : -1.0;
      const V nn = (h.sub & 1) == 0 ? mk(sg, 0.0) : mk(0.0, sg);
      return rot(nn, g.rot[0], g.rot[1]);
    }
    case LG_GEO_SEGMENT: {
      const V e = vsub(mk(g.v[2], g.v[3]), mk(g.v[0], g.v[1]));
      const double le = sqr(dot(e, e));
      return le > 0.0 ? mk(dvd(-e.y, le), dvd(e.x, le)) : mk(0.0, 0.0);
    }
    case LG_GEO_CUBIC: {
      const V dB = cubic_tangent(cubic_of(g.v), h.aux.x);
      const double l = sqr(dot(dB, dB));
      return l > 0.0 ? mk(dvd(-dB.y, l), dvd(dB.x, l)) : unit(mk(-d.y, d.x));
    }
    case LG_GEO_POLYGON: {
      V P[MAX_POLY];
      const int n = poly_vertices(G, g, P);
      const double sgn = poly_orientation(P, n);
      const V e = vsub(P[(h.sub + 1) % n], P[h.sub]);
      return rot(unit(vscl(mk(e.y, -e.x), sgn)), g.rot[0], g.rot[1]);
    }
    case LG_GEO_ELLIPSE: {
      const double A = g.v[0], Bb = g.v[1];
      const V gr = unit(mk(dvd(h.aux.x, mul(A, A)), dvd(h.aux.y, mul(Bb, Bb))));
      return rot(gr, g.rot[0], g.rot[1]);
    }
    default:
      return mk(0.0, 0.0);
  }
}

// ------------------------------------------------------------------ objects (geometry trees)
// One object's tree in preorder, built on the host: node i names its lg_geo, its depth
// (root 0), its parent (-1 for the root), which child of the parent it is (0: a, 1: b), and
// the end of its subtree (preorder index one past its last descendant).  Indices are
// relative to the object's first node.
struct __align__(16) XNode {
  int32_t geo;
  int32_t end;
  int16_t parent;
  uint8_t depth, side;
  uint32_t leaf_ord;  // leaf number of this node in the flattened leaf table (its first
                      // edge for a polygon), as the FP32 scan counts an object's leaves
};
static_assert(sizeof(XNode) == 16, "XNode is 16 B");

// Membership of the subtree [lo, hi) (its root nd[lo]), p in the frame of the root's
// parameters (geo_contains of a Logic node: the point in the node's frame, both children
// evaluated, combined by the op).
static __device__ __noinline__ bool subtree_contains(const lg_geo* G, const XNode* nd, int lo, int hi, V p,
                                                     uint32_t* fl) {
  if (hi - lo == 1) return leaf_contains(G, G[nd[lo].geo], p, fl);
  V pt[MAX_DEPTH + 1];
  bool vs[MAX_DEPTH + 2];
  int ls[MAX_DEPTH + 1];
  int sp = 0, lsp = 0;
  const int base = nd[lo].depth;
  pt[0] = p;
  for (int i = lo; i < hi; ++i) {
    const int D = nd[i].depth - base;
    const lg_geo& g = G[nd[i].geo];
    if (g.kind == LG_GEO_LOGIC) {
      pt[D + 1] = irot(vsub(pt[D], mk(g.origin[0], g.origin[1])), g.rot[0], g.rot[1]);
      ls[lsp++] = i;
    } else {
      vs[sp++] = leaf_contains(G, g, pt[D], fl);
    }
    while (lsp > 0 && nd[ls[lsp - 1]].end == i + 1) {
      const lg_geo& L = G[nd[ls[--lsp]].geo];
      const bool b = vs[--sp], a = vs[--sp];
      vs[sp++] = L.op == LG_OP_AND ? (a && b) : L.op == LG_OP_OR ? (a || b) : (a && !b);
    }
  }
  return vs[0];
}

// All hits of one object's tree with the ray (o, d) in world coordinates, in collision2d
// order (a Logic node lists child a's kept hits, then child b's), each passed to emit(Hit)
// with its point in world coordinates.  A child hit survives a Logic node when the other
// child's membership (at the hit point in the node's frame) makes it a boundary of the
// combination; surviving points move to the parent's frame.
template <class F>
__device__ __forceinline__ void object_hits(const lg_geo* G, const XNode* nd, int nn, V o, V d, double& ev,
                                            F&& emit) {
  if (nn == 1) {
    leaf_hits(G, G[nd[0].geo], o, d, ev, emit);
    return;
  }
  V ro[MAX_DEPTH + 1], rd[MAX_DEPTH + 1];
  ro[0] = o;
  rd[0] = d;
  for (int i = 0; i < nn; ++i) {
    const lg_geo& g = G[nd[i].geo];
    const int D = nd[i].depth;
    if (g.kind == LG_GEO_LOGIC) {
      ro[D + 1] = irot(vsub(ro[D], mk(g.origin[0], g.origin[1])), g.rot[0], g.rot[1]);
      rd[D + 1] = irot(rd[D], g.rot[0], g.rot[1]);
      continue;
    }
    leaf_hits(G, g, ro[D], rd[D], ev, [&](Hit h) {
      h.node = i;
      int cur = i, j = nd[i].parent;
      while (j >= 0) {
        const lg_geo& L = G[nd[j].geo];
        // the other child of j: b's subtree follows a's
        const bool from_a = nd[cur].side == 0;
        const int olo = from_a ? nd[cur].end : j + 1, ohi = from_a ? nd[j].end : cur;
        uint32_t cfl = 0;
        const bool in_other = subtree_contains(G, nd, olo, ohi, h.p, &cfl);
        if (cfl) event(ev, h.t);
        const bool keep = L.op == LG_OP_AND ? in_other : L.op == LG_OP_OR ? !in_other : (from_a ? !in_other : in_other);
        if (!keep) return;
        h.p = vadd(mk(L.origin[0], L.origin[1]), rot(h.p, L.rot[0], L.rot[1]));
        cur = j;
        j = nd[j].parent;
      }
      emit(h);
    });
  }
}

// The world normal of a hit object_hits reported: the leaf's normal, rotated out through the
// Logic frames above it (the ray direction is taken down the same frames for the cubic's
// fallback).
__device__ __forceinline__ V object_normal(const lg_geo* G, const XNode* nd, V d, const Hit& h) {
  int chain[MAX_DEPTH + 1];
  int nc = 0;
  for (int j = nd[h.node].parent; j >= 0 && nc <= MAX_DEPTH; j = nd[j].parent) chain[nc++] = j;
  for (int k = nc - 1; k >= 0; --k) d = irot(d, G[nd[chain[k]].geo].rot[0], G[nd[chain[k]].geo].rot[1]);
  V n = leaf_normal(G, G[nd[h.node].geo], h, d);
  for (int k = 0; k < nc; ++k) n = rot(n, G[nd[chain[k]].geo].rot[0], G[nd[chain[k]].geo].rot[1]);
  return n;
}
// The leaf number (in the flattened leaf table) of a hit.
__device__ __forceinline__ int hit_leaf(const lg_geo* G, const XNode* nd, const Hit& h) {
  return (int)nd[h.node].leaf_ord + (G[nd[h.node].geo].kind == LG_GEO_POLYGON ? h.sub : 0);
}

__device__ __forceinline__ bool object_contains_tree(const lg_geo* G, const XNode* nd, int nn, V p, uint32_t* fl) {
  return subtree_contains(G, nd, 0, nn, p, fl);
}

}  // namespace lgx
