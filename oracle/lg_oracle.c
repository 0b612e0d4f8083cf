/*
 * lg_oracle.c — CPU FP64 restatement of light_garden's trace-and-accumulate path.
 *
 * TEST INFRASTRUCTURE ONLY (see lg_oracle.h).  PARITY UNPINNED: the geometry crate
 * collision2d is absent and the reference has no tests or golden outputs, so the
 * geometry below is restated from mathematics and these definitions are our choice:
 *
 *   T_MIN        hits at ray parameter t <= 1e-9 are ignored (self-intersection rule).
 *   EPSILON      1e-9, the constant SpotLight::set_num_rays compares |dir.x| against.
 *   ray dir      kept as produced (unit up to rounding), never renormalised.
 *   circle       |o + t d - c|^2 = r^2, cancellation-free roots q = -(b + sgn(b) sqrt(disc)),
 *                t1 = q / a, t2 = cc / q (Numerical Recipes 5.6); normal (p - c) / r.
 *   rect         slab test in the rect's local frame; entry and exit are both hits.
 *   segment      2x2 parametric solve, u in [0, 1]; normal = unit left normal of b - a.
 *   cubic        f(s) = cross(d, B(s) - o) on [0, 1], split at the roots of f', each
 *                sign change solved by safeguarded Newton (ten bisection steps, then Newton
 *                kept inside the bracket, Numerical Recipes 9.4, finished by bisection when
 *                it does not converge); normal = perp(B'(s)).
 *   logic        children hit in the node's local frame, kept when the other child's
 *                membership makes the point a boundary of the combination:
 *                And: other inside; Or: other outside; AndNot: a-hits with b outside,
 *                b-hits with a inside.  contains() is closed (boundary points inside).
 *   polygon      convex, vertices in the node's frame: every edge is a segment hit with the
 *                outward normal; contains = on the inner side of every edge (closed).
 *   ellipse      the ray in the ellipse frame scaled by (1/a, 1/b) meets the unit circle
 *                (same ray parameter); normal = normalised gradient (x/a^2, y/b^2).
 *   hit point    o + t d on the ray.
 *   inside test  "obj.contains(ray origin)" (tracer.rs:431) is evaluated at the midpoint
 *                of origin -> hit; it equals the literal test whenever the origin is not
 *                on obj's boundary, and decides the on-boundary case (a ray that just
 *                entered obj) the physical way instead of by rounding.
 *   refract      Snell with TIR; reflectance = unpolarised Fresnel (Rs + Rp) / 2, 1 on TIR.
 *   directional  origins a + (i / n)(b - a), i in [0, n); direction = unit left normal.
 *   canvas exit  nearest hit (t > T_MIN) with the canvas rectangle.
 *   near-degenerate  decisions whose margin is below 1e-10 (relative) are flagged
 *                (LG_PATH_NEAR_DEGENERATE) and the flag is inherited by descendants.
 */
#define _GNU_SOURCE
#include "lg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#define T_MIN 1e-9
#define SPOT_EPSILON 1e-9
#define BAND 1e-10
#define MAX_GEO_HITS 256
#define MAX_DEPTH 64
#define NEAR LG_PATH_NEAR_DEGENERATE

typedef struct { double x, y; } v2;
static inline v2 mk(double x, double y) { v2 r = {x, y}; return r; }
static inline v2 add(v2 a, v2 b) { return mk(a.x + b.x, a.y + b.y); }
static inline v2 sub(v2 a, v2 b) { return mk(a.x - b.x, a.y - b.y); }
static inline v2 scl(v2 a, double s) { return mk(a.x * s, a.y * s); }
static inline double dot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline double cross(v2 a, v2 b) { return a.x * b.y - a.y * b.x; }
static inline v2 unit(v2 a) { double l = sqrt(dot(a, a)); return l > 0 ? scl(a, 1.0 / l) : a; }
/* rotation by (c, s) and its inverse */
static inline v2 rot(v2 a, double c, double s) { return mk(c * a.x - s * a.y, s * a.x + c * a.y); }
static inline v2 irot(v2 a, double c, double s) { return mk(c * a.x + s * a.y, -s * a.x + c * a.y); }

typedef struct { double t; v2 p, n; } ohit;

typedef struct {
  const lg_geo* g;
  uint32_t n_geo;
  const lg_object* o;
  uint32_t n_obj;
  const lg_light* l;
  uint32_t n_light;
  lg_params prm;
  double aspect;
} oscene;

/* ------------------------------------------------------------------ polygons */
#define MAX_POLY 63
/* vertices of a POLYGON node (in its frame), following its VERTICES chain; returns the count */
static int poly_vertices(const lg_geo* G, const lg_geo* g, v2* out) {
  const int n = g->a;
  int k = 0;
  const lg_geo* cur = g;
  while (k < n) {
    for (int i = 0; i < 4 && k < n; ++i, ++k) out[k] = mk(cur->v[2 * i], cur->v[2 * i + 1]);
    if (k < n) cur = &G[cur->b];
  }
  return n;
}
static double poly_orientation(const v2* P, int n) {
  double a = 0.0;
  for (int i = 0; i < n; ++i) a += cross(P[i], P[(i + 1) % n]);
  return a >= 0.0 ? 1.0 : -1.0;
}

/* ------------------------------------------------------------------ geometry: contains */
/* Membership with a near-boundary flag (closed sets). */
static int geo_contains(const lg_geo* G, int gi, v2 p, uint32_t* fl) {
  const lg_geo* g = &G[gi];
  switch (g->kind) {
    case LG_GEO_CIRCLE: {
      v2 d = sub(p, mk(g->origin[0], g->origin[1]));
      double r = g->v[0];
      double m = dot(d, d) - r * r;
      if (fl && fabs(m) <= BAND * r * r) *fl |= NEAR;
      return m <= 0.0;
    }
    case LG_GEO_RECT: {
      v2 l = irot(sub(p, mk(g->origin[0], g->origin[1])), g->rot[0], g->rot[1]);
      double hw = 0.5 * g->v[0], hh = 0.5 * g->v[1];
      double ex = fabs(l.x) - hw, ey = fabs(l.y) - hh;
      double sd = ex > ey ? ex : ey;
      if (fl && fabs(sd) <= BAND * (hw + hh)) *fl |= NEAR;
      return sd <= 0.0;
    }
    case LG_GEO_POLYGON: {
      v2 P[MAX_POLY];
      const int n = poly_vertices(G, g, P);
      const double sgn = poly_orientation(P, n);
      v2 l = irot(sub(p, mk(g->origin[0], g->origin[1])), g->rot[0], g->rot[1]);
      int in = 1;
      for (int i = 0; i < n; ++i) {
        v2 e = sub(P[(i + 1) % n], P[i]);
        double le = sqrt(dot(e, e));
        double sd = -sgn * cross(e, sub(l, P[i])) / (le > 0 ? le : 1.0); /* > 0 outside this edge */
        if (fl && fabs(sd) <= BAND * (le + 1e-300)) *fl |= NEAR;
        if (sd > 0.0) in = 0;
      }
      return in;
    }
    case LG_GEO_ELLIPSE: {
      v2 l = irot(sub(p, mk(g->origin[0], g->origin[1])), g->rot[0], g->rot[1]);
      double u = l.x / g->v[0], w = l.y / g->v[1];
      double m = u * u + w * w - 1.0;
      if (fl && fabs(m) <= BAND) *fl |= NEAR;
      return m <= 0.0;
    }
    case LG_GEO_LOGIC: {
      v2 l = irot(sub(p, mk(g->origin[0], g->origin[1])), g->rot[0], g->rot[1]);
      int a = geo_contains(G, g->a, l, fl);
      int b = geo_contains(G, g->b, l, fl);
      if (g->op == LG_OP_AND) return a && b;
      if (g->op == LG_OP_OR) return a || b;
      return a && !b;
    }
    default: /* segments and cubics enclose nothing */
      return 0;
  }
}

/* ------------------------------------------------------------------ geometry: hits */
static int push_hit(ohit* out, int n, int cap, double t, v2 o, v2 d, v2 nrm) {
  if (n >= cap) return n;
  out[n].t = t;
  out[n].p = add(o, scl(d, t));
  out[n].n = nrm;
  return n + 1;
}

/* Near-degenerate decision events: *ev keeps the smallest ray parameter at which a
 * decision (hit or no hit) fell inside the FP64 band.  Only events at or before the
 * winning hit can change the outcome, so the tracer compares ev against the winner. */
static inline void event(double* ev, double t) {
  if (t < 0.0) t = 0.0;
  if (t < *ev) *ev = t;
}
static void tmin_band(double t, double* ev) {
  if (t > 1e-2 * T_MIN && t < 1e2 * T_MIN) event(ev, t);
}

static int hits_circle(const lg_geo* g, v2 o, v2 d, ohit* out, int cap, double* ev) {
  v2 c = mk(g->origin[0], g->origin[1]);
  double r = g->v[0];
  v2 oc = sub(o, c);
  double a = dot(d, d), b = dot(oc, d), cc = dot(oc, oc) - r * r;
  double disc = b * b - a * cc;
  if (fabs(disc) <= BAND * (b * b + fabs(a * cc)) && -b / a > -T_MIN) event(ev, -b / a);
  if (disc < 0.0) return 0;
  double sq = sqrt(disc);
  double q = -(b + (b >= 0 ? sq : -sq));
  double t1, t2;
  if (q != 0.0) {
    t1 = q / a;
    t2 = cc / q;
  } else {
    t1 = t2 = 0.0;
  }
  if (t1 > t2) { double x = t1; t1 = t2; t2 = x; }
  int n = 0;
  double ts[2] = {t1, t2};
  for (int k = 0; k < 2; ++k) {
    tmin_band(ts[k], ev);
    if (ts[k] > T_MIN) {
      v2 p = add(o, scl(d, ts[k]));
      n = push_hit(out, n, cap, ts[k], o, d, scl(sub(p, c), 1.0 / r));
    }
  }
  return n;
}

static int hits_segment(v2 A, v2 B, v2 o, v2 d, ohit* out, int cap, double* ev) {
  v2 e = sub(B, A);
  double den = cross(d, e);
  double le = sqrt(dot(e, e)), ld = sqrt(dot(d, d));
  v2 w = sub(A, o);
  if (fabs(den) <= BAND * le * ld) event(ev, den != 0.0 ? cross(w, e) / den : 0.0);
  if (den == 0.0) return 0;
  double t = cross(w, e) / den;
  double u = cross(w, d) / den;
  if (fabs(u) <= BAND || fabs(u - 1.0) <= BAND) event(ev, t);
  if (u < 0.0 || u > 1.0) return 0;
  tmin_band(t, ev);
  if (!(t > T_MIN)) return 0;
  v2 nrm = le > 0 ? mk(-e.y / le, e.x / le) : mk(0, 0);
  return push_hit(out, 0, cap, t, o, d, nrm);
}

static int hits_rect(const lg_geo* g, v2 o, v2 d, ohit* out, int cap, double* ev) {
  double c = g->rot[0], s = g->rot[1];
  v2 ctr = mk(g->origin[0], g->origin[1]);
  v2 lo = irot(sub(o, ctr), c, s), ld = irot(d, c, s);
  double h[2] = {0.5 * g->v[0], 0.5 * g->v[1]};
  double O[2] = {lo.x, lo.y}, D[2] = {ld.x, ld.y};
  double tn = -INFINITY, tf = INFINITY;
  int an = -1, af = -1;
  double sn = 0, sf = 0; /* outward sign of the entry / exit face */
  double tn_other = -INFINITY;
  for (int ax = 0; ax < 2; ++ax) {
    if (D[ax] == 0.0) {
      if (fabs(fabs(O[ax]) - h[ax]) <= BAND * h[ax]) event(ev, 0.0);
      if (fabs(O[ax]) > h[ax]) return 0;
      continue;
    }
    double t1 = (-h[ax] - O[ax]) / D[ax];
    double t2 = (h[ax] - O[ax]) / D[ax];
    double s1 = -1.0, s2 = 1.0;
    if (t1 > t2) { double x = t1; t1 = t2; t2 = x; s1 = 1.0; s2 = -1.0; }
    if (t1 > tn) { tn_other = tn; tn = t1; an = ax; sn = s1; } else if (t1 > tn_other) tn_other = t1;
    if (t2 < tf) { tf = t2; af = ax; sf = s2; }
  }
  if (an < 0 || af < 0) return 0; /* degenerate direction */
  double scale = fabs(tn) + fabs(tf) + 1.0;
  if (fabs(tf - tn) <= BAND * scale) event(ev, tn);                         /* corner graze */
  if (tn_other > -INFINITY && fabs(tn - tn_other) <= BAND * scale) event(ev, tn); /* corner entry */
  if (tn > tf) return 0;
  int n = 0;
  v2 nn = an == 0 ? mk(sn, 0) : mk(0, sn);
  v2 nf = af == 0 ? mk(sf, 0) : mk(0, sf);
  tmin_band(tn, ev);
  if (tn > T_MIN) n = push_hit(out, n, cap, tn, o, d, rot(nn, c, s));
  tmin_band(tf, ev);
  if (tf > T_MIN) n = push_hit(out, n, cap, tf, o, d, rot(nf, c, s));
  return n;
}

/* cubic in power basis: B(s) = C3 s^3 + C2 s^2 + C1 s + C0 */
typedef struct { v2 c0, c1, c2, c3; } cubic;
static cubic cubic_of(const double* v) {
  v2 P0 = mk(v[0], v[1]), P1 = mk(v[2], v[3]), P2 = mk(v[4], v[5]), P3 = mk(v[6], v[7]);
  cubic k;
  k.c0 = P0;
  k.c1 = scl(sub(P1, P0), 3.0);
  k.c2 = add(scl(sub(P2, scl(P1, 2.0)), 3.0), scl(P0, 3.0));
  k.c3 = sub(add(P3, scl(sub(P1, P2), 3.0)), P0);
  return k;
}
static double poly3(const double* a, double s) { return ((a[3] * s + a[2]) * s + a[1]) * s + a[0]; }
static double cubic_t(const cubic* k, double s, v2 o, v2 d) {
  v2 B = add(add(add(scl(k->c3, s * s * s), scl(k->c2, s * s)), scl(k->c1, s)), k->c0);
  return dot(sub(B, o), d) / dot(d, d);
}

/* The root of f (monotone on [lo, hi], f(lo) = flo != 0 and f(hi) of the other sign):
 * ten bisection steps, then Newton steps from the bracket's midpoint, each kept inside the
 * bracket (a step that leaves it bisects instead), until a step moves the root by 1e-15 or
 * less (Numerical Recipes 9.4, rtsafe); if twelve steps do not get there, bisection of the
 * remaining bracket to full precision. */
static double cubic_root(const double* a, double lo, double hi, double flo) {
  const int neg_lo = flo < 0;
  for (int it = 0; it < 10; ++it) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) return mid;
    double fm = poly3(a, mid);
    if (fm == 0.0) return mid;
    if ((fm < 0) == neg_lo) lo = mid; else hi = mid;
  }
  double s = 0.5 * (lo + hi);
  for (int it = 0; it < 12; ++it) {
    double f = poly3(a, s);
    if (f == 0.0) return s;
    if ((f < 0) == neg_lo) lo = s; else hi = s;
    double fp = (3.0 * a[3] * s + 2.0 * a[2]) * s + a[1];
    double sn = s - f / fp;
    if (!(sn > lo && sn < hi)) sn = 0.5 * (lo + hi);
    double step = sn - s;
    s = sn;
    if (fabs(step) <= 1e-15) return s;
  }
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) return mid;
    double fm = poly3(a, mid);
    if (fm == 0.0) return mid;
    if ((fm < 0) == neg_lo) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

static int hits_cubic(const lg_geo* g, v2 o, v2 d, ohit* out, int cap, double* ev) {
  cubic k = cubic_of(g->v);
  double a[4] = {cross(d, sub(k.c0, o)), cross(d, k.c1), cross(d, k.c2), cross(d, k.c3)};
  double scale = fabs(a[0]) + fabs(a[1]) + fabs(a[2]) + fabs(a[3]) + 1e-300;
  /* critical points: 3 a3 s^2 + 2 a2 s + a1 = 0 */
  double cr[2];
  int ncr = 0;
  double qa = 3.0 * a[3], qb = 2.0 * a[2], qc = a[1];
  if (qa != 0.0) {
    double disc = qb * qb - 4.0 * qa * qc;
    if (disc >= 0.0) {
      double sq = sqrt(disc);
      double q = -0.5 * (qb + (qb >= 0 ? sq : -sq));
      double r1 = q / qa, r2 = q != 0.0 ? qc / q : r1;
      if (r1 > r2) { double x = r1; r1 = r2; r2 = x; }
      if (r1 > 0.0 && r1 < 1.0) cr[ncr++] = r1;
      if (r2 > 0.0 && r2 < 1.0 && (ncr == 0 || r2 != cr[0])) cr[ncr++] = r2;
    }
  } else if (qb != 0.0) {
    double r = -qc / qb;
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
    double lo = knots[i], hi = knots[i + 1];
    double flo = poly3(a, lo), fhi = poly3(a, hi);
    if (i > 0 && fabs(flo) <= BAND * scale) event(ev, cubic_t(&k, lo, o, d)); /* tangency */
    if (flo == 0.0) {
      if (nr == 0 || roots[nr - 1] != lo) roots[nr++] = lo;
      continue;
    }
    if (fhi == 0.0) {
      if (i + 2 == nk) roots[nr++] = hi;
      continue;
    }
    if ((flo < 0) != (fhi < 0)) roots[nr++] = cubic_root(a, lo, hi, flo);
  }
  if (fabs(a[0]) <= BAND * scale) event(ev, cubic_t(&k, 0.0, o, d)); /* end points */
  if (fabs(poly3(a, 1.0)) <= BAND * scale) event(ev, cubic_t(&k, 1.0, o, d));
  int n = 0;
  double dd = dot(d, d);
  for (int i = 0; i < nr; ++i) {
    double s = roots[i];
    v2 B = add(add(add(scl(k.c3, s * s * s), scl(k.c2, s * s)), scl(k.c1, s)), k.c0);
    double t = dot(sub(B, o), d) / dd;
    tmin_band(t, ev);
    if (!(t > T_MIN)) continue;
    v2 dB = add(add(scl(k.c3, 3.0 * s * s), scl(k.c2, 2.0 * s)), k.c1);
    double l = sqrt(dot(dB, dB));
    if (l == 0.0) event(ev, t);
    v2 nrm = l > 0 ? mk(-dB.y / l, dB.x / l) : unit(mk(-d.y, d.x));
    n = push_hit(out, n, cap, t, o, d, nrm);
  }
  return n;
}

static int hits_polygon(const lg_geo* G, const lg_geo* g, v2 o, v2 d, ohit* out, int cap, double* ev) {
  v2 P[MAX_POLY];
  const int n = poly_vertices(G, g, P);
  const double sgn = poly_orientation(P, n);
  const double c = g->rot[0], s = g->rot[1];
  v2 org = mk(g->origin[0], g->origin[1]);
  v2 lo = irot(sub(o, org), c, s), ld = irot(d, c, s);
  int m = 0;
  for (int i = 0; i < n; ++i) {
    ohit h[1];
    if (hits_segment(P[i], P[(i + 1) % n], lo, ld, h, 1, ev) == 1 && m < cap) {
      v2 e = sub(P[(i + 1) % n], P[i]);
      v2 nrm = unit(scl(mk(e.y, -e.x), sgn)); /* outward */
      out[m].t = h[0].t;
      out[m].p = add(o, scl(d, h[0].t));
      out[m].n = rot(nrm, c, s);
      ++m;
    }
  }
  return m;
}

static int hits_ellipse(const lg_geo* g, v2 o, v2 d, ohit* out, int cap, double* ev) {
  const double c = g->rot[0], s = g->rot[1], A = g->v[0], Bb = g->v[1];
  v2 org = mk(g->origin[0], g->origin[1]);
  v2 lo = irot(sub(o, org), c, s), ld = irot(d, c, s);
  v2 so = mk(lo.x / A, lo.y / Bb), sd = mk(ld.x / A, ld.y / Bb);
  double a = dot(sd, sd), b = dot(so, sd), cc = dot(so, so) - 1.0;
  double disc = b * b - a * cc;
  if (fabs(disc) <= BAND * (b * b + fabs(a * cc)) && -b / a > -T_MIN) event(ev, -b / a);
  if (disc < 0.0) return 0;
  double sq = sqrt(disc);
  double q = -(b + (b >= 0 ? sq : -sq));
  double t1 = 0.0, t2 = 0.0;
  if (q != 0.0) {
    t1 = q / a;
    t2 = cc / q;
  }
  if (t1 > t2) { double x = t1; t1 = t2; t2 = x; }
  int n = 0;
  double ts[2] = {t1, t2};
  for (int k = 0; k < 2; ++k) {
    tmin_band(ts[k], ev);
    if (ts[k] > T_MIN) {
      v2 pl = add(lo, scl(ld, ts[k]));
      v2 gr = unit(mk(pl.x / (A * A), pl.y / (Bb * Bb)));
      n = push_hit(out, n, cap, ts[k], o, d, rot(gr, c, s));
    }
  }
  return n;
}

static int geo_hits(const lg_geo* G, int gi, v2 o, v2 d, ohit* out, int cap, double* ev, int depth) {
  const lg_geo* g = &G[gi];
  switch (g->kind) {
    case LG_GEO_POLYGON: return hits_polygon(G, g, o, d, out, cap, ev);
    case LG_GEO_ELLIPSE: return hits_ellipse(g, o, d, out, cap, ev);
    case LG_GEO_CIRCLE: return hits_circle(g, o, d, out, cap, ev);
    case LG_GEO_RECT: return hits_rect(g, o, d, out, cap, ev);
    case LG_GEO_SEGMENT: return hits_segment(mk(g->v[0], g->v[1]), mk(g->v[2], g->v[3]), o, d, out, cap, ev);
    case LG_GEO_CUBIC: return hits_cubic(g, o, d, out, cap, ev);
    case LG_GEO_LOGIC: {
      if (depth >= MAX_DEPTH) return 0;
      double c = g->rot[0], s = g->rot[1];
      v2 org = mk(g->origin[0], g->origin[1]);
      v2 lo = irot(sub(o, org), c, s), ld = irot(d, c, s);
      ohit tmp[MAX_GEO_HITS];
      int n = 0;
      for (int side = 0; side < 2; ++side) {
        int child = side == 0 ? g->a : g->b;
        int other = side == 0 ? g->b : g->a;
        int nh = geo_hits(G, child, lo, ld, tmp, MAX_GEO_HITS, ev, depth + 1);
        for (int k = 0; k < nh; ++k) {
          uint32_t cfl = 0;
          int in_other = geo_contains(G, other, tmp[k].p, &cfl);
          if (cfl) event(ev, tmp[k].t);
          int keep;
          if (g->op == LG_OP_AND) keep = in_other;
          else if (g->op == LG_OP_OR) keep = !in_other;
          else keep = side == 0 ? !in_other : in_other;
          if (!keep || n >= cap) continue;
          out[n].t = tmp[k].t;
          out[n].p = add(org, rot(tmp[k].p, c, s));
          out[n].n = rot(tmp[k].n, c, s);
          ++n;
        }
      }
      return n;
    }
    default: return 0;
  }
}

/* --------------------------------------------------------------------- objects */
static int object_contains(const oscene* S, uint32_t k, v2 p, uint32_t* fl) {
  const lg_object* ob = &S->o[k];
  if (ob->kind == LG_OBJ_STRAIGHT_MIRROR || ob->kind == LG_OBJ_CURVED_MIRROR) return 0; /* object.rs:243-244 */
  return geo_contains(S->g, ob->geo, p, fl);
}

static int validate_geo(const lg_geo* G, uint32_t n_geo, int gi, int depth) {
  if (gi < 0 || (uint32_t)gi >= n_geo || depth > MAX_DEPTH) return LGO_ERR_INVALID;
  const lg_geo* g = &G[gi];
  switch (g->kind) {
    case LG_GEO_CIRCLE: case LG_GEO_RECT: case LG_GEO_SEGMENT: case LG_GEO_CUBIC: return LGO_OK;
    case LG_GEO_ELLIPSE: return g->v[0] > 0.0 && g->v[1] > 0.0 ? LGO_OK : LGO_ERR_INVALID;
    case LG_GEO_POLYGON: {
      if (g->a < 3 || g->a > MAX_POLY) return LGO_ERR_INVALID;
      int k = 4;
      const lg_geo* cur = g;
      while (k < g->a) {  /* the VERTICES chain */
        if (cur->b < 0 || (uint32_t)cur->b >= n_geo || G[cur->b].kind != LG_GEO_VERTICES) return LGO_ERR_INVALID;
        cur = &G[cur->b];
        k += 4;
      }
      return LGO_OK;
    }
    case LG_GEO_LOGIC: {
      if (g->op < 0 || g->op > 2) return LGO_ERR_INVALID;
      int r = validate_geo(G, n_geo, g->a, depth + 1);
      if (r) return r;
      return validate_geo(G, n_geo, g->b, depth + 1);
    }
    default: return LGO_ERR_UNSUPPORTED;
  }
}

static int validate_scene(const oscene* S) {
  for (uint32_t k = 0; k < S->n_obj; ++k) {
    const lg_object* ob = &S->o[k];
    if (ob->kind < 0 || ob->kind > LG_OBJ_GEO) return LGO_ERR_INVALID;
    int r = validate_geo(S->g, S->n_geo, ob->geo, 0);
    if (r) return r;
    int rk = S->g[ob->geo].kind;
    if ((ob->kind == LG_OBJ_STRAIGHT_MIRROR && rk != LG_GEO_SEGMENT) ||
        (ob->kind == LG_OBJ_CURVED_MIRROR && rk != LG_GEO_CUBIC) ||
        (ob->kind == LG_OBJ_CIRCLE && rk != LG_GEO_CIRCLE) ||
        (ob->kind == LG_OBJ_RECT && rk != LG_GEO_RECT) || (ob->kind == LG_OBJ_LENS && rk != LG_GEO_LOGIC) ||
        (ob->kind == LG_OBJ_CONVEX_POLYGON && rk != LG_GEO_POLYGON) || (ob->kind == LG_OBJ_ELLIPSE && rk != LG_GEO_ELLIPSE))
      return LGO_ERR_INVALID;
  }
  for (uint32_t k = 0; k < S->n_light; ++k)
    if (S->l[k].kind < 0 || S->l[k].kind > LG_LIGHT_SPOT) return LGO_ERR_INVALID;
  if (S->prm.max_bounce > 64 || S->prm.width == 0 || S->prm.height == 0) return LGO_ERR_INVALID;
  return LGO_OK;
}

/* ------------------------------------------------------------------------ lights */
/* sin / cos / atan of the ray generators, restated from published methods with plain
 * IEEE-754 double operations only (every product and sum rounded on its own), so that
 * the same operations give the same bits on every machine and on the GPU:
 *   sincos  Cody-Waite reduction by pi/2 (pi/2 split in three parts of 33, 33 and 53
 *           significant bits, so that k * P1 and k * P2 are exact for |k| < 2^20), then the
 *           Taylor series of sin and cos on [-pi/4, pi/4] (terms to r^19 and r^20, the
 *           truncation below 1e-21) in Horner form, and the quadrant from k mod 4;
 *   atan    atan(x) = pi/2 - atan(1/x) for |x| > 1, atan(a) = pi/6 + atan((a sqrt3 - 1) /
 *           (a + sqrt3)) for a > tan(pi/12), then the Taylor series to a^29 on |a| <= 0.268.
 * They stay within a few ulp of the C library's functions (tests/test_oracle.py), which is
 * what light.rs calls through Rust's f64::sin_cos / atan; the ray directions are a shared
 * definition of this restatement and of the GPU path. */
#define CW_P1 1.5707963267341256
#define CW_P2 6.077100506303966e-11
#define CW_P3 2.0222662487959506e-21
#define TWO_OVER_PI 0.6366197723675814
#define PI2_HI 1.5707963267948966
#define PI2_LO 6.123233995736766e-17
#define PI6_HI 0.5235987755982989
#define PI6_LO (-5.360408832255455e-17)
#define SQRT3 1.7320508075688772
#define TAN_PI12 0.2679491924311227

void lgo_sincos(double x, double* s_out, double* c_out) {
  const double k = rint(x * TWO_OVER_PI);
  const double r = ((x - k * CW_P1) - k * CW_P2) - k * CW_P3;
  const double z = r * r;
  /* sin: r + r z (-1/3! + z (1/5! - ... - z^8/19!)) */
  double ps = -8.22063524662433e-18;        /* -1/19! */
  ps = ps * z + 2.8114572543455206e-15;     /*  1/17! */
  ps = ps * z - 7.647163731819816e-13;      /* -1/15! */
  ps = ps * z + 1.6059043836821613e-10;     /*  1/13! */
  ps = ps * z - 2.505210838544172e-08;      /* -1/11! */
  ps = ps * z + 2.7557319223985893e-06;     /*  1/9!  */
  ps = ps * z - 0.0001984126984126984;      /* -1/7!  */
  ps = ps * z + 0.008333333333333333;       /*  1/5!  */
  ps = ps * z - 0.16666666666666666;        /* -1/3!  */
  const double sn = r + (r * z) * ps;
  /* cos: 1 - z/2 + z^2 (1/4! - z/6! + ... + z^8/20!) */
  double pc = 4.110317623312165e-19;        /*  1/20! */
  pc = pc * z - 1.5619206968586225e-16;     /* -1/18! */
  pc = pc * z + 4.779477332387385e-14;      /*  1/16! */
  pc = pc * z - 1.1470745597729725e-11;     /* -1/14! */
  pc = pc * z + 2.08767569878681e-09;       /*  1/12! */
  pc = pc * z - 2.755731922398589e-07;      /* -1/10! */
  pc = pc * z + 2.48015873015873e-05;       /*  1/8!  */
  pc = pc * z - 0.001388888888888889;       /* -1/6!  */
  pc = pc * z + 0.041666666666666664;       /*  1/4!  */
  const double cs = (1.0 - 0.5 * z) + (z * z) * pc;
  const long long q = ((long long)k % 4 + 4) % 4;
  *s_out = q == 0 ? sn : q == 1 ? cs : q == 2 ? -sn : -cs;
  *c_out = q == 0 ? cs : q == 1 ? -sn : q == 2 ? -cs : sn;
}

double lgo_atan(double x) {
  if (x != x) return x;
  const int neg = x < 0.0;
  double a = fabs(x);
  const int inv = a > 1.0;
  if (inv) a = 1.0 / a;
  const int off = a > TAN_PI12;
  if (off) a = (a * SQRT3 - 1.0) / (a + SQRT3);
  const double z = a * a;
  double p = -0.034482758620689655;         /* -1/29 */
  p = p * z + 0.037037037037037035;         /*  1/27 */
  p = p * z - 0.04;                         /* -1/25 */
  p = p * z + 0.043478260869565216;         /*  1/23 */
  p = p * z - 0.047619047619047616;         /* -1/21 */
  p = p * z + 0.05263157894736842;          /*  1/19 */
  p = p * z - 0.058823529411764705;         /* -1/17 */
  p = p * z + 0.06666666666666667;          /*  1/15 */
  p = p * z - 0.07692307692307693;          /* -1/13 */
  p = p * z + 0.09090909090909091;          /*  1/11 */
  p = p * z - 0.1111111111111111;           /* -1/9  */
  p = p * z + 0.14285714285714285;          /*  1/7  */
  p = p * z - 0.2;                          /* -1/5  */
  p = p * z + 0.3333333333333333;           /*  1/3  */
  double r = a - (a * z) * p;
  if (off) r = PI6_HI + (r + PI6_LO);
  if (inv) r = PI2_HI - (r - PI2_LO);
  return neg ? -r : r;
}

static void light_ray(const lg_light* L, uint64_t i, v2* o, v2* d) {
  double n = (double)L->num_rays;
  switch (L->kind) {
    case LG_LIGHT_POINT: { /* light.rs:163-174 */
      double f = (double)i * M_PI * 2.0 / n;
      double sf, cf;
      lgo_sincos(f, &sf, &cf);
      *o = mk(L->origin[0], L->origin[1]);
      *d = mk(cf, sf);
      break;
    }
    case LG_LIGHT_SPOT: { /* light.rs:225-249 */
      double sx = L->v[0], sy = L->v[1];
      double dir_angle = fabs(sx) < SPOT_EPSILON ? (sy >= 0.0 ? M_PI * 0.5 : -M_PI * 0.5) : lgo_atan(sy / sx);
      double min_angle = dir_angle - 0.5 * L->spot_angle;
      double step = (double)(i + 1);
      double ang = min_angle + (step / n) * L->spot_angle;
      double sign = signbit(sx) ? -1.0 : 1.0; /* f64::signum: -0.0 -> -1 */
      double sa, ca;
      lgo_sincos(ang, &sa, &ca);
      *o = mk(L->origin[0], L->origin[1]);
      *d = mk(sign * ca, sign * sa);
      break;
    }
    default: { /* DIRECTIONAL, light.rs:103-115 with the definition in the header */
      v2 a = mk(L->origin[0], L->origin[1]), b = mk(L->v[0], L->v[1]);
      v2 e = sub(b, a);
      double r = (double)i / n;
      *o = add(a, scl(e, r));
      *d = unit(mk(-e.y, e.x));
      break;
    }
  }
}

int lgo_light_rays(const lg_light* L, double* out, uint64_t cap) {
  if (!L || !out) return LGO_ERR_INVALID;
  if ((uint64_t)L->num_rays > cap) return LGO_ERR_TRUNCATED;
  for (uint64_t i = 0; i < L->num_rays; ++i) {
    v2 o, d;
    light_ray(L, i, &o, &d);
    out[4 * i] = o.x; out[4 * i + 1] = o.y; out[4 * i + 2] = d.x; out[4 * i + 3] = d.y;
  }
  return LGO_OK;
}

static double light_medium(const oscene* S, const lg_light* L) {
  /* tracer.rs:280-287: the last object containing the light origin wins */
  double n = 1.0;
  v2 p = mk(L->origin[0], L->origin[1]);
  for (uint32_t k = 0; k < S->n_obj; ++k)
    if (object_contains(S, k, p, NULL) && S->o[k].has_material) n = S->o[k].refractive_index;
  return n;
}

/* ------------------------------------------------------------------------ refract */
static int refract(v2 d, v2 n, double n1, double n2, v2* refl, v2* refr, double* R, uint32_t* fl) {
  double ci = -dot(d, n);
  if (ci < 0.0) { ci = -ci; n = scl(n, -1.0); }
  *refl = add(d, scl(n, 2.0 * ci));
  double eta = n1 / n2;
  double k = 1.0 - eta * eta * (1.0 - ci * ci);
  if (fabs(k) <= BAND) *fl |= NEAR;
  if (k < 0.0) { *R = 1.0; return 0; }
  double ct = sqrt(k);
  *refr = add(scl(d, eta), scl(n, eta * ci - ct));
  double ds = n1 * ci + n2 * ct, dp = n1 * ct + n2 * ci;
  if (ds == 0.0 || dp == 0.0) { *R = 1.0; return 1; }
  double rs = (n1 * ci - n2 * ct) / ds;
  double rp = (n1 * ct - n2 * ci) / dp;
  *R = 0.5 * (rs * rs + rp * rp);
  return 1;
}

int lgo_refract(double dx, double dy, double nx, double ny, double n1, double n2,
                double* refl_dir, double* refr_dir, double* R) {
  v2 rl, rr = mk(0, 0);
  uint32_t fl = 0;
  int ok = refract(mk(dx, dy), mk(nx, ny), n1, n2, &rl, &rr, R, &fl);
  refl_dir[0] = rl.x; refl_dir[1] = rl.y;
  refr_dir[0] = rr.x; refr_dir[1] = rr.y;
  return ok;
}

/* ------------------------------------------------------------------------ tracing */
typedef struct {
  v2 o, d;
  float c[4];
  double n;
  uint64_t path;
  uint32_t gen;
  uint32_t flags;
} oray;

typedef struct {
  lg_segment* seg;
  lg_path_record* rec;
  double* s64;
  uint64_t n, cap;
  uint64_t visits, near;
} obuf;

static int buf_push(obuf* B, v2 a, v2 b, const float* c, const lg_path_record* r) {
  if (B->n == B->cap) {
    uint64_t nc = B->cap ? 2 * B->cap : 256;
    lg_segment* s = realloc(B->seg, nc * sizeof(lg_segment));
    if (!s) return LGO_ERR_OOM;
    B->seg = s;
    lg_path_record* q = realloc(B->rec, nc * sizeof(lg_path_record));
    if (!q) return LGO_ERR_OOM;
    B->rec = q;
    double* t = realloc(B->s64, nc * 4 * sizeof(double));
    if (!t) return LGO_ERR_OOM;
    B->s64 = t;
    B->cap = nc;
  }
  lg_segment* s = &B->seg[B->n];
  s->x0 = (float)a.x; s->y0 = (float)a.y; s->x1 = (float)b.x; s->y1 = (float)b.y;
  memcpy(s->color, c, 16);
  B->rec[B->n] = *r;
  double* t = &B->s64[4 * B->n];
  t[0] = a.x; t[1] = a.y; t[2] = b.x; t[3] = b.y;
  if (r->flags & NEAR) B->near++;
  B->n++;
  return LGO_OK;
}

static int cutoff(const float* c, const float* k, uint32_t* fl) {
  for (int i = 0; i < 4; ++i)
    if (fabsf(c[i] - k[i]) <= 1e-6f * k[i]) *fl |= NEAR;
  return (c[0] < k[0] && c[1] < k[1] && c[2] < k[2]) || c[3] < k[3];
}

/* tracer.rs:360-493 for one primary ray */
static int trace_one(const oscene* S, obuf* B, uint32_t light, uint32_t prim, v2 o, v2 d,
                     const float* color, double n0) {
  oray* cur = malloc(sizeof(oray) * 16);
  oray* nxt = malloc(sizeof(oray) * 16);
  size_t ncur = 1, nnxt = 0, capc = 16, capn = 16;
  if (!cur || !nxt) { free(cur); free(nxt); return LGO_ERR_OOM; }
  cur[0].o = o; cur[0].d = d; memcpy(cur[0].c, color, 16); cur[0].n = n0;
  cur[0].path = 0; cur[0].gen = 0; cur[0].flags = 0;
  ohit hits[MAX_GEO_HITS];
  int rc = LGO_OK;
  for (uint32_t gen = 0; gen < S->prm.max_bounce && rc == LGO_OK; ++gen) {
    if (ncur == 0) break;
    for (size_t e = 0; e < ncur && rc == LGO_OK; ++e) {
      oray* r = &cur[e];
      uint32_t fl = r->flags;
      if (cutoff(r->c, S->prm.cutoff_color, &fl)) continue;
      B->visits++;
      /* nearest object, strict < in object order (tracer.rs:412-424) */
      double best = INFINITY, second = INFINITY, ev = INFINITY;
      int best_obj = -1;
      ohit bh;
      for (uint32_t k = 0; k < S->n_obj; ++k) {
        int nh = geo_hits(S->g, S->o[k].geo, r->o, r->d, hits, MAX_GEO_HITS, &ev, 0);
        double obj_best = INFINITY;
        int obj_bi = -1;
        for (int h = 0; h < nh; ++h) {
          v2 dv = sub(hits[h].p, r->o);
          double d2 = dot(dv, dv);
          if (d2 < obj_best) { obj_best = d2; obj_bi = h; }
        }
        if (obj_bi < 0) continue;
        if (obj_best < best) {
          second = best;
          best = obj_best;
          best_obj = (int)k;
          bh = hits[obj_bi];
        } else if (obj_best < second) {
          second = obj_best;
        }
      }
      if (best_obj >= 0 && second < INFINITY && second - best <= BAND * best) fl |= NEAR;
      if (best_obj >= 0 ? ev <= bh.t * (1.0 + 1e-6) + 1e-12 : ev < INFINITY) fl |= NEAR;
      lg_path_record rec;
      rec.path = r->path; rec.primary = prim; rec.light = (uint16_t)light;
      rec.gen = (uint8_t)gen; rec.source = LG_SRC_TRACE;
      if (best_obj >= 0) {
        const lg_object* ob = &S->o[best_obj];
        rec.hit = best_obj;
        if (ob->has_material) {
          double n2 = 1.0; /* air */
          v2 mid = scl(add(r->o, bh.p), 0.5);
          if (object_contains(S, (uint32_t)best_obj, mid, &fl)) {
            for (uint32_t k = 0; k < S->n_obj; ++k) {
              if ((int)k != best_obj && object_contains(S, k, bh.p, &fl) && S->o[k].has_material) {
                n2 = S->o[k].refractive_index;
                break;
              }
            }
          } else {
            n2 = ob->refractive_index;
          }
          v2 rl, rr;
          double R;
          int has_refr = refract(r->d, bh.n, r->n, n2, &rl, &rr, &R, &fl);
          rec.flags = (uint8_t)((fl & 0xff) | (has_refr ? 0 : LG_PATH_TIR));
          rc = buf_push(B, r->o, bh.p, r->c, &rec);
          float refl = (float)R;
          float om = 1.0f - refl;
          if (nnxt + 2 > capn) {
            capn *= 2;
            oray* t = realloc(nxt, sizeof(oray) * capn);
            if (!t) { rc = LGO_ERR_OOM; break; }
            nxt = t;
          }
          oray* c1 = &nxt[nnxt++];
          c1->o = bh.p; c1->d = rl; c1->n = r->n; c1->gen = gen + 1; c1->flags = fl;
          c1->path = r->path;
          c1->c[0] = r->c[0] * refl; c1->c[1] = r->c[1] * refl; c1->c[2] = r->c[2] * refl; c1->c[3] = r->c[3];
          if (has_refr) {
            oray* c2 = &nxt[nnxt++];
            c2->o = bh.p; c2->d = rr; c2->n = n2; c2->gen = gen + 1; c2->flags = fl;
            c2->path = r->path | ((uint64_t)1 << gen);
            c2->c[0] = r->c[0] * om; c2->c[1] = r->c[1] * om; c2->c[2] = r->c[2] * om; c2->c[3] = r->c[3];
          }
        } else {
          rec.flags = (uint8_t)(fl & 0xff);
          rc = buf_push(B, r->o, bh.p, r->c, &rec);
          if (nnxt + 1 > capn) {
            capn *= 2;
            oray* t = realloc(nxt, sizeof(oray) * capn);
            if (!t) { rc = LGO_ERR_OOM; break; }
            nxt = t;
          }
          oray* c1 = &nxt[nnxt++];
          double dn = dot(r->d, bh.n);
          c1->o = bh.p; c1->d = sub(r->d, scl(bh.n, 2.0 * dn)); c1->n = r->n;
          c1->gen = gen + 1; c1->flags = fl; c1->path = r->path;
          memcpy(c1->c, r->c, 16);
        }
      } else {
        /* canvas exit (tracer.rs:482-488) */
        lg_geo canvas;
        memset(&canvas, 0, sizeof canvas);
        canvas.kind = LG_GEO_RECT; canvas.rot[0] = 1.0;
        canvas.v[0] = 2.0 * S->aspect; canvas.v[1] = 2.0;
        double cev = INFINITY;
        int nh = hits_rect(&canvas, r->o, r->d, hits, MAX_GEO_HITS, &cev);
        if (nh > 0) {
          int bi = 0;
          for (int h = 1; h < nh; ++h)
            if (hits[h].t < hits[bi].t) bi = h;
          rec.hit = -1;
          rec.flags = (uint8_t)((fl | (cev < INFINITY ? NEAR : 0)) & 0xff);
          rc = buf_push(B, r->o, hits[bi].p, r->c, &rec);
        }
      }
    }
    oray* t = cur; cur = nxt; nxt = t;
    size_t tc = capc; capc = capn; capn = tc;
    ncur = nnxt; nnxt = 0;
  }
  free(cur);
  free(nxt);
  return rc;
}

typedef struct {
  const oscene* S;
  const double* n0;
  uint64_t* chunk_light;  /* light of each chunk */
  uint64_t* chunk_begin;  /* first primary index of each chunk */
  uint64_t n_chunks;
  uint32_t stride, offset;
  obuf* out;              /* one buffer per chunk */
  volatile uint64_t next;
  pthread_mutex_t mu;
  int rc;
} ojob;

#define CHUNK 100 /* Tracer::chunk_size default, tracer.rs:39 */

static void* worker(void* arg) {
  ojob* J = (ojob*)arg;
  for (;;) {
    pthread_mutex_lock(&J->mu);
    uint64_t c = J->next++;
    pthread_mutex_unlock(&J->mu);
    if (c >= J->n_chunks) break;
    uint32_t li = (uint32_t)J->chunk_light[c];
    const lg_light* L = &J->S->l[li];
    uint64_t b = J->chunk_begin[c];
    uint64_t e = b + (uint64_t)CHUNK * J->stride;
    if (e > L->num_rays) e = L->num_rays;
    for (uint64_t i = b; i < e; i += J->stride) {
      v2 o, d;
      light_ray(L, i, &o, &d);
      int rc = trace_one(J->S, &J->out[c], li, (uint32_t)i, o, d, L->color, J->n0[li]);
      if (rc) { J->rc = rc; return NULL; }
    }
  }
  return NULL;
}

static int online_cores(void) {
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

static uint64_t wrapping_pow(uint64_t b, uint64_t e) {
  uint64_t r = 1;
  while (e) {
    if (e & 1) r *= b;
    b *= b;
    e >>= 1;
  }
  return r;
}

/* ---------------------------------------------------------------- string mod
 * string_mod.rs:33-85 (init_points), 104-122 (draw_init_points), 124-150 (get_color).
 * The point angle is (turns * n) as f64 * TAU / m, multiplied before the division as in
 * the reference; sine and cosine are lgo_sincos. */

/* num-complex 0.4.6 (Cargo.lock), Pow<u32> for &Complex<f64>: binary powering that squares
 * the base past the trailing zero bits of the exponent, then multiplies the accumulator by
 * every later square whose bit is set; products (a.re b.re - a.im b.im, a.re b.im + a.im b.re). */
static void cmul(double ar, double ai, double br, double bi, double* r, double* i) {
  *r = ar * br - ai * bi;
  *i = ar * bi + ai * br;
}
static void cpowu(double re, double im, uint32_t e, double* orr, double* oi) {
  if (e == 0) { *orr = 1.0; *oi = 0.0; return; }
  double br = re, bi = im;
  while ((e & 1u) == 0) { cmul(br, bi, br, bi, &br, &bi); e >>= 1; }
  if (e == 1) { *orr = br; *oi = bi; return; }
  double ar = br, ai = bi;
  while (e > 1) {
    e >>= 1;
    cmul(br, bi, br, bi, &br, &bi);
    if (e & 1u) cmul(ar, ai, br, bi, &ar, &ai);
  }
  *orr = ar; *oi = ai;
}

static void string_mod_point(const lg_string_mod* sm, uint64_t n, double* x, double* y) {
  const uint64_t k = sm->turns * n; /* u64, wrapping */
  if (sm->curve == LG_CURVE_COMPLEX_EXP) {
    cpowu(sm->curve_f[0], sm->curve_f[1], (uint32_t)k, x, y);
    return;
  }
  const double angle = (double)k * (2.0 * M_PI) / (double)sm->modulo;
  double s, c;
  if (sm->curve == LG_CURVE_HYPOTROCHOID) {
    const double r = (double)sm->curve_u[0], big = (double)sm->curve_u[1], d = (double)sm->curve_u[2];
    const double smr = big - r, ratio = smr + d;
    double s2, c2;
    lgo_sincos(angle, &s, &c);
    lgo_sincos(angle * smr / r, &s2, &c2);
    *x = (smr * c + d * c2) / ratio;
    *y = (smr * s - d * s2) / ratio;
  } else if (sm->curve == LG_CURVE_LISSAJOUS) {
    double s2, c2;
    lgo_sincos((double)sm->curve_u[0] * angle + sm->curve_f[0], &s, &c);
    lgo_sincos((double)sm->curve_u[1] * angle, &s2, &c2);
    *x = s;
    *y = s2;
  } else {
    lgo_sincos(angle, &s, &c);
    *x = c;
    *y = s;
  }
}

static void string_mod_color(const lg_string_mod* sm, uint64_t ix, float* out) {
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  uint32_t cnt = 0;
  for (uint32_t k = 0; k < sm->n_colors; ++k) {
    const lg_mod_color* e = &sm->colors[k];
    if (ix % e->modulo == e->rem) {
      for (int ch = 0; ch < 4; ++ch) acc[ch] += e->color[ch];
      ++cnt;
    }
  }
  for (int ch = 0; ch < 4; ++ch) out[ch] = cnt ? acc[ch] / (float)cnt : sm->color[ch];
}

/* StringMod::draw_init_points (string_mod.rs:104-122): the point that line iix joins to
 * point iix, by the mod's mode (u64 arithmetic wrapping like Rust's release build). */
static uint64_t string_mod_target(const lg_string_mod* sm, uint64_t iix) {
  const uint64_t m = sm->modulo;
  switch (sm->mode) {
    case LG_SM_ADD: return (iix + sm->num) % m;
    case LG_SM_MUL: return (iix * sm->num) % m;
    case LG_SM_POW: return wrapping_pow(iix, (uint32_t)sm->num) % m;
    default: return wrapping_pow(sm->num, (uint32_t)iix) % m;
  }
}

static int string_mod_check(const lg_string_mod* sm, int nested) {
  if ((!nested && sm->curve > LG_CURVE_LISSAJOUS) || sm->mode > LG_SM_BASE) return LGO_ERR_UNSUPPORTED;
  if (sm->n_colors && !sm->colors) return LGO_ERR_INVALID;
  for (uint32_t k = 0; k < sm->n_colors; ++k)
    if (sm->colors[k].modulo == 0) return LGO_ERR_INVALID;
  return LGO_OK;
}

/* Crossing of segments ab and cd, the definition the library states for lg_string_mod.nested
 * (collision2d's LineSegment::intersect is not vendored): the 2x2 parametric solve
 * a + t (b - a) = c + u (d - c), each FP64 operation rounded on its own; a crossing needs a
 * non-zero determinant and t, u in [0, 1]. */
static int seg_cross(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy,
                     double* px, double* py) {
  const double rx = bx - ax, ry = by - ay, sx = dx - cx, sy = dy - cy;
  const double den = rx * sy - ry * sx;
  if (den == 0.0) return 0;
  const double wx = cx - ax, wy = cy - ay;
  const double t = (wx * sy - wy * sx) / den;
  const double u = (wx * ry - wy * rx) / den;
  if (!(t >= 0.0 && t <= 1.0 && u >= 0.0 && u <= 1.0)) return 0;
  *px = ax + rx * t;
  *py = ay + ry * t;
  return 1;
}

int lgo_seg_cross(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy,
                  double* px, double* py) {
  return seg_cross(ax, ay, bx, by, cx, cy, dx, dy, px, py);
}

/* StringMod::line_crossings_as_points (string_mod.rs:87-102): the lines of the mod's own
 * draw, then for diff = 1 .. m-1 and a = 0 .. m-1 the crossing of line a with line
 * (a + diff) % m.  Writes up to cap points (x, y) to xy; *n_out = all crossings. */
int lgo_string_mod_crossings(const lg_string_mod* sm, double* xy, uint64_t cap, uint64_t* n_out) {
  if (!sm || !n_out) return LGO_ERR_INVALID;
  *n_out = 0;
  const uint64_t m = sm->modulo;
  if (m < 2) return LGO_OK;
  if (m > LG_STRING_MOD_NESTED_MAX) return LGO_ERR_UNSUPPORTED;
  int rc = string_mod_check(sm, 0);
  if (rc) return rc;
  double* L = malloc(4 * m * sizeof(double));
  if (!L) return LGO_ERR_OOM;
  for (uint64_t i = 0; i < m; ++i) {
    string_mod_point(sm, i % m, &L[4 * i], &L[4 * i + 1]);
    string_mod_point(sm, string_mod_target(sm, i) % m, &L[4 * i + 2], &L[4 * i + 3]);
  }
  uint64_t n = 0;
  for (uint64_t diff = 1; diff < m; ++diff)
    for (uint64_t a = 0; a < m; ++a) {
      const double* p = &L[4 * a];
      const double* q = &L[4 * ((a + diff) % m)];
      double x, y;
      if (seg_cross(p[0], p[1], p[2], p[3], q[0], q[1], q[2], q[3], &x, &y)) {
        if (xy && n < cap) { xy[2 * n] = x; xy[2 * n + 1] = y; }
        ++n;
      }
    }
  free(L);
  *n_out = n;
  return xy && n > cap ? LGO_ERR_TRUNCATED : LGO_OK;
}

int lgo_string_mod_chords(const lg_params* prm, lg_chord* out, uint64_t cap, uint64_t* n_out) {
  if (!prm || !n_out) return LGO_ERR_INVALID;
  const lg_string_mod* sm = &prm->string_mod;
  *n_out = 0;
  if (sm->modulo == 0) return LGO_OK;
  int rc = string_mod_check(sm, 0);
  if (rc) return rc;
  if (sm->nested) {  /* StringMod::draw with a nested mod (string_mod.rs:152-155) */
    const lg_string_mod* ns = sm->nested;
    if ((rc = string_mod_check(ns, 1))) return rc;
    uint64_t np = 0;
    if ((rc = lgo_string_mod_crossings(sm, NULL, 0, &np))) return rc;
    const uint64_t n = np ? ns->modulo : 0;
    *n_out = n;
    if (n == 0) return LGO_OK;
    if (cap < n) return LGO_ERR_TRUNCATED;
    double* pts = malloc(2 * np * sizeof(double));
    if (!pts) return LGO_ERR_OOM;
    if ((rc = lgo_string_mod_crossings(sm, pts, np, &np))) { free(pts); return rc; }
    for (uint64_t iix = 0; iix < n; ++iix) {
      const uint64_t ix = string_mod_target(ns, iix);
      const double* a = &pts[2 * (iix % np)];
      const double* b = &pts[2 * (ix % np)];
      lg_chord* c = &out[iix];
      c->x0 = (float)a[0]; c->y0 = (float)a[1]; c->x1 = (float)b[0]; c->y1 = (float)b[1];
      string_mod_color(ns, iix, c->color0);
      string_mod_color(ns, ix, c->color1);
    }
    free(pts);
    return LGO_OK;
  }
  const uint64_t m = sm->modulo;
  *n_out = m;
  if (cap < m) return LGO_ERR_TRUNCATED;
  for (uint64_t iix = 0; iix < m; ++iix) {
    const uint64_t ix = string_mod_target(sm, iix);
    double xa, ya, xb, yb;
    string_mod_point(sm, iix % m, &xa, &ya);
    string_mod_point(sm, ix % m, &xb, &yb);
    lg_chord* c = &out[iix];
    c->x0 = (float)xa; c->y0 = (float)ya; c->x1 = (float)xb; c->y1 = (float)yb;
    string_mod_color(sm, iix, c->color0);
    string_mod_color(sm, ix, c->color1);
  }
  return LGO_OK;
}

int lgo_trace(const lg_geo* geos, uint32_t n_geo, const lg_object* objs, uint32_t n_obj,
              const lg_light* lights, uint32_t n_lights, const lg_params* prm,
              uint32_t ray_stride, uint32_t ray_offset, int n_threads,
              lg_segment* segs, lg_path_record* paths, double* seg64, uint64_t cap,
              uint64_t* n_out, lgo_stats* stats) {
  if (!prm || !n_out || (n_geo && !geos) || (n_obj && !objs) || (n_lights && !lights)) return LGO_ERR_INVALID;
  if (ray_stride == 0) ray_stride = 1;
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  oscene S;
  S.g = geos; S.n_geo = n_geo; S.o = objs; S.n_obj = n_obj; S.l = lights; S.n_light = n_lights;
  S.prm = *prm;
  S.aspect = (double)((float)prm->width / (float)prm->height); /* renderer: f32 aspect */
  int rc = validate_scene(&S);
  if (rc) return rc;
  double* n0 = calloc(n_lights ? n_lights : 1, sizeof(double));
  uint64_t nch = 0;
  for (uint32_t l = 0; l < n_lights; ++l) {
    n0[l] = light_medium(&S, &lights[l]);
    uint64_t span = (uint64_t)CHUNK * ray_stride;
    nch += (lights[l].num_rays + span - 1) / span;
  }
  ojob J;
  memset(&J, 0, sizeof J);
  J.S = &S; J.n0 = n0; J.stride = ray_stride; J.offset = ray_offset;
  J.n_chunks = nch;
  J.chunk_light = calloc(nch ? nch : 1, sizeof(uint64_t));
  J.chunk_begin = calloc(nch ? nch : 1, sizeof(uint64_t));
  J.out = calloc(nch + 1, sizeof(obuf));
  if (!J.chunk_light || !J.chunk_begin || !J.out || !n0) {
    free(n0); free(J.chunk_light); free(J.chunk_begin); free(J.out);
    return LGO_ERR_OOM;
  }
  uint64_t c = 0;
  uint64_t prim_total = 0;
  for (uint32_t l = 0; l < n_lights; ++l) {
    uint64_t span = (uint64_t)CHUNK * ray_stride;
    for (uint64_t b = 0; b < lights[l].num_rays; b += span) {
      J.chunk_light[c] = l;
      J.chunk_begin[c] = b + ray_offset;
      ++c;
    }
    for (uint64_t i = ray_offset; i < lights[l].num_rays; i += ray_stride) ++prim_total;
  }
  pthread_mutex_init(&J.mu, NULL);
  int nt = n_threads > 0 ? n_threads : online_cores();
  if (nt > 256) nt = 256;
  pthread_t th[256];
  for (int i = 0; i < nt; ++i) pthread_create(&th[i], NULL, worker, &J);
  for (int i = 0; i < nt; ++i) pthread_join(th[i], NULL);
  pthread_mutex_destroy(&J.mu);
  rc = J.rc;
  /* overlays: curved-mirror control lines (tracer.rs:341-346, object.rs:355-365) */
  obuf* ov = &J.out[nch];
  if (!rc && ray_offset == 0 && prm->emit_control_lines) {
    const float red[4] = {1.f, 0.f, 0.f, 1.f};
    for (uint32_t k = 0; k < n_obj && !rc; ++k) {
      if (objs[k].kind != LG_OBJ_CURVED_MIRROR) continue;
      const double* v = geos[objs[k].geo].v;
      for (int s = 0; s < 3 && !rc; ++s) {
        lg_path_record r = {0, k, 0xffff, (uint8_t)s, 0, -1, LG_SRC_CONTROL_LINE};
        rc = buf_push(ov, mk(v[2 * s], v[2 * s + 1]), mk(v[2 * s + 2], v[2 * s + 3]), red, &r);
      }
    }
  }
  uint64_t total = 0, visits = 0, nearc = 0;
  for (uint64_t i = 0; i <= nch; ++i) {
    total += J.out[i].n;
    visits += J.out[i].visits;
    nearc += J.out[i].near;
  }
  *n_out = total;
  if (!rc && total > cap) rc = LGO_ERR_TRUNCATED;
  if (!rc) {
    uint64_t w = 0;
    for (uint64_t i = 0; i <= nch; ++i) {
      obuf* b = &J.out[i];
      if (segs) memcpy(segs + w, b->seg, b->n * sizeof(lg_segment));
      if (paths) memcpy(paths + w, b->rec, b->n * sizeof(lg_path_record));
      if (seg64) memcpy(seg64 + 4 * w, b->s64, b->n * 4 * sizeof(double));
      w += b->n;
    }
  }
  for (uint64_t i = 0; i <= nch; ++i) {
    free(J.out[i].seg); free(J.out[i].rec); free(J.out[i].s64);
  }
  free(J.out); free(J.chunk_light); free(J.chunk_begin); free(n0);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (stats) {
    stats->primary_rays = prim_total;
    stats->ray_visits = visits;
    stats->segments = total;
    stats->near_degenerate = nearc;
    stats->pixels = 0;
    stats->seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  }
  return rc;
}

int lgo_geo_hits(const lg_geo* geos, uint32_t n_geo, int32_t root, double ox, double oy,
                 double dx, double dy, lgo_hit* out, int cap, uint32_t* flags) {
  if (validate_geo(geos, n_geo, root, 0)) return LGO_ERR_INVALID;
  ohit tmp[MAX_GEO_HITS];
  double ev = INFINITY;
  int n = geo_hits(geos, root, mk(ox, oy), mk(dx, dy), tmp, MAX_GEO_HITS, &ev, 0);
  if (flags) *flags = ev < INFINITY ? NEAR : 0;
  int w = n < cap ? n : cap;
  for (int i = 0; i < w; ++i) {
    out[i].t = tmp[i].t; out[i].px = tmp[i].p.x; out[i].py = tmp[i].p.y;
    out[i].nx = tmp[i].n.x; out[i].ny = tmp[i].n.y;
  }
  return n;
}

int lgo_geo_contains(const lg_geo* geos, uint32_t n_geo, int32_t root, double px, double py) {
  if (validate_geo(geos, n_geo, root, 0)) return LGO_ERR_INVALID;
  return geo_contains(geos, root, mk(px, py), NULL);
}

double lgo_light_medium(const lg_geo* geos, uint32_t n_geo, const lg_object* objs,
                        uint32_t n_obj, const lg_light* light) {
  oscene S;
  memset(&S, 0, sizeof S);
  S.g = geos; S.n_geo = n_geo; S.o = objs; S.n_obj = n_obj;
  return light_medium(&S, light);
}

/* ---------------------------------------------------------------------- raster */
int64_t lgo_fixed(float v) {
  if (v != v) return 0;
  if (v > 1048576.0f) v = 1048576.0f;
  if (v < -1048576.0f) v = -1048576.0f;
  return llrintf(v * 4294967296.0f);
}

static int blend_ok(const lg_blend_component* b) {
  int op = b->op, sf = b->src_factor, df = b->dst_factor;
  if (op == LG_BO_MIN || op == LG_BO_MAX) return sf == LG_BF_ONE && df == LG_BF_ONE;
  if (op != LG_BO_ADD && op != LG_BO_REVERSE_SUBTRACT) return 0;
  if (df != LG_BF_ONE) return 0;
  return sf == LG_BF_ZERO || sf == LG_BF_ONE || sf == LG_BF_SRC || sf == LG_BF_ONE_MINUS_SRC ||
         sf == LG_BF_SRC_ALPHA || sf == LG_BF_ONE_MINUS_SRC_ALPHA || sf == LG_BF_CONSTANT ||
         sf == LG_BF_ONE_MINUS_CONSTANT;
}

static float factor(int f, int ch, const float* src, const float* k) {
  switch (f) {
    case LG_BF_ZERO: return 0.0f;
    case LG_BF_ONE: return 1.0f;
    case LG_BF_SRC: return src[ch];
    case LG_BF_ONE_MINUS_SRC: return 1.0f - src[ch];
    case LG_BF_SRC_ALPHA: return src[3];
    case LG_BF_ONE_MINUS_SRC_ALPHA: return 1.0f - src[3];
    case LG_BF_CONSTANT: return k[ch];
    default: return 1.0f - k[ch];
  }
}

/* per-channel source term and op of one segment */
static void contribution(const lg_params* P, const float* src, float* val, int* op) {
  for (int ch = 0; ch < 4; ++ch) {
    const lg_blend_component* b = ch < 3 ? &P->color_blend : &P->alpha_blend;
    op[ch] = b->op;
    if (b->op == LG_BO_MIN || b->op == LG_BO_MAX) val[ch] = src[ch];
    else val[ch] = src[ch] * factor(b->src_factor, ch, src, P->blend_constant);
  }
}

int lgo_clear(int64_t* acc, uint32_t w, uint32_t h, const lg_params* P) {
  int64_t c[4];
  for (int i = 0; i < 4; ++i) c[i] = lgo_fixed(P->clear_color[i]);
  for (uint64_t p = 0; p < (uint64_t)w * h; ++p)
    for (int i = 0; i < 4; ++i) acc[4 * p + i] = c[i];
  return LGO_OK;
}

/* raster setup shared by the fixed-point and double rasterisers */
typedef struct {
  int xmajor;
  float ua, va, slope;
  int lo, hi; /* major-axis pixel range [lo, hi) */
} rsetup;

static int raster_setup(const lg_segment* s, uint32_t W, uint32_t H, rsetup* R) {
  float sc = (float)H * 0.5f, cx = (float)W * 0.5f, cy = sc;
  float X0 = fmaf(s->x0, sc, cx), Y0 = fmaf(-s->y0, sc, cy);
  float X1 = fmaf(s->x1, sc, cx), Y1 = fmaf(-s->y1, sc, cy);
  if (!isfinite(X0) || !isfinite(Y0) || !isfinite(X1) || !isfinite(Y1)) return 0;
  float adx = fabsf(X1 - X0), ady = fabsf(Y1 - Y0);
  R->xmajor = adx >= ady;
  float ua, va, ub, vb;
  if (R->xmajor) { ua = X0; va = Y0; ub = X1; vb = Y1; } else { ua = Y0; va = X0; ub = Y1; vb = X1; }
  if (ub < ua) { float t = ua; ua = ub; ub = t; t = va; va = vb; vb = t; }
  float du = ub - ua;
  if (!(du > 0.0f)) return 0;
  R->slope = (vb - va) / du;
  R->ua = ua;
  R->va = va;
  float nmaj = (float)(R->xmajor ? W : H);
  float lo = ceilf(ua - 0.5f), hi = ceilf(ub - 0.5f);
  if (lo < 0.0f) lo = 0.0f;
  if (hi > nmaj) hi = nmaj;
  if (!(lo < hi)) return 0;
  R->lo = (int)lo;
  R->hi = (int)hi;
  return 1;
}

static inline int raster_minor(const rsetup* R, int i) {
  float v = fmaf(((float)i + 0.5f) - R->ua, R->slope, R->va);
  float fv = floorf(v);
  if (!(fv >= -1.0f)) return -1;
  if (fv > 2147483000.0f) return 2147483000;
  return (int)fv;
}

typedef struct {
  const lg_segment* segs;
  uint64_t n;
  const lg_params* P;
  int64_t* acc;
  uint32_t r0, r1; /* band of image rows (y-major: pixel rows; the same for both axes) */
  uint64_t pixels;
} rjob;

static void apply(int64_t* px, const int64_t* q, const int* op) {
  for (int ch = 0; ch < 4; ++ch) {
    switch (op[ch]) {
      case LG_BO_ADD: px[ch] += q[ch]; break;
      case LG_BO_REVERSE_SUBTRACT: px[ch] -= q[ch]; break;
      case LG_BO_MIN: if (q[ch] < px[ch]) px[ch] = q[ch]; break;
      default: if (q[ch] > px[ch]) px[ch] = q[ch]; break;
    }
  }
}

static void* raster_band(void* arg) {
  rjob* J = (rjob*)arg;
  uint32_t W = J->P->width, H = J->P->height;
  for (uint64_t k = 0; k < J->n; ++k) {
    rsetup R;
    if (!raster_setup(&J->segs[k], W, H, &R)) continue;
    float val[4];
    int op[4];
    contribution(J->P, J->segs[k].color, val, op);
    int64_t q[4];
    for (int ch = 0; ch < 4; ++ch) q[ch] = lgo_fixed(val[ch]);
    if (R.xmajor) {
      /* rows of this band: restrict the column range conservatively, then test exactly */
      int lo = R.lo, hi = R.hi;
      if (R.slope != 0.0f) {
        double c0 = R.ua + ((double)J->r0 - R.va) / R.slope - 0.5;
        double c1 = R.ua + ((double)J->r1 - R.va) / R.slope - 0.5;
        double cmin = c0 < c1 ? c0 : c1, cmax = c0 < c1 ? c1 : c0;
        if (cmin - 2.0 > lo) lo = cmin - 2.0 > hi ? hi : (int)(cmin - 2.0);
        if (cmax + 3.0 < hi) hi = cmax + 3.0 < lo ? lo : (int)(cmax + 3.0);
      } else {
        int j = raster_minor(&R, R.lo);
        if (j < (int)J->r0 || j >= (int)J->r1) continue;
      }
      for (int i = lo; i < hi; ++i) {
        int j = raster_minor(&R, i);
        if (j < (int)J->r0 || j >= (int)J->r1) continue;
        apply(&J->acc[4 * ((uint64_t)j * W + (uint64_t)i)], q, op);
        J->pixels++;
      }
    } else {
      int lo = R.lo > (int)J->r0 ? R.lo : (int)J->r0;
      int hi = R.hi < (int)J->r1 ? R.hi : (int)J->r1;
      for (int j = lo; j < hi; ++j) {
        int i = raster_minor(&R, j);
        if (i < 0 || i >= (int)W) continue;
        apply(&J->acc[4 * ((uint64_t)j * W + (uint64_t)i)], q, op);
        J->pixels++;
      }
    }
  }
  return NULL;
}

int lgo_raster(const lg_segment* segs, uint64_t n, const lg_params* P, int64_t* acc,
               int n_threads, uint64_t* pixels) {
  if (!P || !acc || (n && !segs)) return LGO_ERR_INVALID;
  if (!blend_ok(&P->color_blend) || !blend_ok(&P->alpha_blend)) return LGO_ERR_UNSUPPORTED;
  int nt = n_threads > 0 ? n_threads : online_cores();
  if (nt > 256) nt = 256;
  if ((uint32_t)nt > P->height) nt = (int)P->height;
  rjob J[256];
  pthread_t th[256];
  for (int t = 0; t < nt; ++t) {
    J[t].segs = segs; J[t].n = n; J[t].P = P; J[t].acc = acc; J[t].pixels = 0;
    J[t].r0 = (uint32_t)((uint64_t)P->height * t / nt);
    J[t].r1 = (uint32_t)((uint64_t)P->height * (t + 1) / nt);
    pthread_create(&th[t], NULL, raster_band, &J[t]);
  }
  uint64_t px = 0;
  for (int t = 0; t < nt; ++t) {
    pthread_join(th[t], NULL);
    px += J[t].pixels;
  }
  if (pixels) *pixels = px;
  return LGO_OK;
}

/* String-mod lines: the raster rule of the segments, with the colour interpolated along
 * the major axis (f from the unswapped vertex coordinates, clamped to [0, 1]). */
static void chord_setup(const lg_chord* c, uint32_t W, uint32_t H, lg_segment* sg, float* u0, float* du) {
  sg->x0 = c->x0; sg->y0 = c->y0; sg->x1 = c->x1; sg->y1 = c->y1;
  for (int ch = 0; ch < 4; ++ch) sg->color[ch] = c->color0[ch];
  float sc = (float)H * 0.5f, cx = (float)W * 0.5f, cy = sc;
  float X0 = fmaf(c->x0, sc, cx), Y0 = fmaf(-c->y0, sc, cy);
  float X1 = fmaf(c->x1, sc, cx), Y1 = fmaf(-c->y1, sc, cy);
  int xmajor = fabsf(X1 - X0) >= fabsf(Y1 - Y0);
  *u0 = xmajor ? X0 : Y0;
  *du = (xmajor ? X1 : Y1) - *u0;
}

static void chord_color(const lg_chord* c, float u0, float du, int i, float* src) {
  float f = (((float)i + 0.5f) - u0) / du;
  f = f < 0.0f ? 0.0f : (f > 1.0f ? 1.0f : f);
  for (int ch = 0; ch < 4; ++ch) src[ch] = fmaf(f, c->color1[ch] - c->color0[ch], c->color0[ch]);
}

int lgo_raster_chords(const lg_chord* chords, uint64_t n, const lg_params* P, int64_t* acc, uint64_t* pixels) {
  if (!P || !acc || (n && !chords)) return LGO_ERR_INVALID;
  if (!blend_ok(&P->color_blend) || !blend_ok(&P->alpha_blend)) return LGO_ERR_UNSUPPORTED;
  uint32_t W = P->width, H = P->height;
  uint64_t px = 0;
  for (uint64_t k = 0; k < n; ++k) {
    lg_segment sg;
    float u0, du;
    chord_setup(&chords[k], W, H, &sg, &u0, &du);
    rsetup R;
    if (!raster_setup(&sg, W, H, &R)) continue;
    for (int i = R.lo; i < R.hi; ++i) {
      int j = raster_minor(&R, i);
      int x = R.xmajor ? i : j, y = R.xmajor ? j : i;
      if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) continue;
      float src[4], val[4];
      int op[4];
      chord_color(&chords[k], u0, du, i, src);
      contribution(P, src, val, op);
      int64_t q[4];
      for (int ch = 0; ch < 4; ++ch) q[ch] = lgo_fixed(val[ch]);
      apply(&acc[4 * ((uint64_t)y * W + (uint64_t)x)], q, op);
      ++px;
    }
  }
  if (pixels) *pixels = px;
  return LGO_OK;
}

int lgo_raster_chords_f64(const lg_chord* chords, uint64_t n, const lg_params* P, double* acc, uint64_t* pixels) {
  if (!P || !acc || (n && !chords)) return LGO_ERR_INVALID;
  if (!blend_ok(&P->color_blend) || !blend_ok(&P->alpha_blend)) return LGO_ERR_UNSUPPORTED;
  uint32_t W = P->width, H = P->height;
  uint64_t px = 0;
  for (uint64_t k = 0; k < n; ++k) {
    lg_segment sg;
    float u0, du;
    chord_setup(&chords[k], W, H, &sg, &u0, &du);
    rsetup R;
    if (!raster_setup(&sg, W, H, &R)) continue;
    for (int i = R.lo; i < R.hi; ++i) {
      int j = raster_minor(&R, i);
      int x = R.xmajor ? i : j, y = R.xmajor ? j : i;
      if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) continue;
      float src[4], val[4];
      int op[4];
      chord_color(&chords[k], u0, du, i, src);
      contribution(P, src, val, op);
      double* p = &acc[4 * ((uint64_t)y * W + (uint64_t)x)];
      for (int ch = 0; ch < 4; ++ch) {
        switch (op[ch]) {
          case LG_BO_ADD: p[ch] += val[ch]; break;
          case LG_BO_REVERSE_SUBTRACT: p[ch] -= val[ch]; break;
          case LG_BO_MIN: if (val[ch] < p[ch]) p[ch] = val[ch]; break;
          default: if (val[ch] > p[ch]) p[ch] = val[ch]; break;
        }
      }
      ++px;
    }
  }
  if (pixels) *pixels = px;
  return LGO_OK;
}

int lgo_raster_f64(const lg_segment* segs, uint64_t n, const lg_params* P, double* acc, uint64_t* pixels) {
  if (!P || !acc || (n && !segs)) return LGO_ERR_INVALID;
  if (!blend_ok(&P->color_blend) || !blend_ok(&P->alpha_blend)) return LGO_ERR_UNSUPPORTED;
  uint32_t W = P->width, H = P->height;
  uint64_t px = 0;
  for (uint64_t k = 0; k < n; ++k) {
    rsetup R;
    if (!raster_setup(&segs[k], W, H, &R)) continue;
    float val[4];
    int op[4];
    contribution(P, segs[k].color, val, op);
    for (int i = R.lo; i < R.hi; ++i) {
      int j = raster_minor(&R, i);
      int x = R.xmajor ? i : j, y = R.xmajor ? j : i;
      if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) continue;
      double* p = &acc[4 * ((uint64_t)y * W + (uint64_t)x)];
      for (int ch = 0; ch < 4; ++ch) {
        switch (op[ch]) {
          case LG_BO_ADD: p[ch] += val[ch]; break;
          case LG_BO_REVERSE_SUBTRACT: p[ch] -= val[ch]; break;
          case LG_BO_MIN: if (val[ch] < p[ch]) p[ch] = val[ch]; break;
          default: if (val[ch] > p[ch]) p[ch] = val[ch]; break;
        }
      }
      ++px;
    }
  }
  if (pixels) *pixels = px;
  return LGO_OK;
}

/* -------------------------------------------------------------------- resolve */
uint16_t lgo_f32_to_f16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ex = (x >> 23) & 0xffu, man = x & 0x7fffffu;
  if (ex == 0xffu) return (uint16_t)(sign | 0x7c00u | (man ? 0x200u | (man >> 13) : 0u));
  int e = (int)ex - 127 + 15;
  if (e >= 31) return (uint16_t)(sign | 0x7c00u);
  if (e <= 0) {
    if (e < -10) return (uint16_t)sign;
    man |= 0x800000u;
    int shift = 14 - e;
    uint32_t h = man >> shift, rem = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rem > half || (rem == half && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
  }
  uint32_t h = ((uint32_t)e << 10) | (man >> 13), rem = man & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
  return (uint16_t)(sign | h);
}

float lgo_f16_to_f32(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t ex = (h >> 10) & 0x1fu, man = h & 0x3ffu, x;
  if (ex == 0) {
    if (man == 0) x = sign;
    else {
      int e = -1;
      do { ++e; man <<= 1; } while (!(man & 0x400u));
      x = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3ffu) << 13);
    }
  } else if (ex == 31) {
    x = sign | 0x7f800000u | (man << 13);
  } else {
    x = sign | ((ex + 127 - 15) << 23) | (man << 13);
  }
  float f;
  memcpy(&f, &x, 4);
  return f;
}

static float fixed_to_f32(int64_t v) { return (float)v * 2.3283064365386963e-10f; /* 2^-32 */ }

void lgo_resolve_f16(const int64_t* acc, uint32_t w, uint32_t h, uint16_t* out) {
  for (uint64_t p = 0; p < (uint64_t)w * h * 4; ++p) out[p] = lgo_f32_to_f16(fixed_to_f32(acc[p]));
}

void lgo_resolve_rgba8(const int64_t* acc, uint32_t w, uint32_t h, uint8_t* out) {
  for (uint64_t p = 0; p < (uint64_t)w * h * 4; ++p) {
    float f = lgo_f16_to_f32(lgo_f32_to_f16(fixed_to_f32(acc[p])));
    float g = powf(f, 1.0f / 2.2f) * 255.0f;
    uint8_t u = 0;
    if (g != g || g <= 0.0f) u = 0;
    else if (g >= 255.0f) u = 255;
    else u = (uint8_t)g;
    out[p] = u;
  }
}
