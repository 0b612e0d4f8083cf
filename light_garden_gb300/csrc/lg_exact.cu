// lg_exact.cu — the solve and bounce kernels of the exact FP64 precision mode.
//
// In LG_PRECISION_EXACT one generation is k_scan (FP32 search, lg_trace.cu: candidates of
// the nearest hit, in work lists) -> k_solve_x -> k_bounce_x.  Both kernels here evaluate
// the restated collision2d formulas of lg_x64.cuh in IEEE double with every operation
// rounded on its own, so every decision of Tracer::trace (tracer.rs:360-493: nearest hit
// with strict < in object order, medium rule, refract / reflect, colour split, canvas exit)
// is taken on the same FP64 values a CPU evaluation of those formulas computes, and the
// segments and child rays come out bit for bit equal.
//
// Rays and hits keep their FP64 coordinates in the 8-byte df slots of RayRec / HitRec (xd /
// xdf move the bits).
#include "lg_kernels.cuh"
#include "lg_trace_common.cuh"

// CTAs per SM the exact kernels' registers are sized for (build-time, for sweeps)
#ifndef LG_SOLVE_X_BLOCKS
#define LG_SOLVE_X_BLOCKS 4
#endif
#ifndef LG_BOUNCE_X_BLOCKS
#define LG_BOUNCE_X_BLOCKS 4
#endif

namespace lgd {

using lgx::V;

__device__ __forceinline__ V ray_o(const RayRec& r) { return lgx::mk(xd(r.ox), xd(r.oy)); }
__device__ __forceinline__ V ray_d(const RayRec& r) { return lgx::mk(xd(r.dx), xd(r.dy)); }

// Membership of object k (object.rs:240-253): mirrors enclose nothing.
__device__ __forceinline__ bool obj_contains_x(const SceneDev& S, uint32_t k, V p, uint32_t* fl) {
  const ObjInfo& oi = S.info[k];
  if (oi.flags & INFO_NO_CONTAINS) return false;
  return lgx::object_contains_tree(S.xgeo, S.xnode + oi.xnode_begin, (int)oi.xnode_count, p, fl);
}

// Membership of object k at p decided in FP32 where the FP32 copy of its leaves decides it:
// 1 inside, 0 outside, -1 undecided.  The band of leaf_member32 covers the rounding of p and
// of the leaf parameters to FP32 (1e-6 of the coordinates against 6e-8), so a decided answer
// is the one the FP64 tree gives; objects the scan only bounds stay undecided.
__device__ __forceinline__ int obj_member32(const ObjScan& s, float px, float py) {
  if (s.info & INFO_NO_CONTAINS) return 0;
  const uint32_t sk = info_scan(s.info);
  if (sk == SCAN_ONE) {
    const uint32_t ka = info_leaf_a(s.info);
    return ka == LEAF_CUBIC ? -1 : leaf_member32(ka, s.a, px, py, 1e-6f);
  }
  if (sk != SCAN_TWO) return -1;
  const int a = leaf_member32(info_leaf_a(s.info), s.a, px, py, 1e-6f);
  const int b = leaf_member32(info_leaf_b(s.info), s.b, px, py, 1e-6f);
  switch (info_op(s.info)) {
    case LG_OP_AND: return (a == 0 || b == 0) ? 0 : (a == 1 && b == 1 ? 1 : -1);
    case LG_OP_OR: return (a == 1 || b == 1) ? 1 : (a == 0 && b == 0 ? 0 : -1);
    default: return (a == 0 || b == 1) ? 0 : (a == 1 && b == 0 ? 1 : -1);  // a and not b
  }
}

// obj_contains_x behind the FP32 pre-test (k scene-global).
__device__ __forceinline__ bool obj_contains_f(const SceneDev& S, uint32_t k, V p, uint32_t* fl) {
  const int m = obj_member32(S.scan[k], (float)p.x, (float)p.y);
  if (m >= 0) return m == 1;
  return obj_contains_x(S, k, p, fl);
}

// Light start media (tracer.rs:280-287: the last object with a material containing the
// light's position) and spot base angles (light.rs:230-234), once per frame.
template <bool MULTI>
__global__ void k_light_setup_x(SceneDev S) {
  const uint32_t l0 = S.serve ? S.light_lo : 0u, l1 = S.serve ? S.light_hi : S.n_lights;
  for (uint32_t l = l0 + blockIdx.x * blockDim.x + threadIdx.x; l < l1; l += gridDim.x * blockDim.x) {
    LightDev& L = S.lights[l];
    const SceneLoc sl = scene_of<MULTI>(S, L.scene);
    double n = 1.0;
    const V p = lgx::mk(L.ox, L.oy);
    for (uint32_t k = sl.base; k < sl.base + sl.n; ++k)
      if (obj_contains_x(S, k, p, nullptr) && (S.info[k].flags & INFO_MATERIAL)) n = S.info[k].n64;
    L.n0x = n;
    L.dir_angle = lgx::spot_base_angle(L.vx, L.vy);
  }
}
template __global__ void k_light_setup_x<false>(SceneDev);
template __global__ void k_light_setup_x<true>(SceneDev);

// ------------------------------------------------------------------ nearest hit
// Exact hit record in HitRec's slots: t, p, n as FP64, the event parameter ev in (k, ev).
__device__ __forceinline__ void store_hit_x(HitRec& o, int obj, const lgx::Hit& h, V n, int leaf, double ev,
                                            uint8_t flags) {
  o.obj = obj < 0 ? HIT_NONE : (uint16_t)obj;
  o.t = xdf(h.t); o.px = xdf(h.p.x); o.py = xdf(h.p.y); o.nx = xdf(n.x); o.ny = xdf(n.y);
  const df e = xdf(ev);
  o.k = e.hi;
  o.ev = e.lo;
  o.leaf = (uint8_t)leaf;
  o.flags = flags;
}

// Nearest hit of object k (scene-global index) with the ray: the minimum distance_squared
// over the object's hits, the first one on ties (tracer.rs:412-424 per object).  Returns
// that distance (INFINITY: no hit).  Out of line, so the solve kernel keeps one copy of the
// geometry code and its own registers for the ray state.
static __device__ __noinline__ double obj_best_x(const SceneDev& S, uint32_t k, V o, V d, double& ev, lgx::Hit& best) {
  const ObjInfo& oi = S.info[k];
  double ob = INFINITY;
  lgx::object_hits(S.xgeo, S.xnode + oi.xnode_begin, (int)oi.xnode_count, o, d, ev, [&](const lgx::Hit& h) {
    const V dv = lgx::vsub(h.p, o);
    const double d2 = lgx::dot(dv, dv);
    if (lgx::plt(d2, ob)) {
      ob = d2;
      best = h;
    }
  });
  return ob;
}

// The FP64 hit of one leaf at the root the FP32 scan proved (t32; face32: the rect face as
// 2 axis + (outward sign > 0); s32: a cubic's curve parameter): the very operations of
// leaf_hits for that root only.  A circle computes the quotient of its proved root (q / a or
// c / q, told apart by their FP32 values) and not the other; a rect computes the slab quotient
// of its proved face and not the other three; a cubic searches only the bracket that holds
// s32.  Other leaves take leaf_hits and the root nearest t32.  False: no such hit (the caller
// solves the object whole).
__device__ __forceinline__ bool leaf_proved_hit(const lg_geo* G, const lg_geo& g, V o, V d, float t32, int face32,
                                                float s32, double& ev, lgx::Hit& out) {
  using namespace lgx;
  if (g.kind == LG_GEO_CIRCLE) {
    const V oc = vsub(o, mk(g.origin[0], g.origin[1]));
    const double r = g.v[0];
    const double a = dot(d, d), b = dot(oc, d), cc = sub(dot(oc, oc), mul(r, r));
    const double disc = sub(mul(b, b), mul(a, cc));
    if (is_neg(disc)) return false;
    const double sq = sqr(disc);
    const double q = -add(b, b >= 0.0 ? sq : -sq);
    if (is_zero(q)) return false;
    const float ra = (float)q / (float)a, rc = (float)cc / (float)q;  // selection only
    const double t = fabsf(ra - t32) <= fabsf(rc - t32) ? dvd(q, a) : dvd(cc, q);
    if (!gt_pos(t, T_MIN)) return false;
    const V p = vadd(o, vscl(d, t));
    out = Hit{t, p, p, 0, 0};
    return true;
  }
  if (g.kind == LG_GEO_RECT) {
    if (face32 < 0) return false;
    const int ax = face32 >> 1;
    const bool pos = (face32 & 1) != 0;
    const V lo = irot(vsub(o, mk(g.origin[0], g.origin[1])), g.rot[0], g.rot[1]);
    const V ld = irot(d, g.rot[0], g.rot[1]);
    const double h = mul(0.5, g.v[ax]);
    const double O = ax ? lo.y : lo.x, D = ax ? ld.y : ld.x;
    if (is_zero(D)) return false;
    const double t = dvd(sub(pos ? h : -h, O), D);
    if (!gt_pos(t, T_MIN)) return false;
    out = mkhit(t, o, d, mk(0.0, 0.0), ax + (pos ? 2 : 0));
    return true;
  }
  if (g.kind == LG_GEO_CUBIC && s32 > 0.0f) {
    // the bracket between the derivative's roots that holds the proved curve parameter s32:
    // hits_cubic's operations for that bracket only (a parameter within 1e-4 of a knot, or
    // a knot or bracket end that is itself a root, takes the whole leaf below)
    const Cubic k = cubic_of(g.v);
    const double a[4] = {cross(d, vsub(k.c0, o)), cross(d, k.c1), cross(d, k.c2), cross(d, k.c3)};
    double kn[4];
    int nk = 0;
    kn[nk++] = 0.0;
    const double qa = mul(3.0, a[3]), qb = mul(2.0, a[2]), qc = a[1];
    if (qa != 0.0) {
      const double disc = sub(mul(qb, qb), mul(mul(4.0, qa), qc));
      if (disc >= 0.0) {
        const double sq = sqr(disc);
        const double q = mul(-0.5, add(qb, qb >= 0 ? sq : -sq));
        double r1 = dvd(q, qa), r2 = q != 0.0 ? dvd(qc, q) : r1;
        if (r1 > r2) { const double x = r1; r1 = r2; r2 = x; }
        if (r1 > 0.0 && r1 < 1.0) kn[nk++] = r1;
        if (r2 > 0.0 && r2 < 1.0 && (nk == 1 || r2 != kn[1])) kn[nk++] = r2;
      }
    } else if (qb != 0.0) {
      const double r = dvd(-qc, qb);
      if (r > 0.0 && r < 1.0) kn[nk++] = r;
    }
    kn[nk++] = 1.0;
    double lo = -1.0, hi = -1.0;
    for (int i = 0; i + 1 < nk; ++i)
      if ((double)s32 > kn[i] + 1e-4 && (double)s32 < kn[i + 1] - 1e-4) { lo = kn[i]; hi = kn[i + 1]; }
    if (lo >= 0.0) {
      const double flo = poly3(a, lo), fhi = poly3(a, hi);
      if (!is_zero(flo) && !is_zero(fhi) && is_neg(flo) != is_neg(fhi)) {
        const double sr = cubic_root(a, lo, hi, flo);
        const double t = dvd(dot(vsub(cubic_point(k, sr), o), d), dot(d, d));
        if (!gt_pos(t, T_MIN)) return false;
        out = mkhit(t, o, d, mk(sr, 0.0), 0);
        return true;
      }
    }
  }
  double near = INFINITY;
  bool found = false;
  leaf_hits(G, g, o, d, ev, [&](const Hit& h) {
    const double e = fabs(h.t - (double)t32);  // selection only
    if (e < near) {
      near = e;
      out = h;
      found = true;
    }
  });
  return found;
}

// An object whose nearest root the FP32 scan proved (a single candidate with a certain root
// and, for a two-leaf CSG object, certain membership of that root's point in the other
// leaf): only the proved leaf's root is computed in FP64, and a CSG hit point is lifted out
// of the Logic frame with the operations object_hits uses.  The other roots, the other leaf
// and the membership tests cannot change which hit object_hits keeps, so the result is the
// same bits.
static __device__ __noinline__ bool solve_proved_x(const SceneDev& S, const ObjInfo& oi, V o, V d, int side, int face,
                                                   float t32, float s32, double& ev, lgx::Hit& out) {
  const lgx::XNode* nd = S.xnode + oi.xnode_begin;
  const lg_geo& L = S.xgeo[nd[0].geo];
  if (oi.xnode_count == 1) {
    if (side != 0 || !leaf_proved_hit(S.xgeo, L, o, d, t32, face, s32, ev, out)) return false;
    out.node = 0;
    return true;
  }
  if (oi.xnode_count != 3 || L.kind != LG_GEO_LOGIC) return false;
  const V org = lgx::mk(L.origin[0], L.origin[1]);
  const V lo = lgx::irot(lgx::vsub(o, org), L.rot[0], L.rot[1]);
  const V ld = lgx::irot(d, L.rot[0], L.rot[1]);
  const int li = 1 + side;
  if (!leaf_proved_hit(S.xgeo, S.xgeo[nd[li].geo], lo, ld, t32, face, 0.0f, ev, out)) return false;
  out.node = li;
  out.p = lgx::vadd(org, lgx::rot(out.p, L.rot[0], L.rot[1]));
  return true;
}

// Every ray with candidates (the refine lists and the full-solve list of k_scan): the
// nearest hit over its candidates, each object solved whole as tracer.rs:412-424 does
// (the minimum distance_squared over the object's hits, then over objects with ties kept by
// the lower object index), and the near-degenerate flags of tracer.rs's decisions.  The
// CTA's warps take the candidates one solve class (circle, rect, segment, cubic / deep CSG,
// two-leaf CSG) at a time, with a barrier between classes, so that one geometry code path
// is in flight per CTA.
template <bool MULTI>
__global__ void __launch_bounds__(256, LG_SOLVE_X_BLOCKS) k_solve_x(SceneDev S, TraceBufs B, uint32_t gen) {
  __shared__ unsigned long long blk_solves;
  if (threadIdx.x == 0) blk_solves = 0;
  __syncthreads();
  uint64_t off[LIST_FULL + 2];
  off[0] = 0;
  for (int l = 0; l <= LIST_FULL; ++l) {
    const unsigned long long c = B.ctr->list_count[gen][l];
    off[l + 1] = off[l] + (c < B.queue_cap ? c : B.queue_cap);
  }
  const uint64_t total = off[LIST_FULL + 1];
  const RayRec* q = B.queue[gen & 1];
  unsigned long long my_solves = 0;
  // block-uniform loop (the class barrier needs every thread)
  for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x; base < total; base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const bool valid = i < total;
    uint32_t idx = 0;
    if (valid) {
      int l = 0;
      while (i >= off[l + 1]) ++l;
      idx = B.list[l][i - off[l]];
    }
    const RayRec r = q[idx];
    const ScanRec sc = B.scan[idx];
    const SceneLoc sl = scene_of<MULTI>(S, valid ? r.scene : 0u);
    const V o = ray_o(r), d = ray_d(r);
    double best_d2 = INFINITY, second = INFINITY, ev = INFINITY;
    int best = -1;
    lgx::Hit bh{0.0, lgx::mk(0.0, 0.0), lgx::mk(0.0, 0.0), 0, 0};
    auto consider = [&](uint32_t j) {
      lgx::Hit oh;
      ++my_solves;
      const double ob = obj_best_x(S, sl.base + j, o, d, ev, oh);
      if (!lgx::plt(ob, INFINITY)) return;
      if (lgx::plt(ob, best_d2) || (lgx::bits(ob) == lgx::bits(best_d2) && (int)j < best)) {
        second = best_d2;
        best_d2 = ob;
        best = (int)j;
        bh = oh;
      } else if (lgx::plt(ob, second)) {
        second = ob;
      }
    };
    // proved roots (single circle and rect leaves, two-leaf CSG) first, in a phase of their own
    bool proved = false;
    uint32_t pcls = 7u;
    if (valid && i < off[LIST_FULL] && !sc.overflow && sc.nc == 1 && (sc.leaf == 0 || sc.leaf == 1))
      pcls = solve_class(__ldg(&S.scan[sl.base + sc.cand[0]].info));
    // class 3 holds single cubic leaves and deep CSG trees; only a cubic reaches a refine list
    if (pcls == 0u || pcls == 1u || pcls == 4u || (pcls == 3u && sc.leaf == 0)) {
      proved = solve_proved_x(S, S.info[sl.base + sc.cand[0]], o, d, sc.leaf, sc.face, sc.t32, sc.s32, ev, bh);
      if (proved) {
        best = sc.cand[0];
        ++my_solves;
      }
    }
    __syncthreads();
    {
      uint32_t pending = valid && !sc.overflow && !proved ? (1u << sc.nc) - 1u : 0u;
      uint32_t cls[CAND];
      for (int k = 0; k < CAND; ++k)
        cls[k] = (pending >> k) & 1u ? solve_class(__ldg(&S.scan[sl.base + sc.cand[k]].info)) : 7u;
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
    if (sc.overflow) {  // candidate list overflow (rare): every object that passes the FP32 filters
      const ObjScan* sobjs = S.scan + sl.base;
      const float ox = (float)o.x, oy = (float)o.y, dx = (float)d.x, dy = (float)d.y;
      for (uint32_t j = 0; j < sl.n; ++j) {
        const float4 h = *reinterpret_cast<const float4*>(&sobjs[j]);
        float lb;
        if (!bound_test(h, ox, oy, dx, dy, sc.thr, lb)) continue;
        if (!(classify32(sobjs[j], ox, oy, dx, dy, lb, j == r.src_obj ? (int)r.src_leaf : -1).key <= sc.thr)) continue;
        consider(j);
      }
    }
    uint8_t fl = sc.overflow ? LG_PATH_FALLBACK : 0;
    // tracer.rs:404,417 ties within the band, and decisions in the band before the hit
    if (best >= 0 && second < INFINITY && lgx::sub(second, best_d2) <= lgx::mul(lgx::BAND, best_d2)) fl |= lgx::NEAR;
    if (best >= 0 ? ev <= lgx::add(lgx::mul(bh.t, 1.0 + 1e-6), 1e-12) : ev < INFINITY) fl |= lgx::NEAR;
    V n = lgx::mk(0.0, 0.0);
    int leaf = 0;
    if (best >= 0) {  // the normal of the winning hit only
      const ObjInfo& oi = S.info[sl.base + best];
      const lgx::XNode* nd = S.xnode + oi.xnode_begin;
      n = lgx::object_normal(S.xgeo, nd, d, bh);
      leaf = lgx::hit_leaf(S.xgeo, nd, bh);
    }
    store_hit_x(B.hit[idx], best, bh, n, leaf, ev, fl);
  }
  atomicAdd(&blk_solves, my_solves);
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(&B.ctr->fp64_solves, blk_solves);
}
template __global__ void k_solve_x<false>(SceneDev, TraceBufs, uint32_t);
template __global__ void k_solve_x<true>(SceneDev, TraceBufs, uint32_t);

// ------------------------------------------------------------------ bounce
struct BounceX {
  bool emit;
  float x0, y0, x1, y1;
  int hit;
  uint8_t flags;
  int nchild;
  RayRec child[2];
};

// Ray::refract restated (collision2d; called at tracer.rs:444-450): reflected direction,
// refracted direction unless total internal reflection, unpolarised Fresnel reflectance.
__device__ __forceinline__ bool refract_x(V d, V n, double n1, double n2, V& refl, V& refr, double& R,
                                          uint32_t& fl) {
  using namespace lgx;
  double ci = -dot(d, n);
  if (ci < 0.0) {
    ci = -ci;
    n = vscl(n, -1.0);
  }
  refl = vadd(d, vscl(n, mul(2.0, ci)));
  const double eta = dvd(n1, n2);
  const double k = sub(1.0, mul(mul(eta, eta), sub(1.0, mul(ci, ci))));
  if (fabs(k) <= BAND) fl |= NEAR;
  if (k < 0.0) {
    R = 1.0;
    return false;
  }
  const double ct = sqr(k);
  refr = vadd(vscl(d, eta), vscl(n, sub(mul(eta, ci), ct)));
  const double ds = add(mul(n1, ci), mul(n2, ct)), dp = add(mul(n1, ct), mul(n2, ci));
  if (ds == 0.0 || dp == 0.0) {
    R = 1.0;
    return true;
  }
  const double rs = dvd(sub(mul(n1, ci), mul(n2, ct)), ds);
  const double rp = dvd(sub(mul(n1, ct), mul(n2, ci)), dp);
  R = mul(0.5, add(mul(rs, rs), mul(rp, rp)));
  return true;
}

// The canvas exit of a ray whose origin lies strictly inside the canvas [-aspect, aspect] x
// [-1, 1] and whose exit is clear of the corners and of the origin: the same hit and flags as
// the slab test of the canvas rectangle (hits_rect), which needs the far face of each axis
// only: (sign(D) h - O) / D is the very quotient the slab test takes as its exit parameter.
// Returns false (nothing decided) when any of those conditions fails.
__device__ __forceinline__ bool canvas_exit_inside(V o, V d, double aspect, double& ev, lgx::Hit& first, int& nh) {
  using namespace lgx;
  const double h[2] = {aspect, 1.0};
  const double O[2] = {o.x, o.y}, D[2] = {d.x, d.y};
  double far[2];
  float nr[2];
  for (int ax = 0; ax < 2; ++ax) {
    if (is_zero(D[ax]) || !(fabs(O[ax]) < h[ax])) return false;
    far[ax] = dvd(sub(D[ax] > 0.0 ? h[ax] : -h[ax], O[ax]), D[ax]);
    // the near face's parameter, roughly: only needed to rule out a corner-entry event
    nr[ax] = ((float)(D[ax] > 0.0 ? -h[ax] : h[ax]) - (float)O[ax]) / (float)D[ax];
  }
  const double tf = far[1] < far[0] ? far[1] : far[0];
  if (!(tf >= 1e-9)) return false;
  // the slab test's events: a corner entry (the two near parameters within the band of each
  // other) and an exit within the T_MIN band; the corner graze |tf - tn| <= 1e-10 (|tn| + tf + 1)
  // cannot happen for tn < 0 <= 1e-9 <= tf
  const float tn_abs = fmaxf(fabsf(nr[0]), fabsf(nr[1]));
  if (!(fabsf(nr[0] - nr[1]) > 1e-6f * (tn_abs + (float)tf + 1.0f))) return false;
  lgx::tmin_band(tf, ev);
  if (gt_pos(tf, T_MIN)) {
    first = mkhit(tf, o, d, mk(0.0, 0.0), 0);
    nh = 1;
  }
  return true;
}

template <bool MULTI, bool CULL>
__device__ __forceinline__ void bounce_x(const SceneDev& S, const RayRec& r, const ScanRec& sc, const HitRec* hrec,
                                         BounceX& v) {
  using namespace lgx;
  v.emit = false;
  v.nchild = 0;
  const SceneLoc sl = scene_of<MULTI>(S, r.scene);
  uint32_t fl = r.flags;
  if (near_cutoff(r.c, sl.cutoff)) fl |= NEAR;  // tracer.rs:378-384 in the band
  const V o = ray_o(r), d = ray_d(r);
  v.x0 = (float)o.x;
  v.y0 = (float)o.y;
  int best = -1;
  V bp = mk(0.0, 0.0), bn = mk(0.0, 0.0);
  uint8_t leaf = 0;
  if (sc.nc > 0 || sc.overflow) {
    const HitRec h = *hrec;
    fl |= h.flags;
    if (h.obj != HIT_NONE) {
      best = (int)h.obj;
      bp = mk(xd(h.px), xd(h.py));
      bn = mk(xd(h.nx), xd(h.ny));
      leaf = h.leaf;
    }
  }
  if (best >= 0) {
    const ObjInfo& oi = S.info[sl.base + best];
    v.emit = true;
    v.x1 = (float)bp.x;
    v.y1 = (float)bp.y;
    v.hit = best;
    if (oi.flags & INFO_MATERIAL) {
      // the medium on the far side (tracer.rs:428-442); "origin inside obj" at the midpoint
      double n2 = 1.0;
      uint16_t m2 = MEDIUM_AIR;
      const V mid = vscl(vadd(o, bp), 0.5);
      if (obj_contains_f(S, sl.base + (uint32_t)best, mid, &fl)) {
        // the first other object (in table order) that contains the hit point and has a material
        const float px32 = (float)bp.x, py32 = (float)bp.y;
        auto far_side = [&](uint32_t k) -> bool {
          if ((int)k == best) return false;
          const float4 h = MULTI ? __ldg(&S.bounds[sl.base + k]) : __ldg(reinterpret_cast<const float4*>(&S.scan[k]));
          if (__float_as_uint(h.w) & INFO_NO_CONTAINS) return false;
          const float ex = px32 - h.x, ey = py32 - h.y;
          const float tol = 2e-6f * (fabsf(px32) + fabsf(py32) + fabsf(h.x) + fabsf(h.y) + h.z) + 1e-6f;
          if (ex * ex + ey * ey > (h.z + tol) * (h.z + tol)) return false;  // far outside: no member, no band
          if (!obj_contains_f(S, sl.base + k, bp, &fl)) return false;
          if (!(__float_as_uint(h.w) & INFO_MATERIAL)) return false;
          n2 = S.info[sl.base + k].n64;
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
        n2 = oi.n64;
        m2 = (uint16_t)best;
      }
      const double n1 = r.medium == MEDIUM_AIR ? 1.0
                        : r.medium == MEDIUM_LIGHT ? S.lights[sl.light_base + r.light].n0x : S.info[sl.base + r.medium].n64;
      V rl, rr = mk(0.0, 0.0);
      double R;
      const bool refr = refract_x(d, bn, n1, n2, rl, rr, R, fl);
      v.flags = (uint8_t)((fl & 0xffu) | (refr ? 0u : (uint32_t)LG_PATH_TIR));
      const float refl = (float)R;
      const float om = __fsub_rn(1.0f, refl);
      RayRec& a = v.child[0];
      a.ox = xdf(bp.x); a.oy = xdf(bp.y); a.dx = xdf(rl.x); a.dy = xdf(rl.y);
      a.medium = r.medium;
      a.src_obj = (uint16_t)best;
      a.src_leaf = leaf;
      a.c[0] = __fmul_rn(r.c[0], refl); a.c[1] = __fmul_rn(r.c[1], refl); a.c[2] = __fmul_rn(r.c[2], refl);
      a.c[3] = r.c[3];
      a.path = r.path;
      a.flags = (uint8_t)fl;
      a.ex = 0.0f;
      a.ea = 0.0f;
      v.nchild = 1;
      if (refr) {
        RayRec& t = v.child[1];
        t.ox = xdf(bp.x); t.oy = xdf(bp.y); t.dx = xdf(rr.x); t.dy = xdf(rr.y);
        t.medium = m2;
        t.src_obj = (uint16_t)best;
        t.src_leaf = leaf;
        t.c[0] = __fmul_rn(r.c[0], om); t.c[1] = __fmul_rn(r.c[1], om); t.c[2] = __fmul_rn(r.c[2], om);
        t.c[3] = r.c[3];
        t.path = r.path | (1ull << r.gen);
        t.flags = (uint8_t)fl;
        t.ex = 0.0f;
        t.ea = 0.0f;
        v.nchild = 2;
      }
    } else {  // Ray::reflect (tracer.rs:476-480)
      v.flags = (uint8_t)fl;
      const double dn = dot(d, bn);
      const V rd = vsub(d, vscl(bn, mul(2.0, dn)));
      RayRec& a = v.child[0];
      a.ox = xdf(bp.x); a.oy = xdf(bp.y); a.dx = xdf(rd.x); a.dy = xdf(rd.y);
      a.medium = r.medium;
      a.src_obj = (uint16_t)best;
      a.src_leaf = leaf;
      a.c[0] = r.c[0]; a.c[1] = r.c[1]; a.c[2] = r.c[2]; a.c[3] = r.c[3];
      a.path = r.path;
      a.flags = (uint8_t)fl;
      a.ex = 0.0f;
      a.ea = 0.0f;
      v.nchild = 1;
    }
  } else {
    // canvas exit (tracer.rs:482-488): nearest hit with the canvas rectangle
    const double aspect = MULTI ? S.scenes[r.scene].aspect64 : S.aspect64;
    double cev = INFINITY;
    int nh = 0;
    Hit first{INFINITY, mk(0.0, 0.0), mk(0.0, 0.0), 0, 0};
    if (!canvas_exit_inside(o, d, aspect, cev, first, nh)) {
      lg_geo canvas;
      canvas.kind = LG_GEO_RECT;
      canvas.origin[0] = 0.0; canvas.origin[1] = 0.0;
      canvas.rot[0] = 1.0; canvas.rot[1] = 0.0;
      canvas.v[0] = mul(2.0, aspect);
      canvas.v[1] = 2.0;
      hits_rect(canvas, o, d, cev, [&](const Hit& h) {
        if (nh == 0 || h.t < first.t) first = h;
        ++nh;
      });
    }
    if (nh > 0) {
      v.emit = true;
      v.x1 = (float)first.p.x;
      v.y1 = (float)first.p.y;
      v.hit = -1;
      v.flags = (uint8_t)((fl | (cev < INFINITY ? NEAR : 0u)) & 0xffu);
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
    v.child[w++] = c;
  }
  v.nchild = w;
}

// appends one segment per emitting lane with one atomic per warp (all lanes call)
__device__ __forceinline__ void emit_segments_x(const SceneDev& S, const TraceBufs& B, const BounceX& v,
                                                const RayRec& r, unsigned long long& my_near) {
  const unsigned lane = lane_id();
  const unsigned emask = __ballot_sync(0xffffffffu, v.emit);
  if (!emask) return;
  unsigned long long sbase = 0;
  const int leader = __ffs(emask) - 1;
  if ((int)lane == leader) sbase = atomicAdd(&B.ctr->seg_count, (unsigned long long)__popc(emask));
  sbase = __shfl_sync(0xffffffffu, sbase, leader);
  if (!v.emit) return;
  const unsigned long long slot = sbase + __popc(emask & lanemask_lt());
  if (v.flags & LG_PATH_NEAR_DEGENERATE) ++my_near;
  if (slot >= B.seg_cap) return;
  float4* dst = reinterpret_cast<float4*>(B.segs + slot);
  dst[0] = make_float4(v.x0, v.y0, v.x1, v.y1);
  dst[1] = make_float4(r.c[0], r.c[1], r.c[2], r.c[3]);
  if (B.seg_scene) B.seg_scene[slot] = r.scene;
  if (S.record_paths) {
    lg_path_record pr;
    pr.path = r.path; pr.primary = r.prim; pr.light = r.light; pr.gen = r.gen;
    pr.flags = v.flags; pr.hit = v.hit; pr.source = LG_SRC_TRACE;
    B.paths[slot] = pr;
  }
}

template <bool MULTI, bool CULL>
__global__ void __launch_bounds__(256, LG_BOUNCE_X_BLOCKS) k_bounce_x(SceneDev S, TraceBufs B, uint32_t gen) {
  __shared__ unsigned long long blk_visits, blk_near;
  if (threadIdx.x == 0) { blk_visits = 0; blk_near = 0; }
  __syncthreads();
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
  unsigned long long my_visits = 0, my_near = 0;
  for (uint64_t base = warp * 32; base < total; base += nwarps * 32) {
    const uint64_t i = base + lane;
    BounceX v;
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
      r = qin[idx];
      ++my_visits;
      bounce_x<MULTI, CULL>(S, r, sc, &B.hit[idx], v);
    }
    emit_segments_x(S, B, v, r, my_near);
    // children: warp prefix sum of 0..2 per lane, one atomic per warp
    int incl = v.nchild;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += y;
    }
    const int tot = __shfl_sync(0xffffffffu, incl, 31);
    if (tot > 0 && (MULTI || gen + 1 < S.max_bounce)) {
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
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&B.ctr->visits, blk_visits);
    atomicAdd(&B.ctr->near, blk_near);
  }
}
template __global__ void k_bounce_x<false, false>(SceneDev, TraceBufs, uint32_t);
template __global__ void k_bounce_x<false, true>(SceneDev, TraceBufs, uint32_t);
template __global__ void k_bounce_x<true, false>(SceneDev, TraceBufs, uint32_t);
template __global__ void k_bounce_x<true, true>(SceneDev, TraceBufs, uint32_t);

}  // namespace lgd
