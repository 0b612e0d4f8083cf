// lg_api.cu — host side of the C ABI declared in include/lg.h.
//
// Owns the device buffers of one context and drives the kernels:
//   lg_scene_upload  validates and flattens the scene (tracer.rs:48-116 object/light lists)
//   lg_trace         light setup + one wavefront kernel per generation + overlays
//                    (tracer.rs:276-358), growing the ring / queues on overflow
//   lg_accumulate    bin -> scan -> units -> scatter -> tile raster (renderer.rs:164-188)
//   lg_resolve_f16   Q31.32 -> binary16 (renderer.rs:330-418)
//   lg_render        the three above as one captured CUDA graph launch
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lg_ctx.hpp"

using namespace lgd;

namespace lgh {
// ---------------------------------------------------------------- scene flattening
struct Xf {
  double ox, oy, c, s;  // world = (ox, oy) + R(c, s) * local
  void apply(double x, double y, double& wx, double& wy) const {
    wx = ox + c * x - s * y;
    wy = oy + s * x + c * y;
  }
};

lg_status flatten_node(std::string& err, const lg_geo* G, uint32_t n_geo, int32_t gi, const Xf& T, int depth, Flat& F,
                       uint32_t leaf0, std::vector<uint8_t>& prog) {
  if (gi < 0 || (uint32_t)gi >= n_geo) return set_err(err, LG_ERR_INVALID_ARGUMENT, "geometry index out of range");
  if (depth > 32) return set_err(err, LG_ERR_INVALID_ARGUMENT, "geometry tree deeper than 32 (cycle?)");
  const lg_geo& g = G[gi];
  if (g.kind == LG_GEO_LOGIC) {
    if (g.op < 0 || g.op > 2) return set_err(err, LG_ERR_INVALID_ARGUMENT, "unknown logic op");
    Xf T2;
    T.apply(g.origin[0], g.origin[1], T2.ox, T2.oy);
    T2.c = T.c * g.rot[0] - T.s * g.rot[1];
    T2.s = T.s * g.rot[0] + T.c * g.rot[1];
    lg_status st = flatten_node(err, G, n_geo, g.a, T2, depth + 1, F, leaf0, prog);
    if (st) return st;
    st = flatten_node(err, G, n_geo, g.b, T2, depth + 1, F, leaf0, prog);
    if (st) return st;
    prog.push_back(g.op == LG_OP_AND ? PROG_AND : g.op == LG_OP_OR ? PROG_OR : PROG_AND_NOT);
    return LG_OK;
  }
  if (g.kind == LG_GEO_POLYGON) {
    // a convex polygon is the And of its edges' half-planes
    const int n = g.a;
    if (n < 3 || n > 63) return set_err(err, LG_ERR_INVALID_ARGUMENT, "a polygon has 3..63 vertices");
    std::vector<double> vx, vy;
    const lg_geo* cur = &g;
    for (int k = 0; k < n; ++k) {
      if (k > 0 && k % 4 == 0) {
        if (cur->b < 0 || (uint32_t)cur->b >= n_geo || G[cur->b].kind != LG_GEO_VERTICES)
          return set_err(err, LG_ERR_INVALID_ARGUMENT, "polygon vertex chain broken");
        cur = &G[cur->b];
      }
      vx.push_back(cur->v[2 * (k % 4)]);
      vy.push_back(cur->v[2 * (k % 4) + 1]);
    }
    double area = 0.0;
    for (int k = 0; k < n; ++k) area += vx[k] * vy[(k + 1) % n] - vy[k] * vx[(k + 1) % n];
    if (area == 0.0) return set_err(err, LG_ERR_INVALID_ARGUMENT, "degenerate polygon");
    const double sg = area > 0.0 ? 1.0 : -1.0;
    Xf T2;
    T.apply(g.origin[0], g.origin[1], T2.ox, T2.oy);
    T2.c = T.c * g.rot[0] - T.s * g.rot[1];
    T2.s = T.s * g.rot[0] + T.c * g.rot[1];
    std::vector<double> wx(n), wy(n);
    double box[4] = {INFINITY, INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < n; ++k) {
      T2.apply(vx[k], vy[k], wx[k], wy[k]);
      box[0] = std::min(box[0], wx[k]); box[1] = std::min(box[1], wy[k]);
      box[2] = std::max(box[2], wx[k]); box[3] = std::max(box[3], wy[k]);
    }
    for (int k = 0; k < n; ++k) {
      const double ex = wx[(k + 1) % n] - wx[k], ey = wy[(k + 1) % n] - wy[k], l = std::sqrt(ex * ex + ey * ey);
      if (!(l > 0.0)) return set_err(err, LG_ERR_INVALID_ARGUMENT, "polygon with a zero-length edge");
      LeafH H;
      std::memset(&H, 0, sizeof H);
      H.kind = LEAF_HALFPLANE;
      H.p[0] = wx[k];
      H.p[1] = wy[k];
      H.p[2] = sg * ey / l;  // outward: right of a counter-clockwise edge
      H.p[3] = -sg * ex / l;
      for (int i = 0; i < 4; ++i) H.box[i] = box[i];
      const uint32_t li = (uint32_t)F.leaves.size() - leaf0;
      if (li >= (uint32_t)MAX_LEAVES - 1) return set_err(err, LG_ERR_UNSUPPORTED, "more than 63 leaves in one object");
      F.leaves.push_back(H);
      prog.push_back((uint8_t)li);
      if (k > 0) prog.push_back(PROG_AND);
    }
    return LG_OK;
  }
  LeafH L;
  std::memset(&L, 0, sizeof L);
  switch (g.kind) {
    case LG_GEO_ELLIPSE: {
      if (!(g.v[0] > 0.0) || !(g.v[1] > 0.0)) return set_err(err, LG_ERR_INVALID_ARGUMENT, "ellipse axes must be > 0");
      L.kind = LEAF_ELLIPSE;
      T.apply(g.origin[0], g.origin[1], L.p[0], L.p[1]);
      L.p[2] = T.c * g.rot[0] - T.s * g.rot[1];
      L.p[3] = T.s * g.rot[0] + T.c * g.rot[1];
      L.p[4] = g.v[0];
      L.p[5] = g.v[1];
      L.p[6] = 1.0 / g.v[0];
      L.p[7] = 1.0 / g.v[1];
      break;
    }
    case LG_GEO_CIRCLE:
      L.kind = LEAF_CIRCLE;
      T.apply(g.origin[0], g.origin[1], L.p[0], L.p[1]);
      L.p[2] = g.v[0];
      L.p[3] = g.v[0] != 0.0 ? 1.0 / g.v[0] : 0.0;  // normal = (p - c) / r
      break;
    case LG_GEO_RECT:
      L.kind = LEAF_RECT;
      T.apply(g.origin[0], g.origin[1], L.p[0], L.p[1]);
      L.p[2] = T.c * g.rot[0] - T.s * g.rot[1];
      L.p[3] = T.s * g.rot[0] + T.c * g.rot[1];
      L.p[4] = 0.5 * g.v[0];
      L.p[5] = 0.5 * g.v[1];
      break;
    case LG_GEO_SEGMENT: {
      L.kind = LEAF_SEGMENT;
      T.apply(g.v[0], g.v[1], L.p[0], L.p[1]);
      T.apply(g.v[2], g.v[3], L.p[2], L.p[3]);
      const double ex = L.p[2] - L.p[0], ey = L.p[3] - L.p[1], l = std::sqrt(ex * ex + ey * ey);
      L.p[4] = l > 0.0 ? -ey / l : 0.0;  // unit left normal
      L.p[5] = l > 0.0 ? ex / l : 0.0;
      break;
    }
    case LG_GEO_CUBIC:
      L.kind = LEAF_CUBIC;
      for (int k = 0; k < 4; ++k) T.apply(g.v[2 * k], g.v[2 * k + 1], L.p[2 * k], L.p[2 * k + 1]);
      break;
    default:
      return set_err(err, LG_ERR_UNSUPPORTED, "unsupported geometry kind " + std::to_string(g.kind));
  }
  const uint32_t li = (uint32_t)F.leaves.size() - leaf0;
  if (li >= (uint32_t)MAX_LEAVES - 1) return set_err(err, LG_ERR_UNSUPPORTED, "more than 63 leaves in one object");
  F.leaves.push_back(L);
  prog.push_back((uint8_t)li);
  return LG_OK;
}

// bounding circle of one leaf about a centre: returns the max distance
double leaf_extent(const LeafH& L, double cx, double cy) {
  auto d = [&](double x, double y) { return std::hypot(x - cx, y - cy); };
  switch (L.kind) {
    case LEAF_CIRCLE: return d(L.p[0], L.p[1]) + std::fabs(L.p[2]);
    case LEAF_RECT: return d(L.p[0], L.p[1]) + std::hypot(L.p[4], L.p[5]);
    case LEAF_SEGMENT: return std::max(d(L.p[0], L.p[1]), d(L.p[2], L.p[3]));
    case LEAF_ELLIPSE: return d(L.p[0], L.p[1]) + std::max(L.p[4], L.p[5]);
    case LEAF_HALFPLANE:
      return std::max(std::max(d(L.box[0], L.box[1]), d(L.box[2], L.box[3])),
                      std::max(d(L.box[0], L.box[3]), d(L.box[2], L.box[1])));
    default: {
      double m = 0;
      for (int k = 0; k < 4; ++k) m = std::max(m, d(L.p[2 * k], L.p[2 * k + 1]));
      return m;
    }
  }
}

void leaf_box(const LeafH& L, double& x0, double& y0, double& x1, double& y1) {
  auto add = [&](double x, double y) {
    x0 = std::min(x0, x); y0 = std::min(y0, y); x1 = std::max(x1, x); y1 = std::max(y1, y);
  };
  switch (L.kind) {
    case LEAF_CIRCLE: {
      const double r = std::fabs(L.p[2]);
      add(L.p[0] - r, L.p[1] - r);
      add(L.p[0] + r, L.p[1] + r);
      break;
    }
    case LEAF_RECT: {
      const double ex = std::fabs(L.p[2]) * L.p[4] + std::fabs(L.p[3]) * L.p[5];
      const double ey = std::fabs(L.p[3]) * L.p[4] + std::fabs(L.p[2]) * L.p[5];
      add(L.p[0] - ex, L.p[1] - ey);
      add(L.p[0] + ex, L.p[1] + ey);
      break;
    }
    case LEAF_SEGMENT:
      add(L.p[0], L.p[1]);
      add(L.p[2], L.p[3]);
      break;
    case LEAF_ELLIPSE: {
      const double c = L.p[2], s = L.p[3];
      const double ex = std::sqrt(L.p[4] * L.p[4] * c * c + L.p[5] * L.p[5] * s * s);
      const double ey = std::sqrt(L.p[4] * L.p[4] * s * s + L.p[5] * L.p[5] * c * c);
      add(L.p[0] - ex, L.p[1] - ey);
      add(L.p[0] + ex, L.p[1] + ey);
      break;
    }
    case LEAF_HALFPLANE:
      add(L.box[0], L.box[1]);
      add(L.box[2], L.box[3]);
      break;
    default:
      for (int k = 0; k < 4; ++k) add(L.p[2 * k], L.p[2 * k + 1]);
  }
}

void leaf_f32(const LeafH& L, float* a, float* b) {
  if (L.kind == LEAF_CUBIC) {
    for (int k = 0; k < 6; ++k) a[k] = (float)L.p[k];
    b[0] = (float)L.p[6];
    b[1] = (float)L.p[7];
  } else if (L.kind == LEAF_CIRCLE) {
    a[0] = (float)L.p[0]; a[1] = (float)L.p[1]; a[2] = (float)L.p[2];
  } else if (L.kind == LEAF_RECT) {
    for (int k = 0; k < 6; ++k) a[k] = (float)L.p[k];
  } else {
    a[0] = (float)L.p[0]; a[1] = (float)L.p[1];
    a[2] = (float)(L.p[2] - L.p[0]); a[3] = (float)(L.p[3] - L.p[1]);
  }
}

// Box holding every hit an object's membership program keeps (a hit on a leaf counts when
// flipping that leaf's membership flips the combination) and its enclosed region:
// And keeps hits inside both operands (box intersection), AndNot hits inside the first,
// Or the union.  Disjoint operands of an And leave an empty object, boxed by a point.
void csg_box(const Flat& F, uint32_t leaf0, const std::vector<uint8_t>& prog, double& x0, double& y0, double& x1,
             double& y1) {
  struct Box { double x0, y0, x1, y1; };
  std::vector<Box> st;
  for (const uint8_t op : prog) {
    if (op < 0x40) {
      Box b{INFINITY, INFINITY, -INFINITY, -INFINITY};
      leaf_box(F.leaves[leaf0 + op], b.x0, b.y0, b.x1, b.y1);
      st.push_back(b);
      continue;
    }
    const Box b = st.back();
    st.pop_back();
    Box& a = st.back();
    if (op == PROG_AND) {
      Box c{std::max(a.x0, b.x0), std::max(a.y0, b.y0), std::min(a.x1, b.x1), std::min(a.y1, b.y1)};
      if (c.x0 > c.x1 || c.y0 > c.y1) {  // empty: keep a point of the first operand
        const double mx = 0.5 * (a.x0 + a.x1), my = 0.5 * (a.y0 + a.y1);
        c = Box{mx, my, mx, my};
      }
      a = c;
    } else if (op == PROG_OR) {
      a = Box{std::min(a.x0, b.x0), std::min(a.y0, b.y0), std::max(a.x1, b.x1), std::max(a.y1, b.y1)};
    }  // PROG_AND_NOT: the first operand's box
  }
  x0 = st.back().x0; y0 = st.back().y0; x1 = st.back().x1; y1 = st.back().y1;
}

bool blend_supported(const lg_blend_component& b) {
  if (b.op == LG_BO_MIN || b.op == LG_BO_MAX) return b.src_factor == LG_BF_ONE && b.dst_factor == LG_BF_ONE;
  if (b.op != LG_BO_ADD && b.op != LG_BO_REVERSE_SUBTRACT) return false;
  if (b.dst_factor != LG_BF_ONE) return false;
  switch (b.src_factor) {
    case LG_BF_ZERO: case LG_BF_ONE: case LG_BF_SRC: case LG_BF_ONE_MINUS_SRC: case LG_BF_SRC_ALPHA:
    case LG_BF_ONE_MINUS_SRC_ALPHA: case LG_BF_CONSTANT: case LG_BF_ONE_MINUS_CONSTANT: return true;
    default: return false;
  }
}

// Exact mode: the tree under node gi in preorder (indices relative to the object's first
// node), with each leaf's number in the flattened leaf table (flatten_node's order: child a
// before child b, a polygon's edges one by one).
void xtree(const lg_geo* G, int32_t gi, int depth, int parent, int side, std::vector<lgx::XNode>& out,
           uint32_t& leaf_ord, int& max_depth) {
  const lg_geo& g = G[gi];
  lgx::XNode n;
  std::memset(&n, 0, sizeof n);
  n.geo = gi;
  n.parent = (int16_t)parent;
  n.depth = (uint8_t)std::min(depth, 255);
  n.side = (uint8_t)side;
  n.leaf_ord = leaf_ord;
  const int idx = (int)out.size();
  out.push_back(n);
  max_depth = std::max(max_depth, depth);
  if (g.kind == LG_GEO_LOGIC) {
    xtree(G, g.a, depth + 1, idx, 0, out, leaf_ord, max_depth);
    xtree(G, g.b, depth + 1, idx, 1, out, leaf_ord, max_depth);
  } else {
    leaf_ord += g.kind == LG_GEO_POLYGON ? (uint32_t)g.a : 1u;
  }
  out[idx].end = (int32_t)out.size();
}

lg_status validate_exact(std::string& err, const lg_params& p, const Flat& F) {
  if (p.precision != LG_PRECISION_EXACT) return LG_OK;
  if (F.xdepth > lgx::MAX_DEPTH)
    return set_err(err, LG_ERR_UNSUPPORTED, "exact precision: geometry trees deeper than 8 Logic levels");
  return LG_OK;
}

lg_status flatten_scene(std::string& err, const lg_geo* G, uint32_t n_geo, const lg_object* O, uint32_t n_obj,
                        const lg_light* Ls, uint32_t n_lights, Flat& F) {
  F.xgeo.assign(G, G + n_geo);
  for (uint32_t k = 0; k < n_obj; ++k) {
    const lg_object& o = O[k];
    if (o.kind < 0 || o.kind > LG_OBJ_GEO) return set_err(err, LG_ERR_INVALID_ARGUMENT, "object " + std::to_string(k) + ": unknown kind");
    if (o.geo < 0 || (uint32_t)o.geo >= n_geo) return set_err(err, LG_ERR_INVALID_ARGUMENT, "object " + std::to_string(k) + ": geometry index out of range");
    const int rk = G[o.geo].kind;
    const bool ok = (o.kind == LG_OBJ_STRAIGHT_MIRROR && rk == LG_GEO_SEGMENT) ||
                    (o.kind == LG_OBJ_CURVED_MIRROR && rk == LG_GEO_CUBIC) ||
                    (o.kind == LG_OBJ_CIRCLE && rk == LG_GEO_CIRCLE) || (o.kind == LG_OBJ_RECT && rk == LG_GEO_RECT) ||
                    (o.kind == LG_OBJ_LENS && rk == LG_GEO_LOGIC) ||
                    (o.kind == LG_OBJ_CONVEX_POLYGON && rk == LG_GEO_POLYGON) ||
                    (o.kind == LG_OBJ_ELLIPSE && rk == LG_GEO_ELLIPSE) || o.kind == LG_OBJ_GEO;
    if (!ok) return set_err(err, LG_ERR_INVALID_ARGUMENT, "object " + std::to_string(k) + ": kind does not match its geometry");
    if (o.has_material && !(o.refractive_index > 0.0))
      return set_err(err, LG_ERR_INVALID_ARGUMENT, "object " + std::to_string(k) + ": refractive index must be > 0");
    const uint32_t leaf0 = (uint32_t)F.leaves.size();
    std::vector<uint8_t> prog;
    Xf T{0.0, 0.0, 1.0, 0.0};
    lg_status st = flatten_node(err, G, n_geo, o.geo, T, 0, F, leaf0, prog);
    if (st) return st;
    ObjInfo oi;
    std::memset(&oi, 0, sizeof oi);
    oi.leaf_begin = leaf0;
    oi.n_leaves = (uint16_t)(F.leaves.size() - leaf0);
    oi.prog_begin = (uint32_t)F.prog.size();
    oi.prog_len = (uint16_t)prog.size();
    oi.flags = (o.has_material ? INFO_MATERIAL : 0u) |
               ((o.kind == LG_OBJ_STRAIGHT_MIRROR || o.kind == LG_OBJ_CURVED_MIRROR) ? INFO_NO_CONTAINS : 0u);
    oi.n = DF(o.has_material ? o.refractive_index : 1.0);
    oi.n64 = o.has_material ? o.refractive_index : 1.0;
    oi.xnode_begin = (uint32_t)F.xnode.size();
    {
      std::vector<lgx::XNode> nodes;
      uint32_t ord = 0;
      xtree(G, o.geo, 0, -1, 0, nodes, ord, F.xdepth);
      if (nodes.size() > 32767) return set_err(err, LG_ERR_UNSUPPORTED, "object " + std::to_string(k) + ": tree too large");
      oi.xnode_count = (uint32_t)nodes.size();
      F.xnode.insert(F.xnode.end(), nodes.begin(), nodes.end());
    }
    F.prog.insert(F.prog.end(), prog.begin(), prog.end());
    F.info.push_back(oi);
    if (o.kind == LG_OBJ_CURVED_MIRROR) F.cubics.push_back(k);
    // FP32 scan record
    ObjScan s;
    std::memset(&s, 0, sizeof s);
    double x0, y0, x1, y1;
    csg_box(F, leaf0, prog, x0, y0, x1, y1);
    const double cx = 0.5 * (x0 + x1), cy = 0.5 * (y0 + y1);
    // every hit lies in the box and on some leaf: the smaller of the two radii bounds it
    double R = 0.0;
    for (uint32_t i = leaf0; i < F.leaves.size(); ++i) R = std::max(R, leaf_extent(F.leaves[i], cx, cy));
    R = std::min(R, 0.5 * std::hypot(x1 - x0, y1 - y0));
    if (!std::isfinite(cx) || !std::isfinite(cy) || !std::isfinite(R))
      return set_err(err, LG_ERR_INVALID_ARGUMENT, "object " + std::to_string(k) + ": non-finite geometry");
    s.cx = (float)cx;
    s.cy = (float)cy;
    s.R = (float)(R * (1.0 + 1e-6) + 1e-6 * (1.0 + std::fabs(cx) + std::fabs(cy)));
    const uint32_t nl = oi.n_leaves;
    // one leaf of a scanned kind (a cubic takes both inline slots), or two circle / rect /
    // segment leaves; anything else (ellipses, polygons, deeper CSG) is bounded only
    bool no_cubic = true;
    for (uint32_t i = leaf0; i < leaf0 + nl && i < F.leaves.size(); ++i) no_cubic = no_cubic && F.leaves[i].kind < LEAF_CUBIC;
    uint32_t info = SCAN_BOUND;
    float scratch[6];
    if (nl == 1 && F.leaves[leaf0].kind <= LEAF_CUBIC) {
      info = SCAN_ONE | (F.leaves[leaf0].kind << 4);
      leaf_f32(F.leaves[leaf0], s.a, s.b);
    } else if (nl == 2 && no_cubic) {
      const uint8_t op = prog.back();
      info = SCAN_TWO | (F.leaves[leaf0].kind << 4) | (F.leaves[leaf0 + 1].kind << 6) |
             ((uint32_t)(op == PROG_AND ? LG_OP_AND : op == PROG_OR ? LG_OP_OR : LG_OP_AND_NOT) << 8);
      leaf_f32(F.leaves[leaf0], s.a, scratch);
      leaf_f32(F.leaves[leaf0 + 1], s.b, scratch);
    }
    s.info = info | oi.flags;
    F.scan.push_back(s);
  }
  uint64_t first = 0;
  for (uint32_t l = 0; l < n_lights; ++l) {
    const lg_light& L = Ls[l];
    if (L.kind < 0 || L.kind > LG_LIGHT_SPOT) return set_err(err, LG_ERR_INVALID_ARGUMENT, "light " + std::to_string(l) + ": unknown kind");
    LightDev d;
    std::memset(&d, 0, sizeof d);
    d.ox = L.origin[0]; d.oy = L.origin[1]; d.vx = L.v[0]; d.vy = L.v[1];
    d.spot_angle = L.spot_angle;
    d.n0 = DF(1.0);
    for (int i = 0; i < 4; ++i) d.color[i] = L.color[i];
    d.kind = (uint32_t)L.kind;
    d.num_rays = L.num_rays;
    d.first = first;
    first += L.num_rays;
    F.lights.push_back(d);
  }
  return LG_OK;
}


// Uniform grid over the objects' FP32 bounding circles.  The margin covers the FP32 error
// of a walk from an origin within `reach` (a few 1e-7 of the coordinates) and the
// bounding-circle test's own slack (2e-6 of the distances), with room to spare.
void build_grid(const std::vector<ObjScan>& scan, int culling, float density, GridH& G) {
  const size_t n = scan.size();
  std::memset(&G.rec, 0, sizeof G.rec);
  G.cell_start.assign(1, 0u);
  G.cell_obj.clear();
  const bool want = culling == LG_CULL_ON || (culling != LG_CULL_OFF && n >= (size_t)LG_CULL_AUTO_MIN);
  if (!want || n == 0) return;
  double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
  for (const ObjScan& s : scan) {
    x0 = std::min(x0, (double)s.cx - s.R); x1 = std::max(x1, (double)s.cx + s.R);
    y0 = std::min(y0, (double)s.cy - s.R); y1 = std::max(y1, (double)s.cy + s.R);
  }
  const double W = x1 - x0, H = y1 - y0;
  const double scale = 1.0 + std::max(std::fabs(x0), std::fabs(x1)) + std::max(std::fabs(y0), std::fabs(y1)) + W + H;
  const double target = std::max(1.0, (density > 0.0f ? (double)density : 2.0) * (double)n);
  const double ar = std::max(W, 1e-9 * scale) / std::max(H, 1e-9 * scale);
  int nx = (int)std::lround(std::sqrt(target * ar)), ny;
  nx = std::min(1024, std::max(1, nx));
  ny = std::min(1024, std::max(1, (int)std::lround(target / nx)));
  constexpr uint64_t MAX_ENTRIES = 1ull << 24;
  for (;;) {
    const double margin = 4e-5 * scale + 1e-3 * std::min(W / nx, H / ny);
    GridRec& R = G.rec;
    R.x0 = (float)(x0 - 2.0 * margin);
    R.y0 = (float)(y0 - 2.0 * margin);
    R.cw = (float)((x1 + 2.0 * margin - R.x0) / nx);
    R.ch = (float)((y1 + 2.0 * margin - R.y0) / ny);
    R.iw = 1.0f / R.cw;
    R.ih = 1.0f / R.ch;
    R.margin = (float)margin;
    R.nx = (uint32_t)nx;
    R.ny = (uint32_t)ny;
    R.cell_base = 0;
    R.list_base = 0;
    R.reach = (float)scale;
    uint64_t total = 0;
    int rx0, ry0, rx1, ry1;
    for (const ObjScan& o : scan) {
      grid_cell_range(R, o.cx, o.cy, o.R, rx0, ry0, rx1, ry1);
      total += (uint64_t)(rx1 - rx0 + 1) * (uint64_t)(ry1 - ry0 + 1);
    }
    if (total > MAX_ENTRIES && (nx > 1 || ny > 1)) {  // huge objects: coarser cells
      nx = std::max(1, nx / 2);
      ny = std::max(1, ny / 2);
      continue;
    }
    const size_t ncell = (size_t)nx * ny;
    G.cell_start.assign(ncell + 1, 0u);
    for (const ObjScan& o : scan) {
      grid_cell_range(R, o.cx, o.cy, o.R, rx0, ry0, rx1, ry1);
      for (int iy = ry0; iy <= ry1; ++iy)
        for (int ix = rx0; ix <= rx1; ++ix) ++G.cell_start[(size_t)iy * nx + ix + 1];
    }
    for (size_t c = 0; c < ncell; ++c) G.cell_start[c + 1] += G.cell_start[c];
    G.cell_obj.assign(total, 0);
    std::vector<uint32_t> cur(G.cell_start.begin(), G.cell_start.end() - 1);
    for (size_t k = 0; k < n; ++k) {  // ascending object order within every cell
      grid_cell_range(R, scan[k].cx, scan[k].cy, scan[k].R, rx0, ry0, rx1, ry1);
      for (int iy = ry0; iy <= ry1; ++iy)
        for (int ix = rx0; ix <= rx1; ++ix) G.cell_obj[cur[(size_t)iy * nx + ix]++] = (uint16_t)k;
    }
    return;
  }
}

lg_status validate_params(std::string& err, const lg_params& p) {
  if (p.max_bounce > (uint32_t)MAX_GEN) return set_err(err, LG_ERR_INVALID_ARGUMENT, "max_bounce must be <= 64");
  if (p.width == 0 || p.height == 0 || p.width > 32768 || p.height > 32768)
    return set_err(err, LG_ERR_INVALID_ARGUMENT, "canvas must be 1..32768 pixels per side");
  if (p.accum != LG_ACCUM_FIXED64 && p.accum != LG_ACCUM_F32)
    return set_err(err, LG_ERR_INVALID_ARGUMENT, "unknown accum mode");
  if (!blend_supported(p.color_blend) || !blend_supported(p.alpha_blend))
    return set_err(err, LG_ERR_UNSUPPORTED, "blend state reads the destination (order-dependent): not supported");
  const lg_string_mod& sm = p.string_mod;
  if (sm.modulo) {
    if (sm.curve > LG_CURVE_LISSAJOUS) return set_err(err, LG_ERR_INVALID_ARGUMENT, "string mod: unknown curve");
    if (sm.mode > LG_SM_BASE) return set_err(err, LG_ERR_INVALID_ARGUMENT, "string mod: unknown mode");
    if (sm.modulo > (1ull << 26)) return set_err(err, LG_ERR_INVALID_ARGUMENT, "string mod: modulo above 2^26");
    if (sm.n_colors > 4096) return set_err(err, LG_ERR_INVALID_ARGUMENT, "string mod: more than 4096 modulo colours");
    if (sm.n_colors && !sm.colors) return set_err(err, LG_ERR_INVALID_ARGUMENT, "string mod: null modulo colours");
    for (uint32_t k = 0; k < sm.n_colors; ++k)
      if (sm.colors[k].modulo == 0) return set_err(err, LG_ERR_INVALID_ARGUMENT, "string mod: modulo colour with modulo 0");
    if (sm.nested) {
      const lg_string_mod& ns = *sm.nested;
      if (sm.modulo > LG_STRING_MOD_NESTED_MAX)
        return set_err(err, LG_ERR_UNSUPPORTED, "string mod: a nested mod needs modulo <= LG_STRING_MOD_NESTED_MAX");
      if (ns.mode > LG_SM_BASE) return set_err(err, LG_ERR_INVALID_ARGUMENT, "nested string mod: unknown mode");
      if (ns.modulo > (1ull << 26)) return set_err(err, LG_ERR_INVALID_ARGUMENT, "nested string mod: modulo above 2^26");
      if (ns.n_colors > 4096) return set_err(err, LG_ERR_INVALID_ARGUMENT, "nested string mod: more than 4096 modulo colours");
      if (ns.n_colors && !ns.colors) return set_err(err, LG_ERR_INVALID_ARGUMENT, "nested string mod: null modulo colours");
      for (uint32_t k = 0; k < ns.n_colors; ++k)
        if (ns.colors[k].modulo == 0)
          return set_err(err, LG_ERR_INVALID_ARGUMENT, "nested string mod: modulo colour with modulo 0");
    }
  }
  if (p.precision != LG_PRECISION_EXACT && p.precision != LG_PRECISION_FAST)
    return set_err(err, LG_ERR_INVALID_ARGUMENT, "unknown precision");
  if (p.ray_stride > 1 && p.ray_offset >= p.ray_stride)
    return set_err(err, LG_ERR_INVALID_ARGUMENT, "ray_offset must be below ray_stride");
  return LG_OK;
}

// Overlay segments (curved-mirror control lines) and string-mod lines of the context's frame
// (none in a sampled frame with ray_offset != 0).
uint64_t overlay_segments(const lg_ctx* c) {
  if (c->prm.ray_stride > 1 && c->prm.ray_offset != 0) return 0;
  return 3ull * c->n_cubic * (c->prm.emit_control_lines ? 1 : 0);
}
uint64_t string_mod_lines(const lg_ctx* c) {
  if (c->prm.ray_stride > 1 && c->prm.ray_offset != 0) return 0;
  if (c->has_nested) return c->n_cross ? c->nested.modulo : 0;  // no crossings, no lines
  return c->prm.string_mod.modulo;
}

// Primaries of a light with num_rays rays that a sampled frame traces.
uint64_t sampled_rays(uint64_t num_rays, const lg_params& p) {
  if (p.ray_stride <= 1) return num_rays;
  return num_rays > p.ray_offset ? (num_rays - p.ray_offset + p.ray_stride - 1) / p.ray_stride : 0;
}

int raster_mode(const lg_params& p) {
  if (p.accum == LG_ACCUM_F32) return RM_F32_;
  const lg_blend_component* b[2] = {&p.color_blend, &p.alpha_blend};
  for (const lg_blend_component* x : b)
    if (x->op == LG_BO_MIN || x->op == LG_BO_MAX) return RM_FIXED_MINMAX_;
  return RM_FIXED_SPLIT_;
}

void to_device_leaves(const std::vector<LeafH>& in, std::vector<Leaf64>& out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    std::memset(&out[i], 0, sizeof(Leaf64));
    out[i].kind = in[i].kind;
    for (int k = 0; k < 8; ++k) out[i].p[k] = DF(in[i].p[k]);
  }
}

}  // namespace lgh

using namespace lgh;

namespace lgh {

lg_status fail(lg_ctx* c, lg_status st, const std::string& msg) {
  if (c) c->err = msg;
  return st;
}

lg_status cuda_fail(lg_ctx* c, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  (void)cudaGetLastError();
  return fail(c, e == cudaErrorMemoryAllocation ? LG_ERR_OUT_OF_MEMORY : LG_ERR_CUDA, m);
}

lg_status ensure(lg_ctx* c, DevBuf& b, size_t bytes, const char* what) {
  if (bytes <= b.bytes && b.p) return LG_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return cuda_fail(c, e, what);
  }
  b.bytes = bytes;
  c->graph_valid = false;
  return LG_OK;
}

void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

SceneDev scene_dev(lg_ctx* c) {
  SceneDev S;
  S.scan = (const ObjScan*)c->d_scan.p;
  S.info = (const ObjInfo*)c->d_info.p;
  S.leaves = (const Leaf64*)c->d_leaves.p;
  S.prog = (const uint8_t*)c->d_prog.p;
  S.lights = (LightDev*)c->d_lights.p;
  S.n_obj = c->n_obj;
  S.n_lights = c->n_lights;
  S.n_primary = c->n_primary;
  S.aspect = DF(c->aspect);
  for (int i = 0; i < 4; ++i) S.cutoff[i] = c->prm.cutoff_color[i];
  S.max_bounce = c->prm.max_bounce;
  S.record_paths = c->prm.record_paths ? 1u : 0u;
  S.scenes = nullptr;
  S.bounds = nullptr;
  S.n_scenes = 1;
  S.serve = 0;
  S.n_new = 0;
  S.light_lo = 0;
  S.light_hi = 0;
  S.grids = (const GridRec*)c->d_grids.p;
  S.cell_start = (const uint32_t*)c->d_cell_start.p;
  S.cell_obj = (const uint16_t*)c->d_cell_obj.p;
  S.wait_polls = c->wait_polls;
  S.xgeo = (const lg_geo*)c->d_xgeo.p;
  S.xnode = (const lgx::XNode*)c->d_xnode.p;
  S.aspect64 = c->aspect;
  S.ray_stride = c->prm.ray_stride > 1 ? c->prm.ray_stride : 1u;
  S.ray_offset = c->prm.ray_stride > 1 ? c->prm.ray_offset : 0u;
  return S;
}

TraceBufs trace_bufs(lg_ctx* c) {
  TraceBufs B;
  B.queue[0] = (RayRec*)c->d_queue[0].p;
  B.queue[1] = (RayRec*)c->d_queue[1].p;
  B.queue_cap = c->queue_cap;
  B.scan = (ScanRec*)c->d_scanrec.p;
  B.hit = (HitRec*)c->d_hitrec.p;
  for (int i = 0; i < N_LISTS; ++i) B.list[i] = (uint32_t*)c->d_list[i].p;
  B.segs = (lg_segment*)c->d_segs.p;
  B.paths = (lg_path_record*)c->d_paths.p;
  B.seg_scene = nullptr;
  B.order = nullptr;
  B.seg_cap = c->seg_cap;
  B.ctr = (Counters*)c->d_ctr.p;
  return B;
}

RasterArgs raster_args(lg_ctx* c) {
  RasterArgs A;
  std::memset(&A, 0, sizeof A);
  A.segs = (const lg_segment*)c->d_segs.p;
  A.seg_cap = c->seg_cap;
  A.W = c->prm.width;
  A.H = c->prm.height;
  A.ntx = c->ntx;
  A.nty = c->nty;
  A.n_tiles = 2 * c->n_tiles;  // bins: x-major and y-major segments of each tile
  A.unit_refs = c->raster_variant == 2 ? UNIT_REFS_WARP : UNIT_REFS;
  for (int ch = 0; ch < 4; ++ch) {
    const lg_blend_component& b = ch < 3 ? c->prm.color_blend : c->prm.alpha_blend;
    A.blend.src[ch] = b.src_factor;
    A.blend.op[ch] = b.op;
    A.blend.constant[ch] = c->prm.blend_constant[ch];
    A.blend.clear[ch] = c->prm.clear_color[ch];
  }
  A.tile_count = (uint32_t*)c->d_tile_count.p;
  A.tile_off = (uint64_t*)c->d_tile_off.p;
  A.tile_cursor = (unsigned long long*)c->d_tile_cursor.p;
  A.unit_off = (uint64_t*)c->d_unit_off.p;
  A.refs = (uint32_t*)c->d_refs.p;
  A.refs_cap = c->refs_cap;
  A.units = (Unit*)c->d_units.p;
  A.units_cap = c->units_cap;
  A.accum = c->d_accum.p;
  A.ctr = (Counters*)c->d_ctr.p;
  A.cta_hist = cta_hist_for(c, A.n_tiles);
  return A;
}

lg_status upload_grids(lg_ctx* c, const lgh::GridTables& G) {
  // grid records address their cells and lists with 32-bit bases
  if (G.cell_start.size() > 0xffffffffull || G.cell_obj.size() > 0xffffffffull)
    return fail(c, LG_ERR_UNSUPPORTED, "culling grids of more than 2^32 cells or list entries in one upload");
  auto up = [&](DevBuf& b, const void* src, size_t bytes, const char* what) -> lg_status {
    lg_status st = ensure(c, b, bytes + 16, what);
    if (st) return st;
    if (bytes) CK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c->stream), what);
    return LG_OK;
  };
  lg_status st;
  if ((st = up(c->d_grids, G.recs.data(), G.recs.size() * sizeof(GridRec), "culling grids"))) return st;
  if ((st = up(c->d_cell_start, G.cell_start.data(), G.cell_start.size() * 4, "culling grids"))) return st;
  return up(c->d_cell_obj, G.cell_obj.data(), G.cell_obj.size() * 2, "culling grids");
}

lg_status ensure_trace_buffers(lg_ctx* c) {
  lg_status st;
  if ((st = ensure(c, c->d_queue[0], c->queue_cap * sizeof(RayRec), "ray queue"))) return st;
  if ((st = ensure(c, c->d_queue[1], c->queue_cap * sizeof(RayRec), "ray queue"))) return st;
  if ((st = ensure(c, c->d_scanrec, c->queue_cap * sizeof(ScanRec), "scan records"))) return st;
  if ((st = ensure(c, c->d_hitrec, c->queue_cap * sizeof(HitRec), "hit records"))) return st;
  for (int i = 0; i < N_LISTS; ++i)
    if ((st = ensure(c, c->d_list[i], c->queue_cap * 4, "work lists"))) return st;
  if ((st = ensure(c, c->d_segs, c->seg_cap * sizeof(lg_segment), "segment ring"))) return st;
  if (c->prm.record_paths && (st = ensure(c, c->d_paths, c->seg_cap * sizeof(lg_path_record), "path records")))
    return st;
  return LG_OK;
}

lg_status ensure_cta_hist(lg_ctx* c, size_t bins) {
  if (bins > MAX_SMEM_TILES) return LG_OK;
  return ensure(c, c->d_cta_hist, (size_t)scatter_grid(c->n_sm, 1) * bins * 4, "per-CTA bin counts");
}

uint32_t* cta_hist_for(const lg_ctx* c, size_t bins) {
  const size_t need = (size_t)scatter_grid(c->n_sm, 1) * bins * 4;
  return bins <= MAX_SMEM_TILES && c->d_cta_hist.p && c->d_cta_hist.bytes >= need ? (uint32_t*)c->d_cta_hist.p
                                                                                  : nullptr;
}

void launch_bin_count(lg_ctx* c, const RasterArgs& A, int smem_tiles, size_t bsm) {
  if (smem_tiles && A.cta_hist)
    k_bin_count<<<scatter_grid(c->n_sm, 1), SCATTER_THREADS, bsm, c->stream>>>(A, 1);
  else
    k_bin_count<<<c->bin_grid, 256, bsm, c->stream>>>(A, smem_tiles);
}

lg_status ensure_raster_buffers(lg_ctx* c) {
  lg_status st;
  const uint64_t px = (uint64_t)c->prm.width * c->prm.height;
  const size_t elem = c->prm.accum == LG_ACCUM_F32 ? 4 : 8;
  if ((st = ensure(c, c->d_accum, px * 4 * elem, "accumulation image"))) return st;
  const size_t bins = 2 * (size_t)c->n_tiles;
  if ((st = ensure(c, c->d_tile_count, bins * 4, "tile counts"))) return st;
  if ((st = ensure(c, c->d_tile_off, bins * 8, "tile offsets"))) return st;
  if ((st = ensure(c, c->d_tile_cursor, bins * 8, "tile cursors"))) return st;
  if ((st = ensure(c, c->d_unit_off, bins * 8, "unit offsets"))) return st;
  if ((st = ensure(c, c->d_refs, c->refs_cap * 4, "tile refs"))) return st;
  c->units_cap = bins + c->refs_cap / MIN_UNIT_REFS + 1;
  if ((st = ensure(c, c->d_units, c->units_cap * sizeof(Unit), "raster units"))) return st;
  if ((st = ensure_cta_hist(c, bins))) return st;
  return LG_OK;
}

template <int CH>
static TraceKernel scan_kernel_ch(bool multi, bool culled, bool exact) {
  if (exact) {
    if (multi) return culled ? k_scan<true, true, true, CH> : k_scan<true, false, true, CH>;
    return culled ? k_scan<false, true, true, CH> : k_scan<false, false, true, CH>;
  }
  if (multi) return culled ? k_scan<true, true, false, CH> : k_scan<true, false, false, CH>;
  return culled ? k_scan<false, true, false, CH> : k_scan<false, false, false, CH>;
}

TraceKernel scan_kernel(bool multi, bool culled, bool exact, int pairs) {
  return pairs <= 8 ? scan_kernel_ch<8>(multi, culled, exact) : scan_kernel_ch<16>(multi, culled, exact);
}

// The scan's pair slots per lane: the tuned or requested value, else 8 with a culling grid
// and 16 without.
int scan_pairs_of(const lg_ctx* c) { return c->scan_pairs ? c->scan_pairs : (c->scan_walk ? 8 : 16); }

// Occupancy-sized grid of the scan for the context's mode and pair slots.
lg_status scan_grid(lg_ctx* c, bool multi) {
  const bool exact = c->prm.precision == LG_PRECISION_EXACT;
  const int pairs = scan_pairs_of(c);
  int occ = 0;
  if (multi) {
    // serving: the requests' precision is not known yet, the grid fits either kernel
    int occ_x = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, scan_kernel(true, c->scan_walk, c->serve ? false : exact, pairs),
                                                     SCAN_THREADS, (size_t)scan_smem_bytes(pairs)), "occupancy");
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_x, scan_kernel(true, c->scan_walk, c->serve ? true : exact, pairs),
                                                     SCAN_THREADS, (size_t)scan_smem_bytes(pairs)), "occupancy");
    c->batch_grid_scan = c->n_sm * std::max(1, std::min(occ, occ_x));
  } else {
    const size_t tsm = c->smem_fits ? c->obj_smem : 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, scan_kernel(false, c->scan_walk, exact, pairs), SCAN_THREADS,
                                                     (size_t)scan_smem_bytes(pairs) + tsm), "occupancy");
    c->trace_grid[0] = c->n_sm * std::max(1, occ);
  }
  return LG_OK;
}

// Switches the scan to `pairs` slots per lane: new grid, new graph.
lg_status set_scan_pairs(lg_ctx* c, int pairs, bool multi) {
  c->scan_pairs = pairs;
  c->graph_valid = false;
  return scan_grid(c, multi);
}
TraceKernel bounce_kernel(bool multi, bool culled) {
  if (multi) return culled ? k_bounce<true, true> : k_bounce<true, false>;
  return culled ? k_bounce<false, true> : k_bounce<false, false>;
}
TraceKernel3 bounce_x_kernel(bool multi, bool culled) {
  if (multi) return culled ? k_bounce_x<true, true> : k_bounce_x<true, false>;
  return culled ? k_bounce_x<false, true> : k_bounce_x<false, false>;
}

lg_status trace_grids(lg_ctx* c, bool multi, size_t tsm) {
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, multi ? k_refine<true> : k_refine<false>, 256, 0), "occupancy");
  c->trace_grid[1] = c->n_sm * std::max(1, occ);
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, multi ? k_full<true> : k_full<false>, 256, tsm), "occupancy");
  c->trace_grid[2] = c->n_sm * std::max(1, occ);
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bounce_kernel(multi, c->culled), 256, tsm), "occupancy");
  c->trace_grid[3] = c->n_sm * std::max(1, occ);
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, multi ? k_solve_x<true> : k_solve_x<false>, 256, 0), "occupancy");
  c->trace_grid[4] = c->n_sm * std::max(1, occ);
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bounce_x_kernel(multi, c->culled), 256, 0), "occupancy");
  c->trace_grid[5] = c->n_sm * std::max(1, occ);
  return LG_OK;
}

void launch_light_setup(lg_ctx* c, const SceneDev& S, bool multi, int blocks) {
  if (c->prm.precision == LG_PRECISION_EXACT) {
    if (multi) k_light_setup_x<true><<<blocks, 256, 0, c->stream>>>(S);
    else k_light_setup_x<false><<<blocks, 256, 0, c->stream>>>(S);
  } else {
    if (multi) k_light_setup<true><<<blocks, 256, 0, c->stream>>>(S);
    else k_light_setup<false><<<blocks, 256, 0, c->stream>>>(S);
  }
}

// Events around one generation's kernels while lg_render captures its frame graph (kev_on),
// k = 0 before the scan, 1 after it, 2 after the precise solve, 3 after the bounce.
static void kernel_event(lg_ctx* c, uint32_t g, int k) {
  if (!c->kev_on || 4 * g + k >= c->kev.size()) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusActive) return;
  cudaEventRecordWithFlags(c->kev[4 * g + k], c->stream, cudaEventRecordExternal);  // only inside the frame graph
}

void launch_generation(lg_ctx* c, const SceneDev& S, const TraceBufs& B, uint32_t g, bool multi, int scan_grid,
                       size_t scan_smem, size_t tsm, int smem_fits) {
  const bool exact = c->prm.precision == LG_PRECISION_EXACT;
  kernel_event(c, g, 0);
  scan_kernel(multi, c->scan_walk, exact, scan_pairs_of(c))<<<scan_grid, SCAN_THREADS, scan_smem, c->stream>>>(S, B, g,
                                                                                                   smem_fits);
  kernel_event(c, g, 1);
  if (exact) {
    if (multi) k_solve_x<true><<<c->trace_grid[4], 256, 0, c->stream>>>(S, B, g);
    else k_solve_x<false><<<c->trace_grid[4], 256, 0, c->stream>>>(S, B, g);
    kernel_event(c, g, 2);
    bounce_x_kernel(multi, c->culled)<<<c->trace_grid[5], 256, 0, c->stream>>>(S, B, g);
  } else {
    if (multi) {
      k_refine<true><<<c->trace_grid[1], 256, 0, c->stream>>>(S, B, g);
      k_full<true><<<c->trace_grid[2], 256, tsm, c->stream>>>(S, B, g, smem_fits);
    } else {
      k_refine<false><<<c->trace_grid[1], 256, 0, c->stream>>>(S, B, g);
      k_full<false><<<c->trace_grid[2], 256, tsm, c->stream>>>(S, B, g, smem_fits);
    }
    kernel_event(c, g, 2);
    bounce_kernel(multi, c->culled)<<<c->trace_grid[3], 256, tsm, c->stream>>>(S, B, g, smem_fits);
  }
  kernel_event(c, g, 3);
}

// Per-kernel trace times of the last lg_render, from the kernel events of every generation.
static void kernel_times(lg_ctx* c, lg_trace_stats* s) {
  if (!s || !c->kev_on) return;
  float a = 0.f, b = 0.f, d = 0.f;
  for (uint32_t g = 0; g < c->prm.max_bounce && 4 * g + 3 < c->kev.size(); ++g) {
    a += elapsed(c->kev[4 * g], c->kev[4 * g + 1]);
    b += elapsed(c->kev[4 * g + 1], c->kev[4 * g + 2]);
    d += elapsed(c->kev[4 * g + 2], c->kev[4 * g + 3]);
  }
  s->scan_ms = a;
  s->solve_ms = b;
  s->bounce_ms = d;
}

// lg_render's graphs record the kernel events (created once per context).
static lg_status enable_kernel_events(lg_ctx* c) {
  if (c->kev.empty()) {
    c->kev.assign(4 * MAX_GEN, nullptr);
    for (auto& e : c->kev) CK(cudaEventCreate(&e), "event");
  }
  if (!c->kev_on) c->graph_valid = false;  // the captured graph must record them
  c->kev_on = true;
  return LG_OK;
}

lg_status upload_exact(lg_ctx* c, const Flat& F) {
  lg_status st;
  if ((st = ensure(c, c->d_xgeo, F.xgeo.size() * sizeof(lg_geo) + 16, "scene"))) return st;
  if ((st = ensure(c, c->d_xnode, F.xnode.size() * sizeof(lgx::XNode) + 16, "scene"))) return st;
  if (!F.xgeo.empty())
    CK(cudaMemcpyAsync(c->d_xgeo.p, F.xgeo.data(), F.xgeo.size() * sizeof(lg_geo), cudaMemcpyHostToDevice, c->stream), "upload");
  if (!F.xnode.empty())
    CK(cudaMemcpyAsync(c->d_xnode.p, F.xnode.data(), F.xnode.size() * sizeof(lgx::XNode), cudaMemcpyHostToDevice, c->stream), "upload");
  return LG_OK;
}

// Control lines into the segment ring, string-mod lines into their table; records how many
// lines the accumulation draws.
void launch_overlay(lg_ctx* c, const SceneDev& S, const TraceBufs& B) {
  const uint64_t n_ov = overlay_segments(c), n_sm = string_mod_lines(c);
  c->chords_ready = n_sm;
  if (!n_ov && !n_sm) return;
  lg_string_mod sm = c->has_nested ? c->nested : c->prm.string_mod;
  sm.modulo = n_sm;
  ChordArgs CA;
  CA.out = (lg_chord*)c->d_chords.p;
  CA.colors = (const lg_mod_color*)c->d_mod_colors.p;
  CA.n_colors = sm.n_colors;
  CA.pts = c->has_nested ? (const double2*)c->d_cross.p : nullptr;
  CA.n_pts = c->n_cross;
  const int blocks = (int)std::min<uint64_t>((n_ov + n_sm + 255) / 256, 4096);
  k_overlay<<<blocks, 256, 0, c->stream>>>(S, B, (const uint32_t*)c->d_cubics.p, nullptr,
                                           c->prm.emit_control_lines ? c->n_cubic : 0, sm, CA);
}

// The string-mod lines of the last trace, into the image (after its clear).
void launch_chords(lg_ctx* c, const RasterArgs& A) {
  if (!c->chords_ready) return;
  const int blocks = (int)std::min<uint64_t>((c->chords_ready + 7) / 8, (uint64_t)c->n_sm * 8);
  if (c->prm.accum == LG_ACCUM_FIXED64)
    k_raster_chords<true><<<blocks, 256, 0, c->stream>>>(A, (const lg_chord*)c->d_chords.p, c->chords_ready);
  else
    k_raster_chords<false><<<blocks, 256, 0, c->stream>>>(A, (const lg_chord*)c->d_chords.p, c->chords_ready);
}

// The crossing points of a string mod's lines, for its nested mod (StringMod::
// line_crossings_as_points, string_mod.rs:87-102), computed once per upload: the lines, the
// crossings per block of (diff, line) pairs, their scan, then the points in pair order.
lg_status upload_crossings(lg_ctx* c, const lg_string_mod& outer) {
  const uint64_t m = outer.modulo;
  c->n_cross = 0;
  if (m < 2) return LG_OK;
  lg_string_mod sm = outer;
  sm.colors = nullptr;
  sm.nested = nullptr;
  const uint64_t n_pairs = m * (m - 1);
  const uint32_t n_blk = (uint32_t)((n_pairs + CROSS_PAIRS_PER_BLOCK - 1) / CROSS_PAIRS_PER_BLOCK);
  lg_status st;
  if ((st = ensure(c, c->d_sm_lines, 2 * m * sizeof(double2), "string-mod crossings"))) return st;
  if ((st = ensure(c, c->d_cross_blk, (size_t)n_blk * 4 + 16, "string-mod crossings"))) return st;
  double2* lines = (double2*)c->d_sm_lines.p;
  uint32_t* blk = (uint32_t*)c->d_cross_blk.p;
  unsigned long long* d_total = (unsigned long long*)((char*)c->d_cross_blk.p + (((size_t)n_blk * 4 + 7) & ~(size_t)7));
  k_sm_lines<<<(int)((m + 255) / 256), 256, 0, c->stream>>>(sm, lines);
  k_cross_count<<<n_blk, CROSS_THREADS, 0, c->stream>>>(lines, m, blk);
  k_cross_scan<<<1, 1024, 0, c->stream>>>(blk, n_blk, d_total);
  unsigned long long total = 0;
  CK(cudaMemcpyAsync(&total, d_total, sizeof total, cudaMemcpyDeviceToHost, c->stream), "string-mod crossings");
  CK(cudaStreamSynchronize(c->stream), "string-mod crossings");
  if (total) {
    if ((st = ensure(c, c->d_cross, total * sizeof(double2), "string-mod crossings"))) return st;
    k_cross_write<<<n_blk, CROSS_THREADS, 0, c->stream>>>(lines, m, blk, (double2*)c->d_cross.p);
    CK(cudaGetLastError(), "string-mod crossings");
  }
  c->n_cross = total;
  return LG_OK;
}

lg_status enqueue_trace(lg_ctx* c) {
  const SceneDev S = scene_dev(c);
  const TraceBufs B = trace_bufs(c);
  CK(cudaMemsetAsync(c->d_ctr.p, 0, sizeof(Counters), c->stream), "memset counters");
  if (c->n_lights) launch_light_setup(c, S, false, 1);
  const size_t tsm = c->smem_fits ? c->obj_smem : 0;
  for (uint32_t g = 0; g < c->prm.max_bounce; ++g)
    launch_generation(c, S, B, g, false, c->trace_grid[0], (size_t)scan_smem_bytes(scan_pairs_of(c)) + tsm, tsm, c->smem_fits);
  launch_overlay(c, S, B);
  CK(cudaGetLastError(), "trace launch");
  return LG_OK;
}

lg_status stage_event(lg_ctx* c, int i) {
  CK(cudaEventRecordWithFlags(c->ev[i], c->stream, cudaEventRecordExternal), "stage event");
  return LG_OK;
}

// binned_event >= 0 records that stage event between binning and the tile raster
lg_status enqueue_accumulate(lg_ctx* c, int binned_event = -1) {
  const RasterArgs A = raster_args(c);
  const int fixed = c->prm.accum == LG_ACCUM_FIXED64;
  k_clear_accum<<<c->n_sm * 8, 256, 0, c->stream>>>(A, fixed);
  CK(cudaMemsetAsync(c->d_tile_count.p, 0, (size_t)c->n_tiles * 8, c->stream), "memset tile counts");
  CK(cudaMemsetAsync(&((Counters*)c->d_ctr.p)->pixels, 0, sizeof(unsigned long long), c->stream), "memset pixels");
  const uint32_t bins = 2 * c->n_tiles;
  const int smem_tiles = bins <= MAX_SMEM_TILES ? 1 : 0;
  const size_t bsm = smem_tiles ? (size_t)bins * 4 : 0;
  launch_bin_count(c, A, smem_tiles, bsm);
  k_scan_tiles<<<1, 1024, 0, c->stream>>>(A);
  k_build_units<<<std::max(1u, (2 * c->n_tiles + 255) / 256), 256, 0, c->stream>>>(A);
  k_bin_scatter<<<scatter_grid(c->n_sm, smem_tiles), SCATTER_THREADS, bsm, c->stream>>>(A, smem_tiles);
  if (binned_event >= 0) {
    lg_status st = stage_event(c, binned_event);
    if (st) return st;
  }
  const int mode = raster_mode(c->prm);
  const size_t rsm = (size_t)raster_smem_bytes(mode);
  if (c->raster_variant == 2) {
    if (mode == RM_F32_)
      k_raster_warp<RM_F32_><<<c->raster_warp_grid, 32, raster_warp_smem_bytes(), c->stream>>>(A);
    else
      k_raster_warp<RM_FIXED_SPLIT_><<<c->raster_warp_grid, 32, raster_warp_smem_bytes(), c->stream>>>(A);
  } else if (mode == RM_FIXED_SPLIT_)
    k_raster<RM_FIXED_SPLIT_><<<c->raster_grid, 256, rsm, c->stream>>>(A);
  else if (mode == RM_FIXED_MINMAX_)
    k_raster<RM_FIXED_MINMAX_><<<c->raster_grid, 256, rsm, c->stream>>>(A);
  else
    k_raster<RM_F32_><<<c->raster_grid, 256, rsm, c->stream>>>(A);
  launch_chords(c, A);
  CK(cudaGetLastError(), "accumulate launch");
  return LG_OK;
}

lg_status enqueue_resolve(lg_ctx* c, uint16_t* dst, size_t pitch) {
  const int fixed = c->prm.accum == LG_ACCUM_FIXED64;
  k_resolve_f16<<<c->n_sm * 8, 256, 0, c->stream>>>(c->d_accum.p, fixed, c->prm.width, c->prm.height, dst, pitch);
  CK(cudaGetLastError(), "resolve launch");
  return LG_OK;
}

lg_status sync_counters(lg_ctx* c) {
  CK(cudaMemcpyAsync(c->h_ctr, c->d_ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "read counters");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  if (c->h_ctr->error_flags & ERR_TMA_TIMEOUT)
    return fail(c, LG_ERR_TIMEOUT, "object-table bulk copy did not complete within its wait limit");
  return LG_OK;
}

bool trace_overflowed(lg_ctx* c, uint64_t& need_seg, uint64_t& need_q) {
  need_seg = c->h_ctr->seg_count;
  need_q = 0;
  for (int g = 0; g <= MAX_GEN; ++g) need_q = std::max<uint64_t>(need_q, c->h_ctr->queue_count[g]);
  return need_seg > c->seg_cap || need_q > c->queue_cap;
}

lg_status grow_trace(lg_ctx* c, uint64_t need_seg, uint64_t need_q) {
  c->graph_valid = false;  // capacities are baked into the captured launches
  if (need_seg > c->seg_cap) c->seg_cap = need_seg + need_seg / 4 + 1024;
  if (need_q > c->queue_cap) c->queue_cap = need_q + need_q / 2 + 1024;
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const double want = (double)c->seg_cap * (sizeof(lg_segment) + (c->prm.record_paths ? sizeof(lg_path_record) : 0)) +
                      (double)c->queue_cap * (2 * sizeof(RayRec) + sizeof(ScanRec) + sizeof(HitRec) + 4 * N_LISTS);
  if (want > (double)total_b * 0.9)
    return fail(c, LG_ERR_OUT_OF_MEMORY, "trace needs " + std::to_string(want / 1e9) + " GB of segment ring and ray queues");
  return ensure_trace_buffers(c);
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

void fill_stats(lg_ctx* c, lg_trace_stats* s) {
  if (!s) return;
  const Counters& k = *c->h_ctr;
  s->primary_rays = c->n_primary;
  s->ray_visits = k.visits;
  s->segments = std::min<uint64_t>(k.seg_count, c->seg_cap);
  s->fp64_solves = k.fp64_solves;
  s->fp64_fallbacks = k.fallbacks;
  s->near_degenerate = k.near;
  s->ill_conditioned = k.ill;
  s->pixels = k.pixels;
  s->tile_refs = k.tile_refs;
  s->bound_tests = k.bound_tests;
  s->object_tests = k.object_tests;
}

lg_status run_trace_once(lg_ctx* c, uint32_t& retries, uint64_t seg_limit = ~0ull);

lg_status run_trace(lg_ctx* c, uint32_t& retries, uint64_t seg_limit = ~0ull) {
  return run_trace_once(c, retries, seg_limit);
}

// seg_limit: return LG_ERR_TRUNCATED instead of growing the ring past it
lg_status run_trace_once(lg_ctx* c, uint32_t& retries, uint64_t seg_limit) {
  for (int attempt = 0; attempt < 8; ++attempt) {
    lg_status st = enqueue_trace(c);
    if (st) return st;
    if ((st = sync_counters(c))) return st;
    uint64_t ns, nq;
    if (!trace_overflowed(c, ns, nq)) return LG_OK;
    if (ns > seg_limit) return LG_ERR_TRUNCATED;
    ++retries;
    if ((st = grow_trace(c, ns, nq))) return st;
  }
  return fail(c, LG_ERR_OUT_OF_MEMORY, "segment ring / ray queue kept overflowing");
}

lg_status run_accumulate_once(lg_ctx* c, uint32_t& retries);

// Autotuner: the first accumulation of a context runs both tile-raster kernels (each a
// complete, identical accumulation) and keeps the faster for every later launch and graph.
lg_status tune_raster(lg_ctx* c, uint32_t& retries) {
  float best = INFINITY;
  int pick = 1;
  for (int v = 1; v <= 2; ++v) {
    c->raster_variant = v;
    CK(cudaEventRecord(c->ev[4], c->stream), "event");
    lg_status st = run_accumulate_once(c, retries);
    if (st) return st;
    CK(cudaEventRecord(c->ev[5], c->stream), "event");
    CK(cudaEventSynchronize(c->ev[5]), "event");
    const float ms = elapsed(c->ev[4], c->ev[5]);
    if (ms < best) { best = ms; pick = v; }
  }
  c->graph_valid = false;
  if (c->raster_variant != pick) {
    c->raster_variant = pick;
    return run_accumulate_once(c, retries);
  }
  return LG_OK;
}

lg_status run_accumulate(lg_ctx* c, uint32_t& retries) {
  if (c->raster_variant == 0) return tune_raster(c, retries);
  return run_accumulate_once(c, retries);
}

lg_status run_accumulate_once(lg_ctx* c, uint32_t& retries) {
  for (int attempt = 0; attempt < 4; ++attempt) {
    lg_status st = enqueue_accumulate(c);
    if (st) return st;
    if ((st = sync_counters(c))) return st;
    if (c->h_ctr->tile_refs <= c->refs_cap) return LG_OK;
    ++retries;
    c->refs_cap = c->h_ctr->tile_refs + c->h_ctr->tile_refs / 8 + 4096;
    if (c->refs_cap >= 0xffffffffull) return fail(c, LG_ERR_UNSUPPORTED, "more than 2^32 (segment, tile) pairs in one frame");
    c->graph_valid = false;
    if ((st = ensure_raster_buffers(c))) return st;
  }
  return fail(c, LG_ERR_OUT_OF_MEMORY, "tile reference list kept overflowing");
}

lg_status need_scene(lg_ctx* c) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  if (!c->has_scene) return fail(c, LG_ERR_NO_SCENE, "no scene uploaded");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  return LG_OK;
}


}  // namespace lgh

// =============================================================================== C ABI
extern "C" {

uint32_t lg_abi_version(void) { return LG_ABI_VERSION; }

void lg_params_default(lg_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->max_bounce = 5;  // tracer.rs:37
  p->width = 512;
  p->height = 512;
  for (int i = 0; i < 4; ++i) p->cutoff_color[i] = 0.001f;  // tracer.rs:38
  p->clear_color[3] = 1.0f;                                 // wgpu::Color::BLACK
  p->color_blend = {LG_BF_ONE, LG_BF_ONE, LG_BO_ADD};       // mod.rs:67-71
  p->alpha_blend = {LG_BF_SRC_ALPHA, LG_BF_ONE, LG_BO_ADD}; // mod.rs:62-66
  p->accum = LG_ACCUM_FIXED64;
  p->emit_control_lines = 1;
  p->precision = LG_PRECISION_EXACT;
  p->ray_stride = 1;  // every primary
}

const char* lg_last_error(const lg_ctx* c) { return c ? c->err.c_str() : "null context"; }

lg_status lg_create(lg_ctx** out, const lg_device_opts* opts) {
  if (!out) return LG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  lg_ctx* c = new (std::nothrow) lg_ctx();
  if (!c) return LG_ERR_OUT_OF_MEMORY;
  c->device = opts ? opts->device : 0;
  c->seg_cap_hint = opts ? opts->segment_capacity : 0;
  c->raster_variant = opts && (opts->raster_variant == 1 || opts->raster_variant == 2) ? opts->raster_variant : 0;
  c->queue_cap_hint = opts ? opts->queue_capacity : 0;
  if (opts && opts->stream_segments) c->stream_ring = opts->stream_segments;
  if (opts && (opts->culling < LG_CULL_AUTO || opts->culling > LG_CULL_ON || !(opts->grid_density >= 0.0f))) {
    delete c;
    return LG_ERR_INVALID_ARGUMENT;
  }
  c->culling = opts ? opts->culling : LG_CULL_AUTO;
  c->grid_density = opts ? opts->grid_density : 0.0f;
  if (opts && opts->wait_polls) c->wait_polls = opts->wait_polls < 0 ? 0 : opts->wait_polls;
  if (opts && opts->scan_pairs != 0 && opts->scan_pairs != 8 && opts->scan_pairs != 16) {
    delete c;
    return LG_ERR_INVALID_ARGUMENT;
  }
  c->scan_pairs_opt = opts ? opts->scan_pairs : 0;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_ctr, sizeof(Counters));
  if (e == cudaSuccess) e = cudaMalloc(&c->d_ctr.p, sizeof(Counters));
  for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
  for (int pairs : {8, 16})
    for (int m = 0; m < 2; ++m)
      for (int cu = 0; cu < 2; ++cu)
        for (int ex = 0; ex < 2; ++ex)
          if (e == cudaSuccess)
            e = cudaFuncSetAttribute(scan_kernel(m != 0, cu != 0, ex != 0, pairs), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     scan_smem_bytes(pairs) + (m ? 0 : (int)OBJ_SMEM_MAX));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_full<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OBJ_SMEM_MAX);
  for (TraceKernel k : {k_bounce<false, false>, k_bounce<false, true>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OBJ_SMEM_MAX);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_bin_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(MAX_SMEM_TILES * 4));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_bin_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(MAX_SMEM_TILES * 4));
  if (e != cudaSuccess) {
    lg_status st = e == cudaErrorMemoryAllocation ? LG_ERR_OUT_OF_MEMORY : LG_ERR_CUDA;
    (void)cudaGetLastError();
    lg_destroy(c);
    return st;
  }
  c->d_ctr.bytes = sizeof(Counters);
  std::memset(c->h_ctr, 0, sizeof(Counters));
  lg_params_default(&c->prm);
  *out = c;
  return LG_OK;
}

lg_status lg_destroy(lg_ctx* c) {
  if (!c) return LG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  serve_free(c);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  DevBuf* bufs[] = {&c->d_scan, &c->d_info, &c->d_leaves, &c->d_prog, &c->d_lights, &c->d_cubics, &c->d_queue[0],
                    &c->d_queue[1], &c->d_scanrec, &c->d_hitrec, &c->d_list[0], &c->d_list[1], &c->d_list[2],
                    &c->d_list[3], &c->d_list[4], &c->d_list[5], &c->d_segs, &c->d_paths, &c->d_ctr, &c->d_tile_count, &c->d_tile_off,
                    &c->d_tile_cursor, &c->d_unit_off, &c->d_refs, &c->d_units, &c->d_accum, &c->d_stage,
                    &c->d_scenes, &c->d_canvases, &c->d_seg_scene, &c->d_cubic_scene, &c->d_part,
                    &c->d_bounds, &c->d_order, &c->d_scene_count, &c->d_scene_off,
                    &c->d_grids, &c->d_cell_start, &c->d_cell_obj, &c->d_cta_hist};
  for (DevBuf* b : bufs) release(*b);
  if (c->h_ctr) cudaFreeHost(c->h_ctr);
  for (int i = 0; i < 6; ++i)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  for (cudaEvent_t e : c->bev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->kev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return LG_OK;
}

lg_status lg_scene_upload(lg_ctx* c, const lg_geo* geos, uint32_t n_geo, const lg_object* objects, uint32_t n_objects,
                          const lg_light* lights, uint32_t n_lights, const lg_params* params) {
  if (!c || !params || (n_geo && !geos) || (n_objects && !objects) || (n_lights && !lights))
    return c ? fail(c, LG_ERR_INVALID_ARGUMENT, "null pointer") : LG_ERR_INVALID_ARGUMENT;
  if (c->serve) return fail(c, LG_ERR_INVALID_ARGUMENT, "serving in progress: lg_serve_end first");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const lg_params& p = *params;
  lg_status st = validate_params(c->err, p);
  if (st) return st;
  if (n_lights > 65535) return fail(c, LG_ERR_INVALID_ARGUMENT, "at most 65535 lights");
  if (n_objects > 65535) return fail(c, LG_ERR_UNSUPPORTED, "at most 65535 objects");
  Flat F;
  st = flatten_scene(c->err, geos, n_geo, objects, n_objects, lights, n_lights, F);
  if (st) return st;
  if ((st = validate_exact(c->err, p, F))) return st;
  lg_params pk = p;  // kept without the caller's colour-table and nested-mod pointers
  pk.string_mod.colors = nullptr;
  pk.string_mod.nested = nullptr;
  const bool nested = p.string_mod.modulo && p.string_mod.nested;
  lg_string_mod nk{};  // the nested mod, kept without its pointers
  if (nested) {
    nk = *p.string_mod.nested;
    nk.colors = nullptr;
    nk.nested = nullptr;
  }
  const bool same_shape = c->has_scene && c->n_obj == n_objects && c->n_leaves == F.leaves.size() &&
                          c->n_prog == F.prog.size() && c->n_lights == n_lights && c->n_cubic == F.cubics.size() &&
                          std::memcmp(&c->prm, &pk, sizeof pk) == 0 && c->has_nested == nested &&
                          std::memcmp(&c->nested, &nk, sizeof nk) == 0;
  // From here on the device tables are replaced: until this upload completes there is no scene
  // to trace, so a failure below leaves LG_ERR_NO_SCENE rather than a mix of two scenes (whose
  // line counts could exceed the line table).
  c->has_scene = false;
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  if ((st = upload_exact(c, F))) return st;
  if (p.string_mod.modulo) {
    // the mod drawn: the nested one (between the crossings of this mod's lines), else this one
    const lg_string_mod& drawn = nested ? *p.string_mod.nested : p.string_mod;
    if ((st = ensure(c, c->d_chords, std::max<uint64_t>(drawn.modulo, 1) * sizeof(lg_chord), "string-mod lines")))
      return st;
    if ((st = ensure(c, c->d_mod_colors, (size_t)std::max<uint32_t>(drawn.n_colors, 1) * sizeof(lg_mod_color),
                     "string-mod colours"))) return st;
    if (drawn.n_colors)
      CK(cudaMemcpyAsync(c->d_mod_colors.p, drawn.colors, drawn.n_colors * sizeof(lg_mod_color),
                         cudaMemcpyHostToDevice, c->stream), "upload");
  }
  c->has_nested = false;  // set again below once the crossings are in place
  c->n_cross = 0;
  if (nested && (st = upload_crossings(c, p.string_mod))) return st;
  c->has_nested = nested;
  c->nested = nk;
  if ((st = ensure(c, c->d_scan, F.scan.size() * sizeof(ObjScan), "scene"))) return st;
  if ((st = ensure(c, c->d_info, F.info.size() * sizeof(ObjInfo), "scene"))) return st;
  std::vector<Leaf64> dleaves;
  to_device_leaves(F.leaves, dleaves);
  if ((st = ensure(c, c->d_leaves, F.leaves.size() * sizeof(Leaf64), "scene"))) return st;
  if ((st = ensure(c, c->d_prog, F.prog.size() + 16, "scene"))) return st;
  if ((st = ensure(c, c->d_lights, F.lights.size() * sizeof(LightDev), "scene"))) return st;
  if ((st = ensure(c, c->d_cubics, F.cubics.size() * 4, "scene"))) return st;
  if (!F.scan.empty()) CK(cudaMemcpyAsync(c->d_scan.p, F.scan.data(), F.scan.size() * sizeof(ObjScan), cudaMemcpyHostToDevice, c->stream), "upload");
  if (!F.info.empty()) CK(cudaMemcpyAsync(c->d_info.p, F.info.data(), F.info.size() * sizeof(ObjInfo), cudaMemcpyHostToDevice, c->stream), "upload");
  if (!dleaves.empty()) CK(cudaMemcpyAsync(c->d_leaves.p, dleaves.data(), dleaves.size() * sizeof(Leaf64), cudaMemcpyHostToDevice, c->stream), "upload");
  if (!F.prog.empty()) CK(cudaMemcpyAsync(c->d_prog.p, F.prog.data(), F.prog.size(), cudaMemcpyHostToDevice, c->stream), "upload");
  if (p.ray_stride > 1) {  // a sampled frame numbers only the primaries it traces
    uint64_t first = 0;
    for (uint32_t l = 0; l < n_lights; ++l) {
      F.lights[l].first = first;
      first += sampled_rays(lights[l].num_rays, p);
    }
  }
  if (!F.lights.empty()) CK(cudaMemcpyAsync(c->d_lights.p, F.lights.data(), F.lights.size() * sizeof(LightDev), cudaMemcpyHostToDevice, c->stream), "upload");
  if (!F.cubics.empty()) CK(cudaMemcpyAsync(c->d_cubics.p, F.cubics.data(), F.cubics.size() * 4, cudaMemcpyHostToDevice, c->stream), "upload");
  build_grid(F.scan, c->culling, c->grid_density, F.grid);
  GridTables GT;
  GT.append(F.grid);
  if ((st = upload_grids(c, GT))) return st;
  CK(cudaStreamSynchronize(c->stream), "upload");
  if (c->multi) {  // leaving batch mode: every captured launch and launch shape is stale
    c->multi = false;
    c->graph_valid = false;
    c->n_scenes = 0;
  }
  if (c->culled != (F.grid.rec.nx > 0)) {  // the captured graph holds the other kernels
    c->culled = F.grid.rec.nx > 0;
    c->graph_valid = false;
  }
  // a new scene's scan walks the grid from LG_CULL_WALK_MIN objects until the autotuner measures
  // it (the bounce's medium test takes the grid whenever there is one); the same scene again keeps
  // what was tuned
  const bool walk = c->culled && (n_objects >= LG_CULL_WALK_MIN || c->culling == LG_CULL_ON);
  if ((!same_shape || !c->culled) && c->scan_walk != walk) {
    c->scan_walk = walk;
    c->graph_valid = false;
  }
  c->n_obj = n_objects;
  c->n_leaves = (uint32_t)F.leaves.size();
  c->n_prog = (uint32_t)F.prog.size();
  c->n_lights = n_lights;
  c->n_cubic = (uint32_t)F.cubics.size();
  c->n_primary = 0;
  for (uint32_t l = 0; l < n_lights; ++l) c->n_primary += sampled_rays(lights[l].num_rays, p);
  c->prm = pk;
  c->chords_ready = 0;
  c->aspect = (double)((float)p.width / (float)p.height);
  c->ntx = (p.width + TILE - 1) / TILE;
  c->nty = (p.height + TILE - 1) / TILE;
  c->n_tiles = c->ntx * c->nty;
  // launch shapes
  c->obj_smem = (size_t)n_objects * sizeof(ObjScan);
  c->smem_fits = c->obj_smem <= OBJ_SMEM_MAX ? 1 : 0;
  int occ = 0;
  const size_t tsm = c->smem_fits ? c->obj_smem : 0;
  if (!same_shape) {  // a new scene: its second lg_render times both scan pair-buffer sizes
    c->scan_pairs = c->scan_pairs_opt;
    c->scan_tune = c->scan_pairs_opt == 0;
    c->renders = 0;
  }
  if ((st = scan_grid(c, false))) return st;
  if ((st = trace_grids(c, false, tsm))) return st;
  const int mode = raster_mode(p);
  const int rsm = raster_smem_bytes(mode);
  if (mode == RM_FIXED_SPLIT_) {
    CK(cudaFuncSetAttribute(k_raster<RM_FIXED_SPLIT_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm), "smem attr");
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_FIXED_SPLIT_>, 256, rsm), "occupancy");
  } else if (mode == RM_FIXED_MINMAX_) {
    CK(cudaFuncSetAttribute(k_raster<RM_FIXED_MINMAX_>, cudaFuncAttributeMaxDynamicSharedMemorySize, rsm), "smem attr");
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_FIXED_MINMAX_>, 256, rsm), "occupancy");
  } else {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<RM_F32_>, 256, rsm), "occupancy");
  }
  c->raster_grid = c->n_sm * std::max(1, occ);
  CK(cudaFuncSetAttribute(k_raster_warp<RM_FIXED_SPLIT_>, cudaFuncAttributeMaxDynamicSharedMemorySize, raster_warp_smem_bytes()), "smem attr");
  CK(cudaFuncSetAttribute(k_raster_warp<RM_F32_>, cudaFuncAttributeMaxDynamicSharedMemorySize, raster_warp_smem_bytes()), "smem attr");
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster_warp<RM_FIXED_SPLIT_>, 32, raster_warp_smem_bytes()), "occupancy");
  c->raster_warp_grid = c->n_sm * std::max(1, occ);
  c->bin_grid = c->n_sm * 8;
  // capacities: first guesses, grown on overflow
  const uint64_t overlays = 3ull * F.cubics.size();
  // an explicit capacity from lg_device_opts is honoured as given (it still grows on overflow)
  const uint64_t want_seg = c->seg_cap_hint ? c->seg_cap_hint : 8 * c->n_primary + overlays + 1024;
  const uint64_t want_q = c->queue_cap_hint ? c->queue_cap_hint : 2 * c->n_primary + 1024;
  c->seg_cap = std::max(c->seg_cap, want_seg);
  c->queue_cap = std::max(c->queue_cap, std::max<uint64_t>(want_q, c->n_primary));  // gen 0 stores every primary
  if ((st = ensure_trace_buffers(c))) return st;
  c->refs_cap = std::max<uint64_t>(c->refs_cap, 1u << 20);
  if ((st = ensure_raster_buffers(c))) return st;
  if ((st = ensure(c, c->d_stage, (size_t)p.width * p.height * 8, "resolve staging"))) return st;
  if (!same_shape) {
    c->graph_valid = false;
    c->streaming = false;  // a new scene starts with one accumulation pass per frame
  }
  c->has_scene = true;
  return LG_OK;
}

lg_status lg_trace(lg_ctx* c, lg_trace_stats* stats) {
  lg_status st = need_scene(c);
  if (st) return st;
  uint32_t retries = 0;
  CK(cudaEventRecord(c->ev[0], c->stream), "event");
  if ((st = run_trace(c, retries))) return st;
  CK(cudaEventRecord(c->ev[1], c->stream), "event");
  CK(cudaEventSynchronize(c->ev[1]), "event");
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    fill_stats(c, stats);
    stats->retries = retries;
    stats->trace_ms = elapsed(c->ev[0], c->ev[1]);
    stats->total_ms = stats->trace_ms;
  }
  return LG_OK;
}

lg_status lg_accumulate(lg_ctx* c, lg_trace_stats* stats) {
  lg_status st = need_scene(c);
  if (st) return st;
  uint32_t retries = 0;
  CK(cudaEventRecord(c->ev[0], c->stream), "event");
  if ((st = run_accumulate(c, retries))) return st;
  CK(cudaEventRecord(c->ev[1], c->stream), "event");
  CK(cudaEventSynchronize(c->ev[1]), "event");
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    fill_stats(c, stats);
    stats->retries = retries;
    stats->accumulate_ms = elapsed(c->ev[0], c->ev[1]);
    stats->total_ms = stats->accumulate_ms;
  }
  return LG_OK;
}

lg_status lg_accumulate_segments(lg_ctx* c, const lg_segment* segs, uint64_t n, lg_trace_stats* stats) {
  lg_status st = need_scene(c);
  if (st) return st;
  if (n && !segs) return fail(c, LG_ERR_INVALID_ARGUMENT, "null segments");
  if (n > c->seg_cap) {
    c->seg_cap = n;
    if ((st = ensure_trace_buffers(c))) return st;
  }
  if (n) CK(cudaMemcpyAsync(c->d_segs.p, segs, n * sizeof(lg_segment), cudaMemcpyHostToDevice, c->stream), "upload segments");
  Counters* d = (Counters*)c->d_ctr.p;
  CK(cudaMemsetAsync(d, 0, sizeof(Counters), c->stream), "memset counters");
  unsigned long long nn = n;
  CK(cudaMemcpyAsync(&d->seg_count, &nn, sizeof nn, cudaMemcpyHostToDevice, c->stream), "segment count");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  c->graph_valid = false;  // the ring no longer holds a trace
  c->chords_ready = 0;
  return lg_accumulate(c, stats);
}

lg_status lg_resolve_f16(lg_ctx* c, uint16_t* dst, size_t pitch, int32_t dst_is_device) {
  lg_status st = need_scene(c);
  if (st) return st;
  const size_t row = (size_t)c->prm.width * 8;
  if (!dst || pitch < row) return fail(c, LG_ERR_INVALID_ARGUMENT, "destination null or pitch < width * 8");
  if (dst_is_device) {
    if ((st = enqueue_resolve(c, dst, pitch))) return st;
  } else {
    if ((st = enqueue_resolve(c, (uint16_t*)c->d_stage.p, row))) return st;
    CK(cudaMemcpy2DAsync(dst, pitch, c->d_stage.p, row, row, c->prm.height, cudaMemcpyDeviceToHost, c->stream), "download image");
  }
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return LG_OK;
}

lg_status lg_resolve_rgba8(lg_ctx* c, uint8_t* dst, size_t pitch, int32_t dst_is_device) {
  lg_status st = need_scene(c);
  if (st) return st;
  const size_t row = (size_t)c->prm.width * 4;
  if (!dst || pitch < row) return fail(c, LG_ERR_INVALID_ARGUMENT, "destination null or pitch < width * 4");
  const int fixed = c->prm.accum == LG_ACCUM_FIXED64;
  uint8_t* out = dst_is_device ? dst : (uint8_t*)c->d_stage.p;
  k_resolve_rgba8<<<c->n_sm * 8, 256, 0, c->stream>>>(c->d_accum.p, fixed, c->prm.width, c->prm.height, out,
                                                       dst_is_device ? pitch : row);
  CK(cudaGetLastError(), "resolve launch");
  if (!dst_is_device)
    CK(cudaMemcpy2DAsync(dst, pitch, c->d_stage.p, row, row, c->prm.height, cudaMemcpyDeviceToHost, c->stream), "download image");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return LG_OK;
}

// The whole frame with the accumulation interleaved: after each generation the segment ring
// is accumulated if it could not take the next generation (k_stream_decide), so the ring
// and the tile lists hold a bounded part of the frame.  ev: 2 * max_bounce + 2 events.
static lg_status enqueue_stream_frame(lg_ctx* c, uint16_t* dst, size_t row, cudaEvent_t* ev) {
  const SceneDev S = scene_dev(c);
  const TraceBufs B = trace_bufs(c);
  const RasterArgs A = raster_args(c);
  const int fixed = c->prm.accum == LG_ACCUM_FIXED64;
  CK(cudaEventRecordWithFlags(ev[0], c->stream, cudaEventRecordExternal), "stage event");
  CK(cudaMemsetAsync(c->d_ctr.p, 0, sizeof(Counters), c->stream), "memset counters");
  k_clear_accum<<<c->n_sm * 8, 256, 0, c->stream>>>(A, fixed);
  if (c->n_lights) launch_light_setup(c, S, false, 1);
  const size_t tsm = c->smem_fits ? c->obj_smem : 0;
  const uint32_t bins = 2 * c->n_tiles;
  const int smem_tiles = bins <= MAX_SMEM_TILES ? 1 : 0;
  const size_t bsm = smem_tiles ? (size_t)bins * 4 : 0;
  const uint32_t n_part = (bins + TILE_SCAN_CHUNK - 1) / TILE_SCAN_CHUNK;
  const int mode = raster_mode(c->prm);
  const size_t rsm = (size_t)raster_smem_bytes(mode);
  const uint32_t G = c->prm.max_bounce;
  for (uint32_t g = 0; g < G; ++g) {
    launch_generation(c, S, B, g, false, c->trace_grid[0], (size_t)scan_smem_bytes(scan_pairs_of(c)) + tsm, tsm, c->smem_fits);
    if (g == 0) {
      launch_overlay(c, S, B);
      launch_chords(c, A);
    }
    CK(cudaEventRecordWithFlags(ev[1 + 2 * g], c->stream, cudaEventRecordExternal), "stage event");
    k_stream_decide<<<1, 1, 0, c->stream>>>((Counters*)c->d_ctr.p, g, c->seg_cap, c->queue_cap, g + 1 == G ? 1 : 0);
    k_clear_counts<<<c->n_sm * 4, 256, 0, c->stream>>>(A);
    launch_bin_count(c, A, smem_tiles, bsm);
    if (bins <= 32768) {
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
  k_resolve_f16<<<c->n_sm * 8, 256, 0, c->stream>>>(c->d_accum.p, fixed, c->prm.width, c->prm.height, dst, row);
  CK(cudaEventRecordWithFlags(ev[1 + 2 * G], c->stream, cudaEventRecordExternal), "stage event");
  CK(cudaGetLastError(), "stream frame launch");
  return LG_OK;
}

// Switches a context to the streaming frame: a ring of stream_ring segments instead of one
// that holds the whole frame.
static lg_status start_streaming(lg_ctx* c) {
  c->streaming = true;
  c->graph_valid = false;
  if (c->raster_variant == 0) c->raster_variant = 1;
  const uint64_t n_ov = 3ull * c->n_cubic;
  c->seg_cap = std::max<uint64_t>(c->stream_ring, c->queue_cap + n_ov + 1024);
  c->refs_cap = std::min<uint64_t>(4 * c->seg_cap, 0xfffffff0ull);
  if (c->bev.empty()) {
    c->bev.assign(2 * MAX_GEN + 2, nullptr);
    for (auto& e : c->bev) CK(cudaEventCreate(&e), "event");
  }
  lg_status st = ensure_trace_buffers(c);
  if (st) return st;
  if ((st = ensure_raster_buffers(c))) return st;
  const size_t parts = (2 * (size_t)c->n_tiles + TILE_SCAN_CHUNK - 1) / TILE_SCAN_CHUNK;
  return ensure(c, c->d_part, std::max<size_t>(parts, 1) * 16, "tile scan partials");
}

static lg_status render_streaming(lg_ctx* c, uint16_t* dst, size_t pitch, int32_t dst_is_device, lg_trace_stats* stats,
                              uint32_t retries) {
  const size_t row = (size_t)c->prm.width * 8;
  std::vector<cudaEvent_t>& ev = c->bev;
  const uint32_t G = c->prm.max_bounce;
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (!c->graph_valid) {
      if (c->gexec) cudaGraphExecDestroy(c->gexec);
      c->gexec = nullptr;
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      lg_status s1 = enqueue_stream_frame(c, (uint16_t*)c->d_stage.p, row, ev.data());
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
    const Counters& k = *c->h_ctr;
    if (k.error_flags & ERR_TMA_TIMEOUT)
      return fail(c, LG_ERR_TIMEOUT, "object-table bulk copy did not complete within its wait limit");
    uint64_t nq = 0;
    for (int g = 0; g <= MAX_GEN; ++g) nq = std::max<uint64_t>(nq, k.queue_count[g]);
    if (nq > c->queue_cap || k.seg_max > c->seg_cap || k.refs_max > c->refs_cap) {
      ++retries;
      c->graph_valid = false;
      if (nq > c->queue_cap) c->queue_cap = nq + nq / 2 + 1024;
      c->seg_cap = std::max<uint64_t>(c->seg_cap, c->queue_cap + 3ull * c->n_cubic + 1024);
      if (k.refs_max > c->refs_cap) c->refs_cap = k.refs_max + k.refs_max / 4 + 4096;
      if (c->refs_cap >= 0xffffffffull) return fail(c, LG_ERR_UNSUPPORTED, "more than 2^32 (segment, tile) pairs in one pass");
      lg_status st = ensure_trace_buffers(c);
      if (st) return st;
      if ((st = ensure_raster_buffers(c))) return st;
      continue;
    }
    CK(cudaMemcpy2DAsync(dst, pitch, c->d_stage.p, row, row, c->prm.height,
                         dst_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream), "copy image");
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (stats) {
      std::memset(stats, 0, sizeof *stats);
      fill_stats(c, stats);
      stats->segments = k.seg_total;
      stats->tile_refs = k.refs_total;
      stats->retries = retries;
      float tr = 0.f, ac = 0.f;
      for (uint32_t g = 0; g < G; ++g) {
        tr += elapsed(g == 0 ? ev[0] : ev[2 * g], ev[1 + 2 * g]);
        ac += elapsed(ev[1 + 2 * g], ev[2 + 2 * g]);
      }
      stats->trace_ms = tr;
      stats->accumulate_ms = ac;
      stats->raster_ms = ac;
      stats->resolve_ms = elapsed(ev[2 * G], ev[1 + 2 * G]);
      stats->total_ms = elapsed(ev[0], ev[1 + 2 * G]);
      kernel_times(c, stats);
    }
    return LG_OK;
  }
  return fail(c, LG_ERR_OUT_OF_MEMORY, "render buffers kept overflowing");
}

static lg_status render_frame(lg_ctx* c, uint16_t* dst, size_t pitch, int32_t dst_is_device, lg_trace_stats* stats);

// The second frame of a scene (unless lg_device_opts.scan_pairs fixes the size) renders with
// each scan pair-buffer size and keeps the one whose scan kernels ran faster; the frames are
// identical, so the caller's image is simply the last one.  A scene rendered once keeps the
// default (8 slots with a culling grid, 16 without) and pays no tuning.
lg_status lg_render(lg_ctx* c, uint16_t* dst, size_t pitch, int32_t dst_is_device, lg_trace_stats* stats) {
  lg_status st = need_scene(c);
  if (st) return st;
  if (c->renders < 0xffffffffu) ++c->renders;
  if (c->scan_tune && c->renders >= 2) {
    // with a culling grid: the grid walk with 8 pair slots against the table scan with 16; without
    // one: the table scan with 8 against 16
    c->scan_tune = false;
    float best = INFINITY;
    int pick = scan_pairs_of(c);
    bool pick_walk = c->scan_walk;
    const int opts[2][2] = {{c->culled ? 1 : 0, 8}, {0, 16}};
    for (const auto& o : opts) {
      c->scan_walk = o[0] != 0;
      if ((st = set_scan_pairs(c, o[1], false))) return st;
      lg_trace_stats s;
      if ((st = render_frame(c, dst, pitch, dst_is_device, &s))) return st;
      const float ms = s.trace_ms > 0.0f ? s.trace_ms : s.total_ms;  // the walk also moves work to the solve
      if (ms < best) { best = ms; pick = o[1]; pick_walk = o[0] != 0; }
    }
    c->scan_walk = pick_walk;
    if ((st = set_scan_pairs(c, pick, false))) return st;
  }
  return render_frame(c, dst, pitch, dst_is_device, stats);
}

static lg_status render_frame(lg_ctx* c, uint16_t* dst, size_t pitch, int32_t dst_is_device, lg_trace_stats* stats) {
  lg_status st = LG_OK;
  const size_t row = (size_t)c->prm.width * 8;
  if (!dst || pitch < row) return fail(c, LG_ERR_INVALID_ARGUMENT, "destination null or pitch < width * 8");
  uint32_t retries = 0;
  if ((st = enable_kernel_events(c))) return st;
  if (c->streaming) return render_streaming(c, dst, pitch, dst_is_device, stats, retries);
  if (c->raster_variant == 0) {  // pick the raster kernel before it is baked into the graph
    st = run_trace(c, retries, c->stream_ring);
    if (st == LG_ERR_TRUNCATED) {  // more segments than one pass takes: stream the frame
      if ((st = start_streaming(c))) return st;
      return render_streaming(c, dst, pitch, dst_is_device, stats, retries);
    }
    if (st) return st;
    if ((st = tune_raster(c, retries))) return st;
  }
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (!c->graph_valid) {
      if (c->gexec) cudaGraphExecDestroy(c->gexec);
      c->gexec = nullptr;
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      // timing events recorded as graph nodes: start, traced, binned, rasterised, resolved
      lg_status s1 = stage_event(c, 0);
      if (!s1) s1 = enqueue_trace(c);
      if (!s1) s1 = stage_event(c, 1);
      if (!s1) s1 = enqueue_accumulate(c, 2);
      if (!s1) s1 = stage_event(c, 3);
      if (!s1) s1 = enqueue_resolve(c, (uint16_t*)c->d_stage.p, row);
      if (!s1) s1 = stage_event(c, 4);
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
    uint64_t ns, nq;
    if (trace_overflowed(c, ns, nq)) {
      ++retries;
      if (ns > c->stream_ring) {
        if ((st = start_streaming(c))) return st;
        return render_streaming(c, dst, pitch, dst_is_device, stats, retries);
      }
      if ((st = grow_trace(c, ns, nq))) return st;
      continue;
    }
    if (c->h_ctr->tile_refs > c->refs_cap) {
      ++retries;
      c->refs_cap = c->h_ctr->tile_refs + c->h_ctr->tile_refs / 8 + 4096;
      if (c->refs_cap >= 0xfffffff0ull) {
        if ((st = start_streaming(c))) return st;
        return render_streaming(c, dst, pitch, dst_is_device, stats, retries);
      }
      if ((st = ensure_raster_buffers(c))) return st;
      c->graph_valid = false;
      continue;
    }
    if (dst_is_device) {
      CK(cudaMemcpy2DAsync(dst, pitch, c->d_stage.p, row, row, c->prm.height, cudaMemcpyDeviceToDevice, c->stream), "copy image");
    } else {
      CK(cudaMemcpy2DAsync(dst, pitch, c->d_stage.p, row, row, c->prm.height, cudaMemcpyDeviceToHost, c->stream), "download image");
    }
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (stats) {
      std::memset(stats, 0, sizeof *stats);
      fill_stats(c, stats);
      stats->retries = retries;
      stats->trace_ms = elapsed(c->ev[0], c->ev[1]);
      stats->bin_ms = elapsed(c->ev[1], c->ev[2]);
      stats->raster_ms = elapsed(c->ev[2], c->ev[3]);
      stats->accumulate_ms = elapsed(c->ev[1], c->ev[3]);
      stats->resolve_ms = elapsed(c->ev[3], c->ev[4]);
      stats->total_ms = elapsed(c->ev[0], c->ev[4]);
      kernel_times(c, stats);
    }
    return LG_OK;
  }
  return fail(c, LG_ERR_OUT_OF_MEMORY, "render buffers kept overflowing");
}

lg_status lg_segments_download(lg_ctx* c, lg_segment* out, lg_path_record* paths, uint64_t cap, uint64_t* n_out) {
  lg_status st = need_scene(c);
  if (st) return st;
  if (!n_out) return fail(c, LG_ERR_INVALID_ARGUMENT, "null n_out");
  CK(cudaMemcpyAsync(c->h_ctr, c->d_ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream), "read counters");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  const uint64_t n = std::min<uint64_t>(c->h_ctr->seg_count, c->seg_cap);
  *n_out = n;
  if (cap < n) return fail(c, LG_ERR_TRUNCATED, "buffer holds fewer segments than the ring");
  if (paths && !c->prm.record_paths) return fail(c, LG_ERR_INVALID_ARGUMENT, "path records need params.record_paths");
  if (n && out) CK(cudaMemcpyAsync(out, c->d_segs.p, n * sizeof(lg_segment), cudaMemcpyDeviceToHost, c->stream), "download segments");
  if (n && paths) CK(cudaMemcpyAsync(paths, c->d_paths.p, n * sizeof(lg_path_record), cudaMemcpyDeviceToHost, c->stream), "download paths");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return LG_OK;
}

lg_status lg_chords_download(lg_ctx* c, lg_chord* out, uint64_t cap, uint64_t* n_out) {
  lg_status st = need_scene(c);
  if (st) return st;
  if (!n_out) return fail(c, LG_ERR_INVALID_ARGUMENT, "null n_out");
  const uint64_t n = c->chords_ready;
  *n_out = n;
  if (cap < n) return fail(c, LG_ERR_TRUNCATED, "buffer holds fewer lines than the frame");
  if (n && out) CK(cudaMemcpyAsync(out, c->d_chords.p, n * sizeof(lg_chord), cudaMemcpyDeviceToHost, c->stream), "download lines");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return LG_OK;
}

lg_status lg_accum_download(lg_ctx* c, void* out, uint64_t cap_bytes) {
  lg_status st = need_scene(c);
  if (st) return st;
  const uint64_t bytes = (uint64_t)c->prm.width * c->prm.height * 4 * (c->prm.accum == LG_ACCUM_F32 ? 4 : 8);
  if (!out) return fail(c, LG_ERR_INVALID_ARGUMENT, "null output");
  if (cap_bytes < bytes) return fail(c, LG_ERR_TRUNCATED, "output smaller than the accumulation image");
  CK(cudaMemcpyAsync(out, c->d_accum.p, bytes, cudaMemcpyDeviceToHost, c->stream), "download accumulation image");
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return LG_OK;
}


}  // extern "C"
