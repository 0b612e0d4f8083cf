// lg_host.hpp — host-side scene flattening shared by the single-scene context
// (lg_api.cu) and the multi-scene batch / serving engine (lg_batch.cu).
#pragma once
#include <string>
#include <vector>

#include "lg_kernels.cuh"

namespace lgh {

using namespace lgd;

inline lg_status set_err(std::string& e, lg_status st, const std::string& m) {
  e = m;
  return st;
}

// host FP64 leaf; converted to the device's double-float Leaf64 at upload
struct LeafH {
  uint32_t kind;
  double p[8];
  double box[4];  // HALFPLANE: the world box of its polygon (the leaf itself is unbounded)
};

// Culling grid of one scene: the record (bases 0), its cell offsets and object lists.
struct GridH {
  GridRec rec;
  std::vector<uint32_t> cell_start;  // nx * ny + 1 (one entry when there is no grid)
  std::vector<uint16_t> cell_obj;
};

// One scene (or several, concatenated) in the layout of the device tables.
struct Flat {
  std::vector<ObjScan> scan;
  std::vector<ObjInfo> info;
  std::vector<LeafH> leaves;
  std::vector<uint8_t> prog;
  std::vector<LightDev> lights;
  std::vector<uint32_t> cubics;
  GridH grid;
  // exact mode: the geometry nodes as given, each object's tree in preorder (ObjInfo::
  // xnode_begin / xnode_count index xnode; XNode::geo indexes xgeo) and the deepest node
  std::vector<lg_geo> xgeo;
  std::vector<lgx::XNode> xnode;
  int xdepth = 0;
  // appends another scene's exact-mode tables, moving its node indices past this one's;
  // the caller adds the returned base to that scene's ObjInfo::xnode_begin
  uint32_t append_exact(const Flat& o) {
    const uint32_t g0 = (uint32_t)xgeo.size(), n0 = (uint32_t)xnode.size();
    xgeo.insert(xgeo.end(), o.xgeo.begin(), o.xgeo.end());
    for (lgx::XNode n : o.xnode) {
      n.geo += (int32_t)g0;
      xnode.push_back(n);
    }
    xdepth = xdepth > o.xdepth ? xdepth : o.xdepth;
    return n0;
  }
};

// Several scenes' grids, concatenated in the order of their object tables.
struct GridTables {
  std::vector<GridRec> recs;
  std::vector<uint32_t> cell_start;
  std::vector<uint16_t> cell_obj;
  // appends a scene's cells and object lists; returns its record with the bases set
  GridRec add(const GridH& g) {
    GridRec r = g.rec;
    r.cell_base = (uint32_t)cell_start.size();
    r.list_base = (uint32_t)cell_obj.size();
    cell_start.insert(cell_start.end(), g.cell_start.begin(), g.cell_start.end());
    cell_obj.insert(cell_obj.end(), g.cell_obj.begin(), g.cell_obj.end());
    return r;
  }
  void append(const GridH& g) { recs.push_back(add(g)); }
};


// Validates and flattens one scene: geometry trees into leaves + postfix CSG programs,
// FP32 scan records with bounding circles, lights with their first primary index.
lg_status flatten_scene(std::string& err, const lg_geo* G, uint32_t n_geo, const lg_object* O, uint32_t n_obj,
                        const lg_light* Ls, uint32_t n_lights, Flat& F);
lg_status validate_params(std::string& err, const lg_params& p);
// Exact mode's limits on a flattened scene (trees of at most lgx::MAX_DEPTH levels).
lg_status validate_exact(std::string& err, const lg_params& p, const Flat& F);
bool blend_supported(const lg_blend_component& b);
int raster_mode(const lg_params& p);
void to_device_leaves(const std::vector<LeafH>& in, std::vector<Leaf64>& out);
// Builds the culling grid of a flattened scene (culling: lg_culling; density: cells per
// object, 0 = default).
void build_grid(const std::vector<ObjScan>& scan, int culling, float density, GridH& G);

}  // namespace lgh
