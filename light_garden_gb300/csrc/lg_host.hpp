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

// One scene (or several, concatenated) in the layout of the device tables.
struct Flat {
  std::vector<ObjScan> scan;
  std::vector<ObjInfo> info;
  std::vector<LeafH> leaves;
  std::vector<uint8_t> prog;
  std::vector<LightDev> lights;
  std::vector<uint32_t> cubics;
};


// Validates and flattens one scene: geometry trees into leaves + postfix CSG programs,
// FP32 scan records with bounding circles, lights with their first primary index.
lg_status flatten_scene(std::string& err, const lg_geo* G, uint32_t n_geo, const lg_object* O, uint32_t n_obj,
                        const lg_light* Ls, uint32_t n_lights, Flat& F);
lg_status validate_params(std::string& err, const lg_params& p);
bool blend_supported(const lg_blend_component& b);
int raster_mode(const lg_params& p);
void to_device_leaves(const std::vector<LeafH>& in, std::vector<Leaf64>& out);

}  // namespace lgh
