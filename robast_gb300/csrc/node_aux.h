// node_aux.h -- device-only tables derived from a flattened scene for the
// mixed-precision tracer: FP32 screens need float boxes and float copies of
// the shape parameters, and most nodes of a telescope are placed without a
// rotation, so their master->local transform can be skipped or reduced to a
// translation.  Built once per scene on the host (scene.cpp), uploaded with
// the other tables; not part of the flattened-scene C view.
#pragma once
#include <cstdint>

enum : int32_t {
  RBG_XFORM_IDENTITY = 0,     // local == master
  RBG_XFORM_TRANSLATION = 1,  // local = master - t
  RBG_XFORM_GENERAL = 2       // rotation and translation
};

enum : int32_t {
  // aspheric disk whose two faces share curvature, conic constant and
  // polynomial and differ only by their vertex z (a thin mirror shell)
  RBG_AUX_ASPH_TWIN_FACES = 1
};

struct rbg_node_aux {
  float lo[3], hi[3];  // master-frame bounding box, rounded outward to float
  int32_t xform;       // RBG_XFORM_*
  int32_t flags;       // RBG_AUX_*
};
static_assert(sizeof(rbg_node_aux) == 32, "rbg_node_aux layout");

struct rbg_scene;
namespace rbg {
// fills s->node_aux and s->fparams from the flattened tables (scene.cpp)
void build_node_aux(rbg_scene* s);
}  // namespace rbg
