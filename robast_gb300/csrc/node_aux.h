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
  RBG_AUX_ASPH_TWIN_FACES = 1,
  // the node has AGeoAsphericDisk daughters: its boundary search brackets
  // their crossings in FP32 first (find_next_boundary_and_step_f)
  RBG_AUX_ASPH_CHILDREN = 2
};

struct rbg_node_aux {
  float lo[3], hi[3];  // master-frame bounding box, rounded outward to float
  int32_t xform;       // RBG_XFORM_*
  int32_t flags;       // RBG_AUX_*
};
static_assert(sizeof(rbg_node_aux) == 32, "rbg_node_aux layout");

// Per-shape trigonometric constants (rbg_scene::trig at trig_off[shape]),
// so that no shape query evaluates sin/cos/tan/atan2 of a fixed angle:
//   TUBE, PCON : [0..3] phi-plane normals (-sin a1, cos a1, -sin a2, cos a2),
//                a1 = phi1, a2 = phi1 + dphi
//   SPHERE     : [0..3] phi-plane normals, [4] cos th1, [5] cos th2,
//                [6] cos^2 th1, [7] cos^2 th2
//   PGON       : [0..3] phi-plane normals, then per edge e (cos pe, sin pe)
//                with pe = phi1 + (e + 1/2) dphi / nedges
//   WINSTON    : [0] cos theta, [1] sin theta, [2] tan(pi / n), then per face
//                k (cos 2 pi k / n, sin 2 pi k / n)
//   ASPHERIC   : [0] z2 - z1 (the face separation), then the derivative
//                coefficients (j + 1) K_j of face 1 (npol1) and of face 2
//                (npol2), so that d sag / d r^2 is a plain FMA Horner sum
enum : int32_t {
  RBG_TRIG_PHI = 0,
  RBG_TRIG_SPH_COS = 4,
  RBG_TRIG_SPH_COS2 = 6,
  RBG_TRIG_PGON_EDGE = 4,
  RBG_TRIG_WIN_COS = 0,
  RBG_TRIG_WIN_SIN = 1,
  RBG_TRIG_WIN_TANHALF = 2,
  RBG_TRIG_WIN_FACE = 3,
  RBG_TRIG_ASPH_DZ = 0,
  RBG_TRIG_ASPH_DK = 1
};

struct rbg_scene;
namespace rbg {
// fills s->node_aux, s->fparams, s->trig and s->trig_off from the
// flattened tables (scene.cpp)
void build_node_aux(rbg_scene* s);
}  // namespace rbg
