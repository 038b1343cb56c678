// scene_internal.h -- host-side representation of a flattened scene.
#pragma once
#include <cstdint>
#include <vector>

#include "robast_gb.h"
#include "robast_gb_layout.h"
#include "node_aux.h"

struct rbg_device_scene;  // defined in device_state.cuh

struct rbg_scene {
  // canonical description tables (ids identical to the user description)
  std::vector<rbg_shape_desc> shapes;
  std::vector<double> params;
  std::vector<rbg_volume_desc> volumes;
  std::vector<rbg_table_desc> tables;
  std::vector<rbg_index_desc> indices;
  std::vector<rbg_layer_desc> layers;
  std::vector<rbg_multilayer_desc> multilayers;
  std::vector<rbg_border_desc> borders;
  // physical tree
  std::vector<rbg_node> nodes;
  std::vector<int32_t> children;
  std::vector<rbg_bvh_node> bvh;
  std::vector<int32_t> bvh_items;
  // local bounding boxes per shape: lo[3], hi[3]
  std::vector<double> shape_box;
  // kFeat* bits (trace_features.h) the scene uses
  uint32_t features = 0;
  // device-only tables of the mixed-precision tracer (node_aux.h)
  std::vector<rbg_node_aux> node_aux;
  std::vector<float> fparams;
  // per-shape trigonometric constants (node_aux.h), offsets per shape or -1
  std::vector<double> trig;
  std::vector<int32_t> trig_off;
  // precalculated thin-film tables: R then T per multilayer at tmm_off (or
  // -1); filled on the GPU at the first upload (tmm.cu), then kept here
  std::vector<double> tmm_tables;
  std::vector<int64_t> tmm_off;
  bool tmm_ready = true;

  // device mirror, owned by the CUDA side (capi.cu)
  rbg_device_scene* dev = nullptr;
  int dev_id = -1;
  int last_launches = 0;
  // kernel timing of rbg_trace (rbg_scene_set_timing): CUDA events around
  // the tracer kernel, its last duration in ms
  bool timing = false;
  void* tev[2] = {nullptr, nullptr};
  float last_kernel_ms = -1.f;
  int tuned_compaction = 0;  // rbg_scene_autotune's choice, 0: none yet
  int tuned_block = 0;       // its block size for the lean mixed instance, 0: none yet
  void* workspace = nullptr;
  size_t workspace_bytes = 0;
  // rbg_trace's ray-order workspace (grown on demand, freed with the scene)
  void* order_ws = nullptr;
  size_t order_ws_bytes = 0;
};

// host helpers shared with the C-ABI implementation
namespace rbg {
void release_device(rbg_scene* s);  // capi.cu
}
