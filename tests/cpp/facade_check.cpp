// facade_check.cpp -- exercises the C++ facade (include/robast_gb.hpp).
//
//   facade_check cpu   scene creation, error translation, ray shooters and
//                      the status bins (no device needed)
//   facade_check gpu   TraceNonSequential on a world box holding one focal
//                      box: rays over the box focus on its top face, the
//                      others leave the world; rays that are not running on
//                      entry are left untouched
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "robast_gb.hpp"

namespace rg = robast_gb;

static int failures = 0;
#define EXPECT(cond)                                                 \
  do {                                                               \
    if (!(cond)) {                                                   \
      std::fprintf(stderr, "%s:%d: failed: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                    \
    }                                                                \
  } while (0)

struct BoxWorld {
  std::vector<rbg_shape_desc> shapes;
  std::vector<double> matrices, params;
  std::vector<rbg_volume_desc> volumes;
  std::vector<rbg_placement_desc> placements;
  rbg_scene_desc desc{};

  BoxWorld() {
    // world box 100 cm half size; focal box 50 x 50 x 1 cm centred at z = -50
    params = {100, 100, 100, 0, 0, 0, 50, 50, 1, 0, 0, 0};
    shapes.resize(2);
    std::memset(shapes.data(), 0, sizeof(rbg_shape_desc) * 2);
    for (int i = 0; i < 2; ++i) {
      shapes[i].type = RBG_SHAPE_BOX;
      shapes[i].param_offset = 6 * i;
      shapes[i].n_params = 6;
      shapes[i].left = shapes[i].right = shapes[i].left_matrix = shapes[i].right_matrix = -1;
    }
    matrices = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, -50};
    volumes.resize(2);
    for (int i = 0; i < 2; ++i) {
      volumes[i].shape = i;
      volumes[i].kind = i == 0 ? RBG_KIND_OPT : RBG_KIND_FOCUS;
      volumes[i].reflectance = 1.0;
      volumes[i].refl_table = volumes[i].index = -1;
      volumes[i].qe_lambda_table = volumes[i].qe_angle_table = -1;
    }
    placements.push_back(rbg_placement_desc{0, 1, 0, 1, 0});
    desc.n_shapes = 2, desc.shapes = shapes.data();
    desc.n_matrices = 1, desc.matrices = matrices.data();
    desc.n_volumes = 2, desc.volumes = volumes.data();
    desc.n_placements = 1, desc.placements = placements.data();
    desc.top_volume = 0;
    desc.n_params = (int64_t)params.size(), desc.params = params.data();
  }
};

static rg::RayArray line_of_rays(int n) {
  rg::RayArray rays;
  for (int i = 0; i < n; ++i) {
    double x = -90.0 + 180.0 * i / (n - 1);
    rays.Add(400 * rg::units::nm, x, 0.0, 50.0, 0.0, 0.0, 0.0, -2.0);  // direction normalised by the tracer
  }
  return rays;
}

static void check_cpu() {
  BoxWorld w;
  rg::Scene scene(w.desc);
  EXPECT(scene.n_nodes() == 2);

  // a description whose top volume does not exist is refused with a status
  BoxWorld bad;
  bad.desc.top_volume = 7;
  int status = -1;
  try {
    rg::Scene s(bad.desc);
  } catch (const rg::Error& e) {
    status = e.status();
  }
  EXPECT(status != -1 && status != RBG_OK);

  // ARayShooter::RandomCircle: n rays inside the disk, all running, along +z
  rg::RayArray disk = rg::RayShooter::RandomCircle(400 * rg::units::nm, 10.0, 1000, nullptr, nullptr, nullptr, 7);
  EXPECT(disk.size() == 1000);
  bool inside = true;
  for (size_t i = 0; i < disk.size(); ++i)
    inside = inside && std::hypot(disk.x[i], disk.y[i]) <= 10.0 && disk.dz[i] == 1.0;
  EXPECT(inside);
  EXPECT(disk.GetRunning().size() == 1000);
  // the same seed gives the same rays
  rg::RayArray disk2 = rg::RayShooter::RandomCircle(400 * rg::units::nm, 10.0, 1000, nullptr, nullptr, nullptr, 7);
  EXPECT(disk2.x == disk.x && disk2.y == disk.y);
  // ARayShooter::Square: n x n grid
  EXPECT(rg::RayShooter::Square(400 * rg::units::nm, 1.0, 5).size() == 25);

  rg::RayArray rays = line_of_rays(11);
  rays.status[3] = rg::kStop;
  EXPECT(rays.GetStopped().size() == 1 && rays.GetRunning().size() == 10);
  rg::RayArray more = line_of_rays(4);
  rays.Merge(more);
  EXPECT(rays.size() == 15 && rays.GetRunning().size() == 14);

  rg::OpticsManager man(scene);
  EXPECT(man.GetLimit() == 100);
  man.SetLimit(7);
  man.DisableFresnelReflection(true);
  EXPECT(man.GetLimit() == 7 && man.IsFresnelReflectionDisabled());
  man.SetCompaction(32);
  man.SetRayOrder(RBG_ORDER_INPUT);
  man.SetRayOrder(RBG_ORDER_SPATIAL);
}

static void check_gpu() {
  BoxWorld w;
  rg::Scene scene(w.desc);
  rg::OpticsManager man(scene);
  const int n = 101;  // x0 = -90 + 1.8 i: no ray on the box's edges at x = +-50
  rg::RayArray rays = line_of_rays(n);
  // ray 0 is already stopped: the trace must leave it as it is
  rays.status[0] = rg::kStop;
  man.TraceNonSequential(rays);
  EXPECT(rays.status[0] == rg::kStop && rays.x[0] == -90.0 && rays.z[0] == 50.0 && rays.npoints[0] == 1);
  EXPECT(rays.GetRunning().empty());
  size_t focused = 0, exited = 0;
  for (int i = 1; i < n; ++i) {
    double x0 = -90.0 + 180.0 * i / (n - 1);
    if (std::fabs(x0) < 50.0) {
      ++focused;
      EXPECT(rays.status[i] == rg::kFocus);
      EXPECT(std::fabs(rays.z[i] + 49.0) < 1e-6);
      EXPECT(std::fabs(rays.x[i] - x0) < 1e-9);
      EXPECT(std::fabs(rays.dz[i] + 1.0) < 1e-15);
      EXPECT(rays.last_node[i] == 1);
    } else {
      ++exited;
      EXPECT(rays.status[i] == rg::kExit);
    }
  }
  EXPECT(rays.GetFocused().size() == focused && rays.GetExited().size() == exited);
  EXPECT(focused > 0 && exited > 0);
}

int main(int argc, char** argv) {
  const char* mode = argc > 1 ? argv[1] : "cpu";
  try {
    if (std::strcmp(mode, "gpu") == 0)
      check_gpu();
    else
      check_cpu();
  } catch (const rg::Error& e) {
    std::fprintf(stderr, "unexpected error: %s (status %d)\n", e.what(), e.status());
    return 2;
  }
  if (failures) return 1;
  std::printf("facade_check %s: OK\n", mode);
  return 0;
}
