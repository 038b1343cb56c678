/*
 * robast_gb.hpp -- header-only C++ facade over the C ABI (robast_gb.h).
 *
 * Mirrors the reference's host interface for the traced path so that a ROOT
 * macro's tracing section reads the same:
 *   AOpticsManager::SetLimit / DisableFresnelReflection /
 *     TraceNonSequential(ARayArray&)        include/AOpticsManager.h:73-100
 *   ARayArray::Add / GetExited / GetFocused / GetStopped / GetSuspended /
 *     GetAbsorbed / GetRunning              include/ARayArray.h, src/ARayArray.cxx:41-73
 *   ARayShooter::RandomCircle / Circle / RandomCone / RandomRectangle /
 *     RandomSphere / RandomSphericalCone / Rectangle / Square / RandomSquare
 *                                           include/ARayShooter.h:25-51
 * Differences a caller sees: the geometry is a flattened rbg_scene built
 * from an rbg_scene_desc (the TGeo tree as plain arrays) instead of a
 * TGeoManager; the ray array is a structure of arrays and the status bins
 * are index lists into it; errors throw robast_gb::Error carrying the C
 * status code instead of printing through ROOT's Error().
 *
 * Link with librobast_gb.so (built in robast_gb300/_build).
 */
#ifndef ROBAST_GB_HPP
#define ROBAST_GB_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "robast_gb.h"

namespace robast_gb {

class Error : public std::runtime_error {
 public:
  explicit Error(int status)
      : std::runtime_error(std::string("robast_gb: ") + rbg_status_string(status)), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status) {
  if (status != RBG_OK) throw Error(status);
}

// ROBAST length/time units (include/AOpticsManager.h:59-71): cm and s.
namespace units {
constexpr double cm = 1.0, m = 100.0, km = 1e5, mm = 0.1, um = 1e-4, nm = 1e-7;
constexpr double inch = 2.54;
constexpr double s = 1.0, ms = 1e-3, us = 1e-6, ns = 1e-9;
constexpr double rad = 1.0, deg = 3.14159265358979323846 / 180.0;
}  // namespace units

// Ray fates, numbered as ARay's enum (include/ARay.h:26).
enum Status : uint8_t {
  kRun = RBG_RUN,
  kStop = RBG_STOP,
  kExit = RBG_EXIT,
  kFocus = RBG_FOCUS,
  kSuspend = RBG_SUSPEND,
  kAbsorb = RBG_ABSORB
};

// A flattened, immutable scene (the closed geometry).  Move-only owner of
// the rbg_scene handle; the description's arrays are copied at construction.
class Scene {
 public:
  explicit Scene(const rbg_scene_desc& desc) { check(rbg_scene_create(&desc, &s_)); }
  ~Scene() { rbg_scene_destroy(s_); }
  Scene(const Scene&) = delete;
  Scene& operator=(const Scene&) = delete;
  Scene(Scene&& o) noexcept : s_(std::exchange(o.s_, nullptr)) {}
  Scene& operator=(Scene&& o) noexcept {
    if (this != &o) {
      rbg_scene_destroy(s_);
      s_ = std::exchange(o.s_, nullptr);
    }
    return *this;
  }
  rbg_scene* get() const { return s_; }
  rbg_flat_scene flat() const {
    rbg_flat_scene f;
    check(rbg_scene_flat(s_, &f));
    return f;
  }
  int32_t n_nodes() const { return flat().n_nodes; }

 private:
  rbg_scene* s_ = nullptr;
};

// ARayArray as a structure of arrays.  Add() appends a running ray (ARay's
// constructor argument order: lambda, x, y, z, t, dx, dy, dz; the direction
// is normalised by the tracer exactly as ARay::SetDirection does).  After
// TraceNonSequential the position, time and direction arrays hold each
// ray's last point and direction, status() its fate and the Get* bins the
// indices of the rays in each fate.
class RayArray {
 public:
  std::vector<double> x, y, z, t, dx, dy, dz, lambda;
  std::vector<uint8_t> status;
  std::vector<int32_t> npoints, last_node;

  RayArray() = default;
  explicit RayArray(size_t n) { resize(n); }

  size_t size() const { return x.size(); }
  void resize(size_t n) {
    for (auto* v : {&x, &y, &z, &t, &dx, &dy, &dz, &lambda}) v->resize(n, 0.0);
    status.resize(n, kRun);
    npoints.resize(n, 1);
    last_node.resize(n, -2);
  }
  void Add(double lam, double px, double py, double pz, double pt, double ux, double uy, double uz) {
    lambda.push_back(lam);
    x.push_back(px);
    y.push_back(py);
    z.push_back(pz);
    t.push_back(pt);
    dx.push_back(ux);
    dy.push_back(uy);
    dz.push_back(uz);
    status.push_back(kRun);
    npoints.push_back(1);
    last_node.push_back(-2);
  }
  void Merge(const RayArray& o) {
    auto cat = [](auto& a, const auto& b) { a.insert(a.end(), b.begin(), b.end()); };
    cat(x, o.x), cat(y, o.y), cat(z, o.z), cat(t, o.t), cat(dx, o.dx), cat(dy, o.dy), cat(dz, o.dz);
    cat(lambda, o.lambda), cat(status, o.status), cat(npoints, o.npoints), cat(last_node, o.last_node);
  }
  std::vector<int64_t> Bin(Status s) const {
    std::vector<int64_t> idx;
    for (size_t i = 0; i < status.size(); ++i)
      if (status[i] == s) idx.push_back((int64_t)i);
    return idx;
  }
  std::vector<int64_t> GetAbsorbed() const { return Bin(kAbsorb); }
  std::vector<int64_t> GetExited() const { return Bin(kExit); }
  std::vector<int64_t> GetFocused() const { return Bin(kFocus); }
  std::vector<int64_t> GetRunning() const { return Bin(kRun); }
  std::vector<int64_t> GetStopped() const { return Bin(kStop); }
  std::vector<int64_t> GetSuspended() const { return Bin(kSuspend); }

  rbg_rays rays() const {
    rbg_rays r;
    r.n = (int64_t)size();
    r.x = x.data(), r.y = y.data(), r.z = z.data(), r.t = t.data();
    r.dx = dx.data(), r.dy = dy.data(), r.dz = dz.data();
    r.lambda = lambda.data();
    return r;
  }
  rbg_result result() {
    rbg_result o{};
    o.status = status.data();
    o.npoints = npoints.data();
    o.last_node = last_node.data();
    o.x = x.data(), o.y = y.data(), o.z = z.data(), o.t = t.data();
    o.dx = dx.data(), o.dy = dy.data(), o.dz = dz.data();
    return o;
  }
};

// AOpticsManager's tracing controls over a closed Scene.
class OpticsManager {
 public:
  explicit OpticsManager(const Scene& scene) : scene_(&scene) { rbg_trace_opts_default(&opts_); }

  void SetLimit(int n) { opts_.limit = n; }
  int GetLimit() const { return opts_.limit; }
  void DisableFresnelReflection(bool disable) { opts_.disable_fresnel = disable ? 1 : 0; }
  bool IsFresnelReflectionDisabled() const { return opts_.disable_fresnel != 0; }
  // Philox key of every random draw; results depend only on (seed, ray id).
  void SetSeed(uint64_t seed) { opts_.seed = seed; }
  void SetRayIdOffset(uint64_t first_id) { opts_.ray_id_offset = first_id; }
  void SetPrecision(int precision) { opts_.precision = precision; }
  // mixed tracer: refill threshold (0: the scene's tuned value) and the
  // take-up order (RBG_ORDER_SPATIAL / RBG_ORDER_INPUT); neither changes
  // a result
  void SetCompaction(int threshold) { opts_.compaction = threshold; }
  void SetRayOrder(int order) { opts_.ray_order = order; }
  const rbg_trace_opts& options() const { return opts_; }

  // Traces the rays still running in `rays` (host buffers) and updates them
  // in place.  Rays already in a terminal fate are left untouched, as the
  // reference only drains the running bin (src/AOpticsManager.cxx:525-527).
  void TraceNonSequential(RayArray& rays) const {
    std::vector<int64_t> run = rays.GetRunning();
    if (run.empty()) return;
    if (run.size() == rays.size()) {
      rbg_rays in = rays.rays();
      rbg_result out = rays.result();
      check(rbg_trace_host(scene_->get(), &in, &out, &opts_));
      return;
    }
    RayArray sub(run.size());
    for (size_t k = 0; k < run.size(); ++k) copy_ray(rays, run[k], sub, (int64_t)k);
    TraceNonSequential(sub);
    for (size_t k = 0; k < run.size(); ++k) copy_ray(sub, (int64_t)k, rays, run[k]);
  }

 private:
  static void copy_ray(const RayArray& a, int64_t i, RayArray& b, int64_t j) {
    b.x[j] = a.x[i], b.y[j] = a.y[i], b.z[j] = a.z[i], b.t[j] = a.t[i];
    b.dx[j] = a.dx[i], b.dy[j] = a.dy[i], b.dz[j] = a.dz[i], b.lambda[j] = a.lambda[i];
    b.status[j] = a.status[i], b.npoints[j] = a.npoints[i], b.last_node[j] = a.last_node[i];
  }
  const Scene* scene_;
  rbg_trace_opts opts_;
};

// ARayShooter generators.  rot: row-major 3x3 (nullptr = identity), tr: 3
// (nullptr = 0), dir: local direction (nullptr = +z).
class RayShooter {
 public:
  static RayArray Shoot(int kind, const std::vector<double>& params, int64_t n, double lam,
                        const double* rot = nullptr, const double* tr = nullptr, const double* dir = nullptr,
                        uint64_t seed = 0, uint64_t first_id = 0) {
    RayArray a((size_t)n);
    rbg_rays r = a.rays();
    check(rbg_shoot(kind, params.data(), n, rot, tr, dir, seed, first_id, lam, &r));
    a.resize((size_t)r.n);
    return a;
  }
  static RayArray Circle(double lam, double rmax, int nr, int nphi, const double* rot = nullptr,
                         const double* tr = nullptr, const double* dir = nullptr) {
    return Shoot(RBG_SHOOT_CIRCLE, {rmax, (double)nr, (double)nphi}, 1 + (int64_t)(nr - 1) * nphi, lam, rot, tr,
                 dir);
  }
  static RayArray RandomCircle(double lam, double rmax, int64_t n, const double* rot = nullptr,
                               const double* tr = nullptr, const double* dir = nullptr, uint64_t seed = 0,
                               uint64_t first_id = 0) {
    return Shoot(RBG_SHOOT_RANDOM_CIRCLE, {rmax}, n, lam, rot, tr, dir, seed, first_id);
  }
  static RayArray RandomCone(double lam, double r, double d, int64_t n, const double* rot = nullptr,
                             const double* tr = nullptr, uint64_t seed = 0, uint64_t first_id = 0) {
    return Shoot(RBG_SHOOT_RANDOM_CONE, {r, d}, n, lam, rot, tr, nullptr, seed, first_id);
  }
  static RayArray RandomRectangle(double lam, double dx, double dy, int64_t n, const double* rot = nullptr,
                                  const double* tr = nullptr, const double* dir = nullptr, uint64_t seed = 0,
                                  uint64_t first_id = 0) {
    return Shoot(RBG_SHOOT_RANDOM_RECTANGLE, {dx, dy}, n, lam, rot, tr, dir, seed, first_id);
  }
  static RayArray RandomSquare(double lam, double d, int64_t n, const double* rot = nullptr,
                               const double* tr = nullptr, const double* dir = nullptr, uint64_t seed = 0,
                               uint64_t first_id = 0) {
    return RandomRectangle(lam, d, d, n, rot, tr, dir, seed, first_id);
  }
  static RayArray RandomSphere(double lam, int64_t n, const double* tr = nullptr, uint64_t seed = 0,
                               uint64_t first_id = 0) {
    return Shoot(RBG_SHOOT_RANDOM_SPHERE, {}, n, lam, nullptr, tr, nullptr, seed, first_id);
  }
  static RayArray RandomSphericalCone(double lam, int64_t n, double theta_deg, const double* rot = nullptr,
                                      const double* tr = nullptr, uint64_t seed = 0, uint64_t first_id = 0) {
    return Shoot(RBG_SHOOT_RANDOM_SPHERICAL_CONE, {theta_deg}, n, lam, rot, tr, nullptr, seed, first_id);
  }
  static RayArray Rectangle(double lam, double dx, double dy, int nx, int ny, const double* rot = nullptr,
                            const double* tr = nullptr, const double* dir = nullptr) {
    return Shoot(RBG_SHOOT_RECTANGLE, {dx, dy, (double)nx, (double)ny}, (int64_t)nx * ny, lam, rot, tr, dir);
  }
  static RayArray Square(double lam, double d, int n, const double* rot = nullptr, const double* tr = nullptr,
                         const double* dir = nullptr) {
    return Rectangle(lam, d, d, n, n, rot, tr, dir);
  }
};

}  // namespace robast_gb

#endif  // ROBAST_GB_HPP
