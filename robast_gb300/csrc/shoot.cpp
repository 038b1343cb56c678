// shoot.cpp -- ARayShooter generators (src/ARayShooter.cxx:122-459) on the
// host.  The reference draws from the global gRandom; here ray i draws from
// the Philox stream (seed, first_id + i, stream 1), so a batch can be
// generated in any order or in shards and still be reproducible.
#include <cmath>
#include <cstring>

#include "philox.h"
#include "robast_gb.h"

namespace {

struct Frame {
  double R[9];
  double t[3];
  double dir[3];
  bool has_rot;
};

void rot_apply(const Frame& f, const double* v, double* o) {
  if (!f.has_rot) {
    std::memcpy(o, v, 3 * sizeof(double));
    return;
  }
  for (int i = 0; i < 3; ++i) o[i] = f.R[i * 3] * v[0] + f.R[i * 3 + 1] * v[1] + f.R[i * 3 + 2] * v[2];
}

struct Writer {
  rbg_rays* out;
  int64_t cap, n = 0;
  double lambda;
  bool put(const double* x, const double* d) {
    if (n >= cap) return false;
    const_cast<double*>(out->x)[n] = x[0];
    const_cast<double*>(out->y)[n] = x[1];
    const_cast<double*>(out->z)[n] = x[2];
    if (out->t) const_cast<double*>(out->t)[n] = 0.0;
    const_cast<double*>(out->dx)[n] = d[0];
    const_cast<double*>(out->dy)[n] = d[1];
    const_cast<double*>(out->dz)[n] = d[2];
    const_cast<double*>(out->lambda)[n] = lambda;
    ++n;
    return true;
  }
};

// position: rotation then translation (LocalToMaster of rot, then of tr)
void place(const Frame& f, const double* local, double* master) {
  double tmp[3];
  rot_apply(f, local, tmp);
  for (int k = 0; k < 3; ++k) master[k] = tmp[k] + f.t[k];
}

}  // namespace

extern "C" int rbg_shoot(int32_t kind, const double* p, int64_t n, const double* rot, const double* tr,
                         const double* dir, uint64_t seed, uint64_t first_id, double lambda,
                         rbg_rays* out) {
  if (!out || !out->x || !out->y || !out->z || !out->dx || !out->dy || !out->dz || !out->lambda)
    return RBG_ERR_ARG;
  if (n < 0 || out->n < 0) return RBG_ERR_ARG;
  Frame f;
  f.has_rot = rot != nullptr;
  if (rot) std::memcpy(f.R, rot, sizeof(f.R));
  for (int k = 0; k < 3; ++k) f.t[k] = tr ? tr[k] : 0.0;
  f.dir[0] = dir ? dir[0] : 0.0;
  f.dir[1] = dir ? dir[1] : 0.0;
  f.dir[2] = dir ? dir[2] : 1.0;
  double new_dir[3];
  rot_apply(f, f.dir, new_dir);
  Writer w{out, out->n, 0, lambda};
  const double kTwoPi = 2.0 * M_PI;

  switch (kind) {
    case RBG_SHOOT_CIRCLE: {  // src/ARayShooter.cxx:122-183
      if (!p) return RBG_ERR_ARG;
      double rmax = p[0];
      int nr = (int)p[1], nphi = (int)p[2];
      if (0 > rmax || nr < 1 || nphi < 1) break;
      double c[3] = {0, 0, 0}, x[3];
      for (int k = 0; k < 3; ++k) x[k] = c[k] + f.t[k];
      if (!w.put(x, new_dir)) return RBG_ERR_ARG;
      for (int i = 0; i < nr; i++) {
        double r = rmax * (i + 1) / nr;
        for (int j = 0; j < nphi * (i + 1); j++) {
          double phi = 2 * M_PI / nphi / (i + 1) * j;
          double l[3] = {r * std::cos(phi), r * std::sin(phi), 0};
          place(f, l, x);
          if (!w.put(x, new_dir)) return RBG_ERR_ARG;
        }
      }
      break;
    }
    case RBG_SHOOT_RANDOM_CIRCLE: {  // :186-237
      if (!p) return RBG_ERR_ARG;
      double rmax = p[0];
      if (0 > rmax) break;
      for (int64_t i = 0; i < n; ++i) {
        rbg::RayRng g;
        g.init(seed, first_id + (uint64_t)i, 1);
        double rx = 0, ry = 0;
        for (int tries = 0; tries < 1000; ++tries) {
          rbg::Philox4 b = g.next();
          rx = -rmax + 2 * rmax * rbg::u53(b.v[0], b.v[1]);
          ry = -rmax + 2 * rmax * rbg::u53(b.v[2], b.v[3]);
          if (std::sqrt(rx * rx + ry * ry) <= rmax) break;
        }
        double l[3] = {rx, ry, 0}, x[3];
        place(f, l, x);
        if (!w.put(x, new_dir)) return RBG_ERR_ARG;
      }
      break;
    }
    case RBG_SHOOT_RANDOM_CONE: {  // :240-287
      if (!p) return RBG_ERR_ARG;
      double r = p[0], d = p[1];
      for (int64_t i = 0; i < n; ++i) {
        rbg::RayRng g;
        g.init(seed, first_id + (uint64_t)i, 1);
        double x = 0, y = 0;
        for (int tries = 0; tries < 1000; ++tries) {
          rbg::Philox4 b = g.next();
          x = -r + 2 * r * rbg::u53(b.v[0], b.v[1]);
          y = -r + 2 * r * rbg::u53(b.v[2], b.v[3]);
          if (!(x * x + y * y > r * r)) break;
        }
        double goal[3] = {x, y, d}, tmp[3];
        rot_apply(f, goal, tmp);
        double start[3] = {f.t[0], f.t[1], f.t[2]};
        for (int k = 0; k < 3; ++k) goal[k] = tmp[k] + f.t[k];
        double dd[3] = {goal[0] - start[0], goal[1] - start[1], goal[2] - start[2]};
        if (!w.put(start, dd)) return RBG_ERR_ARG;
      }
      break;
    }
    case RBG_SHOOT_RANDOM_RECTANGLE: {  // :290-330
      if (!p) return RBG_ERR_ARG;
      double dx = p[0], dy = p[1];
      if (dx < 0 || dy < 0 || n < 1) break;
      for (int64_t i = 0; i < n; ++i) {
        rbg::RayRng g;
        g.init(seed, first_id + (uint64_t)i, 1);
        rbg::Philox4 b = g.next();
        double l[3] = {-dx / 2. + dx * rbg::u53(b.v[0], b.v[1]), -dy / 2. + dy * rbg::u53(b.v[2], b.v[3]), 0};
        double x[3];
        place(f, l, x);
        if (!w.put(x, new_dir)) return RBG_ERR_ARG;
      }
      break;
    }
    case RBG_SHOOT_RANDOM_SPHERE: {  // :333-351 (uniform directions)
      for (int64_t i = 0; i < n; ++i) {
        rbg::RayRng g;
        g.init(seed, first_id + (uint64_t)i, 1);
        rbg::Philox4 b = g.next();
        double z = -1 + 2 * rbg::u53(b.v[0], b.v[1]);
        double phi = kTwoPi * rbg::u53(b.v[2], b.v[3]);
        double s = std::sqrt(1 - z * z);
        double d[3] = {s * std::cos(phi), s * std::sin(phi), z};
        double x[3] = {f.t[0], f.t[1], f.t[2]};
        if (!w.put(x, d)) return RBG_ERR_ARG;
      }
      break;
    }
    case RBG_SHOOT_RANDOM_SPHERICAL_CONE: {  // :354-384
      if (!p) return RBG_ERR_ARG;
      double theta = p[0];
      for (int64_t i = 0; i < n; ++i) {
        rbg::RayRng g;
        g.init(seed, first_id + (uint64_t)i, 1);
        rbg::Philox4 b = g.next();
        double c0 = std::cos(theta * M_PI / 180.0);
        double ran = c0 + (1 - c0) * rbg::u53(b.v[0], b.v[1]);
        double th = std::acos(ran);
        double phi = kTwoPi * rbg::u53(b.v[2], b.v[3]);
        double l[3] = {std::sin(th) * std::cos(phi), std::sin(th) * std::sin(phi), std::cos(th)};
        double d[3];
        rot_apply(f, l, d);
        double x[3] = {f.t[0], f.t[1], f.t[2]};
        if (!w.put(x, d)) return RBG_ERR_ARG;
      }
      break;
    }
    case RBG_SHOOT_RECTANGLE: {  // :394-453
      if (!p) return RBG_ERR_ARG;
      double dx = p[0], dy = p[1];
      int nx = (int)p[2], ny = (int)p[3];
      if (dx < 0 || dy < 0 || nx < 1 || ny < 1) break;
      double deltax = nx == 1 ? dx / 2 : dx / (nx - 1);
      double deltay = ny == 1 ? dy / 2 : dy / (ny - 1);
      for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
          double l[3] = {i * deltax - dx / 2, j * deltay - dy / 2, 0}, x[3];
          place(f, l, x);
          if (!w.put(x, new_dir)) return RBG_ERR_ARG;
        }
      break;
    }
    default:
      return RBG_ERR_ARG;
  }
  out->n = w.n;
  return RBG_OK;
}
