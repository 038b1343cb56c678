// scene.cpp -- flattening of a TGeo-style volume description into the
// physical node table, bounding boxes and per-mother BVHs that the GPU
// kernels (and any CPU checker) navigate.
//
// Replaces TGeoManager::CloseGeometry() + ROOT's voxelisation for the
// scenes ROBAST builds (e.g. tutorials/SimpleParabolicTelescope.C:22-83,
// tutorials/DaviesCotton.C:30-160, tutorials/SchwarzschildCouder.C:19-81).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include "trace_features.h"
#include "scene_internal.h"

namespace {

constexpr double kBig = RBG_BIG;
constexpr int kMaxNodes = 1 << 24;
constexpr int kMaxDepth = 64;
constexpr int kBvhLeaf = 4;
// SAH splits only while the tree stays shallower than this (the device
// traverses with a 32-entry stack)
constexpr int kBvhSahDepth = 28;
constexpr int kBvhMinChildren = 9;
constexpr int kMaxCompositeDepth = RBG_MAX_COMPOSITE_DEPTH;

struct Box {
  double lo[3], hi[3];
};

void mat_identity(double* m) {
  std::memset(m, 0, 12 * sizeof(double));
  m[0] = m[4] = m[8] = 1.0;
}

// c = a * b  (apply b first, then a): master = Ra (Rb x + tb) + ta
void mat_mul(const double* a, const double* b, double* c) {
  double r[12];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      r[i * 3 + j] = a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j] +
                     a[i * 3 + 2] * b[2 * 3 + j];
    r[9 + i] = a[i * 3 + 0] * b[9] + a[i * 3 + 1] * b[10] + a[i * 3 + 2] * b[11] + a[9 + i];
  }
  std::memcpy(c, r, sizeof(r));
}

Box box_transform(const Box& b, const double* m) {
  Box o;
  double c[3], h[3];
  for (int k = 0; k < 3; ++k) {
    c[k] = 0.5 * (b.lo[k] + b.hi[k]);
    h[k] = 0.5 * (b.hi[k] - b.lo[k]);
  }
  for (int i = 0; i < 3; ++i) {
    double ci = m[9 + i], hi = 0;
    for (int j = 0; j < 3; ++j) {
      ci += m[i * 3 + j] * c[j];
      hi += std::fabs(m[i * 3 + j]) * h[j];
    }
    o.lo[i] = ci - hi;
    o.hi[i] = ci + hi;
  }
  return o;
}

Box box_pad(Box b) {
  for (int k = 0; k < 3; ++k) {
    double e = (b.hi[k] - b.lo[k]) * 1e-6 + 1e-6;
    b.lo[k] -= e;
    b.hi[k] += e;
  }
  return b;
}

// --- AGeoAsphericDisk sag, restated from src/AGeoAsphericDisk.cxx:126-153
// (returns false where the reference throws) -----------------------------
bool asph_sag(double r, double z0, double c, double kappa, int npol, const double* k,
              double* f) {
  double p = r * r * c * c * kappa;
  if (1 - p < 0) return false;
  double ret = z0 + r * r * c / (1 + std::sqrt(1 - p));
  for (int i = 0; i < npol; ++i) ret += k[i] * std::pow(r, 2 * (i + 1));
  *f = ret;
  return true;
}

// AGeoAsphericDisk::ComputeBBox grid search (src/AGeoAsphericDisk.cxx:164-243)
void asph_bbox(const double* p, double* origin_z, double* dz, int steps, int repeat) {
  const double z1 = p[RBG_ASPH_Z1], z2 = p[RBG_ASPH_Z2];
  const double c1 = p[RBG_ASPH_C1], c2 = p[RBG_ASPH_C2];
  const double ka1 = p[RBG_ASPH_KAPPA1], ka2 = p[RBG_ASPH_KAPPA2];
  const double rmin = p[RBG_ASPH_RMIN], rmax = p[RBG_ASPH_RMAX];
  const int n1 = (int)p[RBG_ASPH_NPOL1], n2 = (int)p[RBG_ASPH_NPOL2];
  const double* k1 = p + RBG_ASPH_K;
  const double* k2 = p + RBG_ASPH_K + n1;

  double zmax = -kBig;
  if (n2 == 0) {
    double f1, f2;
    if (!asph_sag(rmin, z2, c2, ka2, n2, k2, &f1) || !asph_sag(rmax, z2, c2, ka2, n2, k2, &f2)) {
      f1 = kBig;
      f2 = kBig;
    }
    zmax = f1 > f2 ? f1 : f2;
  } else {
    double r1 = rmin, r2 = rmax;
    for (int i = 0; i < repeat; ++i) {
      double step = (r2 - r1) / steps;
      double r_ = r1;
      for (int j = 0; j <= steps + 1; ++j) {
        double r = r1 + j * step, f;
        if (!asph_sag(r, z2, c2, ka2, n2, k2, &f)) f = -kBig;
        if (f > zmax) {
          zmax = f;
          r_ = r;
        }
      }
      r1 = r_ == rmin ? rmin : r_ - step;
      r2 = r_ == rmax ? rmax : r_ + step;
    }
  }
  double zmin = kBig;
  if (n1 == 0) {
    double f1, f2;
    if (!asph_sag(rmin, z1, c1, ka1, n1, k1, &f1) || !asph_sag(rmax, z1, c1, ka1, n1, k1, &f2)) {
      f1 = -kBig;
      f2 = -kBig;
    }
    zmin = f1 < f2 ? f1 : f2;
  } else {
    double r1 = rmin, r2 = rmax;
    for (int i = 0; i < repeat; ++i) {
      double step = (r2 - r1) / steps;
      double r_ = r1;
      for (int j = 0; j <= steps + 1; ++j) {
        double r = r1 + j * step, f;
        if (!asph_sag(r, z1, c1, ka1, n1, k1, &f)) f = kBig;
        if (f < zmin) {
          zmin = f;
          r_ = r;
        }
      }
      r1 = r_ == rmin ? rmin : r_ - step;
      r2 = r_ == rmax ? rmax : r_ + step;
    }
  }
  *origin_z = (zmax + zmin) / 2;
  *dz = (zmax - zmin) / 2;
}

struct Builder {
  const rbg_scene_desc* d;
  rbg_scene* s;
  std::vector<int> shape_state;  // 0 = todo, 1 = in progress, 2 = done
  std::vector<int> composite_depth;

  int fail(int code) { return code; }

  bool matrix_ok(int id) const { return id >= -1 && id < d->n_matrices; }
  void get_matrix(int id, double* m) const {
    if (id < 0) mat_identity(m);
    else std::memcpy(m, d->matrices + 12 * (size_t)id, 12 * sizeof(double));
  }

  // Canonicalise one shape (recursing into composite operands).
  int canon_shape(int id) {
    if (id < 0 || id >= d->n_shapes) return RBG_ERR_SCENE;
    if (shape_state[id] == 2) return RBG_OK;
    if (shape_state[id] == 1) return RBG_ERR_SCENE;  // cycle
    shape_state[id] = 1;
    const rbg_shape_desc& u = d->shapes[id];
    if (u.param_offset < 0 || u.n_params < 0 || (int64_t)u.param_offset + u.n_params > d->n_params)
      return RBG_ERR_SCENE;
    const double* p = d->params + u.param_offset;
    rbg_shape_desc c = u;
    c.param_offset = (int32_t)s->params.size();
    std::vector<double> q;
    Box b;
    switch (u.type) {
      case RBG_SHAPE_BOX: {
        if (u.n_params < 3) return RBG_ERR_SCENE;
        q.assign(RBG_BOX_NP, 0.0);
        for (int k = 0; k < 3; ++k) q[k] = std::fabs(p[k]);
        for (int k = 3; k < 6 && k < u.n_params; ++k) q[k] = p[k];
        for (int k = 0; k < 3; ++k) {
          b.lo[k] = q[3 + k] - q[k];
          b.hi[k] = q[3 + k] + q[k];
        }
        break;
      }
      case RBG_SHAPE_TUBE: {
        if (u.n_params < 3) return RBG_ERR_SCENE;
        double rmin = p[0], rmax = p[1], dz = std::fabs(p[2]);
        double phi1 = u.n_params >= 5 ? p[3] : 0.0, phi2 = u.n_params >= 5 ? p[4] : 360.0;
        if (rmin < 0 || rmax <= rmin) return RBG_ERR_SCENE;
        double dphi = phi2 - phi1;
        if (!std::isfinite(dphi)) return RBG_ERR_SCENE;
        while (dphi <= 0) dphi += 360.0;
        q = {rmin, rmax, dz, phi1, dphi >= 360.0 ? 360.0 : dphi};
        b = {{-rmax, -rmax, -dz}, {rmax, rmax, dz}};
        break;
      }
      case RBG_SHAPE_SPHERE: {
        if (u.n_params < 2) return RBG_ERR_SCENE;
        double rmin = p[0], rmax = p[1];
        double th1 = u.n_params >= 4 ? p[2] : 0.0, th2 = u.n_params >= 4 ? p[3] : 180.0;
        double ph1 = u.n_params >= 6 ? p[4] : 0.0, ph2 = u.n_params >= 6 ? p[5] : 360.0;
        if (rmin < 0 || rmax <= rmin || th1 < 0 || th2 > 180 || th2 <= th1) return RBG_ERR_SCENE;
        double dphi = ph2 - ph1;
        if (!std::isfinite(dphi)) return RBG_ERR_SCENE;
        while (dphi <= 0) dphi += 360.0;
        q = {rmin, rmax, th1, th2, ph1, dphi >= 360.0 ? 360.0 : dphi};
        const double d2r = M_PI / 180.0;
        double ct1 = std::cos(th1 * d2r), ct2 = std::cos(th2 * d2r);
        double zhi = ct1 >= 0 ? rmax * ct1 : rmin * ct1;
        double zlo = ct2 <= 0 ? rmax * ct2 : rmin * ct2;
        double smax = (th1 <= 90.0 && th2 >= 90.0) ? 1.0
                                                   : std::max(std::sin(th1 * d2r), std::sin(th2 * d2r));
        double rho = rmax * smax;
        b = {{-rho, -rho, zlo}, {rho, rho, zhi}};
        break;
      }
      case RBG_SHAPE_PARABOLOID: {
        if (u.n_params < 3) return RBG_ERR_SCENE;
        double rlo = std::fabs(p[0]), rhi = std::fabs(p[1]), dz = std::fabs(p[2]);
        if (rlo == rhi || dz <= 0) return RBG_ERR_SCENE;
        double a = 2 * dz / (rhi * rhi - rlo * rlo);
        double bb = -dz - a * rlo * rlo;
        q = {rlo, rhi, dz, a, bb};
        double r = std::max(rlo, rhi);
        b = {{-r, -r, -dz}, {r, r, dz}};
        break;
      }
      case RBG_SHAPE_PGON:
      case RBG_SHAPE_PCON: {
        bool pg = u.type == RBG_SHAPE_PGON;
        int head = pg ? 4 : 3;
        if (u.n_params < head) return RBG_ERR_SCENE;
        int nz = (int)p[pg ? 3 : 2];
        int nedges = pg ? (int)p[2] : 0;
        if (nz < 2 || u.n_params < head + 3 * nz || (pg && nedges < 3)) return RBG_ERR_SCENE;
        q.assign(p, p + head + 3 * nz);
        double dphi = q[1];
        if (dphi <= 0 || dphi > 360.0) dphi = 360.0;
        q[1] = dphi;
        double rmax = 0, zlo = kBig, zhi = -kBig;
        for (int i = 0; i < nz; ++i) {
          double z = q[head + i], r0 = q[head + nz + i], r1 = q[head + 2 * nz + i];
          if (i > 0 && z < q[head + i - 1]) return RBG_ERR_SCENE;
          if (r0 < 0 || r1 < r0) return RBG_ERR_SCENE;
          rmax = std::max(rmax, r1);
          zlo = std::min(zlo, z);
          zhi = std::max(zhi, z);
        }
        if (pg) rmax /= std::cos(M_PI * (dphi / 360.0) / nedges);
        b = {{-rmax, -rmax, zlo}, {rmax, rmax, zhi}};
        break;
      }
      case RBG_SHAPE_ASPHERIC_DISK: {
        if (u.n_params < 12) return RBG_ERR_SCENE;
        double z1 = p[0], cu1 = p[1], z2 = p[2], cu2 = p[3], rmax = p[4], rmin = p[5];
        double conic1 = p[6], conic2 = p[7];
        int n1 = (int)p[8], n2 = (int)p[9];
        int steps = (int)p[10], repeat = (int)p[11];
        if (n1 < 0 || n2 < 0 || n1 > RBG_ASPH_MAXPOL || n2 > RBG_ASPH_MAXPOL ||
            u.n_params < 12 + n1 + n2)
          return RBG_ERR_SCENE;
        if (steps <= 0) steps = 100;
        if (repeat <= 0) repeat = 4;
        q.assign(RBG_ASPH_K + n1 + n2, 0.0);
        // SetAsphDimensions (src/AGeoAsphericDisk.cxx:971-1005)
        if (z1 < z2) {
          q[RBG_ASPH_Z1] = z1; q[RBG_ASPH_Z2] = z2; q[RBG_ASPH_C1] = cu1; q[RBG_ASPH_C2] = cu2;
        } else {
          q[RBG_ASPH_Z1] = z2; q[RBG_ASPH_Z2] = z1; q[RBG_ASPH_C1] = cu2; q[RBG_ASPH_C2] = cu1;
        }
        if (rmax < 0) rmax = -rmax;
        if (rmin < 0) rmin = -rmin;
        if (rmax > rmin) {
          q[RBG_ASPH_RMAX] = rmax; q[RBG_ASPH_RMIN] = rmin;
        } else {
          q[RBG_ASPH_RMAX] = rmin; q[RBG_ASPH_RMIN] = rmax;
        }
        q[RBG_ASPH_RSEG] = q[RBG_ASPH_RMIN] > 0 ? 1.0 : 0.0;
        // SetConicConstants (src/AGeoAsphericDisk.cxx:1007-1013)
        q[RBG_ASPH_KAPPA1] = conic1 + 1;
        q[RBG_ASPH_KAPPA2] = conic2 + 1;
        // SetPolynomials (src/AGeoAsphericDisk.cxx:1187-1204)
        q[RBG_ASPH_NPOL1] = n1;
        q[RBG_ASPH_NPOL2] = n2;
        for (int i = 0; i < n1 + n2; ++i) q[RBG_ASPH_K + i] = p[12 + i];
        double oz, dz;
        asph_bbox(q.data(), &oz, &dz, steps, repeat);
        q[RBG_ASPH_ORIGIN_Z] = oz;
        q[RBG_ASPH_DZ] = dz;
        {
          const double* k1 = q.data() + RBG_ASPH_K;
          const double* k2 = k1 + n1;
          const double nan = std::numeric_limits<double>::quiet_NaN();
          double f;
          const double rr[2] = {q[RBG_ASPH_RMIN], q[RBG_ASPH_RMAX]};
          for (int w = 0; w < 2; ++w) {
            q[RBG_ASPH_F1RMIN + 2 * w] =
                asph_sag(rr[w], q[RBG_ASPH_Z1], q[RBG_ASPH_C1], q[RBG_ASPH_KAPPA1], n1, k1, &f) ? f : nan;
            q[RBG_ASPH_F2RMIN + 2 * w] =
                asph_sag(rr[w], q[RBG_ASPH_Z2], q[RBG_ASPH_C2], q[RBG_ASPH_KAPPA2], n2, k2, &f) ? f : nan;
          }
        }
        double r = q[RBG_ASPH_RMAX];
        // conservative box for culling only: the sampled extremum can miss
        // the true one by a grid step, so pad generously
        double pad = 1e-3 * std::max(dz, 1.0) + 1e-4;
        b = {{-r, -r, oz - dz - pad}, {r, r, oz + dz + pad}};
        break;
      }
      case RBG_SHAPE_WINSTON_POLY: {
        if (u.n_params < 3) return RBG_ERR_SCENE;
        double r1 = p[0], r2 = p[1];
        int n = (int)p[2];
        if (r1 == r2 || r1 == 0 || r2 == 0 || n <= 0) return RBG_ERR_SCENE;
        // SetWinstonDimensions (src/AGeoWinstonConePoly.cxx:356-386)
        double R1, R2;
        if (std::fabs(r1) > std::fabs(r2)) {
          R1 = std::fabs(r1); R2 = std::fabs(r2);
        } else {
          R1 = std::fabs(r2); R2 = std::fabs(r1);
        }
        int N = n >= 3 ? n : 3;
        double rr = r1 / std::cos(M_PI / n);
        double dx = 0, dy = 0;
        for (int i = 0; i < N; ++i) dx = std::max(std::fabs(rr * std::cos(M_PI / n * (2 * i + 1))), dx);
        for (int i = 0; i < N; ++i) dy = std::max(std::fabs(rr * std::sin(M_PI / n * (2 * i + 1))), dy);
        double theta = std::asin(R2 / R1);
        double dz = (R1 + R2) / std::tan(theta) / 2.;
        double f = R2 * (1 + std::sin(theta));
        q = {R1, R2, (double)N, theta, f, dz, dx, dy};
        double rc = R1 / std::cos(M_PI / N);
        b = {{-rc, -rc, -dz}, {rc, rc, dz}};
        break;
      }
      case RBG_SHAPE_WINSTON_2D: {
        if (u.n_params < 3) return RBG_ERR_SCENE;
        const double r1 = p[0], r2 = p[1], y = std::fabs(p[2]);
        if (r1 == r2 || r1 == 0 || r2 == 0) return RBG_ERR_SCENE;
        // AGeoWinstonCone2D::SetWinstonDimensions (src/AGeoWinstonCone2D.cxx:551-567)
        const double R1 = std::max(std::fabs(r1), std::fabs(r2)), R2 = std::min(std::fabs(r1), std::fabs(r2));
        const double theta = std::asin(R2 / R1);
        const double dz = (R1 + R2) / std::tan(theta) / 2.;
        const double f = R2 * (1 + std::sin(theta));
        q = {R1, R2, 2.0, theta, f, dz, R1, y};
        b = {{-R1, -y, -dz}, {R1, y, dz}};  // ComputeBBox (:109-117)
        break;
      }
      case RBG_SHAPE_COMPOSITE: {
        if (u.op < RBG_OP_UNION || u.op > RBG_OP_SUBTRACTION) return RBG_ERR_SCENE;
        if (!matrix_ok(u.left_matrix) || !matrix_ok(u.right_matrix)) return RBG_ERR_SCENE;
        int rc;
        if ((rc = canon_shape(u.left)) != RBG_OK) return rc;
        if ((rc = canon_shape(u.right)) != RBG_OK) return rc;
        // the device walks composite trees with fixed-size stacks: bound their depth
        int depth = 1 + std::max(composite_depth[u.left], composite_depth[u.right]);
        if (depth > kMaxCompositeDepth) return RBG_ERR_UNSUPPORTED;
        composite_depth[id] = depth;
        for (int opnd : {u.left, u.right}) {
          int t = d->shapes[opnd].type;
          if (t == RBG_SHAPE_ASPHERIC_DISK || t == RBG_SHAPE_WINSTON_POLY || t == RBG_SHAPE_WINSTON_2D)
            return RBG_ERR_UNSUPPORTED;
        }
        q.assign(RBG_COMP_NP, 0.0);
        get_matrix(u.left_matrix, q.data() + RBG_COMP_ML);
        get_matrix(u.right_matrix, q.data() + RBG_COMP_MR);
        Box bl, br;
        std::memcpy(bl.lo, &s->shape_box[6 * u.left], 3 * sizeof(double));
        std::memcpy(bl.hi, &s->shape_box[6 * u.left + 3], 3 * sizeof(double));
        std::memcpy(br.lo, &s->shape_box[6 * u.right], 3 * sizeof(double));
        std::memcpy(br.hi, &s->shape_box[6 * u.right + 3], 3 * sizeof(double));
        bl = box_transform(bl, q.data() + RBG_COMP_ML);
        br = box_transform(br, q.data() + RBG_COMP_MR);
        for (int k = 0; k < 3; ++k) {
          if (u.op == RBG_OP_UNION) {
            b.lo[k] = std::min(bl.lo[k], br.lo[k]);
            b.hi[k] = std::max(bl.hi[k], br.hi[k]);
          } else if (u.op == RBG_OP_INTERSECTION) {
            b.lo[k] = std::max(bl.lo[k], br.lo[k]);
            b.hi[k] = std::min(bl.hi[k], br.hi[k]);
            if (b.hi[k] < b.lo[k]) b.hi[k] = b.lo[k];
          } else {
            b.lo[k] = bl.lo[k];
            b.hi[k] = bl.hi[k];
          }
        }
        break;
      }
      default:
        return RBG_ERR_SCENE;
    }
    c.n_params = (int32_t)q.size();
    c.param_offset = (int32_t)s->params.size();
    s->params.insert(s->params.end(), q.begin(), q.end());
    s->shapes[id] = c;
    std::memcpy(&s->shape_box[6 * id], b.lo, 3 * sizeof(double));
    std::memcpy(&s->shape_box[6 * id + 3], b.hi, 3 * sizeof(double));
    shape_state[id] = 2;
    return RBG_OK;
  }

  int copy_tables() {
    s->tables.assign(d->tables, d->tables + d->n_tables);
    for (auto& t : s->tables) {
      if (t.kind != RBG_TABLE_1D && t.kind != RBG_TABLE_2D) return RBG_ERR_SCENE;
      int64_t need = t.kind == RBG_TABLE_1D ? 2LL * t.nx : (int64_t)t.nx + t.ny + (int64_t)t.nx * t.ny;
      if (t.nx < 1 || (t.kind == RBG_TABLE_2D && t.ny < 1) || t.param_offset < 0 ||
          t.param_offset + need > d->n_params)
        return RBG_ERR_SCENE;
      const double* src = d->params + t.param_offset;
      rbg_table_desc c = t;
      c.param_offset = (int32_t)s->params.size();
      if (t.kind == RBG_TABLE_1D) {
        // TGraph points sorted by x (stable), as TGraph::Eval's neighbour
        // search assumes
        std::vector<int> order(t.nx);
        for (int i = 0; i < t.nx; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return src[a] < src[b]; });
        for (int i = 0; i < t.nx; ++i) s->params.push_back(src[order[i]]);
        for (int i = 0; i < t.nx; ++i) s->params.push_back(src[t.nx + order[i]]);
      } else {
        for (int64_t i = 0; i < need; ++i) s->params.push_back(src[i]);
        for (int i = 1; i < t.nx; ++i)
          if (src[i] <= src[i - 1]) return RBG_ERR_SCENE;
        for (int i = 1; i < t.ny; ++i)
          if (src[t.nx + i] <= src[t.nx + i - 1]) return RBG_ERR_SCENE;
      }
      t = c;
    }
    return RBG_OK;
  }

  int build_tree() {
    // node 0 = top volume
    rbg_node top{};
    top.parent = -1;
    top.volume = d->top_volume;
    top.depth = 0;
    mat_identity(top.m);
    s->nodes.push_back(top);
    // placements grouped by mother, in insertion order
    std::vector<std::vector<int>> by_mother(d->n_volumes);
    for (int i = 0; i < d->n_placements; ++i) {
      const rbg_placement_desc& pl = d->placements[i];
      if (pl.mother < 0 || pl.mother >= d->n_volumes || pl.daughter < 0 ||
          pl.daughter >= d->n_volumes || !matrix_ok(pl.matrix))
        return RBG_ERR_SCENE;
      by_mother[pl.mother].push_back(i);
    }
    // breadth-first expansion: the children of a node get consecutive ids
    for (size_t cur = 0; cur < s->nodes.size(); ++cur) {
      rbg_node n = s->nodes[cur];
      const auto& pls = by_mother[n.volume];
      int first = (int)s->nodes.size();
      if (!pls.empty() && n.depth + 1 >= kMaxDepth) return RBG_ERR_SCENE;
      if (s->nodes.size() + pls.size() > (size_t)kMaxNodes) return RBG_ERR_SCENE;
      for (int pi : pls) {
        const rbg_placement_desc& pl = d->placements[pi];
        rbg_node c{};
        c.parent = (int32_t)cur;
        c.volume = pl.daughter;
        c.depth = n.depth + 1;
        double m[12];
        get_matrix(pl.matrix, m);
        mat_mul(n.m, m, c.m);
        s->nodes.push_back(c);
      }
      s->nodes[cur].child_begin = (int32_t)s->children.size();
      s->nodes[cur].child_count = (int32_t)pls.size();
      for (size_t k = 0; k < pls.size(); ++k) s->children.push_back(first + (int)k);
    }
    for (auto& n : s->nodes) {
      const rbg_volume_desc& v = s->volumes[n.volume];
      n.shape = v.shape;
      n.kind = v.kind;
      n.bvh_root = -1;
      Box b;
      std::memcpy(b.lo, &s->shape_box[6 * v.shape], 3 * sizeof(double));
      std::memcpy(b.hi, &s->shape_box[6 * v.shape + 3], 3 * sizeof(double));
      b = box_pad(box_transform(b, n.m));
      std::memcpy(n.lo, b.lo, sizeof(b.lo));
      std::memcpy(n.hi, b.hi, sizeof(b.hi));
    }
    return RBG_OK;
  }

  // Binary BVH over item ids [b, e) of `items`.  Splits minimise the
  // surface-area cost SA(left) n_left + SA(right) n_right over every
  // centroid-sorted split on each axis (SAH, full sweep).  A median split on
  // the widest centroid axis would cut a telescope's mirror field into
  // rings when a camera far above it stretches the z extent: every ring box
  // spans the whole dish and a vertical ray then overlaps most leaves.
  // Where the remaining items might not fit the device's 32-entry
  // traversal stack under further unbalanced splits, the median split
  // (depth log2 of the items) takes over.  Returns the created node's index.
  static double box_area(const double* lo, const double* hi) {
    const double x = std::max(0.0, hi[0] - lo[0]), y = std::max(0.0, hi[1] - lo[1]),
                 z = std::max(0.0, hi[2] - lo[2]);
    return 2.0 * (x * y + y * z + z * x);
  }

  int bvh_build(std::vector<int>& items, int b, int e, int depth = 0) {
    rbg_bvh_node bn{};
    double lo[3] = {kBig, kBig, kBig}, hi[3] = {-kBig, -kBig, -kBig};
    double clo[3] = {kBig, kBig, kBig}, chi[3] = {-kBig, -kBig, -kBig};
    for (int i = b; i < e; ++i) {
      const rbg_node& n = s->nodes[items[i]];
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], n.lo[k]);
        hi[k] = std::max(hi[k], n.hi[k]);
        double c = 0.5 * (n.lo[k] + n.hi[k]);
        clo[k] = std::min(clo[k], c);
        chi[k] = std::max(chi[k], c);
      }
    }
    for (int k = 0; k < 3; ++k) {
      float fl = (float)lo[k], fh = (float)hi[k];
      if ((double)fl > lo[k]) fl = std::nextafter(fl, -std::numeric_limits<float>::infinity());
      if ((double)fh < hi[k]) fh = std::nextafter(fh, std::numeric_limits<float>::infinity());
      bn.lo[k] = fl;
      bn.hi[k] = fh;
    }
    int self = (int)s->bvh.size();
    s->bvh.push_back(bn);
    const int n = e - b;
    if (n <= kBvhLeaf) {
      s->bvh[self].left = -1;
      s->bvh[self].right = n;
      s->bvh[self].item_begin = (int)s->bvh_items.size();
      for (int i = b; i < e; ++i) s->bvh_items.push_back(items[i]);
      return self;
    }
    auto by_axis = [&](int axis) {
      return [&, axis](int x, int y) {
        const rbg_node& nx = s->nodes[x];
        const rbg_node& ny = s->nodes[y];
        double cx = nx.lo[axis] + nx.hi[axis], cy = ny.lo[axis] + ny.hi[axis];
        return cx < cy || (cx == cy && x < y);
      };
    };
    int median_depth = 0;
    for (int m = n; m > kBvhLeaf; m = (m + 1) / 2) ++median_depth;
    int axis = 0, mid = (b + e) / 2;
    if (depth + 1 + median_depth < kBvhSahDepth) {
      double best_cost = std::numeric_limits<double>::infinity();
      std::vector<double> right_area(n);
      for (int k = 0; k < 3; ++k) {
        if (!(chi[k] > clo[k])) continue;
        std::sort(items.begin() + b, items.begin() + e, by_axis(k));
        double rlo[3] = {kBig, kBig, kBig}, rhi[3] = {-kBig, -kBig, -kBig};
        for (int i = n - 1; i > 0; --i) {
          const rbg_node& nd = s->nodes[items[b + i]];
          for (int q = 0; q < 3; ++q) {
            rlo[q] = std::min(rlo[q], nd.lo[q]);
            rhi[q] = std::max(rhi[q], nd.hi[q]);
          }
          right_area[i] = box_area(rlo, rhi);
        }
        double llo[3] = {kBig, kBig, kBig}, lhi[3] = {-kBig, -kBig, -kBig};
        for (int i = 1; i < n; ++i) {
          const rbg_node& nd = s->nodes[items[b + i - 1]];
          for (int q = 0; q < 3; ++q) {
            llo[q] = std::min(llo[q], nd.lo[q]);
            lhi[q] = std::max(lhi[q], nd.hi[q]);
          }
          const double cost = box_area(llo, lhi) * i + right_area[i] * (n - i);
          if (cost < best_cost) {
            best_cost = cost;
            axis = k;
            mid = b + i;
          }
        }
      }
      std::sort(items.begin() + b, items.begin() + e, by_axis(axis));
    } else {
      for (int k = 1; k < 3; ++k)
        if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
      std::nth_element(items.begin() + b, items.begin() + mid, items.begin() + e, by_axis(axis));
    }
    int l = bvh_build(items, b, mid, depth + 1);
    int r = bvh_build(items, mid, e, depth + 1);
    s->bvh[self].left = l;
    s->bvh[self].right = r;
    s->bvh[self].item_begin = -1;
    return self;
  }

  int run() {
    if (d->n_shapes <= 0 || d->n_volumes <= 0 || !d->shapes || !d->volumes) return RBG_ERR_SCENE;
    if (d->top_volume < 0 || d->top_volume >= d->n_volumes) return RBG_ERR_SCENE;
    if ((d->n_matrices > 0 && !d->matrices) || (d->n_placements > 0 && !d->placements) ||
        (d->n_params > 0 && !d->params) || (d->n_tables > 0 && !d->tables) ||
        (d->n_indices > 0 && !d->indices) || (d->n_layers > 0 && !d->layers) ||
        (d->n_multilayers > 0 && !d->multilayers) || (d->n_borders > 0 && !d->borders))
      return RBG_ERR_ARG;
    s->shapes.assign(d->shapes, d->shapes + d->n_shapes);
    s->shape_box.assign(6 * (size_t)d->n_shapes, 0.0);
    shape_state.assign(d->n_shapes, 0);
    composite_depth.assign(d->n_shapes, 0);
    int rc;
    for (int i = 0; i < d->n_shapes; ++i)
      if ((rc = canon_shape(i)) != RBG_OK) return rc;
    if ((rc = copy_tables()) != RBG_OK) return rc;
    auto table_ok = [&](int t) { return t >= -1 && t < d->n_tables; };
    s->indices.assign(d->indices, d->indices + d->n_indices);
    for (int i = 0; i < d->n_indices; ++i) {
      const rbg_index_desc& x = s->indices[i];
      if (x.kind < RBG_INDEX_TABLE || x.kind > RBG_INDEX_MIXED) return RBG_ERR_SCENE;
      if (!table_ok(x.n_table) || !table_ok(x.k_table)) return RBG_ERR_SCENE;
      for (int t : {x.n_table, x.k_table})
        if (t >= 0 && s->tables[t].kind != RBG_TABLE_1D) return RBG_ERR_SCENE;
      // mixtures may only refer to earlier, non-mixed entries (no cycles)
      if (x.kind == RBG_INDEX_MIXED &&
          (x.mix_a < 0 || x.mix_a >= i || x.mix_b < 0 || x.mix_b >= i ||
           s->indices[x.mix_a].kind == RBG_INDEX_MIXED || s->indices[x.mix_b].kind == RBG_INDEX_MIXED))
        return RBG_ERR_SCENE;
    }
    s->layers.assign(d->layers, d->layers + d->n_layers);
    for (auto& l : s->layers)
      if (l.index < 0 || l.index >= d->n_indices) return RBG_ERR_SCENE;
    s->multilayers.assign(d->multilayers, d->multilayers + d->n_multilayers);
    s->tmm_off.assign(s->multilayers.size(), -1);
    int64_t tmm_cells = 0;
    for (size_t i = 0; i < s->multilayers.size(); ++i) {
      const auto& m = s->multilayers[i];
      if (m.n_layers < 2 || m.n_layers > 64 || m.layer_offset < 0 || m.layer_offset + m.n_layers > d->n_layers)
        return RBG_ERR_SCENE;
      if (m.precalc < 0 || m.precalc > 2) return RBG_ERR_SCENE;
      if (m.precalc != 0) {
        if (m.lam_nbins < 1 || m.th_nbins < 1 || (int64_t)m.lam_nbins * m.th_nbins > (int64_t)1 << 24 ||
            !(m.lam_max > m.lam_min) || !(m.th_max > m.th_min))
          return RBG_ERR_SCENE;
        s->tmm_off[i] = tmm_cells;
        tmm_cells += 2 * (int64_t)m.lam_nbins * m.th_nbins;
      }
    }
    s->tmm_tables.assign((size_t)tmm_cells, 0.0);
    s->tmm_ready = tmm_cells == 0;
    s->borders.assign(d->borders, d->borders + d->n_borders);
    for (auto& b : s->borders)
      if (b.component1 < 0 || b.component1 >= d->n_volumes || b.component2 < -1 ||
          b.component2 >= d->n_volumes || b.multilayer < -1 || b.multilayer >= d->n_multilayers)
        return RBG_ERR_SCENE;
    s->volumes.assign(d->volumes, d->volumes + d->n_volumes);
    for (auto& v : s->volumes) {
      if (v.shape < 0 || v.shape >= d->n_shapes) return RBG_ERR_SCENE;
      if (v.kind < RBG_KIND_LENS || v.kind > RBG_KIND_OTHER) return RBG_ERR_SCENE;
      if (!table_ok(v.refl_table) || !table_ok(v.qe_lambda_table) || !table_ok(v.qe_angle_table))
        return RBG_ERR_SCENE;
      if (v.index < -1 || v.index >= d->n_indices) return RBG_ERR_SCENE;
      for (int t : {v.qe_lambda_table, v.qe_angle_table})
        if (t >= 0 && s->tables[t].kind != RBG_TABLE_1D) return RBG_ERR_SCENE;
    }
    if ((rc = build_tree()) != RBG_OK) return rc;
    for (size_t i = 0; i < s->nodes.size(); ++i) {
      rbg_node& n = s->nodes[i];
      if (n.child_count >= kBvhMinChildren) {
        std::vector<int> items(s->children.begin() + n.child_begin,
                               s->children.begin() + n.child_begin + n.child_count);
        n.bvh_root = bvh_build(items, 0, (int)items.size());
        s->features |= rbg::kFeatBVH;
      }
    }
    for (const auto& sh : s->shapes) {
      if (sh.type == RBG_SHAPE_WINSTON_POLY || sh.type == RBG_SHAPE_WINSTON_2D) s->features |= rbg::kFeatWinston;
      else if (sh.type != RBG_SHAPE_BOX && sh.type != RBG_SHAPE_ASPHERIC_DISK) s->features |= rbg::kFeatCSG;
    }
    for (const auto& v : s->volumes)
      if (v.kind == RBG_KIND_LENS) s->features |= rbg::kFeatLens;
    for (const auto& b : s->borders) {
      if (b.multilayer >= 0) s->features |= rbg::kFeatMultilayer;
      if (b.sigma != 0 || b.lambertian) s->features |= rbg::kFeatRough;
    }
    rbg::build_node_aux(s);
    return RBG_OK;
  }
};

// largest float <= v (smallest float >= v when up)
float round_to_float(double v, bool up) {
  float f = (float)v;
  if (std::isnan(v)) return f;
  if (up && (double)f < v) f = std::nextafter(f, std::numeric_limits<float>::infinity());
  if (!up && (double)f > v) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
  return f;
}

}  // namespace

void rbg::build_node_aux(rbg_scene* s) {
  const double d2r = M_PI / 180.0;
  s->trig.clear();
  s->trig_off.assign(s->shapes.size(), -1);
  for (size_t i = 0; i < s->shapes.size(); ++i) {
    const rbg_shape_desc& sh = s->shapes[i];
    const double* P = s->params.data() + sh.param_offset;
    auto phi_planes = [&](double phi1, double dphi) {
      const double a1 = phi1 * d2r, a2 = (phi1 + dphi) * d2r;
      s->trig.insert(s->trig.end(), {-std::sin(a1), std::cos(a1), -std::sin(a2), std::cos(a2)});
    };
    const int32_t off = (int32_t)s->trig.size();
    switch (sh.type) {
      case RBG_SHAPE_TUBE:
        phi_planes(P[RBG_TUBE_PHI1], P[RBG_TUBE_DPHI]);
        break;
      case RBG_SHAPE_PCON:
        phi_planes(P[RBG_PCON_PHI1], P[RBG_PCON_DPHI]);
        break;
      case RBG_SHAPE_SPHERE: {
        phi_planes(P[RBG_SPH_PHI1], P[RBG_SPH_DPHI]);
        const double c1 = std::cos(P[RBG_SPH_TH1] * d2r), c2 = std::cos(P[RBG_SPH_TH2] * d2r);
        s->trig.insert(s->trig.end(), {c1, c2, c1 * c1, c2 * c2});
        break;
      }
      case RBG_SHAPE_PGON: {
        phi_planes(P[RBG_PGON_PHI1], P[RBG_PGON_DPHI]);
        const int ned = (int)P[RBG_PGON_NEDGES];
        const double sector = P[RBG_PGON_DPHI] / ned;
        for (int e = 0; e < ned; ++e) {
          const double pe = (P[RBG_PGON_PHI1] + (e + 0.5) * sector) * d2r;
          s->trig.insert(s->trig.end(), {std::cos(pe), std::sin(pe)});
        }
        break;
      }
      case RBG_SHAPE_WINSTON_POLY:
      case RBG_SHAPE_WINSTON_2D: {
        const int n = (int)P[RBG_WIN_N];
        const double th = P[RBG_WIN_THETA];
        s->trig.insert(s->trig.end(), {std::cos(th), std::sin(th), std::tan(M_PI / n)});
        for (int k = 0; k < n; ++k) {
          const double a = k * 2 * M_PI / n;
          s->trig.insert(s->trig.end(), {std::cos(a), std::sin(a)});
        }
        break;
      }
      case RBG_SHAPE_ASPHERIC_DISK: {
        const int n1 = (int)P[RBG_ASPH_NPOL1], n2 = (int)P[RBG_ASPH_NPOL2];
        s->trig.push_back(P[RBG_ASPH_Z2] - P[RBG_ASPH_Z1]);
        for (int j = 0; j < n1; ++j) s->trig.push_back((j + 1) * P[RBG_ASPH_K + j]);
        for (int j = 0; j < n2; ++j) s->trig.push_back((j + 1) * P[RBG_ASPH_K + n1 + j]);
        break;
      }
      default:
        break;
    }
    if ((int32_t)s->trig.size() > off) s->trig_off[i] = off;
  }
  s->fparams.resize(s->params.size());
  for (size_t i = 0; i < s->params.size(); ++i) s->fparams[i] = (float)s->params[i];
  s->node_aux.assign(s->nodes.size(), rbg_node_aux{});
  for (size_t i = 0; i < s->nodes.size(); ++i) {
    const rbg_node& n = s->nodes[i];
    rbg_node_aux& a = s->node_aux[i];
    for (int k = 0; k < 3; ++k) {
      a.lo[k] = round_to_float(n.lo[k], false);
      a.hi[k] = round_to_float(n.hi[k], true);
    }
    const bool rot_identity = n.m[0] == 1 && n.m[1] == 0 && n.m[2] == 0 && n.m[3] == 0 && n.m[4] == 1 &&
                              n.m[5] == 0 && n.m[6] == 0 && n.m[7] == 0 && n.m[8] == 1;
    const bool no_shift = n.m[9] == 0 && n.m[10] == 0 && n.m[11] == 0;
    a.xform = !rot_identity ? RBG_XFORM_GENERAL : (no_shift ? RBG_XFORM_IDENTITY : RBG_XFORM_TRANSLATION);
    a.flags = 0;
    const rbg_shape_desc& sh = s->shapes[n.shape];
    if (sh.type == RBG_SHAPE_ASPHERIC_DISK) {
      const double* P = s->params.data() + sh.param_offset;
      const int n1 = (int)P[RBG_ASPH_NPOL1], n2 = (int)P[RBG_ASPH_NPOL2];
      bool twin = n1 == n2 && P[RBG_ASPH_C1] == P[RBG_ASPH_C2] && P[RBG_ASPH_KAPPA1] == P[RBG_ASPH_KAPPA2];
      for (int j = 0; twin && j < n1; ++j) twin = P[RBG_ASPH_K + j] == P[RBG_ASPH_K + n1 + j];
      if (twin) a.flags |= RBG_AUX_ASPH_TWIN_FACES;
    }
    for (int c = 0; c < n.child_count; ++c)
      if (s->shapes[s->nodes[s->children[n.child_begin + c]].shape].type == RBG_SHAPE_ASPHERIC_DISK)
        a.flags |= RBG_AUX_ASPH_CHILDREN;
  }
}

extern "C" {

int rbg_abi_version(void) { return RBG_ABI_VERSION; }

const char* rbg_status_string(int status) {
  switch (status) {
    case RBG_OK: return "ok";
    case RBG_ERR_ARG: return "invalid argument";
    case RBG_ERR_SCENE: return "inconsistent scene description";
    case RBG_ERR_CUDA: return "CUDA runtime error";
    case RBG_ERR_NAN: return "ray with NaN or zero direction";
    case RBG_ERR_CAP: return "bounded loop hit its iteration cap";
    case RBG_ERR_UNSUPPORTED: return "unsupported feature";
    case RBG_ERR_NOMEM: return "out of memory";
    case RBG_ERR_NODEVICE: return "no CUDA device";
    case RBG_ERR_TOO_LARGE: return "scene larger than the no-allocation trace array (4 MiB)";
    default: return "unknown status";
  }
}

void rbg_trace_opts_default(rbg_trace_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->limit = 100;
  o->disable_fresnel = 0;
  o->seed = 0x5eed5eedULL;
  o->ray_id_offset = 0;
  o->precision = RBG_PREC_FP64;
  o->block_size = 0;
}

int rbg_scene_create(const rbg_scene_desc* desc, rbg_scene** out) {
  if (!desc || !out) return RBG_ERR_ARG;
  *out = nullptr;
  rbg_scene* s = new (std::nothrow) rbg_scene();
  if (!s) return RBG_ERR_NOMEM;
  Builder b{desc, s, {}};
  int rc;
  try {
    rc = b.run();
  } catch (const std::bad_alloc&) {
    rc = RBG_ERR_NOMEM;
  }
  if (rc != RBG_OK) {
    delete s;
    return rc;
  }
  *out = s;
  return RBG_OK;
}

void rbg_scene_destroy(rbg_scene* s) {
  if (!s) return;
  rbg::release_device(s);
  delete s;
}

int rbg_scene_flat(const rbg_scene* s, rbg_flat_scene* o) {
  if (!s || !o) return RBG_ERR_ARG;
  o->n_nodes = (int32_t)s->nodes.size();
  o->nodes = s->nodes.data();
  o->n_children = (int32_t)s->children.size();
  o->children = s->children.data();
  o->n_bvh = (int32_t)s->bvh.size();
  o->bvh = s->bvh.data();
  o->n_bvh_items = (int32_t)s->bvh_items.size();
  o->bvh_items = s->bvh_items.data();
  o->n_shapes = (int32_t)s->shapes.size();
  o->shapes = s->shapes.data();
  o->n_volumes = (int32_t)s->volumes.size();
  o->volumes = s->volumes.data();
  o->n_tables = (int32_t)s->tables.size();
  o->tables = s->tables.data();
  o->n_indices = (int32_t)s->indices.size();
  o->indices = s->indices.data();
  o->n_layers = (int32_t)s->layers.size();
  o->layers = s->layers.data();
  o->n_multilayers = (int32_t)s->multilayers.size();
  o->multilayers = s->multilayers.data();
  o->n_borders = (int32_t)s->borders.size();
  o->borders = s->borders.data();
  o->n_params = (int64_t)s->params.size();
  o->params = s->params.data();
  o->top_node = 0;
  return RBG_OK;
}

}  // extern "C"
