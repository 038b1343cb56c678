// device_scene.cuh -- device view of a flattened scene and small FP64
// helpers shared by the tracer kernels.
#pragma once
#include <cstdint>

#include "trace_features.h"
#include "philox.h"
#include "robast_gb.h"
#include "robast_gb_layout.h"
#include "node_aux.h"
#include "events.h"

#define RBG_D __device__ __forceinline__

namespace rbg {

struct DevScene {
  const rbg_node* nodes;
  const int32_t* children;
  const rbg_bvh_node* bvh;
  const int32_t* bvh_items;
  const rbg_shape_desc* shapes;
  const rbg_volume_desc* volumes;
  const rbg_table_desc* tables;
  const rbg_index_desc* indices;
  const rbg_layer_desc* layers;
  const rbg_multilayer_desc* multilayers;
  const rbg_border_desc* borders;
  const double* params;
  // mixed-precision tracer only: per-node float boxes and transform kind,
  // float copy of params (same offsets)
  const rbg_node_aux* aux;
  const float* fparams;
  // per-shape trigonometric constants (node_aux.h), both tracers
  const double* trig;
  const int32_t* trig_off;
  // precalculated thin-film tables (R then T per multilayer), offsets per
  // multilayer or -1
  const double* tmm_tables;
  const int64_t* tmm_off;
  int32_t n_nodes, n_borders, n_multilayers, n_tables;
  uint32_t features;  // kFeat* bits present in the scene
};



// error bits raised by kernels (read back by the C ABI)
enum : unsigned { ERR_BIT_NAN = 1u, ERR_BIT_CAP = 2u };

struct d3 {
  double x, y, z;
};
RBG_D d3 mk(double x, double y, double z) { return d3{x, y, z}; }
RBG_D d3 operator+(d3 a, d3 b) { return d3{a.x + b.x, a.y + b.y, a.z + b.z}; }
RBG_D d3 operator-(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
RBG_D d3 operator*(double s, d3 a) { return d3{s * a.x, s * a.y, s * a.z}; }
RBG_D double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RBG_D d3 neg(d3 a) { return d3{-a.x, -a.y, -a.z}; }
RBG_D d3 normalized(d3 a) {
  double m = sqrt(dot(a, a));
  return m > 0 ? d3{a.x / m, a.y / m, a.z / m} : a;
}

// matrices: row-major R then t, master = R local + t
RBG_D d3 to_local(const double* m, d3 p) {
  double x = p.x - m[9], y = p.y - m[10], z = p.z - m[11];
  return d3{m[0] * x + m[3] * y + m[6] * z, m[1] * x + m[4] * y + m[7] * z, m[2] * x + m[5] * y + m[8] * z};
}
RBG_D d3 dir_to_local(const double* m, d3 d) {
  return d3{m[0] * d.x + m[3] * d.y + m[6] * d.z, m[1] * d.x + m[4] * d.y + m[7] * d.z,
            m[2] * d.x + m[5] * d.y + m[8] * d.z};
}
RBG_D d3 dir_to_master(const double* m, d3 l) {
  return d3{m[0] * l.x + m[1] * l.y + m[2] * l.z, m[3] * l.x + m[4] * l.y + m[5] * l.z,
            m[6] * l.x + m[7] * l.y + m[8] * l.z};
}
// c = a * b for 12-double matrices held in registers
struct M12 {
  double v[12];
};
RBG_D M12 mat_mul(const double* a, const double* b) {
  M12 r;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) r.v[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
    r.v[9 + i] = a[i * 3] * b[9] + a[i * 3 + 1] * b[10] + a[i * 3 + 2] * b[11] + a[9 + i];
  }
  return r;
}
RBG_D M12 mat_identity() {
  M12 r;
#pragma unroll
  for (int i = 0; i < 12; ++i) r.v[i] = 0;
  r.v[0] = r.v[4] = r.v[8] = 1;
  return r;
}

// cancellation-safe real roots of A t^2 + B t + C = 0
RBG_D int quad_roots(double A, double B, double C, double* r) {
  if (A == 0) {
    if (B == 0) return 0;
    r[0] = -C / B;
    return 1;
  }
  double disc = B * B - 4 * A * C;
  if (disc < 0) return 0;
  double sq = sqrt(disc);
  double q = -0.5 * (B + (B >= 0 ? sq : -sq));
  if (q == 0) {
    r[0] = 0;
    return 1;
  }
  r[0] = q / A;
  r[1] = C / q;
  return 2;
}

// ---- tables: TGraph::Eval, bilinear 2D -------------------------------
RBG_D double table1d(const DevScene& S, int id, double x) {
  const rbg_table_desc t = S.tables[id];
  const double* X = S.params + t.param_offset;
  const double* Y = X + t.nx;
  int n = t.nx;
  if (n == 1) return Y[0];
  for (int i = 0; i < n; ++i)
    if (X[i] == x) return Y[i];
  int lo, hi;
  if (x < X[0]) {
    lo = 0;
    hi = 1;
  } else if (x > X[n - 1]) {
    lo = n - 2;
    hi = n - 1;
  } else {
    hi = 1;
    while (hi < n - 1 && X[hi] < x) ++hi;
    lo = hi - 1;
  }
  if (X[hi] == X[lo]) return Y[lo];
  return Y[lo] + (x - X[lo]) * (Y[hi] - Y[lo]) / (X[hi] - X[lo]);
}
RBG_D double table2d(const DevScene& S, int id, double x, double y) {
  const rbg_table_desc t = S.tables[id];
  const double* X = S.params + t.param_offset;
  const double* Y = X + t.nx;
  const double* Z = Y + t.ny;
  int nx = t.nx, ny = t.ny, ix = 0, iy = 0;
  double fx = 0, fy = 0;
  if (nx > 1) {
    if (x <= X[0]) {
      ix = 0;
      fx = 0;
    } else if (x >= X[nx - 1]) {
      ix = nx - 2;
      fx = 1;
    } else {
      while (ix < nx - 2 && X[ix + 1] < x) ++ix;
      fx = (x - X[ix]) / (X[ix + 1] - X[ix]);
    }
  }
  if (ny > 1) {
    if (y <= Y[0]) {
      iy = 0;
      fy = 0;
    } else if (y >= Y[ny - 1]) {
      iy = ny - 2;
      fy = 1;
    } else {
      while (iy < ny - 2 && Y[iy + 1] < y) ++iy;
      fy = (y - Y[iy]) / (Y[iy + 1] - Y[iy]);
    }
  }
  int ix1 = nx > 1 ? ix + 1 : ix, iy1 = ny > 1 ? iy + 1 : iy;
  double z00 = Z[ix * ny + iy], z01 = Z[ix * ny + iy1], z10 = Z[ix1 * ny + iy], z11 = Z[ix1 * ny + iy1];
  return (1 - fx) * (1 - fy) * z00 + (1 - fx) * fy * z01 + fx * (1 - fy) * z10 + fx * fy * z11;
}

// ---- refractive index models ------------------------------------------
RBG_D double index_n_base(const DevScene& S, const rbg_index_desc& x, double lam) {
  double l = lam / 1e-4;
  switch (x.kind) {
    case RBG_INDEX_TABLE:
      return x.n_table >= 0 ? table1d(S, x.n_table, lam) : 1.0;
    case RBG_INDEX_SELLMEIER: {
      double l2 = l * l;
      return sqrt(1 + x.coef[0] * l2 / (l2 - x.coef[3]) + x.coef[1] * l2 / (l2 - x.coef[4]) +
                  x.coef[2] * l2 / (l2 - x.coef[5]));
    }
    case RBG_INDEX_CAUCHY: {
      double il2 = 1.0 / (l * l);
      return x.coef[0] + x.coef[1] * il2 + x.coef[2] * il2 * il2;
    }
    case RBG_INDEX_SCHOTT: {
      double l2 = l * l, il2 = 1.0 / l2;
      return sqrt(x.coef[0] + x.coef[1] * l2 + x.coef[2] * il2 + x.coef[3] * il2 * il2 +
                  x.coef[4] * il2 * il2 * il2 + x.coef[5] * il2 * il2 * il2 * il2);
    }
  }
  return 1.0;
}
RBG_D double index_n(const DevScene& S, int id, double lam) {
  if (id < 0) return 1.0;
  const rbg_index_desc x = S.indices[id];
  if (x.kind == RBG_INDEX_MIXED)
    return index_n_base(S, S.indices[x.mix_a], lam) * x.coef[0] + index_n_base(S, S.indices[x.mix_b], lam) * x.coef[1];
  return index_n_base(S, x, lam);
}
RBG_D double index_k(const DevScene& S, int id, double lam) {
  if (id < 0) return 0.0;
  const rbg_index_desc x = S.indices[id];
  if (x.kind == RBG_INDEX_MIXED) {
    const rbg_index_desc a = S.indices[x.mix_a], b = S.indices[x.mix_b];
    double ka = a.k_table >= 0 ? table1d(S, a.k_table, lam) : 0.0;
    double kb = b.k_table >= 0 ? table1d(S, b.k_table, lam) : 0.0;
    return ka * x.coef[0] + kb * x.coef[1];
  }
  return x.k_table >= 0 ? table1d(S, x.k_table, lam) : 0.0;
}

}  // namespace rbg
