// geometry.cuh -- device shape queries in a node's local frame.
//
// TGeo primitives (box, tube, sphere, paraboloid, pgon, pcon) and their CSG
// composites are exact solids: every ray/surface root is collected with a
// compact surface code, the roots are sorted, and each segment between two
// roots is classified with the point-containment test.  The first root that
// enters (leaves) the solid past t = 0 is DistFromOutside (DistFromInside).
// The normal is recomputed only for that root.
//
// AGeoAsphericDisk and AGeoWinstonConePoly follow the reference's own
// algorithms (src/AGeoAsphericDisk.cxx, src/AGeoWinstonCone2D.cxx,
// src/AGeoWinstonConePoly.cxx), including their single-root Newton and
// parabola solvers.
#pragma once
#include "device_scene.cuh"

// out-of-line device helpers (one copy per translation unit)
#define RBG_NOINLINE static __device__ __noinline__

namespace rbg {

constexpr double kBig = RBG_BIG;
constexpr double kPi = 3.14159265358979323846;
constexpr double kD2R = kPi / 180.0;

RBG_D const double* SP(const DevScene& S, int shape) { return S.params + S.shapes[shape].param_offset; }
// the shape's trigonometric constants (node_aux.h), or null
RBG_D const double* ST(const DevScene& S, int shape) {
  const int o = S.trig_off[shape];
  return o < 0 ? nullptr : S.trig + o;
}

// --------------------------------------------------------------------
// containment
// --------------------------------------------------------------------
// phi in [phi1, phi1 + dphi] from the two phi-plane normals T[0..3]
// (n1 = (-sin a1, cos a1), n2 = (-sin a2, cos a2)): the point is on the
// inner side of both planes for dphi <= 180, of either plane above
RBG_D bool phi_in(double x, double y, const double* T, double dphi) {
  if (dphi >= 360.0) return true;
  const double s1 = x * T[0] + y * T[1], s2 = x * T[2] + y * T[3];
  return dphi <= 180.0 ? (s1 >= 0 && s2 <= 0) : (s1 >= 0 || s2 <= 0);
}

RBG_D bool pxcon_contains(const double* P, const double* T, bool pg, d3 p) {
  const int head = pg ? 4 : 3;
  const int nz = (int)P[pg ? 3 : 2];
  const double* Z = P + head;
  const double* RMIN = Z + nz;
  const double* RMAX = RMIN + nz;
  if (p.z < Z[0] || p.z > Z[nz - 1]) return false;
  if (!phi_in(p.x, p.y, T + RBG_TRIG_PHI, P[1])) return false;
  double rho;
  if (pg) {
    const int ned = (int)P[2];
    const double* E = T + RBG_TRIG_PGON_EDGE;
    if (P[1] >= 360.0) {
      // the edge whose angular sector holds the point has the largest
      // projection p . n_e (regular polygon)
      rho = p.x * E[0] + p.y * E[1];
      for (int e = 1; e < ned; ++e) rho = fmax(rho, p.x * E[2 * e] + p.y * E[2 * e + 1]);
    } else {
      double sector = P[1] / ned;
      double rel = atan2(p.y, p.x) / kD2R - P[0];
      while (rel < 0) rel += 360.0;
      while (rel >= 360.0) rel -= 360.0;
      int e = (int)floor(rel / sector);
      if (e >= ned) e = ned - 1;
      rho = p.x * E[2 * e] + p.y * E[2 * e + 1];
    }
  } else {
    rho = sqrt(p.x * p.x + p.y * p.y);
  }
  for (int k = 0; k < nz - 1; ++k) {
    if (p.z < Z[k] || p.z > Z[k + 1]) continue;
    double h = Z[k + 1] - Z[k];
    double rmn, rmx;
    if (h == 0) {
      rmn = fmin(RMIN[k], RMIN[k + 1]);
      rmx = fmax(RMAX[k], RMAX[k + 1]);
    } else {
      double f = (p.z - Z[k]) / h;
      rmn = RMIN[k] + f * (RMIN[k + 1] - RMIN[k]);
      rmx = RMAX[k] + f * (RMAX[k + 1] - RMAX[k]);
    }
    if (rho >= rmn && rho <= rmx) return true;
  }
  return false;
}

// theta in [th1, th2] (degrees, polar angle from +z) from the cosines
// c1 = cos th1, c2 = cos th2: th < th1 <=> z > c1 r and th > th2 <=> z < c2 r,
// compared squared with the signs taken apart
RBG_D bool theta_in(double z, double r2, double th1, double th2, double c1, double c2) {
  if (th1 > 0) {
    const bool below = c1 >= 0 ? (z > 0 && z * z > c1 * c1 * r2) : (z >= 0 || z * z < c1 * c1 * r2);
    if (below) return false;
  }
  if (th2 < 180) {
    const bool above = c2 <= 0 ? (z < 0 && z * z > c2 * c2 * r2) : (z < 0 || z * z < c2 * c2 * r2);
    if (above) return false;
  }
  return true;
}

RBG_D bool prim_contains(int type, const double* P, const double* T, d3 p) {
  switch (type) {
    case RBG_SHAPE_BOX:
      return fabs(p.x - P[RBG_BOX_OX]) <= P[RBG_BOX_DX] && fabs(p.y - P[RBG_BOX_OY]) <= P[RBG_BOX_DY] &&
             fabs(p.z - P[RBG_BOX_OZ]) <= P[RBG_BOX_DZ];
    case RBG_SHAPE_TUBE: {
      if (fabs(p.z) > P[RBG_TUBE_DZ]) return false;
      double r2 = p.x * p.x + p.y * p.y;
      if (r2 > P[RBG_TUBE_RMAX] * P[RBG_TUBE_RMAX] || r2 < P[RBG_TUBE_RMIN] * P[RBG_TUBE_RMIN]) return false;
      return phi_in(p.x, p.y, T + RBG_TRIG_PHI, P[RBG_TUBE_DPHI]);
    }
    case RBG_SHAPE_SPHERE: {
      double r2 = dot(p, p);
      if (r2 > P[RBG_SPH_RMAX] * P[RBG_SPH_RMAX] || r2 < P[RBG_SPH_RMIN] * P[RBG_SPH_RMIN]) return false;
      if (!theta_in(p.z, r2, P[RBG_SPH_TH1], P[RBG_SPH_TH2], T[RBG_TRIG_SPH_COS], T[RBG_TRIG_SPH_COS + 1]))
        return false;
      return phi_in(p.x, p.y, T + RBG_TRIG_PHI, P[RBG_SPH_DPHI]);
    }
    case RBG_SHAPE_PARABOLOID: {
      if (fabs(p.z) > P[RBG_PARA_DZ]) return false;
      double f = P[RBG_PARA_A] * (p.x * p.x + p.y * p.y) + P[RBG_PARA_B];
      return P[RBG_PARA_A] > 0 ? f <= p.z : f >= p.z;
    }
    case RBG_SHAPE_PGON:
      return pxcon_contains(P, T, true, p);
    case RBG_SHAPE_PCON:
      return pxcon_contains(P, T, false, p);
  }
  return false;
}

// CSG containment.  A primitive, or a composite of two primitives (the
// common case: every composite of the telescope scenes), is resolved
// from the composite's own operand matrices; deeper trees are walked with
// an explicit stack (depth <= RBG_MAX_COMPOSITE_DEPTH, checked when the
// scene is flattened), left operand first, with TGeo's short cuts: an
// intersection or subtraction whose left operand does not contain the point
// does not, a union whose left operand does, does.  Both are compiled once,
// out of line.
RBG_NOINLINE bool csg_contains_deep(const DevScene& S, int shape, d3 p) {
  constexpr int kFrames = RBG_MAX_COMPOSITE_DEPTH + 1;
  int fs[kFrames], stage[kFrames];
  d3 fp[kFrames];
  int sp = 0;
  fs[0] = shape;
  stage[0] = 0;
  fp[0] = p;
  bool ret = false;  // the value of the frame popped last
  while (sp >= 0) {
    const int id = fs[sp];
    const rbg_shape_desc sh = S.shapes[id];
    if (sh.type != RBG_SHAPE_COMPOSITE) {
      ret = prim_contains(sh.type, SP(S, id), ST(S, id), fp[sp]);
      --sp;
      continue;
    }
    const double* P = SP(S, id);
    if (stage[sp] == 2) {  // right operand evaluated
      if (sh.op == RBG_OP_SUBTRACTION) ret = !ret;
      --sp;
      continue;
    }
    if (stage[sp] == 1) {  // left operand evaluated
      if ((sh.op == RBG_OP_INTERSECTION || sh.op == RBG_OP_SUBTRACTION) && !ret) {
        --sp;
        continue;
      }
      if (sh.op == RBG_OP_UNION && ret) {
        --sp;
        continue;
      }
    }
    if (sp + 1 >= kFrames) return false;  // deeper than the flattener allows: never
    const bool right = stage[sp] == 1;
    stage[sp] = right ? 2 : 1;
    fs[sp + 1] = right ? sh.right : sh.left;
    stage[sp + 1] = 0;
    fp[sp + 1] = to_local(P + (right ? RBG_COMP_MR : RBG_COMP_ML), fp[sp]);
    ++sp;
  }
  return ret;
}

RBG_NOINLINE bool csg_contains(const DevScene& S, int shape, d3 p) {
  const rbg_shape_desc& sh = S.shapes[shape];
  if (sh.type != RBG_SHAPE_COMPOSITE) return prim_contains(sh.type, SP(S, shape), ST(S, shape), p);
  const int lt = S.shapes[sh.left].type, rt = S.shapes[sh.right].type;
  if (lt == RBG_SHAPE_COMPOSITE || rt == RBG_SHAPE_COMPOSITE) return csg_contains_deep(S, shape, p);
  const double* P = SP(S, shape);
  bool a = prim_contains(lt, SP(S, sh.left), ST(S, sh.left), to_local(P + RBG_COMP_ML, p));
  if (sh.op == RBG_OP_INTERSECTION && !a) return false;
  if (sh.op == RBG_OP_SUBTRACTION && !a) return false;
  if (sh.op == RBG_OP_UNION && a) return true;
  bool b = prim_contains(rt, SP(S, sh.right), ST(S, sh.right), to_local(P + RBG_COMP_MR, p));
  if (sh.op == RBG_OP_SUBTRACTION) return !b;
  return b;
}

// --------------------------------------------------------------------
// crossing lists
// --------------------------------------------------------------------
struct XList {
  double t[RBG_MAX_XINGS];
  uint32_t code[RBG_MAX_XINGS];  // leaf << 16 | surface
  int n;
  bool overflow;
};

RBG_D void xl_add(XList& L, double t, uint32_t code) {
  if (!isfinite(t)) return;
  if (L.n >= RBG_MAX_XINGS) {
    L.overflow = true;
    return;
  }
  L.t[L.n] = t;
  L.code[L.n] = code;
  ++L.n;
}

RBG_D void add_plane(XList& L, d3 o, d3 d, d3 n, double rhs, uint32_t code) {
  double den = dot(n, d);
  if (den == 0) return;
  xl_add(L, (rhs - dot(n, o)) / den, code);
}

// surface codes per primitive:
//  BOX 0..5 (axis*2+side) | TUBE 0,1 z, 2 rmax, 3 rmin, 4,5 phi
//  SPHERE 0 rmax, 1 rmin, 2 th1, 3 th2, 4,5 phi | PARABOLOID 0,1 z, 2 surface
//  PGON k<nz z-plane k; nz + (k*2+w)*ned + e face; 0x3ffe/0x3fff phi
//  PCON k<nz z-plane k; nz + k*2+w cone face; 0x3ffe/0x3fff phi
constexpr uint32_t kPhi1 = 0x3ffe, kPhi2 = 0x3fff;

// the two phi planes from their normals T[0..3]
RBG_D void add_phi(XList& L, d3 o, d3 d, const double* T, double dphi, uint32_t leaf) {
  if (dphi >= 360.0) return;
  add_plane(L, o, d, mk(T[0], T[1], 0), 0.0, leaf | kPhi1);
  add_plane(L, o, d, mk(T[2], T[3], 0), 0.0, leaf | kPhi2);
}

RBG_D void prim_collect(int type, const double* P, const double* T, d3 o, d3 d, uint32_t leaf, XList& L) {
  double r[2];
  switch (type) {
    case RBG_SHAPE_BOX: {
      const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (dd[k] == 0) continue;
        xl_add(L, (P[3 + k] - P[k] - oo[k]) / dd[k], leaf | (uint32_t)(2 * k));
        xl_add(L, (P[3 + k] + P[k] - oo[k]) / dd[k], leaf | (uint32_t)(2 * k + 1));
      }
      break;
    }
    case RBG_SHAPE_TUBE: {
      if (d.z != 0) {
        xl_add(L, (-P[RBG_TUBE_DZ] - o.z) / d.z, leaf | 0u);
        xl_add(L, (P[RBG_TUBE_DZ] - o.z) / d.z, leaf | 1u);
      }
      double A = d.x * d.x + d.y * d.y, B = 2 * (o.x * d.x + o.y * d.y), C0 = o.x * o.x + o.y * o.y;
      int k = quad_roots(A, B, C0 - P[RBG_TUBE_RMAX] * P[RBG_TUBE_RMAX], r);
      for (int i = 0; i < k; ++i) xl_add(L, r[i], leaf | 2u);
      if (P[RBG_TUBE_RMIN] > 0) {
        k = quad_roots(A, B, C0 - P[RBG_TUBE_RMIN] * P[RBG_TUBE_RMIN], r);
        for (int i = 0; i < k; ++i) xl_add(L, r[i], leaf | 3u);
      }
      add_phi(L, o, d, T + RBG_TRIG_PHI, P[RBG_TUBE_DPHI], leaf);
      break;
    }
    case RBG_SHAPE_SPHERE: {
      double A = dot(d, d), B = 2 * dot(o, d), C0 = dot(o, o);
      int k = quad_roots(A, B, C0 - P[RBG_SPH_RMAX] * P[RBG_SPH_RMAX], r);
      for (int i = 0; i < k; ++i) xl_add(L, r[i], leaf | 0u);
      if (P[RBG_SPH_RMIN] > 0) {
        k = quad_roots(A, B, C0 - P[RBG_SPH_RMIN] * P[RBG_SPH_RMIN], r);
        for (int i = 0; i < k; ++i) xl_add(L, r[i], leaf | 1u);
      }
      for (int w = 0; w < 2; ++w) {
        double th = w == 0 ? P[RBG_SPH_TH1] : P[RBG_SPH_TH2];
        if ((w == 0 && th <= 0) || (w == 1 && th >= 180)) continue;
        const double c2 = T[RBG_TRIG_SPH_COS2 + w];
        double s2 = 1 - c2;
        double Ac = d.z * d.z * s2 - c2 * (d.x * d.x + d.y * d.y);
        double Bc = 2 * (o.z * d.z * s2 - c2 * (o.x * d.x + o.y * d.y));
        double Cc = o.z * o.z * s2 - c2 * (o.x * o.x + o.y * o.y);
        k = quad_roots(Ac, Bc, Cc, r);
        for (int i = 0; i < k; ++i) xl_add(L, r[i], leaf | (uint32_t)(2 + w));
      }
      add_phi(L, o, d, T + RBG_TRIG_PHI, P[RBG_SPH_DPHI], leaf);
      break;
    }
    case RBG_SHAPE_PARABOLOID: {
      if (d.z != 0) {
        xl_add(L, (-P[RBG_PARA_DZ] - o.z) / d.z, leaf | 0u);
        xl_add(L, (P[RBG_PARA_DZ] - o.z) / d.z, leaf | 1u);
      }
      double a = P[RBG_PARA_A], b = P[RBG_PARA_B];
      double A = a * (d.x * d.x + d.y * d.y);
      double B = 2 * a * (o.x * d.x + o.y * d.y) - d.z;
      double C = a * (o.x * o.x + o.y * o.y) + b - o.z;
      int k = quad_roots(A, B, C, r);
      for (int i = 0; i < k; ++i) xl_add(L, r[i], leaf | 2u);
      break;
    }
    case RBG_SHAPE_PGON: {
      const int ned = (int)P[2], nz = (int)P[3];
      const double* Z = P + 4;
      const double* RMIN = Z + nz;
      const double* RMAX = RMIN + nz;
      if (d.z != 0)
        for (int k = 0; k < nz; ++k) xl_add(L, (Z[k] - o.z) / d.z, leaf | (uint32_t)k);
      const double* E = T + RBG_TRIG_PGON_EDGE;
      for (int k = 0; k < nz - 1; ++k) {
        double h = Z[k + 1] - Z[k];
        if (h <= 0) continue;
        // a face plane crossed outside its own section's z range is no
        // boundary point of the solid: dropping it changes no midpoint
        // classification and keeps the list short
        const double tol = 1e-6 * (h + fabs(Z[k]) + fabs(Z[k + 1])) + 1e-9;
        for (int w = 0; w < 2; ++w) {
          const double* R = w ? RMIN : RMAX;
          if (w && R[k] == 0 && R[k + 1] == 0) continue;
          double s = (R[k + 1] - R[k]) / h;
          for (int e = 0; e < ned; ++e) {
            const d3 n = mk(E[2 * e], E[2 * e + 1], -s);
            const double den = dot(n, d);
            if (den == 0) continue;
            const double t = (R[k] - s * Z[k] - dot(n, o)) / den, zt = o.z + t * d.z;
            if (zt < Z[k] - tol || zt > Z[k + 1] + tol) continue;
            xl_add(L, t, leaf | (uint32_t)(nz + (k * 2 + w) * ned + e));
          }
        }
      }
      add_phi(L, o, d, T + RBG_TRIG_PHI, P[1], leaf);
      break;
    }
    case RBG_SHAPE_PCON: {
      const int nz = (int)P[2];
      const double* Z = P + 3;
      const double* RMIN = Z + nz;
      const double* RMAX = RMIN + nz;
      if (d.z != 0)
        for (int k = 0; k < nz; ++k) xl_add(L, (Z[k] - o.z) / d.z, leaf | (uint32_t)k);
      for (int k = 0; k < nz - 1; ++k) {
        double h = Z[k + 1] - Z[k];
        if (h <= 0) continue;
        for (int w = 0; w < 2; ++w) {
          const double* R = w ? RMIN : RMAX;
          if (w && R[k] == 0 && R[k + 1] == 0) continue;
          double s = (R[k + 1] - R[k]) / h;
          double c0 = R[k] - s * Z[k];
          double A = d.x * d.x + d.y * d.y - s * s * d.z * d.z;
          double B = 2 * (o.x * d.x + o.y * d.y - s * d.z * (c0 + s * o.z));
          double C = o.x * o.x + o.y * o.y - (c0 + s * o.z) * (c0 + s * o.z);
          int m = quad_roots(A, B, C, r);
          const double tol = 1e-6 * (h + fabs(Z[k]) + fabs(Z[k + 1])) + 1e-9;
          for (int i = 0; i < m; ++i) {
            const double zt = o.z + r[i] * d.z;
            if (zt < Z[k] - tol || zt > Z[k + 1] + tol) continue;  // not on this section's cone
            xl_add(L, r[i], leaf | (uint32_t)(nz + k * 2 + w));
          }
        }
      }
      add_phi(L, o, d, T + RBG_TRIG_PHI, P[1], leaf);
      break;
    }
  }
}

// local normal of a primitive surface at point p (leaf frame)
RBG_D d3 prim_normal(int type, const double* P, const double* T, uint32_t surf, d3 p) {
  if (surf == kPhi1 || surf == kPhi2) {
    const double* n = T + RBG_TRIG_PHI + (surf == kPhi1 ? 0 : 2);
    return mk(n[0], n[1], 0);
  }
  switch (type) {
    case RBG_SHAPE_BOX: {
      int axis = surf / 2;
      return mk(axis == 0, axis == 1, axis == 2);
    }
    case RBG_SHAPE_TUBE:
      if (surf < 2) return mk(0, 0, 1);
      return mk(p.x, p.y, 0);
    case RBG_SHAPE_SPHERE:
      if (surf < 2) return p;
      {
        const double c2 = T[RBG_TRIG_SPH_COS2 + (surf == 2 ? 0 : 1)];
        return mk(-c2 * p.x, -c2 * p.y, (1 - c2) * p.z);
      }
    case RBG_SHAPE_PARABOLOID:
      if (surf < 2) return mk(0, 0, 1);
      return mk(2 * P[RBG_PARA_A] * p.x, 2 * P[RBG_PARA_A] * p.y, -1);
    case RBG_SHAPE_PGON: {
      const int ned = (int)P[2], nz = (int)P[3];
      if ((int)surf < nz) return mk(0, 0, 1);
      int f = (int)surf - nz;
      int e = f % ned, kw = f / ned, k = kw / 2, w = kw % 2;
      const double* Z = P + 4;
      const double* R = (w ? Z + nz : Z + 2 * nz);
      double s = (R[k + 1] - R[k]) / (Z[k + 1] - Z[k]);
      const double* E = T + RBG_TRIG_PGON_EDGE;
      return mk(E[2 * e], E[2 * e + 1], -s);
    }
    case RBG_SHAPE_PCON: {
      const int nz = (int)P[2];
      if ((int)surf < nz) return mk(0, 0, 1);
      int f = (int)surf - nz;
      int k = f / 2, w = f % 2;
      const double* Z = P + 3;
      const double* R = (w ? Z + nz : Z + 2 * nz);
      double s = (R[k + 1] - R[k]) / (Z[k + 1] - Z[k]);
      double c0 = R[k] - s * Z[k];
      return mk(p.x, p.y, -s * (c0 + s * p.z));
    }
  }
  return mk(0, 0, 1);
}

// Leaves of a composite tree in depth-first order (left operand first),
// each with the matrix from its frame to the query frame (M maps the
// tree's own frame there).  An explicit stack holds the pending right
// operands: at most one per level, RBG_MAX_COMPOSITE_DEPTH + 1 entries.
struct CsgWalk {
  int shape[RBG_MAX_COMPOSITE_DEPTH + 1];
  M12 m[RBG_MAX_COMPOSITE_DEPTH + 1];
  int sp;
};
RBG_D void csg_walk_begin(CsgWalk& w, int shape, const double* M) {
  w.sp = 0;
  w.shape[0] = shape;
#pragma unroll
  for (int i = 0; i < 12; ++i) w.m[0].v[i] = M[i];
}
// next leaf (shape id and matrix); false when the walk is done
RBG_D bool csg_walk_next(const DevScene& S, CsgWalk& w, int& leaf_shape, M12& leafM) {
  while (w.sp >= 0) {
    const int id = w.shape[w.sp];
    const M12 M = w.m[w.sp];
    const rbg_shape_desc sh = S.shapes[id];
    if (sh.type != RBG_SHAPE_COMPOSITE) {
      --w.sp;
      leaf_shape = id;
      leafM = M;
      return true;
    }
    const double* P = SP(S, id);
    if (w.sp + 1 >= RBG_MAX_COMPOSITE_DEPTH + 1) return false;  // deeper than the flattener allows: never
    // replace the composite by its right operand, then push its left one
    w.shape[w.sp] = sh.right;
    w.m[w.sp] = mat_mul(M.v, P + RBG_COMP_MR);
    ++w.sp;
    w.shape[w.sp] = sh.left;
    w.m[w.sp] = mat_mul(M.v, P + RBG_COMP_ML);
  }
  return false;
}

// Collect crossings of a composite tree deeper than two primitives; leaves
// are numbered in depth-first order.
RBG_NOINLINE void csg_collect_deep(const DevScene& S, int shape, const double* M, d3 o, d3 d, uint32_t& leaf,
                                   XList& L) {
  CsgWalk w;
  csg_walk_begin(w, shape, M);
  int ls;
  M12 LM;
  while (csg_walk_next(S, w, ls, LM)) {
    prim_collect(S.shapes[ls].type, SP(S, ls), ST(S, ls), to_local(LM.v, o), dir_to_local(LM.v, d), leaf << 16, L);
    ++leaf;
  }
}

// find leaf #target (depth-first) and its matrix
RBG_NOINLINE bool csg_find_leaf(const DevScene& S, int shape, const double* M, uint32_t target, uint32_t& leaf,
                                int& leaf_shape, M12& leafM) {
  CsgWalk w;
  csg_walk_begin(w, shape, M);
  while (csg_walk_next(S, w, leaf_shape, leafM)) {
    if (leaf == target) return true;
    ++leaf;
  }
  return false;
}

// Distance to enter (exit = false) or leave (exit = true) a TGeo primitive or
// composite; on success code/normal describe the crossed surface (normal in
// the shape frame, not oriented).  Every ray/surface root is collected with
// its surface code, the roots are sorted, and each segment between two is
// classified by containment of its midpoint.  Primitives and two-primitive
// composites take their operand matrices straight from the parameters.
RBG_NOINLINE double csg_dist(const DevScene& S, int shape, d3 o, d3 d, bool exit, d3& nrm, unsigned& err) {
  XList L;
  L.n = 0;
  L.overflow = false;
  const rbg_shape_desc& sh = S.shapes[shape];
  const double* P = SP(S, shape);
  // 0: primitive, 1: composite of two primitives, 2: deeper composite
  int form = 0;
  if (sh.type == RBG_SHAPE_COMPOSITE)
    form = (S.shapes[sh.left].type == RBG_SHAPE_COMPOSITE || S.shapes[sh.right].type == RBG_SHAPE_COMPOSITE) ? 2 : 1;
  if (form == 0) {
    prim_collect(sh.type, P, ST(S, shape), o, d, 0u, L);
  } else if (form == 1) {
    prim_collect(S.shapes[sh.left].type, SP(S, sh.left), ST(S, sh.left), to_local(P + RBG_COMP_ML, o),
                 dir_to_local(P + RBG_COMP_ML, d), 0u << 16, L);
    prim_collect(S.shapes[sh.right].type, SP(S, sh.right), ST(S, sh.right), to_local(P + RBG_COMP_MR, o),
                 dir_to_local(P + RBG_COMP_MR, d), 1u << 16, L);
  } else {
    uint32_t leaf = 0;
    M12 I = mat_identity();
    csg_collect_deep(S, shape, I.v, o, d, leaf, L);
  }
  if (L.overflow) {
    err |= ERR_BIT_CAP;
    return kBig;
  }
  // insertion sort on t
  for (int i = 1; i < L.n; ++i) {
    double t = L.t[i];
    uint32_t c = L.code[i];
    int j = i - 1;
    while (j >= 0 && L.t[j] > t) {
      L.t[j + 1] = L.t[j];
      L.code[j + 1] = L.code[j];
      --j;
    }
    L.t[j + 1] = t;
    L.code[j + 1] = c;
  }
  int j0 = 0;
  while (j0 < L.n && L.t[j0] <= 0) ++j0;
  if (j0 == L.n) return kBig;
  bool in_prev = false;
  if (j0 > 0) {
    double tm = 0.5 * (L.t[j0 - 1] + L.t[j0]);
    in_prev = csg_contains(S, shape, o + tm * d);
  }
  for (int j = j0; j < L.n; ++j) {
    bool in_next = false;
    if (j + 1 < L.n) {
      double tm = 0.5 * (L.t[j] + L.t[j + 1]);
      in_next = csg_contains(S, shape, o + tm * d);
    }
    if ((!exit && !in_prev && in_next) || (exit && in_prev && !in_next)) {
      double t = L.t[j];
      uint32_t target = L.code[j] >> 16, surf = L.code[j] & 0xffffu;
      const d3 q = o + t * d;
      if (form == 0) {
        nrm = normalized(prim_normal(sh.type, P, ST(S, shape), surf, q));
      } else if (form == 1) {
        const double* M = P + (target == 0 ? RBG_COMP_ML : RBG_COMP_MR);
        const int ls = target == 0 ? sh.left : sh.right;
        nrm = dir_to_master(M, normalized(prim_normal(S.shapes[ls].type, SP(S, ls), ST(S, ls), surf, to_local(M, q))));
      } else {
        uint32_t cnt = 0;
        int ls = shape;
        M12 I = mat_identity(), LM = mat_identity();
        csg_find_leaf(S, shape, I.v, target, cnt, ls, LM);
        nrm = dir_to_master(LM.v, normalized(prim_normal(S.shapes[ls].type, SP(S, ls), ST(S, ls), surf,
                                                         to_local(LM.v, q))));
      }
      return t;
    }
    in_prev = in_next;
  }
  return kBig;
}

// --------------------------------------------------------------------
// AGeoAsphericDisk (src/AGeoAsphericDisk.cxx)
// --------------------------------------------------------------------
struct Asph {
  const double* P;
  RBG_D double z(int s) const { return P[s == 1 ? RBG_ASPH_Z1 : RBG_ASPH_Z2]; }
  RBG_D double c(int s) const { return P[s == 1 ? RBG_ASPH_C1 : RBG_ASPH_C2]; }
  RBG_D double kap(int s) const { return P[s == 1 ? RBG_ASPH_KAPPA1 : RBG_ASPH_KAPPA2]; }
  RBG_D int npol(int s) const { return (int)P[s == 1 ? RBG_ASPH_NPOL1 : RBG_ASPH_NPOL2]; }
  RBG_D const double* K(int s) const {
    return P + RBG_ASPH_K + (s == 1 ? 0 : (int)P[RBG_ASPH_NPOL1]);
  }
  RBG_D double rmin() const { return P[RBG_ASPH_RMIN]; }
  RBG_D double rmax() const { return P[RBG_ASPH_RMAX]; }
  RBG_D bool rseg() const { return P[RBG_ASPH_RSEG] != 0; }
};

// CalcF1/CalcF2 (:126-153): Horner in r^2 for the polynomial terms
RBG_D bool asph_F(const Asph& a, int s, double r, double& f) {
  double c = a.c(s), k = a.kap(s);
  double p = r * r * c * c * k;
  if (1 - p < 0) return false;
  double r2 = r * r;
  int n = a.npol(s);
  const double* K = a.K(s);
  double poly = 0;
  for (int i = n - 1; i >= 0; --i) poly = (poly + K[i]) * r2;
  f = a.z(s) + r2 * c / (1 + sqrt(1 - p)) + poly;
  return true;
}
// CalcdF1dr/CalcdF2dr (:96-123)
RBG_D bool asph_dF(const Asph& a, int s, double r, double& f) {
  double c = a.c(s), k = a.kap(s);
  double p = r * r * c * c * k;
  if (1 - p <= 0) return false;
  double r2 = r * r;
  int n = a.npol(s);
  const double* K = a.K(s);
  double poly = 0;  // sum 2 i K_i r^(2i-1)
  for (int i = n - 1; i >= 0; --i) poly = poly * r2 + 2 * (i + 1) * K[i];
  f = r * c / sqrt(1 - p) + poly * r;
  return true;
}
RBG_D bool asph_contains(const Asph& a, d3 p) {
  double r = sqrt(p.x * p.x + p.y * p.y);
  if (r > a.rmax() || r < a.rmin()) return false;
  double f1, f2;
  if (!asph_F(a, 1, r, f1) || !asph_F(a, 2, r, f2)) return false;
  return !(p.z < f1 || f2 < p.z);
}

// DistToAsphere (:415-526)
RBG_D double asph_dist_surface(const Asph& a, int n, d3 point, d3 dir) {
  const double curve = a.c(n), kappa = a.kap(n);
  const int npol = a.npol(n);
  const double* K = a.K(n);
  double H2 = point.x * point.x + point.y * point.y;
  const double d = a.z(n);
  double p = -((point.z - d) * dir.z + point.x * dir.x + point.y * dir.y);
  double M = p * dir.z + point.z - d;
  double M2 = (point.z - d) * (point.z - d) + H2 - p * p;
  double check = 1 - (M2 * curve - 2 * M) * curve / dir.z / dir.z;
  if (check < 0) return kBig;
  double q = p + (M2 * curve - 2 * M) / (dir.z * (1 + sqrt(check)));
  d3 np = mk(point.x + q * dir.x, point.y + q * dir.y, point.z + q * dir.z - d);
  for (int i = 0;; i++) {
    if (i > 100) return kBig;
    H2 = np.x * np.x + np.y * np.y;
    check = 1 - kappa * H2 * curve * curve;
    if (check < 0) return kBig;
    double l = sqrt(check);
    // x = conic sag + sum K_j H2^(j+1); v = sum 2(j+1) K_j H2^j
    double x = 0, v = 0;
    for (int j = npol - 1; j >= 0; --j) {
      x = (x + K[j]) * H2;
      v = v * H2 + 2 * (j + 1) * K[j];
    }
    if (curve != 0) x += (1 - l) / curve / kappa;
    v = curve * kappa + l * v;
    double m = -np.x * v, nn = -np.y * v;
    double norm = sqrt(l * l + m * m + nn * nn);
    l /= norm;
    m /= norm;
    nn /= norm;
    check = dir.z * l + dir.x * m + dir.y * nn;
    if (check == 0) return kBig;
    double e = l * (x - np.z) / check;
    np = np + e * dir;
    if (fabs(e) < 1e-10) break;
  }
  np.z += d;
  d3 dv = np - point;
  if (dot(dir, dv) < 0) return kBig;
  double rz = sqrt(np.x * np.x + np.y * np.y);
  if (rz < a.rmin() || rz > a.rmax()) return kBig;
  return sqrt(dot(dv, dv));
}

// DistToInner / DistToOuter (:529-684)
RBG_D double asph_dist_wall(const Asph& a, bool outer, d3 point, d3 dir) {
  if (!outer && !a.rseg()) return kBig;
  double rsq = point.x * point.x + point.y * point.y;
  double nsq = dir.x * dir.x + dir.y * dir.y;
  if (sqrt(nsq) < 1e-10) return kBig;
  double rdotn = point.x * dir.x + point.y * dir.y;
  double R = outer ? a.rmax() : a.rmin();
  // TGeoTube::DistToTube
  double b = rdotn / nsq;
  double delta = b * b - (rsq - R * R) / nsq;
  delta = delta > 0 ? sqrt(delta) : -1;
  if (delta < 0) return kBig;
  double t1 = -b + delta, t2 = -b - delta;
  if (t1 < 0 && t2 < 0) return kBig;
  const double zmin = a.P[outer ? RBG_ASPH_F1RMAX : RBG_ASPH_F1RMIN];
  const double zmax = a.P[outer ? RBG_ASPH_F2RMAX : RBG_ASPH_F2RMIN];
  if (isnan(zmin) || isnan(zmax)) return kBig;
  if (t2 > 0) {
    if (t1 > 0) {
      double z1 = t1 * dir.z + point.z, z2 = t2 * dir.z + point.z;
      if (z1 < zmin || zmax < z1) t1 = kBig;
      if (z2 < zmin || zmax < z2) t2 = kBig;
      return t1 < t2 ? t1 : t2;
    }
  } else if (t2 == 0) {
    if (t1 > 0) {
      if (zmin <= point.z && point.z <= zmax) return 0;
      double z1 = t1 * dir.z + point.z;
      if (zmin <= z1 && z1 <= zmax) return t1;
    } else if (t1 == 0) {
      if (zmin <= point.z && point.z <= zmax) return 0;
    }
  } else {
    if (t1 > 0) {
      double z1 = t1 * dir.z + point.z;
      if (zmin <= z1 && z1 <= zmax) return t1;
    } else if (t1 == 0) {
      if (zmin <= point.z && point.z <= zmax) return 0;
    }
  }
  return kBig;
}

// Sag F(H2) and dF/dH2 of face s in FP64 without the conic square roots
// when the curvature is zero (the SC and light-guide surfaces); the values
// equal CalcF1/CalcF2 to rounding.
RBG_D bool asph_sag_fast(const Asph& a, int s, double H2, double& F, double& dF) {
  const double c = a.c(s);
  const int n = a.npol(s);
  const double* K = a.K(s);
  double p = 0, dp = 0;
  for (int j = n - 1; j >= 0; --j) {
    p = (p + K[j]) * H2;
    dp = dp * H2 + (j + 1) * K[j];
  }
  if (c == 0) {
    F = a.z(s) + p;
    dF = dp;
    return true;
  }
  double chk = 1 - a.kap(s) * c * c * H2;
  if (chk < 0) return false;
  double sq = sqrt(chk);
  F = a.z(s) + H2 * c / (1 + sq) + p;
  dF = chk > 0 ? c / (2 * sq) + dp : dp;
  return true;
}

// Contains without the radius square root (H2 against rmin^2, rmax^2)
RBG_D bool asph_contains_fast(const Asph& a, d3 p) {
  double H2 = p.x * p.x + p.y * p.y;
  if (H2 > a.rmax() * a.rmax() || H2 < a.rmin() * a.rmin()) return false;
  double f1, f2, d;
  if (!asph_sag_fast(a, 1, H2, f1, d) || !asph_sag_fast(a, 2, H2, f2, d)) return false;
  return !(p.z < f1 || f2 < p.z);
}

// ComputeNormal of the mixed path: the same closest-surface choice, made on
// FP64 safety distances (|dF/dr| = 2 r |F'| with F' the derivative in H2),
// with the normal of a face taken as its exact gradient (-2x F', -2y F', 1)
// (no atan2 / RotateZ).  The choice must be FP64: a point within half an
// FP32 ulp (1.5e-5 cm at r = 270 cm) of a rim reads as ON the rim in FP32,
// and the wall would win over a face crossed 1e-9 cm ago.
RBG_D d3 asph_normal_fast(const Asph& a, d3 point, d3 dir) {
  const double H2 = point.x * point.x + point.y * point.y;
  const double r = sqrt(H2);
  double saf[4];
  saf[0] = a.rseg() ? fabs(r - a.rmin()) : kBig;
  saf[1] = fabs(r - a.rmax());
  double F1, F2, dF1 = 0, dF2 = 0;
  bool ok1 = asph_sag_fast(a, 1, H2, F1, dF1), ok2 = asph_sag_fast(a, 2, H2, F2, dF2);
  saf[2] = ok1 ? fabs(F1 - point.z) / sqrt(1.0 + 4.0 * H2 * (dF1 * dF1)) : kBig;
  saf[3] = ok2 ? fabs(F2 - point.z) / sqrt(1.0 + 4.0 * H2 * (dF2 * dF2)) : kBig;
  int i = 0;
  for (int k = 1; k < 4; ++k)
    if (saf[k] < saf[i]) i = k;
  d3 n;
  if (i <= 1) {
    if (H2 > 0) {
      double inv = 1.0 / r;
      n = mk(point.x * inv, point.y * inv, 0);
    } else {
      n = mk(1, 0, 0);
    }
  } else {
    double dF = i == 2 ? dF1 : dF2;
    if (dF == 0) n = mk(0, 0, 1);
    else n = normalized(mk(-2 * point.x * dF, -2 * point.y * dF, 1));
  }
  if (dot(n, dir) < 0) n = neg(n);
  return n;
}

// DistFromInside (:363-380): nearest of the two faces and the two walls
RBG_D double asph_dist4(const Asph& a, d3 p, d3 d) {
  double best = asph_dist_surface(a, 1, p, d);
  double v = asph_dist_surface(a, 2, p, d);
  if (v < best) best = v;
  v = asph_dist_wall(a, false, p, d);
  if (v < best) best = v;
  v = asph_dist_wall(a, true, p, d);
  if (v < best) best = v;
  return best;
}

// reach of the bounding hollow tube (rmin, rmax, dz) at t >= 0 (the
// TGeoTube::DistFromOutsideS test of DistFromOutside, :393-395)
RBG_D bool tube_reached(d3 o, d3 d, double rmin, double rmax, double dz) {
  double P[RBG_TUBE_NP] = {rmin, rmax, dz, 0, 360};
  if (prim_contains(RBG_SHAPE_TUBE, P, nullptr, o)) return true;
  XList L;
  L.n = 0;
  L.overflow = false;
  prim_collect(RBG_SHAPE_TUBE, P, nullptr, o, d, 0u, L);
  for (int i = 1; i < L.n; ++i) {
    double t = L.t[i];
    int j = i - 1;
    while (j >= 0 && L.t[j] > t) {
      L.t[j + 1] = L.t[j];
      --j;
    }
    L.t[j + 1] = t;
  }
  for (int j = 0; j + 1 < L.n; ++j) {
    if (L.t[j + 1] <= 0) continue;
    double tm = 0.5 * (L.t[j] + L.t[j + 1]);
    if (prim_contains(RBG_SHAPE_TUBE, P, nullptr, o + tm * d)) return true;
  }
  return false;
}

// DistFromOutside (:383-412): the bounding-tube test, then the faces
RBG_D double asph_dist_out(const Asph& a, d3 p, d3 d) {
  d3 pp = mk(p.x, p.y, p.z - a.P[RBG_ASPH_ORIGIN_Z]);
  if (!tube_reached(pp, d, a.rmin(), a.rmax(), a.P[RBG_ASPH_DZ])) return kBig;
  return asph_dist4(a, p, d);
}

// ComputeNormal (:246-327)
RBG_D d3 asph_normal(const Asph& a, d3 point, d3 dir) {
  double r = sqrt(point.x * point.x + point.y * point.y);
  double phi = atan2(point.y, point.x);
  double saf[4];
  saf[0] = a.rseg() ? fabs(r - a.rmin()) : kBig;
  saf[1] = fabs(r - a.rmax());
  double f1, f2, df1 = kBig, df2 = kBig;
  if (!asph_F(a, 1, r, f1)) f1 = -kBig;
  if (f1 == -kBig) saf[2] = kBig;
  else saf[2] = asph_dF(a, 1, r, df1) ? fabs(f1 - point.z) / sqrt(1 + df1 * df1) : kBig;
  if (!asph_F(a, 2, r, f2)) f2 = kBig;
  if (f2 == kBig) saf[3] = kBig;
  else saf[3] = asph_dF(a, 2, r, df2) ? fabs(f2 - point.z) / sqrt(1 + df2 * df2) : kBig;
  int i = 0;
  for (int k = 1; k < 4; ++k)
    if (saf[k] < saf[i]) i = k;
  d3 nv = mk(0, 0, 0);
  if (i <= 1) {
    nv.x = 1;
  } else {
    double df = i == 2 ? df1 : df2;
    if (df == 0) nv.z = 1;
    else {
      nv.x = df / sqrt(1 + df * df);
      nv.z = -1 / sqrt(1 + df * df);
    }
  }
  double c = cos(phi), s = sin(phi);
  d3 n = mk(c * nv.x - s * nv.y, s * nv.x + c * nv.y, nv.z);
  if (dot(n, dir) < 0) n = neg(n);
  return n;
}

// --------------------------------------------------------------------
// AGeoWinstonConePoly
// --------------------------------------------------------------------
// The face angles 2 pi k / n, the cone angle theta and pi / n enter only
// through constants precomputed per shape (T): face normals (cos, sin),
// cos theta, sin theta and tan(pi / n).  Angular tests become sign tests.
struct Win {
  double r1, r2, theta, f, dz;
  int n;
  double ct, st, tan_half;  // cos theta, sin theta, tan(pi / n)
  const double* face;       // (cos 2 pi k / n, sin 2 pi k / n) per face k
};
RBG_D Win win_load(const double* P, const double* T) {
  Win w;
  w.r1 = P[RBG_WIN_R1];
  w.r2 = P[RBG_WIN_R2];
  w.n = (int)P[RBG_WIN_N];
  w.theta = P[RBG_WIN_THETA];
  w.f = P[RBG_WIN_F];
  w.dz = P[RBG_WIN_DZ];
  w.ct = T[RBG_TRIG_WIN_COS];
  w.st = T[RBG_TRIG_WIN_SIN];
  w.tan_half = T[RBG_TRIG_WIN_TANHALF];
  w.face = T + RBG_TRIG_WIN_FACE;
  return w;
}
// CalcR (AGeoWinstonCone2D.cxx:82-98)
RBG_D bool win_R(const Win& w, double z, double& r) {
  if (fabs(z) > w.dz + 1e-10) return false;
  const double sint = w.st, cost = w.ct;
  double t = z + w.dz;
  double a0 = t * t * sint * sint - 4. * w.f * (t * cost + w.f);
  double a1 = 2. * t * sint * cost + 4. * w.f * sint;
  double a2 = cost * cost;
  r = (-a1 + sqrt(a1 * a1 - 4. * a0 * a2)) / (2 * a2) - w.r2;
  return true;
}
// CalcdRdZ (:59-79)
RBG_D double win_dRdZ(const Win& w, double z) {
  const double sint = w.st, cost = w.ct;
  double t = z + w.dz;
  double a0 = t * t * sint * sint - 4. * w.f * (t * cost + w.f);
  double a1 = 2. * t * sint * cost + 4. * w.f * sint;
  double a2 = cost * cost;
  double da0dt = 2 * t * sint * sint - 4 * w.f * cost;
  double da1dt = 2 * sint * cost;
  return (-da1dt + (a1 * da1dt - 2 * da0dt * a2) / sqrt(a1 * a1 - 4 * a0 * a2)) / (2 * a2);
}
// Projection of (x, y) on the normal of the face whose sector holds it:
// the reference reduces atan2(y, x) into [-pi/n, pi/n] and takes
// sqrt(x^2 + y^2) cos(reduced angle), which is max_k (x, y) . n_k for the n
// face normals of a regular polygon.  `k` receives the face.
RBG_D double win_face_proj(const Win& w, double x, double y, int& k) {
  double best = x * w.face[0] + y * w.face[1];
  k = 0;
  for (int i = 1; i < w.n; ++i) {
    const double v = x * w.face[2 * i] + y * w.face[2 * i + 1];
    if (v > best) {
      best = v;
      k = i;
    }
  }
  return best;
}
// InsidePolygon (ConePoly.cxx:293-309)
RBG_D bool win_inside_polygon(const Win& w, double x, double y, double r) {
  int k;
  return !(win_face_proj(w, x, y, k) > r);
}
RBG_NOINLINE bool win_contains(const Win& w, d3 p) {
  if (fabs(p.z) > w.dz) return false;
  double r;
  if (!win_R(w, p.z, r)) return false;
  return win_inside_polygon(w, p.x, p.y, r);
}
// DistToParabola (Cone2D.cxx:325-428) for face k.  tan(alpha - theta) with
// alpha = atan2(pz, px) is (pz cos theta - px sin theta) / (px cos theta +
// pz sin theta); the angular window |atan2(yc, xc)| <= open / 2 is xc >= 0
// for open = pi and xc > 0, |yc| <= xc tan(pi / n) for open = 2 pi / n.
RBG_D double win_dist_parabola(const Win& w, d3 point, d3 dir, int k, bool half_space) {
  const double cp = w.face[2 * k], sp = w.face[2 * k + 1];
  double x = cp * point.x + sp * point.y;
  double y = -sp * point.x + cp * point.y;
  double z = point.z;
  double px = cp * dir.x + sp * dir.y;
  double py = -sp * dir.x + cp * dir.y;
  double pz = dir.z;
  if (px == 0 && pz == 0) return kBig;
  const double cost = w.ct, sint = w.st;
  double X = cost * (x + w.r2) + (z + w.dz) * sint;
  double Z = -sint * (x + w.r2) + (z + w.dz) * cost + w.f;
  const double den = px * cost + pz * sint;
  if (den == 0) return kBig;
  double tanA = (pz * cost - px * sint) / den;
  double tmp = tanA * tanA - (X * tanA - Z) / w.f;
  if (tmp < 0) return kBig;
  double Xp, Xm;
  if (w.dz * 2 / fabs(tanA) < 1e-10) {
    Xp = X;
    Xm = X;
  } else {
    double sq = sqrt(tmp);
    Xp = 2 * w.f * (tanA + sq);
    Xm = 2 * w.f * (tanA - sq);
  }
  double best = kBig;
  for (int s = 0; s < 2; ++s) {
    double Xc = s == 0 ? Xp : Xm;
    double Zc = Xc * Xc / 4. / w.f;
    double xc = cost * Xc - sint * (Zc - w.f) - w.r2;
    double zc = sint * Xc + cost * (Zc - w.f) - w.dz;
    double yc;
    if (fabs(px) <= fabs(pz) && fabs(py) <= fabs(pz)) yc = y + (zc - z) * py / pz;
    else if (fabs(py) <= fabs(px) && fabs(pz) <= fabs(px)) yc = y + (xc - x) * py / px;
    else yc = y + (fabs(px) < 1e-5 ? (zc - z) * py / pz : (xc - x) * py / px);
    double dx = xc - x, dy = yc - y, dz = zc - z;
    double v;
    if (xc < w.r2 || w.r1 < xc || zc < -w.dz || w.dz < zc || dx * px + dz * pz < 0) {
      v = kBig;
    } else {
      const bool in_window = half_space ? xc >= 0 : (xc > 0 && fabs(yc) <= xc * w.tan_half);
      v = in_window ? sqrt(dx * dx + dy * dy + dz * dz) : kBig;
    }
    if (v < best) best = v;
  }
  return best;
}
RBG_NOINLINE double win_dist_in(const Win& w, d3 p, d3 d) {
  double best = kBig;
  if (d.z < 0) best = (-p.z - w.dz) / d.z;
  else if (d.z > 0) best = (w.dz - p.z) / d.z;
  for (int i = 0; i < w.n; i++) {
    double v = win_dist_parabola(w, p, d, i, true);
    if (v < best) best = v;
  }
  return best;
}
RBG_NOINLINE double win_dist_out(const Win& w, d3 p, d3 d) {
  if (p.z <= -w.dz) {
    if (d.z <= 0) return kBig;
    double s = -(w.dz + p.z) / d.z;
    if (win_inside_polygon(w, p.x + s * d.x, p.y + s * d.y, w.r2)) return s;
  } else if (p.z >= w.dz) {
    if (d.z >= 0) return kBig;
    double s = (w.dz - p.z) / d.z;
    if (win_inside_polygon(w, p.x + s * d.x, p.y + s * d.y, w.r1)) return s;
  }
  double best = kBig;
  for (int i = 0; i < w.n; i++) {
    double v = win_dist_parabola(w, p, d, i, false);
    if (v < best) best = v;
  }
  return best;
}
// ComputeNormal (ConePoly.cxx:67-122): the face of the point's sector
RBG_NOINLINE d3 win_normal(const Win& w, d3 point, d3 dir) {
  double x = point.x, y = point.y, z = point.z;
  double saf0 = fabs(fabs(w.dz) - fabs(z)), saf1;
  int k;
  const double proj = win_face_proj(w, x, y, k);
  double R;
  saf1 = win_R(w, z, R) ? fabs(R - proj) : kBig;
  d3 n;
  if (saf0 <= saf1) n = mk(0, 0, 1);
  else n = mk(w.face[2 * k], w.face[2 * k + 1], -win_dRdZ(w, z));
  n = normalized(n);
  if (dot(n, dir) < 0) n = neg(n);
  return n;
}

// --------------------------------------------------------------------
// AGeoWinstonCone2D (src/AGeoWinstonCone2D.cxx): the trough between the
// parabolic walls x = +-R(z), |y| <= dy -- a two-face Win (faces at phi = 0
// and pi, each DistToParabola with a half-space window) plus two y slabs
// --------------------------------------------------------------------
// Contains (:175-190)
RBG_NOINLINE bool win2d_contains(const Win& w, double dy, d3 p) {
  if (fabs(p.y) > dy || fabs(p.z) > w.dz) return false;
  double r;
  if (!win_R(w, p.z, r)) return false;
  return !(fabs(p.x) > r);
}
// DistFromInside (:203-238)
RBG_NOINLINE double win2d_dist_in(const Win& w, double dy, d3 p, d3 d) {
  double v[4];
  v[0] = kBig;
  if (d.z < 0) v[0] = -(p.z + w.dz) / d.z;
  else if (d.z > 0) v[0] = (w.dz - p.z) / d.z;
  v[1] = kBig;
  if (d.y < 0) v[1] = -(p.y + dy) / d.y;
  else if (d.y > 0) v[1] = (dy - p.y) / d.y;
  v[2] = win_dist_parabola(w, p, d, 0, true);
  v[3] = win_dist_parabola(w, p, d, 1, true);
  int k = 0;
  for (int i = 1; i < 4; ++i)
    if (v[i] < v[k]) k = i;
  return v[k];
}
// DistFromOutside (:241-322)
RBG_NOINLINE double win2d_dist_out(const Win& w, double dy, d3 p, d3 d) {
  if (p.z <= -w.dz) {
    if (d.z <= 0) return kBig;
    const double s = -(w.dz + p.z) / d.z;
    if (fabs(p.x + s * d.x) <= w.r2 && fabs(p.y + s * d.y) <= dy) return s;
  } else if (p.z >= w.dz) {
    if (d.z >= 0) return kBig;
    const double s = (w.dz - p.z) / d.z;
    if (fabs(p.x + s * d.x) <= w.r1 && fabs(p.y + s * d.y) <= dy) return s;
  }
  double r;
  if (p.y <= -dy) {
    if (d.y <= 0) return kBig;
    const double s = -(dy + p.y) / d.y, zn = p.z + s * d.z;
    if (fabs(zn) <= w.dz && win_R(w, zn, r) && fabs(p.x + s * d.x) <= r) return s;
  } else if (p.y >= dy) {
    if (d.y >= 0) return kBig;
    const double s = (dy - p.y) / d.y, zn = p.z + s * d.z;
    if (fabs(zn) <= w.dz && win_R(w, zn, r) && fabs(p.x + s * d.x) <= r) return s;
  }
  double s = win_dist_parabola(w, p, d, 0, true);
  const double a = fabs(p.y + s * d.y) <= dy ? s : kBig;
  s = win_dist_parabola(w, p, d, 1, true);
  const double b = fabs(p.y + s * d.y) <= dy ? s : kBig;
  return a < b ? a : b;
}
// ComputeNormal (:120-172)
RBG_NOINLINE d3 win2d_normal(const Win& w, double dy, d3 p, d3 dir) {
  double saf[3], r;
  saf[0] = fabs(fabs(dy) - fabs(p.y));
  saf[1] = fabs(fabs(w.dz) - fabs(p.z));
  saf[2] = win_R(w, p.z, r) ? fabs(r - fabs(p.x)) : kBig;
  int i = 0;
  for (int k = 1; k < 3; ++k)
    if (saf[k] < saf[i]) i = k;
  d3 n;
  if (i == 0) n = mk(0, 1, 0);
  else if (i == 1) n = mk(0, 0, 1);
  else n = mk(1, 0, p.x > 0 ? -win_dRdZ(w, p.z) : win_dRdZ(w, p.z));
  n = normalized(n);
  if (dot(n, dir) < 0) n = neg(n);
  return n;
}

// --------------------------------------------------------------------
// dispatch
// --------------------------------------------------------------------
// Reciprocal seeded in FP32 and refined by one FP64 Newton step (relative
// error ~1e-14): the mixed path's replacement for FP64 divisions by the
// direction cosines.
RBG_D double rcp_refined(double v) {
  double r = (double)(1.0f / (float)v);
  return r * (2.0 - v * r);
}

// TGeoBBox distances for the mixed path (slabs; the same crossings the
// exact-solid method finds for a box).
RBG_D double box_dist_fast(const double* P, d3 p, d3 d, bool exit, d3& nrm) {
  RBG_EVENT(EV_BOX64);
  const double o[3] = {p.x - P[RBG_BOX_OX], p.y - P[RBG_BOX_OY], p.z - P[RBG_BOX_OZ]};
  const double dd[3] = {d.x, d.y, d.z};
  if (exit) {
    double best = kBig;
    int axis = -1;
    for (int k = 0; k < 3; ++k) {
      if (dd[k] == 0) continue;
      double plane = dd[k] > 0 ? P[k] : -P[k];
      double t = (plane - o[k]) * rcp_refined(dd[k]);
      if (t < best) {
        best = t;
        axis = k;
      }
    }
    if (axis < 0 || best <= 0) return kBig;
    nrm = mk(axis == 0, axis == 1, axis == 2);
    return best;
  }
  double tnear = -kBig, tfar = kBig;
  int axis = -1;
  for (int k = 0; k < 3; ++k) {
    if (dd[k] == 0) {
      if (fabs(o[k]) > P[k]) return kBig;
      continue;
    }
    double inv = rcp_refined(dd[k]);
    double ta = (-P[k] - o[k]) * inv, tb = (P[k] - o[k]) * inv;
    if (ta > tb) {
      double s = ta;
      ta = tb;
      tb = s;
    }
    if (ta > tnear) {
      tnear = ta;
      axis = k;
    }
    tfar = fmin(tfar, tb);
  }
  if (axis < 0 || tnear > tfar || tnear <= 0) return kBig;
  nrm = mk(axis == 0, axis == 1, axis == 2);
  return tnear;
}

// shape queries of the FP64 path (the mixed path has its own, below).  In
// kernels with optional features the dispatch is compiled once, out of line
// (shape_contains / shape_dist below): every inlined copy of it multiplies
// the code the instruction cache must hold and the time ptxas takes.
template <unsigned F = kFeatAll>
RBG_D bool shape_contains_body(const DevScene& S, int shape, d3 p) {
  const int type = S.shapes[shape].type;
  if (type == RBG_SHAPE_ASPHERIC_DISK) return asph_contains(Asph{SP(S, shape)}, p);
  if (type == RBG_SHAPE_WINSTON_POLY)
    return (F & kFeatWinston) ? win_contains(win_load(SP(S, shape), ST(S, shape)), p) : false;
  if (type == RBG_SHAPE_WINSTON_2D)
    return (F & kFeatWinston) ? win2d_contains(win_load(SP(S, shape), ST(S, shape)), SP(S, shape)[RBG_WIN_DY], p)
                              : false;
  if (!(F & kFeatCSG) && type == RBG_SHAPE_BOX) return prim_contains(RBG_SHAPE_BOX, SP(S, shape), nullptr, p);
  return (F & kFeatCSG) ? csg_contains(S, shape, p) : false;
}

template <unsigned F = kFeatAll>
RBG_D double shape_dist_body(const DevScene& S, int shape, d3 p, d3 d, bool exit, d3& nrm, unsigned& err) {
  const int type = S.shapes[shape].type;
  if (type == RBG_SHAPE_ASPHERIC_DISK) {
    Asph a{SP(S, shape)};
    return exit ? asph_dist4(a, p, d) : asph_dist_out(a, p, d);
  }
  if (type == RBG_SHAPE_WINSTON_POLY || type == RBG_SHAPE_WINSTON_2D) {
    if (!(F & kFeatWinston)) return kBig;
    Win w = win_load(SP(S, shape), ST(S, shape));
    if (type == RBG_SHAPE_WINSTON_2D) {
      const double dy = SP(S, shape)[RBG_WIN_DY];
      return exit ? win2d_dist_in(w, dy, p, d) : win2d_dist_out(w, dy, p, d);
    }
    return exit ? win_dist_in(w, p, d) : win_dist_out(w, p, d);
  }
  return (F & kFeatCSG) ? csg_dist(S, shape, p, d, exit, nrm, err) : kBig;
}

template <unsigned F>
RBG_NOINLINE bool shape_contains_call(const DevScene& S, int shape, d3 p) {
  return shape_contains_body<F>(S, shape, p);
}
template <unsigned F>
RBG_NOINLINE double shape_dist_call(const DevScene& S, int shape, d3 p, d3 d, bool exit, d3& nrm, unsigned& err) {
  return shape_dist_body<F>(S, shape, p, d, exit, nrm, err);
}
template <unsigned F = kFeatAll>
RBG_D bool shape_contains(const DevScene& S, int shape, d3 p) {
  return F == 0 ? shape_contains_body<F>(S, shape, p) : shape_contains_call<F>(S, shape, p);
}
template <unsigned F = kFeatAll>
RBG_D double shape_dist(const DevScene& S, int shape, d3 p, d3 d, bool exit, d3& nrm, unsigned& err) {
  return F == 0 ? shape_dist_body<F>(S, shape, p, d, exit, nrm, err) : shape_dist_call<F>(S, shape, p, d, exit, nrm, err);
}

RBG_D bool is_ageo(int type) {
  return type == RBG_SHAPE_ASPHERIC_DISK || type == RBG_SHAPE_WINSTON_POLY || type == RBG_SHAPE_WINSTON_2D;
}

// ====================================================================
// Mixed-precision fast paths.
//
// The mixed tracer spends its time in the FP64 pipe, which on this part
// runs at 1/64 of the FP32 rate, and in instruction fetch.  The functions
// below keep every decision the FP64 algorithm makes, but take it with an
// FP32 screen where the screen's error bound leaves no doubt, and fall back
// to the exact FP64 test (compiled once, out of line) where it does.  The
// ray's float position and direction are converted once per step and
// passed along with the FP64 ones.
// ====================================================================

struct f3 {
  float x, y, z;
};
RBG_D f3 to_f3(d3 a) { return f3{(float)a.x, (float)a.y, (float)a.z}; }

// a ray (or point, with d unused) in a node's local frame, FP64 and FP32
struct LRay {
  d3 p, d;
  f3 pf, df;
};

// master -> local for node k, using its transform kind.  The float local
// point is always converted from the FP64 local point, so its error stays
// relative to the local coordinates the screens compare.
RBG_D LRay local_ray(const DevScene& S, int k, d3 p, d3 d, f3 pf, f3 df) {
  const int xf = S.aux[k].xform;
  if (xf == RBG_XFORM_IDENTITY) return LRay{p, d, pf, df};
  const rbg_node& N = S.nodes[k];
  if (xf == RBG_XFORM_TRANSLATION) {
    RBG_EVENT(EV_XFORM_T);
    d3 lp = mk(p.x - N.m[9], p.y - N.m[10], p.z - N.m[11]);
    return LRay{lp, d, to_f3(lp), df};
  }
  RBG_EVENT(EV_XFORM_G);
  d3 lp = to_local(N.m, p), ld = dir_to_local(N.m, d);
  return LRay{lp, ld, to_f3(lp), to_f3(ld)};
}
RBG_D LRay local_point(const DevScene& S, int k, d3 p, f3 pf) {
  const int xf = S.aux[k].xform;
  if (xf == RBG_XFORM_IDENTITY) return LRay{p, p, pf, pf};
  const rbg_node& N = S.nodes[k];
  RBG_EVENT(xf == RBG_XFORM_TRANSLATION ? EV_XFORM_T : EV_XFORM_G);
  d3 lp = xf == RBG_XFORM_TRANSLATION ? mk(p.x - N.m[9], p.y - N.m[10], p.z - N.m[11]) : to_local(N.m, p);
  f3 lpf = to_f3(lp);
  return LRay{lp, lp, lpf, lpf};
}

// 1/sqrt(m2) for m2 >= ~1e-30: FP32 seed, two FP64 Newton steps
// (relative error 2^-23 -> ~1e-14 -> FP64 rounding)
RBG_D double rsqrt_refined(double m2) {
  double r = (double)rsqrtf((float)m2);
  double h = 0.5 * m2;
  r = r * (1.5 - h * r * r);
  r = r * (1.5 - h * r * r);
  return r;
}

// sum_{j<n} K_j h^(j+1) (the polynomial part of CalcF1/CalcF2) with FMAs
RBG_D double asph_poly(const double* K, int n, double h) {
  if (n <= 0) return 0.0;
  double q = K[n - 1];
  for (int j = n - 2; j >= 0; --j) q = fma(q, h, K[j]);
  return q * h;
}
// sum_{j<n} (j+1) K_j h^j = d poly / d h
RBG_D double asph_dpoly(const double* K, int n, double h) {
  if (n <= 0) return 0.0;
  double q = n * K[n - 1];
  for (int j = n - 2; j >= 0; --j) q = fma(q, h, (j + 1) * K[j]);
  return q;
}
// FP32 sag of a face with c == 0 and the sum of its terms' magnitudes
// (the scale of its rounding error)
RBG_D float asph_poly_f(const float* K, int n, float h, float& mag) {
  float q = 0.f, m = 0.f;
  for (int j = n - 1; j >= 0; --j) {
    q = (q + K[j]) * h;
    m = (m + fabsf(K[j])) * h;
  }
  mag = m;
  return q;
}

// the FP64 reference algorithms, out of line: taken only when a screen
// cannot decide or the FP32 iteration breaks down
RBG_NOINLINE double asph_dist_surface_exact(const double* P, int n, d3 point, d3 dir) {
  RBG_EVENT(EV_DIST_EXACT);
  return asph_dist_surface(Asph{P}, n, point, dir);
}
RBG_NOINLINE double asph_dist_wall_exact(const double* P, bool outer, d3 point, d3 dir) {
  RBG_EVENT(EV_WALL_EXACT);
  return asph_dist_wall(Asph{P}, outer, point, dir);
}
// Contains in FP64: for faces with c == 0 the sags are z + sum K_j H2^(j+1)
// by FMA Horner (one sum when both faces share it); conic faces take the
// full evaluation
RBG_NOINLINE bool asph_contains_exact(const double* P, d3 p, bool twin) {
  RBG_EVENT(EV_CONTAINS_EXACT);
  RBG_EVENT_N(EV_HORNER64, (int)P[RBG_ASPH_NPOL1] + (twin ? 0 : (int)P[RBG_ASPH_NPOL2]));
  const double H2 = p.x * p.x + p.y * p.y;
  const double rmin = P[RBG_ASPH_RMIN], rmax = P[RBG_ASPH_RMAX];
  if (H2 > rmax * rmax || H2 < rmin * rmin) return false;
  if (P[RBG_ASPH_C1] != 0 || P[RBG_ASPH_C2] != 0) return asph_contains_fast(Asph{P}, p);
  const int n1 = (int)P[RBG_ASPH_NPOL1], n2 = (int)P[RBG_ASPH_NPOL2];
  const double p1 = asph_poly(P + RBG_ASPH_K, n1, H2);
  if (p.z < P[RBG_ASPH_Z1] + p1) return false;
  const double p2 = twin ? p1 : asph_poly(P + RBG_ASPH_K + n1, n2, H2);
  return !(P[RBG_ASPH_Z2] + p2 < p.z);
}
RBG_NOINLINE d3 asph_normal_exact(const double* P, d3 point, d3 dir) {
  RBG_EVENT(EV_NORMAL_EXACT);
  RBG_EVENT_N(EV_HORNER64, 4 * ((int)P[RBG_ASPH_NPOL1] + (int)P[RBG_ASPH_NPOL2]) / 2);
  return asph_normal_fast(Asph{P}, point, dir);
}

// DistToAsphere (src/AGeoAsphericDisk.cxx:415-526), mixed precision, in
// three parts.
//
// asph_newton_f: the reference's iteration (spherical first guess, Newton
// along the ray) in FP32 from the float parameters, relative to the face
// vertex, tracking the distance t.  Returns false when it breaks down.
RBG_D bool asph_newton_f(const float* Pf, int n, const LRay& L, float& t_out, float& scale_out,
                         float* err_out = nullptr) {
  const int npol1 = (int)Pf[RBG_ASPH_NPOL1];
  const int npol = n == 1 ? npol1 : (int)Pf[RBG_ASPH_NPOL2];
  const float* Kf = Pf + RBG_ASPH_K + (n == 1 ? 0 : npol1);
  const float curve = Pf[n == 1 ? RBG_ASPH_C1 : RBG_ASPH_C2], kappa = Pf[n == 1 ? RBG_ASPH_KAPPA1 : RBG_ASPH_KAPPA2];
  const float px = L.pf.x, py = L.pf.y, pz = L.pf.z - Pf[n == 1 ? RBG_ASPH_Z1 : RBG_ASPH_Z2];
  const float dx = L.df.x, dy = L.df.y, dz = L.df.z;
  float H2 = px * px + py * py;
  const float p = -(pz * dz + px * dx + py * dy);
  const float M = p * dz + pz;
  // the spherical first guess; a flat vertex (curve 0) takes the plane
  float tf;
  if (curve != 0.f) {
    const float M2 = pz * pz + H2 - p * p;
    const float idz = __frcp_rn(dz);
    const float check = 1.f - (M2 * curve - 2.f * M) * curve * idz * idz;
    if (!(check >= 0.f)) return false;
    tf = p + __fdividef((M2 * curve - 2.f * M) * idz, 1.f + sqrtf(check));
  } else {
    tf = p - __fdividef(M, dz);
  }
  const float ick = curve != 0.f ? __frcp_rn(curve * kappa) : 0.f;
  float nx = px + tf * dx, ny = py + tf * dy, nz = pz + tf * dz;
  for (int i = 0; i < 40; i++) {
    RBG_EVENT(EV_NEWTON32);
    RBG_EVENT_N(EV_HORNER32, npol);
    H2 = nx * nx + ny * ny;
    float l = 1.f;
    if (curve != 0.f) {
      const float ch = 1.f - kappa * H2 * curve * curve;
      if (ch < 0) return false;
      l = sqrtf(ch);
    }
    // x = sum K_j H2^(j+1) (+ the conic), v = sum (j+1) K_j H2^j
    float x = 0.f, v = 0.f, jf = (float)npol;
    for (int j = npol - 1; j >= 0; --j) {
      x = (x + Kf[j]) * H2;
      v = fmaf(v, H2, jf * Kf[j]);
      jf -= 1.f;
    }
    if (curve != 0.f) x += (1.f - l) * ick;
    // the surface gradient (l, m, nn) up to a factor; the Newton step along
    // the ray needs only the ratio of its z component to its projection
    // on the direction, so it is not normalised
    const float g = curve * kappa + l * 2.f * v;
    const float m = -nx * g, nn = -ny * g;
    const float check = dz * l + dx * m + dy * nn;
    if (check == 0.f) return false;
    const float scale = __fdividef(l, check);  // dt per unit sag residual
    const float e = scale * (x - nz);
    tf += e;
    nx += e * dx;
    ny += e * dy;
    nz += e * dz;
    if (fabsf(e) < 4e-6f * (1.f + fabsf(nz) + fabsf(nx) + fabsf(ny))) {
      if (!isfinite(tf)) return false;
      t_out = tf;
      scale_out = scale;
      if (err_out) {
        // bound on |tf - t64| (t64: the FP64 root the polish converges
        // to): the last step, plus the slope times the rounding of the
        // FP32 residual -- the float inputs (the ray's local point, the
        // vertex, the coefficients) and the Horner sum, ~10 ulps of each
        // magnitude involved -- plus the rounding of t, all four-fold
        float mag;
        asph_poly_f(Kf, npol, H2, mag);
        const float eps_r = 1.2e-6f * (mag + fabsf(x) + fabsf(L.pf.z) +
                                       fabsf(Pf[n == 1 ? RBG_ASPH_Z1 : RBG_ASPH_Z2]) + fabsf(nz) + 1.f);
        *err_out = 4.f * (fabsf(e) + fabsf(scale) * eps_r + 1e-6f * (fabsf(tf) + 1.f));
      }
      return true;
    }
  }
  return false;
}

// asph_polish: FP64 steps t += s (x(h2) - z) with the FP32 slope s from t
// until |step| < 1e-10 (the reference's stopping rule), or after a first
// step that the FP32 root leaves small (below).  Returns false when it does
// not converge in 8 steps or leaves the conic's domain.
RBG_D bool asph_polish(const double* P, int n, const LRay& L, double sc, double& t, bool fast = true) {
  const int s1 = n == 1;
  const int npol1 = (int)P[RBG_ASPH_NPOL1];
  const int npol = s1 ? npol1 : (int)P[RBG_ASPH_NPOL2];
  const double* K = P + RBG_ASPH_K + (s1 ? 0 : npol1);
  const double c64 = P[s1 ? RBG_ASPH_C1 : RBG_ASPH_C2];
  const double kap64 = P[s1 ? RBG_ASPH_KAPPA1 : RBG_ASPH_KAPPA2];
  const double pz0 = L.p.z - P[s1 ? RBG_ASPH_Z1 : RBG_ASPH_Z2];
  for (int it = 0; it < 8; ++it) {
    RBG_EVENT(EV_POLISH);
    RBG_EVENT_N(EV_HORNER64, npol > 0 ? npol - 1 : 0);
    double qx = fma(t, L.d.x, L.p.x), qy = fma(t, L.d.y, L.p.y), qz = fma(t, L.d.z, pz0);
    double h2 = fma(qx, qx, qy * qy);
    double x = asph_poly(K, npol, h2);
    if (c64 != 0) {
      double chk = 1 - kap64 * h2 * c64 * c64;
      if (chk < 0) return false;
      x += (1 - sqrt(chk)) / c64 / kap64;
    }
    double e = sc * (x - qz);
    t += e;
    if (fabs(e) < 1e-10) return true;
    // A first step below 1e-3 cm at a slope that is not grazing leaves t
    // within (the slope's relative error) x |e| of the root, ~1e-13 cm with
    // the face's own FP32 slope.  Stopping there saves the evaluation that
    // would only confirm it.  (A twin face polished with the other face's
    // slope is not `fast`: across a 1 mm shell met at 56 deg that slope is
    // ~1 % off.)
    if (fast && it == 0 && fabs(e) < 1e-3 && fabs(sc) < 10) return true;
  }
  return false;
}

// asph_accept: the distance to a converged root is t itself (the
// reference's |np - point| for a unit direction), rejected when t < 0 (its
// dot(dir, np - point) < 0) or when the hit radius lies outside
// [rmin, rmax] (compared squared)
RBG_D double asph_accept(const double* P, const LRay& L, double t) {
  if (t < 0) return kBig;
  RBG_EVENT(EV_ACCEPT);
  double qx = fma(t, L.d.x, L.p.x), qy = fma(t, L.d.y, L.p.y);
  double h2 = fma(qx, qx, qy * qy);
  const double rmin = P[RBG_ASPH_RMIN], rmax = P[RBG_ASPH_RMAX];
  if (h2 < rmin * rmin || h2 > rmax * rmax) return kBig;
  return t;
}

// Both faces.  With twin faces (same polynomial, c and kappa; vertex z
// apart by dz) the residual of face 2 at face 1's root is exactly dz, so
// face 2's polish starts from t1 + s dz without a second FP32 iteration.
RBG_D void asph_faces_f(const double* P, const float* Pf, const LRay& L, bool twin, double& d1, double& d2) {
  float tf, sf;
  double t1 = 0, sc = 1;
  bool ok1 = asph_newton_f(Pf, 1, L, tf, sf);
  if (ok1) {
    t1 = (double)tf;
    sc = (double)sf;
    ok1 = asph_polish(P, 1, L, sc, t1);
  }
  d1 = ok1 ? asph_accept(P, L, t1) : asph_dist_surface_exact(P, 1, L.p, L.d);
  double t2;
  bool ok2;
  if (twin && ok1) {
    t2 = t1 + sc * (P[RBG_ASPH_Z2] - P[RBG_ASPH_Z1]);
    ok2 = asph_polish(P, 2, L, sc, t2, false);
  } else {
    ok2 = asph_newton_f(Pf, 2, L, tf, sf);
    if (ok2) {
      t2 = (double)tf;
      ok2 = asph_polish(P, 2, L, (double)sf, t2);
    }
  }
  d2 = ok2 ? asph_accept(P, L, t2) : asph_dist_surface_exact(P, 2, L.p, L.d);
}

// FP32 screen of DistToInner/DistToOuter from the float parameters (the
// test asph_wall_maybe makes, without conversions)
RBG_D bool asph_wall_maybe_f(const float* Pf, bool outer, const LRay& L, float limit) {
  if (!outer && Pf[RBG_ASPH_RSEG] == 0.f) return false;
  RBG_EVENT(EV_SCREEN32);
  const float R = outer ? Pf[RBG_ASPH_RMAX] : Pf[RBG_ASPH_RMIN];
  const float px = L.pf.x, py = L.pf.y, pz = L.pf.z;
  const float dx = L.df.x, dy = L.df.y, dz = L.df.z;
  float nsq = dx * dx + dy * dy;
  if (nsq < 1e-20f) return false;
  float rsq = px * px + py * py, rdotn = px * dx + py * dy;
  const float insq = __frcp_rn(nsq);
  float b = rdotn * insq, delta = b * b - (rsq - R * R) * insq;
  const float pad = 1e-3f + 1e-5f * (R + fabsf(pz));
  if (delta < -pad) return false;
  float sq = sqrtf(fmaxf(delta, 0.f));
  float t1 = -b + sq, t2 = -b - sq;
  if (t1 < -pad && t2 < -pad) return false;
  const float zlo = Pf[outer ? RBG_ASPH_F1RMAX : RBG_ASPH_F1RMIN];
  const float zhi = Pf[outer ? RBG_ASPH_F2RMAX : RBG_ASPH_F2RMIN];
  if (isnan(zlo) || isnan(zhi)) return false;
  float lim = limit + pad + 1e-5f * limit;
  for (int k = 0; k < 2; ++k) {
    float t = k == 0 ? t1 : t2;
    if (t < -pad - 1e-5f * fabsf(t) || t > lim) continue;
    float z = pz + t * dz;
    if (z >= zlo - pad && z <= zhi + pad) return true;
  }
  return false;
}

// DistFromInside (:363-380): nearest of the two faces and the two walls;
// `face` = 1, 2 (faces), 3 (inner wall), 4 (outer wall) of the minimum
RBG_D double asph_dist4_f(const double* P, const float* Pf, const LRay& L, bool twin, int& face) {
  double best, v;
  asph_faces_f(P, Pf, L, twin, best, v);
  face = 1;
  if (v < best) {
    best = v;
    face = 2;
  }
  const float lim = best >= kBig ? 3e38f : (float)best;
  if (asph_wall_maybe_f(Pf, false, L, lim)) {
    v = asph_dist_wall_exact(P, false, L.p, L.d);
    if (v < best) {
      best = v;
      face = 3;
    }
  }
  if (asph_wall_maybe_f(Pf, true, L, best >= kBig ? 3e38f : (float)best)) {
    v = asph_dist_wall_exact(P, true, L.p, L.d);
    if (v < best) {
      best = v;
      face = 4;
    }
  }
  return best;
}

// DistFromOutside (:383-412): the bounding-tube screen in FP32 (enlarged,
// never rejecting a ray the exact TGeoTube test accepts), then the faces
RBG_D double asph_dist_out_f(const double* P, const float* Pf, const LRay& L, bool twin, int& face) {
  RBG_EVENT(EV_SCREEN32);
  // pad: 1e-4 cm, plus 1e-5 of the tube size and 1e-6 of the coordinates
  // (the float position and origin carry ~6e-8 relative error each)
  const float pad = 1e-4f + 1e-5f * (Pf[RBG_ASPH_RMAX] + Pf[RBG_ASPH_DZ]) +
                    1e-6f * (fabsf(L.pf.x) + fabsf(L.pf.y) + fabsf(L.pf.z) + fabsf(Pf[RBG_ASPH_ORIGIN_Z]));
  const float R = Pf[RBG_ASPH_RMAX] + pad, Z = Pf[RBG_ASPH_DZ] + pad;
  const float ox = L.pf.x, oy = L.pf.y, oz = L.pf.z - Pf[RBG_ASPH_ORIGIN_Z];
  const float dx = L.df.x, dy = L.df.y, dzz = L.df.z;
  float t0 = 0.f, t1 = 3.0e38f;
  if (dzz != 0.f) {
    const float idz = __frcp_rn(dzz);
    float ta = (-Z - oz) * idz, tb = (Z - oz) * idz;
    t0 = fmaxf(t0, fminf(ta, tb));
    t1 = fminf(t1, fmaxf(ta, tb));
  } else if (fabsf(oz) > Z) {
    return kBig;
  }
  if (t0 > t1) return kBig;
  float A = dx * dx + dy * dy, B = ox * dx + oy * dy, C = ox * ox + oy * oy - R * R;
  if (A == 0.f) {
    if (C > 0.f) return kBig;
  } else {
    float disc = B * B - A * C;
    if (disc < 0.f) return kBig;
    float sq = sqrtf(disc);
    const float iA = __frcp_rn(A);
    float c0 = (-B - sq) * iA, c1 = (-B + sq) * iA;
    const float lo = fmaxf(t0, c0), hi = fminf(t1, c1);
    if (lo > hi + pad + 1e-5f * (fabsf(lo) + fabsf(hi))) return kBig;
  }
  return asph_dist4_f(P, Pf, L, twin, face);
}

// Contains (:330-347) behind FP32 screens of the radius and of both sags
// (faces with c == 0; the screen margin is 2e-5 of the sum of the sag's term
// magnitudes plus the coordinates, >10x the FP32 rounding of the sums)
RBG_D bool asph_contains_f(const double* P, const float* Pf, const LRay& L, bool twin) {
  RBG_EVENT(EV_SCREEN32);
  const float h = L.pf.x * L.pf.x + L.pf.y * L.pf.y;
  const float rmax = Pf[RBG_ASPH_RMAX], rmin = Pf[RBG_ASPH_RMIN];
  const float hr = 4e-6f * h + 1e-12f;
  if (h > rmax * rmax * (1.f + 4e-6f) + hr) return false;
  if (h < rmin * rmin * (1.f - 4e-6f) - hr) return false;
  const bool radial_in = h < rmax * rmax * (1.f - 4e-6f) - hr && h > rmin * rmin * (1.f + 4e-6f) + hr;
  if (Pf[RBG_ASPH_C1] == 0.f && Pf[RBG_ASPH_C2] == 0.f) {
    const int n1 = (int)Pf[RBG_ASPH_NPOL1], n2 = (int)Pf[RBG_ASPH_NPOL2];
    float m1, m2;
    const float f1 = Pf[RBG_ASPH_Z1] + asph_poly_f(Pf + RBG_ASPH_K, n1, h, m1);
    const float f2 = Pf[RBG_ASPH_Z2] + asph_poly_f(Pf + RBG_ASPH_K + n1, n2, h, m2);
    const float z = L.pf.z;
    const float e1 = 2e-5f * (m1 + fabsf(Pf[RBG_ASPH_Z1]) + fabsf(z)) + 1e-7f;
    const float e2 = 2e-5f * (m2 + fabsf(Pf[RBG_ASPH_Z2]) + fabsf(z)) + 1e-7f;
    if (z < f1 - e1 || z > f2 + e2) return false;
    if (radial_in && z > f1 + e1 && z < f2 - e2) return true;
  }
  return asph_contains_exact(P, L.p, twin);
}

// TGeoBBox::Contains behind an FP32 screen
RBG_D bool box_contains_f(const double* P, const float* Pf, const LRay& L) {
  RBG_EVENT(EV_SCREEN32);
  const float ax = fabsf(L.pf.x - Pf[RBG_BOX_OX]), ay = fabsf(L.pf.y - Pf[RBG_BOX_OY]),
              az = fabsf(L.pf.z - Pf[RBG_BOX_OZ]);
  const float ex = 1e-6f * (fabsf(L.pf.x) + fabsf(Pf[RBG_BOX_OX]) + Pf[RBG_BOX_DX]) + 1e-30f;
  const float ey = 1e-6f * (fabsf(L.pf.y) + fabsf(Pf[RBG_BOX_OY]) + Pf[RBG_BOX_DY]) + 1e-30f;
  const float ez = 1e-6f * (fabsf(L.pf.z) + fabsf(Pf[RBG_BOX_OZ]) + Pf[RBG_BOX_DZ]) + 1e-30f;
  if (ax > Pf[RBG_BOX_DX] + ex || ay > Pf[RBG_BOX_DY] + ey || az > Pf[RBG_BOX_DZ] + ez) return false;
  if (ax < Pf[RBG_BOX_DX] - ex && ay < Pf[RBG_BOX_DY] - ey && az < Pf[RBG_BOX_DZ] - ez) return true;
  return prim_contains(RBG_SHAPE_BOX, P, nullptr, L.p);
}

// Lower and upper bounds of TGeoBBox::DistFromInside (the slab exit
// distance box_dist_fast computes in FP64) from the float ray.  Each
// axis's bound allows 1e-6 of the terms it is made of (the float inputs
// carry ~6e-8 relative error, three float operations follow).  Returns
// false when an axis's direction underflows to zero in float while it is
// not zero in FP64 (then only the FP64 distance is valid).
RBG_D bool box_exit_bounds_f(const float* Pf, const LRay& L, float& lo, float& hi) {
  RBG_EVENT(EV_SCREEN32);
  const float pf[3] = {L.pf.x, L.pf.y, L.pf.z}, df[3] = {L.df.x, L.df.y, L.df.z};
  const double dd[3] = {L.d.x, L.d.y, L.d.z};
  lo = 3e38f;
  hi = 3e38f;
  bool any = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (df[k] == 0.f) {
      if (dd[k] != 0.0) return false;
      continue;
    }
    const float o = pf[k] - Pf[RBG_BOX_OX + k];
    const float half = Pf[RBG_BOX_DX + k];
    const float inv = __frcp_rn(df[k]);
    const float t = ((df[k] > 0.f ? half : -half) - o) * inv;
    const float e = 1e-6f * ((fabsf(pf[k]) + fabsf(Pf[RBG_BOX_OX + k]) + half) * fabsf(inv) + fabsf(t)) + 1e-30f;
    lo = fminf(lo, t - e);
    hi = fminf(hi, t + e);
    any = true;
  }
  return any;
}

// Node-local normal of an aspheric disk at a point just past face `face`
// (1 or 2) of a crossing.  ComputeNormal (:246-327) takes the surface with
// the smallest safety distance: the crossed face is within the 1e-9 cm
// push, so a wall can only win when the point lies that close to a rim.
// When both faces share their polynomial with c == 0 (a thin shell), both
// faces have the same gradient (-2x F', -2y F', 1), and a point clearly away
// from both rims (FP32 radius test, 1e-4 cm + 1e-5 relative margin) takes
// it directly; anything else runs the full FP64 choice.
RBG_D d3 asph_normal_f(const DevScene& S, int node, const double* P, const float* Pf, const LRay& L, int face) {
  if ((face == 1 || face == 2) && (S.aux[node].flags & RBG_AUX_ASPH_TWIN_FACES) && Pf[RBG_ASPH_C1] == 0.f) {
    const float r = sqrtf(L.pf.x * L.pf.x + L.pf.y * L.pf.y);
    const float rmax = Pf[RBG_ASPH_RMAX], rmin = Pf[RBG_ASPH_RMIN];
    const float pad = 1e-4f + 1e-5f * rmax;
    const bool rim = fabsf(r - rmax) < pad || (Pf[RBG_ASPH_RSEG] != 0.f && fabsf(r - rmin) < pad);
    if (!rim) {
      const int n1 = (int)Pf[RBG_ASPH_NPOL1];
      const double H2 = L.p.x * L.p.x + L.p.y * L.p.y;
      // the derivative coefficients (j + 1) K_j come precomputed
      const double* dK = ST(S, S.nodes[node].shape) + RBG_TRIG_ASPH_DK;
      RBG_EVENT(EV_NORMAL);
      RBG_EVENT_N(EV_HORNER64, n1 > 0 ? n1 - 1 : 0);
      double dF = 0.0;
      if (n1 > 0) {
        dF = dK[n1 - 1];
        for (int j = n1 - 2; j >= 0; --j) dF = fma(dF, H2, dK[j]);
      }
      d3 n;
      if (dF == 0) {
        n = mk(0, 0, 1);
      } else {
        const double gx = -2 * L.p.x * dF, gy = -2 * L.p.y * dF;
        const double inv = rsqrt_refined(fma(gx, gx, fma(gy, gy, 1.0)));
        n = mk(gx * inv, gy * inv, inv);
      }
      if (dot(n, L.d) < 0) n = neg(n);
      return n;
    }
  }
  return asph_normal_exact(P, L.p, L.d);
}

}  // namespace rbg
