// adjoint.cu -- reverse-mode derivative of traced ray end points with respect
// to scene parameters (aspheric coefficients, rigid motions of nodes).
//
// The forward trace records every point and node of each ray (the ARay
// point/node history).  The backward pass recomputes the segments from
// those hit records -- no other state is stored -- and walks them from the
// last point to the first:
//   * intersection P = o + t d with the crossed surface f(P; theta) = 0
//     (implicit function theorem):  dP = A (do + t dd) - d f_theta dtheta / (g.d),
//     A = I - d g^T / (g.d), g = grad f;
//   * reflection d' = d - 2 (d.n) n with n = g / |g| (DoReflection,
//     src/AOpticsManager.cxx:226-230), including the curvature term
//     dn = (I - n n^T) H dP / |g| and the parameter term of g;
//   * the 1e-6 + 1e-6 cm step back after a reflection (o' = P - eps d).
//   * refraction d' = eta d + (c2 - eta c1) n at a lens face (DoFresnel's
//     transmitted direction, src/AOpticsManager.cxx:146-155; c1 = d.n with n
//     oriented along d, c2 = sqrt(1 - eta^2 (1 - c1^2)), eta = n1 / n2 at
//     the ray's wavelength), with the boundary push o' = P + 1e-9 cm d;
//     which branch a ray took (transmit, Fresnel reflection, total internal
//     reflection) is read from its recorded path and held fixed, as the
//     random draws are.
// Straight-through crossings (entering an AOpticalComponent, or a medium of
// the same index) do not change the path and are collapsed.
#include <cuda_runtime.h>

#include <cstring>

#include "scene_internal.h"
#include "device_state.cuh"
#include "tracer.cuh"

namespace rbg {

constexpr int kAdjMaxParams = 64;
constexpr int kAdjMaxEvents = 24;
constexpr int kAdjThreads = 128;            // threads per block
constexpr int kAdjTile = 16 * kAdjThreads;  // rays per tile

struct Surf {
  d3 g;         // gradient of f in the master frame
  // Hessian of f = Q Hl Q^T: Q (row-major, local -> master) the frame the
  // surface is written in, Hl its symmetric local Hessian (h00 h01 h02 h11
  // h12 h22)
  double Q[9];
  double h[6];
  // for aspheric faces: local point, face and polynomial length
  int face;     // 1 lower, 2 upper, 0 not an aspheric face
  int npol;
  double H2, x, y;
};

RBG_D d3 cross(d3 a, d3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
RBG_D double comp(d3 v, int a) { return a == 0 ? v.x : a == 1 ? v.y : v.z; }

// H v = Q (Hl (Q^T v)); also returns Q^T v (the local components of v)
RBG_D d3 hess_vec(const Surf& sf, d3 v, d3& vl) {
  vl = dir_to_local(sf.Q, v);
  const double* h = sf.h;
  const d3 hl = mk(h[0] * vl.x + h[1] * vl.y + h[2] * vl.z, h[1] * vl.x + h[3] * vl.y + h[4] * vl.z,
                   h[2] * vl.x + h[4] * vl.y + h[5] * vl.z);
  return dir_to_master(sf.Q, hl);
}

// The nearest surface among the leaves of a TGeo primitive or composite
// (spheres, paraboloids, cylinders, planes; each leaf's Hessian is diagonal
// in its own frame): fills out.Q and out.h and returns the gradient in the
// leaf's frame.  Kept out of line: its traversal stack stays out of the
// aspheric path's registers and frame.
__device__ __noinline__ d3 leaf_surface(const DevScene& S, const rbg_node& N, d3 p, Surf& out) {
  d3 gl;
  // nearest surface among the leaves (spheres, paraboloids, cylinders,
  // planes); each leaf's Hessian is diagonal in its own frame
  double best = kBig;
  M12 bestM = mat_identity();
  d3 bg = mk(0, 0, 1);
  double bh0 = 0, bh4 = 0, bh8 = 0;
  int stack_shape[8];
  M12 stack_m[8];
  int sp = 0;
  stack_shape[sp] = N.shape;
  stack_m[sp] = mat_identity();
  ++sp;
  while (sp > 0) {
    --sp;
    int sid = stack_shape[sp];
    M12 M = stack_m[sp];
    const rbg_shape_desc ss = S.shapes[sid];
    const double* Pp = SP(S, sid);
    if (ss.type == RBG_SHAPE_COMPOSITE) {
      if (sp + 2 > 8) continue;
      stack_shape[sp] = ss.left;
      stack_m[sp] = mat_mul(M.v, Pp + RBG_COMP_ML);
      ++sp;
      stack_shape[sp] = ss.right;
      stack_m[sp] = mat_mul(M.v, Pp + RBG_COMP_MR);
      ++sp;
      continue;
    }
    d3 q = to_local(M.v, p);
    auto consider = [&](double dist, d3 g, double h0, double h4, double h8) {
      if (dist < best) {
        best = dist;
        bestM = M;
        bg = g;
        bh0 = h0;
        bh4 = h4;
        bh8 = h8;
      }
    };
    switch (ss.type) {
      case RBG_SHAPE_SPHERE: {
        double rq = sqrt(dot(q, q));
        consider(fabs(rq - Pp[RBG_SPH_RMAX]), 2.0 * q, 2, 2, 2);
        if (Pp[RBG_SPH_RMIN] > 0) consider(fabs(rq - Pp[RBG_SPH_RMIN]), 2.0 * q, 2, 2, 2);
        break;
      }
      case RBG_SHAPE_PARABOLOID: {
        double A = Pp[RBG_PARA_A];
        d3 g = mk(2 * A * q.x, 2 * A * q.y, -1);
        consider(fabs(A * (q.x * q.x + q.y * q.y) + Pp[RBG_PARA_B] - q.z) / sqrt(dot(g, g)), g, 2 * A, 2 * A, 0);
        consider(fabs(fabs(q.z) - Pp[RBG_PARA_DZ]), mk(0, 0, 1), 0, 0, 0);
        break;
      }
      case RBG_SHAPE_BOX: {
        consider(fabs(fabs(q.x - Pp[RBG_BOX_OX]) - Pp[RBG_BOX_DX]), mk(1, 0, 0), 0, 0, 0);
        consider(fabs(fabs(q.y - Pp[RBG_BOX_OY]) - Pp[RBG_BOX_DY]), mk(0, 1, 0), 0, 0, 0);
        consider(fabs(fabs(q.z - Pp[RBG_BOX_OZ]) - Pp[RBG_BOX_DZ]), mk(0, 0, 1), 0, 0, 0);
        break;
      }
      case RBG_SHAPE_TUBE: {
        double rq = sqrt(q.x * q.x + q.y * q.y);
        consider(fabs(rq - Pp[RBG_TUBE_RMAX]), mk(2 * q.x, 2 * q.y, 0), 2, 2, 0);
        if (Pp[RBG_TUBE_RMIN] > 0) consider(fabs(rq - Pp[RBG_TUBE_RMIN]), mk(2 * q.x, 2 * q.y, 0), 2, 2, 0);
        consider(fabs(fabs(q.z) - Pp[RBG_TUBE_DZ]), mk(0, 0, 1), 0, 0, 0);
        break;
      }
      case RBG_SHAPE_PGON: {
        // flat faces only (the prism sides and the section planes)
        const int ned = (int)Pp[2], nz = (int)Pp[3];
        const double* Z = Pp + 4;
        for (int k = 0; k < nz; ++k) consider(fabs(q.z - Z[k]), mk(0, 0, 1), 0, 0, 0);
        const double* RMAX = Z + 2 * nz;
        for (int k = 0; k + 1 < nz; ++k) {
          double h = Z[k + 1] - Z[k];
          if (h <= 0) continue;
          double s = (RMAX[k + 1] - RMAX[k]) / h;
          for (int e = 0; e < ned; ++e) {
            double pe = (Pp[0] + (e + 0.5) * (Pp[1] / ned)) * kD2R;
            d3 nn = mk(cos(pe), sin(pe), -s);
            double v = dot(nn, q) - (RMAX[k] - s * Z[k]);
            consider(fabs(v) / sqrt(dot(nn, nn)), nn, 0, 0, 0);
          }
        }
        break;
      }
      default:
        break;
    }
  }
  // the leaf's frame in the master frame: Q = R_node R_leaf
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      out.Q[i * 3 + j] = N.m[i * 3] * bestM.v[j] + N.m[i * 3 + 1] * bestM.v[3 + j] + N.m[i * 3 + 2] * bestM.v[6 + j];
  out.h[0] = bh0;
  out.h[3] = bh4;
  out.h[5] = bh8;
  gl = bg;
  return gl;
}

// Implicit function of the surface of node `node` nearest to the master
// point P: value is ignored, only g and H are needed.  Returns false for
// shapes whose surfaces the adjoint does not differentiate.
//
// Aspheric face f = z - F(H2), H2 = x^2 + y^2,
// F = z0 + c H2 / (1 + s) + sum K_j H2^(j+1), s = sqrt(1 - kappa c^2 H2);
// the conic part equals (1 - s) / (kappa c), so dF/dH2 = c / (2 s) + ...
// and d2F/dH2^2 = kappa c^3 / (4 s^3) + ...  The face nearest to P is the
// one of least |z - F| / sqrt(1 + 4 H2 F'^2), compared without roots.
RBG_D bool surface_at(const DevScene& S, int node, d3 P, Surf& out) {
  const rbg_node& N = S.nodes[node];
  const rbg_shape_desc sh = S.shapes[N.shape];
  const d3 p = to_local(N.m, P);
  out.face = 0;
  out.npol = 0;
  out.H2 = out.x = out.y = 0;
  for (int i = 0; i < 6; ++i) out.h[i] = 0;
  d3 gl;
  if (sh.type == RBG_SHAPE_ASPHERIC_DISK) {
    for (int i = 0; i < 9; ++i) out.Q[i] = N.m[i];
    Asph a{SP(S, N.shape)};
    const double H2 = p.x * p.x + p.y * p.y;
    // nearest face: dist^2 = dz^2 / q, compared as dz_a^2 q_b < dz_b^2 q_a.
    // Twin faces (the same curvature, conic and polynomial, the vertices
    // z2 - z1 apart: a thin mirror shell) share F - z0, F' and q, so one
    // evaluation decides between them.
    double best_dz2 = kBig * kBig, best_q = 1.0, best_dF = 0, best_rs = 0;
    int face = 0;
    const bool twin = (S.aux[node].flags & RBG_AUX_ASPH_TWIN_FACES) != 0;
    for (int f = 1; f <= (twin ? 1 : 2); ++f) {
      const double c = a.c(f), k = a.kap(f);
      const double chk = 1 - k * c * c * H2;
      if (chk <= 0) continue;
      const double s = sqrt(chk);
      const double inv = 1.0 / (s * (1 + s));  // 1/s = (1 + s) inv, 1/(1 + s) = s inv
      const double rs = (1 + s) * inv;
      const int n = a.npol(f);
      const double* K = a.K(f);
      double pp = 0, dp = 0;
      for (int j = n - 1; j >= 0; --j) {
        pp = (pp + K[j]) * H2;
        dp = dp * H2 + (j + 1) * K[j];
      }
      const double F = a.z(f) + H2 * c * (s * inv) + pp;
      const double dF = 0.5 * c * rs + dp;
      const double dz = p.z - F, q = 1 + 4 * H2 * dF * dF;
      if (dz * dz * best_q < best_dz2 * q) {
        best_dz2 = dz * dz;
        best_q = q;
        best_dF = dF;
        best_rs = rs;
        face = f;
      }
      if (twin) {
        const double dz2 = dz - (a.z(2) - a.z(1));  // p.z - F2
        if (dz2 * dz2 < best_dz2) {
          best_dz2 = dz2 * dz2;
          face = 2;
        }
      }
    }
    const double r = sqrt(H2);
    double wall = fabs(r - a.rmax());
    if (a.rseg()) wall = fmin(wall, fabs(r - a.rmin()));
    if (face == 0 || wall * wall * best_q < best_dz2) {
      // side wall: f = x^2 + y^2 - R^2
      gl = mk(2 * p.x, 2 * p.y, 0);
      out.h[0] = 2;
      out.h[3] = 2;
    } else {
      // f = z - F(x^2 + y^2)
      const double c = a.c(face), k = a.kap(face);
      const int n = a.npol(face);
      const double* K = a.K(face);
      double d2p = 0;  // sum (j+1) j K_j H2^(j-1)
      for (int j = n - 1; j >= 1; --j) d2p = d2p * H2 + (j + 1) * j * K[j];
      const double dF = best_dF, rs3 = best_rs * best_rs * best_rs;
      const double d2F = 0.25 * k * c * c * c * rs3 + d2p;
      gl = mk(-2 * p.x * dF, -2 * p.y * dF, 1);
      out.h[0] = -2 * dF - 4 * p.x * p.x * d2F;
      out.h[1] = -4 * p.x * p.y * d2F;
      out.h[3] = -2 * dF - 4 * p.y * p.y * d2F;
      out.face = face;
      out.npol = n;
      out.H2 = H2;
      out.x = p.x;
      out.y = p.y;
    }
  } else if (sh.type == RBG_SHAPE_COMPOSITE || sh.type == RBG_SHAPE_SPHERE || sh.type == RBG_SHAPE_BOX ||
             sh.type == RBG_SHAPE_TUBE || sh.type == RBG_SHAPE_PARABOLOID || sh.type == RBG_SHAPE_PGON) {
    gl = leaf_surface(S, N, p, out);
  } else {
    return false;
  }
  out.g = dir_to_master(out.Q, gl);
  return true;
}

// true if `anc` is node k or one of its ancestors
RBG_D bool moves_with(const DevScene& S, int anc, int k) {
  for (int d = 0; k >= 0 && d < 64; ++d) {
    if (k == anc) return true;
    k = S.nodes[k].parent;
  }
  return false;
}

// the parameter list travels by value in the launch's parameter space
struct AdjParams {
  rbg_adjoint_param p[kAdjMaxParams];
};

// true if `anc` is an ancestor of node k (or k itself)
RBG_D bool is_within(const DevScene& S, int anc, int k) { return anc >= 0 && moves_with(S, anc, k); }

// refractive index of the medium of node k at lam (1 outside lenses)
RBG_D double medium_n(const DevScene& S, int k, double lam) {
  if (k < 0 || S.nodes[k].kind != RBG_KIND_LENS) return 1.0;
  return index_n(S, S.volumes[S.nodes[k].volume].index, lam);
}

// Event kinds of a recorded path: a point where the direction changes by a
// reflection (mirror, Fresnel or total internal reflection) or by a
// refraction; straight crossings between media of equal index are collapsed
enum { kEvStart = 0, kEvReflect = 1, kEvRefract = 2, kEvFinal = 3 };

// acc[k] += gbar . dg_k + c df_k over the parameters, with dg_k, df_k the
// derivatives of the implicit function's gradient and value (unrolled to
// MAXP so that the accumulators stay in registers):
//   * coefficient K_j of the hit face:  df = -H2^(j+1), dg = Q (-2 (j+1)
//     H2^j (x, y, 0)), so the term is H2^j (-2 (j+1) u - c H2) with
//     u = (Q^T gbar) . (x, y, 0);
//   * shift of a node the surface moves with, along axis a:  df = -g_a,
//     dg = -H e_a, so the term is -w_a with w = H gbar + c g;
//   * rotation about axis a through pivot o:  df = (g x r)_a, dg = e_a x g +
//     H (r x e_a), r = P - o, so the term is (g x gbar)_a + (w x r)_a.
// moves_with is evaluated once per distinct parameter node.
// coefficient terms H2^j (-2 (j + 1) u - c H2) tabulated for j < kCoefTab
// once per event, when a parameter needs one
constexpr int kCoefTab = 8;

template <int MAXP>
RBG_D void add_terms(const DevScene& S, const rbg_adjoint_param* params, int n_params, int node, d3 P, const Surf& sf,
                     double u, d3 w, d3 gxgbar, double c, double* acc) {
  int last_node = -1, last_moves = 0;
  bool coef = false;
  if (sf.face != 0)
    for (int k = 0; k < n_params; ++k) coef |= params[k].kind == RBG_ADJ_ASPH_COEF && params[k].node == node;
  double tab[kCoefTab];
  if (coef) {
    const double cH2 = c * sf.H2;
    double pw = 1.0;
#pragma unroll
    for (int j = 0; j < kCoefTab; ++j) {
      tab[j] = pw * (-2.0 * (j + 1) * u - cH2);
      pw *= sf.H2;
    }
  }
#pragma unroll
  for (int k = 0; k < MAXP; ++k) {
    if (k >= n_params) break;
    const rbg_adjoint_param& p = params[k];
    const int a = p.index;
    if (p.kind == RBG_ADJ_ASPH_COEF) {
      if (p.node != node || sf.face == 0 || !(p.faces & (1 << (sf.face - 1))) || a < 0 || a >= sf.npol) continue;
      double term = tab[0];
      if (a < kCoefTab) {
#pragma unroll
        for (int j = 1; j < kCoefTab; ++j) term = a == j ? tab[j] : term;
      } else {
        double hj = 1, b = sf.H2;  // H2^j by squaring
        for (int e = a; e; e >>= 1, b *= b)
          if (e & 1) hj *= b;
        term = hj * (-2.0 * (a + 1) * u - c * sf.H2);
      }
      acc[k] += term;
      continue;
    }
    if (p.node != last_node) {
      last_node = p.node;
      last_moves = moves_with(S, p.node, node);
    }
    if (!last_moves) continue;
    if (p.kind == RBG_ADJ_NODE_SHIFT) {
      acc[k] -= comp(w, a);
    } else if (p.kind == RBG_ADJ_NODE_ROTATE) {
      const d3 r = P - mk(p.pivot[0], p.pivot[1], p.pivot[2]);
      acc[k] += comp(gxgbar, a) + comp(cross(w, r), a);
    }
  }
}

template <int MAXP>
__global__ void __launch_bounds__(kAdjThreads) adjoint_kernel(DevScene S, int64_t n, const uint8_t* status, const int32_t* npoints,
                               int32_t hist_cap, const double* hist_xyzt, const int32_t* hist_node,
                               const double* lambda, const double* gx, const double* gy, const double* gz,
                               const double* gpts, int n_params, const __grid_constant__ AdjParams params_v, double* out,
                               unsigned long long* skipped) {
  __shared__ rbg_adjoint_param params[kAdjMaxParams];
  for (int k = threadIdx.x; k < n_params; k += blockDim.x) params[k] = params_v.p[k];
  __syncthreads();
  double acc[MAXP];
#pragma unroll
  for (int k = 0; k < MAXP; ++k) acc[k] = 0;
  unsigned long long nskip = 0;
  // Rays are taken in tiles of kAdjTile: the rays of a tile with a
  // non-zero cotangent are listed in shared memory first (a warp ballot and
  // one shared atomic per warp), then the block's threads walk that list,
  // so no lane idles on a ray that contributes nothing (rays that missed
  // the focal surface, rays outside the loss)
  __shared__ int32_t tile[kAdjTile];
  __shared__ int tile_n;
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * kAdjTile; base < n; base += (int64_t)gridDim.x * kAdjTile) {
    if (threadIdx.x == 0) tile_n = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < kAdjTile; k += blockDim.x) {
      const int64_t i = base + k;
      bool act = false;
      if (i < n) {
        bool any = (gx && gx[i] != 0) || (gy && gy[i] != 0) || (gz && gz[i] != 0);
        const int np = npoints[i];
        // cotangents of the recorded points (hit records), when given
        const double* gp = gpts ? gpts + (size_t)i * hist_cap * 3 : nullptr;
        for (int j = 0; gp && !any && j < np && j < hist_cap; ++j)
          any = gp[3 * j] != 0 || gp[3 * j + 1] != 0 || gp[3 * j + 2] != 0;
        if (any) {
          if (np < 2 || np > hist_cap) ++nskip;
          else act = true;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, act);
      int slot = 0;
      if (lane == 0 && m) slot = atomicAdd(&tile_n, __popc(m));
      slot = __shfl_sync(0xffffffffu, slot, 0);
      if (act) tile[slot + __popc(m & ((1u << lane) - 1u))] = k;
    }
    __syncthreads();
    const int count = tile_n;
    for (int t = threadIdx.x; t < count; t += blockDim.x) {
      const int64_t i = base + tile[t];
      d3 Pbar = mk(gx ? gx[i] : 0.0, gy ? gy[i] : 0.0, gz ? gz[i] : 0.0);
      const int np = npoints[i];
      const double* gp = gpts ? gpts + (size_t)i * hist_cap * 3 : nullptr;
      auto gpt = [&](int j) { return gp ? mk(gp[3 * j], gp[3 * j + 1], gp[3 * j + 2]) : mk(0, 0, 0); };
      const double* h = hist_xyzt + (size_t)i * hist_cap * 4;
      const int32_t* hn = hist_node + (size_t)i * hist_cap;
      auto pt = [&](int j) { return mk(h[4 * j], h[4 * j + 1], h[4 * j + 2]); };
      const double lam = lambda ? lambda[i] : 0.0;
      const bool lenses = S.features & kFeatLens;
      // events: the start, every reflection and refraction, the final point.
      // Media (for refractions) are located at the midpoints of the recorded
      // segments; a point between two media of equal index is straight.
      int ev[kAdjMaxEvents], evk[kAdjMaxEvents], evs[kAdjMaxEvents];
      double eta[kAdjMaxEvents];
      int ne = 0;
      bool ok = true;
      ev[ne] = 0;
      evk[ne] = kEvStart;
      evs[ne] = -1;
      eta[ne] = 1.0;
      ++ne;
      int m_prev = lenses ? locate_from_top(S, 0.5 * (pt(0) + pt(1))) : -1;
      for (int j = 1; j < np - 1 && ok; ++j) {
        const int k = hn[j];
        const int kind = k >= 0 ? S.nodes[k].kind : kNull;
        int m_next = -1;
        if (lenses) m_next = locate_from_top(S, 0.5 * (pt(j) + pt(j + 1)));
        int ekind = -1, snode = -1;
        double e_eta = 1.0;
        if (kind == RBG_KIND_MIRROR) {
          ekind = kEvReflect;
          snode = k;
        } else if (lenses) {
          const double n_in = medium_n(S, m_prev, lam), n_out = medium_n(S, m_next, lam);
          const d3 din = normalized(pt(j) - pt(j - 1)), dout = normalized(pt(j + 1) - pt(j));
          if (m_prev == m_next && dot(din - dout, din - dout) > 1e-18) {
            // Fresnel or total internal reflection at a lens face
            ekind = kEvReflect;
            snode = (m_prev >= 0 && S.nodes[m_prev].kind == RBG_KIND_LENS) ? m_prev : k;
          } else if (n_in != n_out) {
            ekind = kEvRefract;
            e_eta = n_in / n_out;
            // the crossed surface belongs to the node entered, or to the one left
            snode = is_within(S, m_prev, m_next) && m_next != m_prev ? m_next : m_prev;
          }
        }
        if (ekind >= 0) {
          if (ne >= kAdjMaxEvents - 1 || snode < 0) {
            ok = false;
            break;
          }
          ev[ne] = j;
          evk[ne] = ekind;
          evs[ne] = snode;
          eta[ne] = e_eta;
          ++ne;
        }
        m_prev = m_next;
      }
      if (!ok) {
        ++nskip;
        continue;
      }
      ev[ne] = np - 1;
      evk[ne] = kEvFinal;
      ++ne;
      // final point: intersection with the surface of the entered node (or
      // the top volume when the ray left it)
      int m = ne - 1;
      Pbar = Pbar + gpt(ev[m]);
      d3 Pm = pt(ev[m]);
      d3 Pprev = pt(ev[m - 1]);
      d3 dseg = normalized(Pm - Pprev);
      double tseg = sqrt(dot(Pm - Pprev, Pm - Pprev));
      int fnode = hn[ev[m]];
      if (fnode < 0) fnode = 0;
      Surf sf;
      if (!surface_at(S, fnode, Pm, sf)) {
        ++nskip;
        continue;
      }
      double gd = dot(sf.g, dseg);
      if (gd == 0) {
        ++nskip;
        continue;
      }
      const double cf = -dot(Pbar, dseg) / gd;
      // at the final point gbar = 0: only the value terms c df remain
      add_terms<MAXP>(S, params, n_params, fnode, Pm, sf, 0.0, cf * sf.g, mk(0, 0, 0), cf, acc);
      d3 obar = Pbar + cf * sf.g;
      d3 dbar = tseg * obar;
      for (int e = m - 1; e >= 1; --e) {
        const d3 Prec = pt(ev[e]);
        const d3 Pin = pt(ev[e - 1]);
        const d3 seg = Prec - Pin;
        const double L = sqrt(dot(seg, seg));
        if (!(L > 0)) {
          ok = false;
          break;
        }
        const d3 din = (1.0 / L) * seg;
        const bool refl = evk[e] == kEvReflect;
        // recorded point: reflection = hit - eps d_in (the step back),
        // refraction = hit + push d_in (the boundary push)
        const double off = refl ? -RBG_REFLECT_BACKSTEP : RBG_BOUNDARY_PUSH;
        const d3 Phit = Prec - off * din;
        const double t_in = L - off;
        const int node = evs[e];
        if (!surface_at(S, node, Phit, sf)) {
          ok = false;
          break;
        }
        const double rgn = rsqrt(dot(sf.g, sf.g));  // 1 / |g|
        // o_next = the recorded point = Phit + off d_in, with its own cotangent
        const d3 Precbar = obar + gpt(ev[e]);
        d3 Phbar = Precbar;
        d3 dinbar = off * Precbar;
        d3 gbar;
        if (refl) {
          const d3 nrm = rgn * sf.g;
          // d_out = din - 2 (din.n) n
          const double dn = dot(din, nrm), ndb = dot(nrm, dbar);
          dinbar = dinbar + dbar - (2 * ndb) * nrm;
          const d3 nbar = (-2.0) * (dn * dbar + ndb * din);
          gbar = rgn * (nbar - dot(nrm, nbar) * nrm);
        } else {
          // d_out = eta din + (c2 - eta c1) nh, nh = s g / |g| oriented along
          // din, c1 = din.nh, c2 = sqrt(1 - eta^2 (1 - c1^2))
          const double sgn = dot(sf.g, din) < 0 ? -1.0 : 1.0;
          const d3 nh = (sgn * rgn) * sf.g;
          const double et = eta[e];
          const double c1 = dot(din, nh);
          const double s2 = 1 - et * et * (1 - c1 * c1);
          if (!(s2 > 0)) {
            ok = false;
            break;
          }
          const double c2 = sqrt(s2);
          const double kk = et * et * c1 / c2 - et, sd = dot(nh, dbar);
          dinbar = dinbar + et * dbar + (kk * sd) * nh;
          const d3 nhbar = (c2 - et * c1) * dbar + (kk * sd) * din;
          gbar = (sgn * rgn) * (nhbar - dot(nh, nhbar) * nh);
        }
        d3 gbl;  // gbar in the surface's frame
        const d3 Hgbar = hess_vec(sf, gbar, gbl);
        Phbar = Phbar + Hgbar;
        const double gdi = dot(sf.g, din);
        if (gdi == 0) {
          ok = false;
          break;
        }
        const double c = -dot(Phbar, din) / gdi;
        add_terms<MAXP>(S, params, n_params, node, Phit, sf, gbl.x * sf.x + gbl.y * sf.y, Hgbar + c * sf.g,
                        cross(sf.g, gbar), c, acc);
        obar = Phbar + c * sf.g;
        dbar = dinbar + t_in * obar;
      }
      if (!ok) ++nskip;
    }
    __syncthreads();  // the tile list is rewritten next
  }
  // warp reduction, one atomic per warp and parameter
#pragma unroll
  for (int k = 0; k < MAXP; ++k) {
    if (k >= n_params) break;
    double v = acc[k];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0 && v != 0) atomicAdd(out + k, v);
  }
  for (int off = 16; off > 0; off >>= 1) nskip += __shfl_down_sync(0xffffffffu, nskip, off);
  if ((threadIdx.x & 31) == 0 && nskip) atomicAdd(skipped, nskip);
  (void)status;
}

}  // namespace rbg

using namespace rbg;

extern "C" int rbg_trace_adjoint(rbg_scene* s, int64_t n, const rbg_result* fwd, const double* lambda,
                                 const double* gx, const double* gy, const double* gz, const double* g_points,
                                 int32_t n_params,
                                 const rbg_adjoint_param* params, double* dL_dparams, int64_t* n_skipped,
                                 void* stream) {
  if (!s || !fwd || n < 0 || n_params < 0 || n_params > kAdjMaxParams || (n_params > 0 && (!params || !dL_dparams)))
    return RBG_ERR_ARG;
  if (!fwd->npoints || fwd->hist_cap <= 0 || !fwd->hist_xyzt || !fwd->hist_node) return RBG_ERR_ARG;
  if ((s->features & kFeatLens) && n > 0 && !lambda) return RBG_ERR_ARG;  // refractive indices need it
  int rc = ensure_device(s);
  if (rc) return rc;
  for (int k = 0; k < n_params; ++k) {
    const rbg_adjoint_param& p = params[k];
    if (p.kind < RBG_ADJ_ASPH_COEF || p.kind > RBG_ADJ_NODE_ROTATE) return RBG_ERR_ARG;
    if (p.node < 0 || p.node >= (int)s->nodes.size()) return RBG_ERR_ARG;
    if (p.kind != RBG_ADJ_ASPH_COEF && (p.index < 0 || p.index > 2)) return RBG_ERR_ARG;
  }
  if (n == 0 || n_params == 0) {
    if (n_skipped) *n_skipped = 0;
    return RBG_OK;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the parameters go by value with the launch; the skip counter is a word
  // of the scene's own error block (allocated with its tables)
  AdjParams pv;
  std::memset(&pv, 0, sizeof(pv));
  for (int k = 0; k < n_params; ++k) pv.p[k] = params[k];
  unsigned long long* dskip = s->dev->adj_skip;
  if (cudaMemsetAsync(dskip, 0, sizeof(unsigned long long), st) != cudaSuccess) return RBG_ERR_CUDA;
  const int block = kAdjThreads;
  const int blocks = (int)std::min<int64_t>((n + kAdjTile - 1) / kAdjTile, (int64_t)sm_count() * 8);
  // a small parameter list keeps its accumulators in registers
  if (n_params <= 24)
    adjoint_kernel<24><<<blocks, block, 0, st>>>(s->dev->view, n, fwd->status, fwd->npoints, fwd->hist_cap,
                                                 fwd->hist_xyzt, fwd->hist_node, lambda, gx, gy, gz, g_points,
                                                 n_params, pv, dL_dparams, dskip);
  else
    adjoint_kernel<kAdjMaxParams><<<blocks, block, 0, st>>>(s->dev->view, n, fwd->status, fwd->npoints,
                                                            fwd->hist_cap, fwd->hist_xyzt, fwd->hist_node, lambda,
                                                            gx, gy, gz, g_points, n_params, pv, dL_dparams, dskip);
  if (cudaGetLastError() != cudaSuccess) return RBG_ERR_CUDA;
  unsigned long long sk = 0;
  if (cudaMemcpyAsync(&sk, dskip, sizeof(sk), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return RBG_ERR_CUDA;
  if (n_skipped) *n_skipped = (int64_t)sk;
  return RBG_OK;
}
