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

struct Surf {
  d3 g;         // gradient of f in the master frame
  double H[9];  // Hessian of f in the master frame
  // for aspheric faces: local point, face and derivative ingredients
  int face;     // 1 lower, 2 upper, 0 not an aspheric face
  double H2, x, y;
  const double* R;  // node rotation (local -> master)
};

RBG_D d3 mat_vec(const double* R, d3 v) {
  return mk(R[0] * v.x + R[1] * v.y + R[2] * v.z, R[3] * v.x + R[4] * v.y + R[5] * v.z,
            R[6] * v.x + R[7] * v.y + R[8] * v.z);
}
RBG_D d3 sym_vec(const double* H, d3 v) {
  return mk(H[0] * v.x + H[1] * v.y + H[2] * v.z, H[3] * v.x + H[4] * v.y + H[5] * v.z,
            H[6] * v.x + H[7] * v.y + H[8] * v.z);
}
RBG_D d3 cross(d3 a, d3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

// H_w = R Hl R^T
RBG_D void rotate_hessian(const double* R, const double* Hl, double* Hw) {
  double T[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T[i * 3 + j] = R[i * 3] * Hl[j] + R[i * 3 + 1] * Hl[3 + j] + R[i * 3 + 2] * Hl[6 + j];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Hw[i * 3 + j] = T[i * 3] * R[j * 3] + T[i * 3 + 1] * R[j * 3 + 1] + T[i * 3 + 2] * R[j * 3 + 2];
}

// Sag of an aspheric face and its first two derivatives in H2 = x^2 + y^2:
// F = z0 + c H2 / (1 + s) + sum K_j H2^(j+1), s = sqrt(1 - kappa c^2 H2);
// the conic part equals (1 - s) / (kappa c), so dF = c / (2 s) + ..., and
// d2F = kappa c^3 / (4 s^3) + ...
RBG_D bool asph_sag2(const Asph& a, int face, double H2, double& F, double& dF, double& d2F) {
  double c = a.c(face), k = a.kap(face);
  double chk = 1 - k * c * c * H2;
  if (chk <= 0) return false;
  double s = sqrt(chk);
  int n = a.npol(face);
  const double* K = a.K(face);
  double p = 0, dp = 0, d2p = 0;
  for (int j = n - 1; j >= 0; --j) {
    p = (p + K[j]) * H2;
    dp = dp * H2 + (j + 1) * K[j];
    d2p = j >= 1 ? d2p * H2 + (j + 1) * j * K[j] : d2p;
  }
  // d2p above accumulates sum (j+1) j K_j H2^(j-1) by Horner over j >= 1
  F = a.z(face) + H2 * c / (1 + s) + p;
  dF = c / (2 * s) + dp;
  d2F = k * c * c * c / (4 * s * s * s) + d2p;
  return true;
}

// Implicit function of the surface of node `node` nearest to the master
// point P: value is ignored, only g and H are needed.  Returns false for
// shapes whose surfaces the adjoint does not differentiate.
RBG_D bool surface_at(const DevScene& S, int node, d3 P, Surf& out) {
  const rbg_node& N = S.nodes[node];
  const rbg_shape_desc sh = S.shapes[N.shape];
  d3 p = to_local(N.m, P);
  out.R = N.m;
  out.face = 0;
  double Hl[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  d3 gl;
  if (sh.type == RBG_SHAPE_ASPHERIC_DISK) {
    Asph a{SP(S, N.shape)};
    double H2 = p.x * p.x + p.y * p.y;
    double best = kBig;
    int face = 0;
    double dF = 0, d2F = 0;
    for (int f = 1; f <= 2; ++f) {
      double Ff, dFf, d2Ff;
      if (!asph_sag2(a, f, H2, Ff, dFf, d2Ff)) continue;
      double dist = fabs(p.z - Ff) / sqrt(1 + 4 * H2 * dFf * dFf);
      if (dist < best) {
        best = dist;
        face = f;
        dF = dFf;
        d2F = d2Ff;
      }
    }
    double r = sqrt(H2);
    double wall = fabs(r - a.rmax());
    if (a.rseg()) wall = fmin(wall, fabs(r - a.rmin()));
    if (face == 0 || wall < best) {
      // side wall: f = x^2 + y^2 - R^2
      gl = mk(2 * p.x, 2 * p.y, 0);
      Hl[0] = 2;
      Hl[4] = 2;
    } else {
      // f = z - F(x^2 + y^2)
      gl = mk(-2 * p.x * dF, -2 * p.y * dF, 1);
      Hl[0] = -2 * dF - 4 * p.x * p.x * d2F;
      Hl[1] = Hl[3] = -4 * p.x * p.y * d2F;
      Hl[4] = -2 * dF - 4 * p.y * p.y * d2F;
      out.face = face;
      out.H2 = H2;
      out.x = p.x;
      out.y = p.y;
    }
  } else if (sh.type == RBG_SHAPE_COMPOSITE || sh.type == RBG_SHAPE_SPHERE || sh.type == RBG_SHAPE_BOX ||
             sh.type == RBG_SHAPE_TUBE || sh.type == RBG_SHAPE_PARABOLOID || sh.type == RBG_SHAPE_PGON) {
    // nearest surface among the leaves (spheres, paraboloids, cylinders, planes)
    double best = kBig;
    M12 bestM = mat_identity();
    d3 bg = mk(0, 0, 1);
    double bH[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
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
          for (int i = 0; i < 9; ++i) bH[i] = 0;
          bH[0] = h0;
          bH[4] = h4;
          bH[8] = h8;
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
    // leaf frame -> node frame
    gl = dir_to_master(bestM.v, bg);
    rotate_hessian(bestM.v, bH, Hl);
  } else {
    return false;
  }
  out.g = dir_to_master(N.m, gl);
  rotate_hessian(N.m, Hl, out.H);
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

// d f / d theta and d g / d theta of parameter `p` at a hit on `node`
RBG_D bool param_terms(const DevScene& S, const rbg_adjoint_param& p, int node, d3 P, const Surf& sf, double& df,
                       d3& dg, int moves = -1) {
  if (p.kind == RBG_ADJ_ASPH_COEF) {
    if (p.node != node || sf.face == 0 || !(p.faces & (1 << (sf.face - 1)))) return false;
    Asph a{SP(S, S.nodes[node].shape)};
    int j = p.index;
    if (j < 0 || j >= a.npol(sf.face)) return false;
    double hj = 1, b = sf.H2;  // H2^j by squaring
    for (int e = j; e; e >>= 1, b *= b)
      if (e & 1) hj *= b;
    df = -hj * sf.H2;                           // -H2^(j+1)
    d3 gl = mk(-2 * sf.x * (j + 1) * hj, -2 * sf.y * (j + 1) * hj, 0);
    dg = dir_to_master(sf.R, gl);
    return true;
  }
  if (!(moves >= 0 ? moves != 0 : moves_with(S, p.node, node))) return false;
  const int a = p.index;
  d3 e = mk(a == 0, a == 1, a == 2);
  if (p.kind == RBG_ADJ_NODE_SHIFT) {
    const double* H = sf.H;
    df = -(a == 0 ? sf.g.x : a == 1 ? sf.g.y : sf.g.z);
    dg = mk(-H[a], -H[3 + a], -H[6 + a]);
    return true;
  }
  if (p.kind == RBG_ADJ_NODE_ROTATE) {
    d3 r = P - mk(p.pivot[0], p.pivot[1], p.pivot[2]);
    d3 gxr = cross(sf.g, r);
    df = a == 0 ? gxr.x : a == 1 ? gxr.y : gxr.z;
    dg = cross(e, sf.g) + sym_vec(sf.H, cross(r, e));
    return true;
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

// acc[k] += gbar . dg_k + c df_k over the parameters (unrolled to MAXP so
// that the accumulators stay in registers); moves_with is evaluated once
// per distinct parameter node
template <int MAXP>
RBG_D void add_terms(const DevScene& S, const rbg_adjoint_param* params, int n_params, int node, d3 P, const Surf& sf,
                     d3 gbar, double c, double* acc) {
  int last_node = -1, last_moves = 0;
#pragma unroll
  for (int k = 0; k < MAXP; ++k) {
    if (k >= n_params) break;
    const rbg_adjoint_param& p = params[k];
    int mv = -1;
    if (p.kind != RBG_ADJ_ASPH_COEF) {
      if (p.node != last_node) {
        last_node = p.node;
        last_moves = moves_with(S, p.node, node);
      }
      mv = last_moves;
    }
    double df;
    d3 dg;
    if (param_terms(S, p, node, P, sf, df, dg, mv)) acc[k] += dot(gbar, dg) + c * df;
  }
}

template <int MAXP>
__global__ void __launch_bounds__(128) adjoint_kernel(DevScene S, int64_t n, const uint8_t* status, const int32_t* npoints,
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
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    d3 Pbar = mk(gx ? gx[i] : 0.0, gy ? gy[i] : 0.0, gz ? gz[i] : 0.0);
    const int np = npoints[i];
    // cotangents of the recorded points (hit records), when given
    const double* gp = gpts ? gpts + (size_t)i * hist_cap * 3 : nullptr;
    auto gpt = [&](int j) { return gp ? mk(gp[3 * j], gp[3 * j + 1], gp[3 * j + 2]) : mk(0, 0, 0); };
    bool any = !(Pbar.x == 0 && Pbar.y == 0 && Pbar.z == 0);
    for (int j = 0; gp && !any && j < np && j < hist_cap; ++j) {
      const d3 q = gpt(j);
      any = q.x != 0 || q.y != 0 || q.z != 0;
    }
    if (!any) continue;
    if (np < 2 || np > hist_cap) {
      ++nskip;
      continue;
    }
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
    double pd = dot(Pbar, dseg);
    add_terms<MAXP>(S, params, n_params, fnode, Pm, sf, mk(0, 0, 0), -pd / gd, acc);
    d3 obar = Pbar - (pd / gd) * sf.g;
    d3 dbar = tseg * obar;
    for (int e = m - 1; e >= 1; --e) {
      const d3 Prec = pt(ev[e]);
      const d3 Pin = pt(ev[e - 1]);
      const d3 din = normalized(Prec - Pin);
      const bool refl = evk[e] == kEvReflect;
      // recorded point: reflection = hit - eps d_in (the step back),
      // refraction = hit + push d_in (the boundary push)
      const double off = refl ? -RBG_REFLECT_BACKSTEP : RBG_BOUNDARY_PUSH;
      const d3 Phit = Prec - off * din;
      const double t_in = sqrt(dot(Phit - Pin, Phit - Pin));
      const int node = evs[e];
      if (!surface_at(S, node, Phit, sf)) {
        ok = false;
        break;
      }
      const double gn = sqrt(dot(sf.g, sf.g));
      // o_next = the recorded point = Phit + off d_in, with its own cotangent
      const d3 Precbar = obar + gpt(ev[e]);
      d3 Phbar = Precbar;
      d3 dinbar = off * Precbar;
      d3 gbar;
      if (refl) {
        const d3 nrm = (1.0 / gn) * sf.g;
        // d_out = din - 2 (din.n) n
        const double dn = dot(din, nrm), ndb = dot(nrm, dbar);
        dinbar = dinbar + dbar - (2 * ndb) * nrm;
        const d3 nbar = (-2.0) * (dn * dbar + ndb * din);
        gbar = (1.0 / gn) * (nbar - dot(nrm, nbar) * nrm);
      } else {
        // d_out = eta din + (c2 - eta c1) nh, nh = s g / |g| oriented along
        // din, c1 = din.nh, c2 = sqrt(1 - eta^2 (1 - c1^2))
        const double sgn = dot(sf.g, din) < 0 ? -1.0 : 1.0;
        const d3 nh = (sgn / gn) * sf.g;
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
        gbar = (sgn / gn) * (nhbar - dot(nh, nhbar) * nh);
      }
      Phbar = Phbar + sym_vec(sf.H, gbar);
      const double gdi = dot(sf.g, din);
      if (gdi == 0) {
        ok = false;
        break;
      }
      const double phd = dot(Phbar, din);
      add_terms<MAXP>(S, params, n_params, node, Phit, sf, gbar, -phd / gdi, acc);
      obar = Phbar - (phd / gdi) * sf.g;
      dbar = dinbar + t_in * obar;
    }
    if (!ok) ++nskip;
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
  int block = 128;
  int blocks = (int)std::min<int64_t>((n + block - 1) / block, (int64_t)sm_count() * 8);
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
