// tracer.cuh -- navigation and the AOpticsManager state machine on the
// device (src/AOpticsManager.cxx:52-520), one thread per ray.
#pragma once
#include "geometry.cuh"

namespace rbg {

// --------------------------------------------------------------------
// navigation (TGeoNavigator semantics restated)
// --------------------------------------------------------------------
struct Nav {
  int node;   // current node, -1 outside the top volume
  d3 p, d;    // navigator point and direction (master frame)
  int xnode;  // node whose surface the last step crossed
  d3 xn;      // its normal for TGeo primitives (node frame)
  int xface;  // mixed path: face of an aspheric disk the step crossed
};

RBG_D bool in_box(const double* lo, const double* hi, d3 p) {
  return !(p.x < lo[0] || p.x > hi[0] || p.y < lo[1] || p.y > hi[1] || p.z < lo[2] || p.z > hi[2]);
}
RBG_D bool in_fbox(const float* lo, const float* hi, d3 p) {
  return !(p.x < lo[0] || p.x > hi[0] || p.y < lo[1] || p.y > hi[1] || p.z < lo[2] || p.z > hi[2]);
}

template <unsigned F = kFeatAll>
RBG_D bool node_contains(const DevScene& S, int k, d3 p) {
  const rbg_node& N = S.nodes[k];
  if (!in_box(N.lo, N.hi, p)) return false;
  return shape_contains<F>(S, N.shape, to_local(N.m, p));
}

// FP32 segment/box test for the mixed path, enlarged so that it never
// rejects a box the FP64 test accepts
template <typename T>
RBG_D bool seg_box_f32(float ox, float oy, float oz, float ix, float iy, float iz, bool zx, bool zy, bool zz,
                       float smax, const T* lo, const T* hi) {
  RBG_EVENT(EV_SCREEN32);
  float t0 = 0.f, t1 = smax;
  const float o3[3] = {ox, oy, oz}, i3[3] = {ix, iy, iz};
  const bool z3[3] = {zx, zy, zz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float l = (float)lo[a], h = (float)hi[a];
    float pad = 1e-4f + 2e-6f * fmaxf(fabsf(l), fabsf(h));
    l -= pad;
    h += pad;
    if (z3[a]) {
      if (o3[a] < l || o3[a] > h) return false;
      continue;
    }
    float ta = (l - o3[a]) * i3[a], tb = (h - o3[a]) * i3[a];
    t0 = fmaxf(t0, fminf(ta, tb));
    t1 = fminf(t1, fmaxf(ta, tb));
    if (t0 > t1 * 1.000001f + 1e-4f) return false;
  }
  return true;
}

// segment [0, smax] of the ray against a box
template <typename T>
RBG_D bool seg_box(d3 o, d3 inv, d3 d, double smax, const T* lo, const T* hi) {
  double t0 = 0, t1 = smax;
  const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, ii[3] = {inv.x, inv.y, inv.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (dd[a] == 0) {
      if (oo[a] < (double)lo[a] || oo[a] > (double)hi[a]) return false;
      continue;
    }
    double ta = ((double)lo[a] - oo[a]) * ii[a], tb = ((double)hi[a] - oo[a]) * ii[a];
    if (ta > tb) {
      double s = ta;
      ta = tb;
      tb = s;
    }
    t0 = fmax(t0, ta);
    t1 = fmin(t1, tb);
    if (t0 > t1) return false;
  }
  return true;
}

// first child (in placement order) of node k containing p, or -1
template <unsigned F = kFeatAll>
RBG_D int first_child_containing(const DevScene& S, int k, d3 p) {
  const rbg_node& N = S.nodes[k];
  if (!(F & kFeatBVH) || N.bvh_root < 0) {
    for (int i = 0; i < N.child_count; ++i) {
      int c = S.children[N.child_begin + i];
      if (node_contains<F>(S, c, p)) return c;
    }
    return -1;
  }
  int best = -1;
  int stack[32];
  int sp = 0;
  stack[sp++] = N.bvh_root;
  while (sp > 0) {
    const rbg_bvh_node& b = S.bvh[stack[--sp]];
    if (!in_fbox(b.lo, b.hi, p)) continue;
    if (b.left < 0) {
      for (int i = 0; i < b.right; ++i) {
        int c = S.bvh_items[b.item_begin + i];
        if ((best < 0 || c < best) && node_contains<F>(S, c, p)) best = c;
      }
    } else if (sp + 2 <= 32) {
      stack[sp++] = b.left;
      stack[sp++] = b.right;
    }
  }
  return best;
}

template <unsigned F = kFeatAll>
RBG_D int locate_down(const DevScene& S, int k, d3 p) {
  for (int depth = 0; depth < 64; ++depth) {
    int c = first_child_containing<F>(S, k, p);
    if (c < 0) return k;
    k = c;
  }
  return k;
}
template <unsigned F = kFeatAll>
RBG_D int locate_from_top(const DevScene& S, d3 p) {
  if (!node_contains<F>(S, 0, p)) return -1;
  return locate_down<F>(S, 0, p);
}

// ---- mixed-precision navigation: the same tree walks with FP32 screens
// in front of every containment test (geometry.cuh fast paths) ----------
RBG_D bool in_fbox3(const float* lo, const float* hi, f3 p) {
  return !(p.x < lo[0] || p.x > hi[0] || p.y < lo[1] || p.y > hi[1] || p.z < lo[2] || p.z > hi[2]);
}

template <unsigned F>
RBG_D bool shape_contains_f_body(const DevScene& S, int shape, const LRay& L, bool twin) {
  const rbg_shape_desc& sh = S.shapes[shape];
  const double* P = S.params + sh.param_offset;
  const float* Pf = S.fparams + sh.param_offset;
  if (sh.type == RBG_SHAPE_ASPHERIC_DISK) return asph_contains_f(P, Pf, L, twin);
  if (sh.type == RBG_SHAPE_BOX) return box_contains_f(P, Pf, L);
  if (sh.type == RBG_SHAPE_WINSTON_POLY)
    return (F & kFeatWinston) ? win_contains(win_load(P, ST(S, shape)), L.p) : false;
  if (sh.type == RBG_SHAPE_WINSTON_2D)
    return (F & kFeatWinston) ? win2d_contains(win_load(P, ST(S, shape)), P[RBG_WIN_DY], L.p) : false;
  return (F & kFeatCSG) ? csg_contains(S, shape, L.p) : false;
}

// out of line except in the lean (F = 0) instance, as shape_contains
template <unsigned F>
RBG_NOINLINE bool shape_contains_f_call(const DevScene& S, int shape, LRay L, bool twin) {
  return shape_contains_f_body<F>(S, shape, L, twin);
}
template <unsigned F>
RBG_D bool shape_contains_f(const DevScene& S, int shape, const LRay& L, bool twin) {
  return F == 0 ? shape_contains_f_body<F>(S, shape, L, twin) : shape_contains_f_call<F>(S, shape, L, twin);
}

// node k contains p: float box (rounded outward, so it never rejects a
// point of the FP64 box) and the shape's own test in the local frame
template <unsigned F>
RBG_D bool node_contains_f(const DevScene& S, int k, d3 p, f3 pf) {
  const rbg_node_aux& A = S.aux[k];
  if (!in_fbox3(A.lo, A.hi, pf)) return false;
  return shape_contains_f<F>(S, S.nodes[k].shape, local_point(S, k, p, pf), A.flags & RBG_AUX_ASPH_TWIN_FACES);
}

template <unsigned F>
RBG_D int first_child_containing_f(const DevScene& S, int k, d3 p, f3 pf) {
  const rbg_node& N = S.nodes[k];
  if (!(F & kFeatBVH) || N.bvh_root < 0) {
    // box tests of every daughter first, then the shape tests of the
    // survivors in placement order: the lanes of a warp run the same shape
    // code on different daughters instead of taking turns
    for (int base = 0; base < N.child_count; base += 32) {
      const int m = N.child_count - base < 32 ? N.child_count - base : 32;
      unsigned mask = 0;
      for (int i = 0; i < m; ++i) {
        const rbg_node_aux& A = S.aux[S.children[N.child_begin + base + i]];
        if (in_fbox3(A.lo, A.hi, pf)) mask |= 1u << i;
      }
      while (mask) {
        const int i = __ffs(mask) - 1;
        mask &= mask - 1;
        const int c = S.children[N.child_begin + base + i];
        if (shape_contains_f<F>(S, S.nodes[c].shape, local_point(S, c, p, pf),
                                S.aux[c].flags & RBG_AUX_ASPH_TWIN_FACES))
          return c;
      }
    }
    return -1;
  }
  // collect the daughters whose float boxes hold the point, then run the
  // shape tests over the list (the lanes of a warp test candidate j
  // together); the lowest containing id wins whatever the order
  constexpr int kCand = 8;
  int cand[kCand];
  int nc = 0;
  int best = -1;
  auto test = [&](int c) {
    if ((best < 0 || c < best) &&
        shape_contains_f<F>(S, S.nodes[c].shape, local_point(S, c, p, pf), S.aux[c].flags & RBG_AUX_ASPH_TWIN_FACES))
      best = c;
  };
  int stack[32];
  int sp = 0;
  stack[sp++] = N.bvh_root;
  while (sp > 0) {
    const rbg_bvh_node& b = S.bvh[stack[--sp]];
    if (!in_fbox3(b.lo, b.hi, pf)) continue;
    if (b.left < 0) {
      for (int i = 0; i < b.right; ++i) {
        const int c = S.bvh_items[b.item_begin + i];
        if (!in_fbox3(S.aux[c].lo, S.aux[c].hi, pf)) continue;
        if (nc == kCand) {
          for (int j = 0; j < kCand; ++j) test(cand[j]);
          nc = 0;
        }
        cand[nc++] = c;
      }
    } else if (sp + 2 <= 32) {
      stack[sp++] = b.left;
      stack[sp++] = b.right;
    }
  }
  for (int j = 0; j < nc; ++j) test(cand[j]);
  return best;
}

template <unsigned F>
RBG_D int locate_down_f(const DevScene& S, int k, d3 p, f3 pf) {
  for (int depth = 0; depth < 64; ++depth) {
    int c = first_child_containing_f<F>(S, k, p, pf);
    if (c < 0) return k;
    k = c;
  }
  return k;
}
template <unsigned F>
RBG_D int locate_from_top_f(const DevScene& S, d3 p) {
  const f3 pf = to_f3(p);
  if (!node_contains_f<F>(S, 0, p, pf)) return -1;
  return locate_down_f<F>(S, 0, p, pf);
}

// shape distance of node k in the mixed path; `face` receives the aspheric face
template <unsigned F>
RBG_D double shape_dist_f_body(const DevScene& S, int k, const LRay& L, bool exit, d3& nrm, int& face,
                               unsigned& err) {
  const int shape = S.nodes[k].shape;
  const rbg_shape_desc& sh = S.shapes[shape];
  const double* P = S.params + sh.param_offset;
  face = 0;
  if (sh.type == RBG_SHAPE_ASPHERIC_DISK) {
    const float* Pf = S.fparams + sh.param_offset;
    const bool twin = S.aux[k].flags & RBG_AUX_ASPH_TWIN_FACES;
    return exit ? asph_dist4_f(P, Pf, L, twin, face) : asph_dist_out_f(P, Pf, L, twin, face);
  }
  if (sh.type == RBG_SHAPE_WINSTON_POLY || sh.type == RBG_SHAPE_WINSTON_2D) {
    if (!(F & kFeatWinston)) return kBig;
    Win w = win_load(P, ST(S, shape));
    if (sh.type == RBG_SHAPE_WINSTON_2D)
      return exit ? win2d_dist_in(w, P[RBG_WIN_DY], L.p, L.d) : win2d_dist_out(w, P[RBG_WIN_DY], L.p, L.d);
    return exit ? win_dist_in(w, L.p, L.d) : win_dist_out(w, L.p, L.d);
  }
  if (sh.type == RBG_SHAPE_BOX) return box_dist_fast(P, L.p, L.d, exit, nrm);
  return (F & kFeatCSG) ? csg_dist(S, shape, L.p, L.d, exit, nrm, err) : kBig;
}

template <unsigned F>
RBG_NOINLINE double shape_dist_f_call(const DevScene& S, int k, LRay L, bool exit, d3& nrm, int& face,
                                      unsigned& err) {
  return shape_dist_f_body<F>(S, k, L, exit, nrm, face, err);
}
template <unsigned F>
RBG_D double shape_dist_f(const DevScene& S, int k, const LRay& L, bool exit, d3& nrm, int& face, unsigned& err) {
  return F == 0 ? shape_dist_f_body<F>(S, k, L, exit, nrm, face, err)
                : shape_dist_f_call<F>(S, k, L, exit, nrm, face, err);
}

// candidate daughter test shared by the scan and the BVH walk
template <unsigned F = kFeatAll>
RBG_D void try_child(const DevScene& S, int k, d3 p, d3 d, double& best, int& xnode, bool& enter, d3& nbest,
                     unsigned& err) {
  const rbg_node& K = S.nodes[k];
  d3 nrm = mk(0, 0, 1);
  double s = shape_dist<F>(S, K.shape, to_local(K.m, p), dir_to_local(K.m, d), false, nrm, err);
  // ties: leaving the mother first, then the lowest node id (placement order)
  if (s < best || (s == best && enter && k < xnode)) {
    best = s;
    xnode = k;
    enter = true;
    nbest = nrm;
  }
}

// TGeoNavigator::FindNextBoundaryAndStep
template <unsigned F = kFeatAll>
RBG_D int find_next_boundary_and_step(const DevScene& S, Nav& nv, double& step, unsigned& err) {
  const int c = nv.node;
  double best;
  d3 nbest = mk(0, 0, 1);
  int xnode;
  bool enter;
  if (c < 0) {
    const rbg_node& T = S.nodes[0];
    best = shape_dist<F>(S, T.shape, to_local(T.m, nv.p), dir_to_local(T.m, nv.d), false, nbest, err);
    if (best >= kBig) {
      step = 0;
      nv.xnode = -1;
      return -1;
    }
    xnode = 0;
    enter = true;
  } else {
    const rbg_node& N = S.nodes[c];
    best = shape_dist<F>(S, N.shape, to_local(N.m, nv.p), dir_to_local(N.m, nv.d), true, nbest, err);
    xnode = c;
    enter = false;
    const d3 inv = mk(1.0 / nv.d.x, 1.0 / nv.d.y, 1.0 / nv.d.z);
    if (!(F & kFeatBVH) || N.bvh_root < 0) {
      for (int i = 0; i < N.child_count; ++i) {
        int k = S.children[N.child_begin + i];
        const rbg_node& K = S.nodes[k];
        if (!seg_box(nv.p, inv, nv.d, best, K.lo, K.hi)) continue;
        try_child<F>(S, k, nv.p, nv.d, best, xnode, enter, nbest, err);
      }
    } else {
      int stack[32];
      int sp = 0;
      stack[sp++] = N.bvh_root;
      while (sp > 0) {
        const rbg_bvh_node& b = S.bvh[stack[--sp]];
        if (!seg_box(nv.p, inv, nv.d, best, b.lo, b.hi)) continue;
        if (b.left < 0) {
          for (int i = 0; i < b.right; ++i) {
            int k = S.bvh_items[b.item_begin + i];
            const rbg_node& K = S.nodes[k];
            if (!seg_box(nv.p, inv, nv.d, best, K.lo, K.hi)) continue;
            try_child<F>(S, k, nv.p, nv.d, best, xnode, enter, nbest, err);
          }
        } else if (sp + 2 <= 32) {
          stack[sp++] = b.right;
          stack[sp++] = b.left;
        } else {
          err |= ERR_BIT_CAP;
        }
      }
    }
  }
  nv.p = nv.p + (best + RBG_BOUNDARY_PUSH) * nv.d;
  nv.xnode = xnode;
  nv.xn = nbest;
  int next;
  if (enter) {
    next = locate_down<F>(S, xnode, nv.p);
  } else {
    int q = S.nodes[c].parent;
    while (q >= 0 && !node_contains<F>(S, q, nv.p)) q = S.nodes[q].parent;
    next = q < 0 ? -1 : locate_down<F>(S, q, nv.p);
  }
  nv.node = next;
  step = best;
  return next;
}

// TGeoNavigator::FindNextBoundaryAndStep for the mixed path: the same
// candidates, tie rules and relocation as find_next_boundary_and_step, with
// the ray converted to FP32 once for every screen, the daughters culled
// against their float boxes, and the crossed aspheric face recorded for
// find_normal
template <unsigned F>
RBG_D int find_next_boundary_and_step_f(const DevScene& S, Nav& nv, double& step, unsigned& err) {
  const int c = nv.node;
  const f3 pf = to_f3(nv.p), df = to_f3(nv.d);
  double best;
  d3 nbest = mk(0, 0, 1);
  int xnode, face = 0, xface = 0;
  bool enter;
  if (c < 0) {
    best = shape_dist_f<F>(S, 0, local_ray(S, 0, nv.p, nv.d, pf, df), false, nbest, xface, err);
    if (best >= kBig) {
      step = 0;
      nv.xnode = -1;
      return -1;
    }
    xnode = 0;
    enter = true;
  } else {
    const rbg_node& N = S.nodes[c];
    const LRay Lc = local_ray(S, c, nv.p, nv.d, pf, df);
    // A box mother's exit distance is needed only if no daughter is hit
    // before it: start from an FP32 upper bound (it only widens the
    // culling) and take the FP64 distance afterwards unless a daughter
    // lies below the FP32 lower bound.  The result equals taking the FP64
    // exit first: a daughter replaces the mother only when strictly nearer.
    float exit_lo = 0.f, exit_hi = 0.f;
    const bool lazy = S.shapes[N.shape].type == RBG_SHAPE_BOX &&
                      box_exit_bounds_f(S.fparams + S.shapes[N.shape].param_offset, Lc, exit_lo, exit_hi) &&
                      exit_lo > 0.f;
    best = lazy ? (double)exit_hi : shape_dist_f<F>(S, c, Lc, true, nbest, xface, err);
    xnode = c;
    enter = false;
    const bool zx = df.x == 0.f, zy = df.y == 0.f, zz = df.z == 0.f;
    const float ix = zx ? 0.f : __frcp_rn(df.x), iy = zy ? 0.f : __frcp_rn(df.y), iz = zz ? 0.f : __frcp_rn(df.z);
    auto reach = [&](const float* lo, const float* hi) {
      return seg_box_f32(pf.x, pf.y, pf.z, ix, iy, iz, zx, zy, zz, best >= kBig ? 3e38f : (float)best, lo, hi);
    };
    auto visit = [&](int k) {
      const rbg_node_aux& A = S.aux[k];
      if (!reach(A.lo, A.hi)) return;
      d3 nrm = mk(0, 0, 1);
      double s = shape_dist_f<F>(S, k, local_ray(S, k, nv.p, nv.d, pf, df), false, nrm, face, err);
      // ties: leaving the mother first, then the lowest node id (placement order)
      if (s < best || (s == best && enter && k < xnode)) {
        best = s;
        xnode = k;
        enter = true;
        nbest = nrm;
        xface = face;
      }
    };
    if (!(F & kFeatBVH) || N.bvh_root < 0) {
      // cull every daughter first, then test the survivors in placement
      // order (visit re-checks the box against the shrinking distance, so
      // the tested set is the one a single pass would test)
      for (int base = 0; base < N.child_count; base += 32) {
        const int m = N.child_count - base < 32 ? N.child_count - base : 32;
        unsigned mask = 0;
        for (int i = 0; i < m; ++i) {
          const rbg_node_aux& A = S.aux[S.children[N.child_begin + base + i]];
          if (reach(A.lo, A.hi)) mask |= 1u << i;
        }
        while (mask) {
          const int i = __ffs(mask) - 1;
          mask &= mask - 1;
          visit(S.children[N.child_begin + base + i]);
        }
      }
    } else {
      // two phases: the traversal only collects the daughters whose boxes
      // the segment reaches, then the shape distances run over the list.
      // Lanes whose traversals take different turns thus still call the
      // (FP64, often composite) distance together, candidate j at once,
      // instead of one lane at a time from inside the loop.  visit re-checks
      // each box against the distance found so far; the lowest-id tie rule
      // makes the result independent of the order.
      constexpr int kCand = 8;
      int cand[kCand];
      int nc = 0;
      int stack[32];
      int sp = 0;
      stack[sp++] = N.bvh_root;
      while (sp > 0) {
        const rbg_bvh_node& b = S.bvh[stack[--sp]];
        if (!reach(b.lo, b.hi)) continue;
        if (b.left < 0) {
          for (int i = 0; i < b.right; ++i) {
            const int k = S.bvh_items[b.item_begin + i];
            const rbg_node_aux& A = S.aux[k];
            if (!reach(A.lo, A.hi)) continue;
            if (nc == kCand) {
              for (int j = 0; j < kCand; ++j) visit(cand[j]);
              nc = 0;
            }
            cand[nc++] = k;
          }
        } else if (sp + 2 <= 32) {
          stack[sp++] = b.right;
          stack[sp++] = b.left;
        } else {
          err |= ERR_BIT_CAP;
        }
      }
      for (int j = 0; j < nc; ++j) visit(cand[j]);
    }
    if (lazy && !(enter && best < (double)exit_lo)) {
      d3 en = mk(0, 0, 1);
      const double e = box_dist_fast(S.params + S.shapes[N.shape].param_offset, Lc.p, Lc.d, true, en);
      if (!enter || e <= best) {
        best = e;
        xnode = c;
        enter = false;
        nbest = en;
        xface = 0;
      }
    }
  }
  RBG_EVENT(EV_SEGMENT);
  nv.p = nv.p + (best + RBG_BOUNDARY_PUSH) * nv.d;
  nv.xnode = xnode;
  nv.xn = nbest;
  nv.xface = xface;
  const f3 qf = to_f3(nv.p);
  int next;
  if (enter) {
    next = locate_down_f<F>(S, xnode, nv.p, qf);
  } else {
    int q = S.nodes[c].parent;
    while (q >= 0 && !node_contains_f<F>(S, q, nv.p, qf)) q = S.nodes[q].parent;
    next = q < 0 ? -1 : locate_down_f<F>(S, q, nv.p, qf);
  }
  nv.node = next;
  step = best;
  return next;
}

// TGeoNavigator::FindNormal: master-frame normal, n . d >= 0
template <bool MIXED = false, unsigned F = kFeatAll>
RBG_D d3 find_normal(const DevScene& S, const Nav& nv) {
  if (nv.xnode < 0) return mk(0, 0, 1);
  const rbg_node& N = S.nodes[nv.xnode];
  const int type = S.shapes[N.shape].type;
  d3 nl;
  if (MIXED && type == RBG_SHAPE_ASPHERIC_DISK) {
    const int off = S.shapes[N.shape].param_offset;
    const LRay L = local_ray(S, nv.xnode, nv.p, nv.d, to_f3(nv.p), to_f3(nv.d));
    nl = asph_normal_f(S, nv.xnode, S.params + off, S.fparams + off, L, nv.xface);
    const int xf = S.aux[nv.xnode].xform;
    // a rotation keeps the unit length (to rounding); no renormalisation
    d3 n = xf == RBG_XFORM_GENERAL ? dir_to_master(N.m, nl) : nl;
    if (dot(n, nv.d) < 0) n = neg(n);
    return n;
  } else if (type == RBG_SHAPE_ASPHERIC_DISK) {
    Asph a{SP(S, N.shape)};
    d3 pl = to_local(N.m, nv.p), dl = dir_to_local(N.m, nv.d);
    nl = asph_normal(a, pl, dl);
  } else if (type == RBG_SHAPE_WINSTON_POLY) {
    nl = win_normal(win_load(SP(S, N.shape), ST(S, N.shape)), to_local(N.m, nv.p), dir_to_local(N.m, nv.d));
  } else if (type == RBG_SHAPE_WINSTON_2D) {
    nl = win2d_normal(win_load(SP(S, N.shape), ST(S, N.shape)), SP(S, N.shape)[RBG_WIN_DY], to_local(N.m, nv.p),
                      dir_to_local(N.m, nv.d));
  } else {
    nl = nv.xn;
  }
  d3 n = normalized(dir_to_master(N.m, nl));
  if (dot(n, nv.d) < 0) n = neg(n);
  return n;
}

// --------------------------------------------------------------------
// complex arithmetic for the transfer matrices
// --------------------------------------------------------------------
template <typename T>
struct cplxT {
  T re, im;
};
template <typename T>
RBG_D cplxT<T> cx(T r, T i = 0) { return cplxT<T>{r, i}; }
template <typename T>
RBG_D cplxT<T> operator+(cplxT<T> a, cplxT<T> b) { return cplxT<T>{a.re + b.re, a.im + b.im}; }
template <typename T>
RBG_D cplxT<T> operator-(cplxT<T> a, cplxT<T> b) { return cplxT<T>{a.re - b.re, a.im - b.im}; }
template <typename T>
RBG_D cplxT<T> operator*(cplxT<T> a, cplxT<T> b) {
  return cplxT<T>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T>
RBG_D cplxT<T> operator*(T s, cplxT<T> a) { return cplxT<T>{s * a.re, s * a.im}; }
template <typename T>
RBG_D cplxT<T> cdiv(cplxT<T> a, cplxT<T> b) {
  // Smith's algorithm
  if (fabs(b.re) >= fabs(b.im)) {
    T r = b.im / b.re, den = b.re + b.im * r;
    return cplxT<T>{(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  }
  T r = b.re / b.im, den = b.re * r + b.im;
  return cplxT<T>{(a.re * r + a.im) / den, (a.im * r - a.re) / den};
}
template <typename T>
RBG_D T cabs_(cplxT<T> a) { return hypot(a.re, a.im); }
template <typename T>
RBG_D cplxT<T> cexp_(cplxT<T> a) {
  T e = exp(a.re), s, c;
  sincos(a.im, &s, &c);
  return cplxT<T>{e * c, e * s};
}
template <typename T>
RBG_D cplxT<T> ccos_(cplxT<T> a) {
  T s, c;
  sincos(a.re, &s, &c);
  return cplxT<T>{c * cosh(a.im), -s * sinh(a.im)};
}
template <typename T>
RBG_D cplxT<T> csin_(cplxT<T> a) {
  T s, c;
  sincos(a.re, &s, &c);
  return cplxT<T>{s * cosh(a.im), c * sinh(a.im)};
}
template <typename T>
RBG_D cplxT<T> csqrt_(cplxT<T> a) {
  // principal square root
  if (a.re == 0 && a.im == 0) return cplxT<T>{0, a.im};
  T m = hypot(a.re, a.im);
  T t = sqrt(T(0.5) * (m + fabs(a.re)));
  if (a.re >= 0) return cplxT<T>{t, a.im / (2 * t)};
  return cplxT<T>{fabs(a.im) / (2 * t), copysign(t, a.im)};
}
template <typename T>
RBG_D cplxT<T> clog_(cplxT<T> a) { return cplxT<T>{log(hypot(a.re, a.im)), atan2(a.im, a.re)}; }
// principal arcsine: -i log(i z + sqrt(1 - z^2))
template <typename T>
RBG_D cplxT<T> casin_(cplxT<T> z) {
  cplxT<T> one_m = cx<T>(1) - z * z;
  cplxT<T> w = cplxT<T>{-z.im, z.re} + csqrt_(one_m);
  cplxT<T> l = clog_(w);
  return cplxT<T>{l.im, -l.re};
}

template <typename T>
RBG_D bool is_forward_angle(cplxT<T> n, cplxT<T> th) {
  // 100 machine epsilons of the working precision
  const T eps = sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-07);
  cplxT<T> nc = n * ccos_(th);
  if (fabs(nc.im) > 100 * eps) return nc.im > 0;
  return nc.re > 0;
}

// AMultilayer::CoherentTMM (src/AMultilayer.cxx:240-481) in precision T,
// for the m media S.layers[base + a + k dir], k = 0..m-1 (dir = +1 front to
// back, -1 reversed as CoherentTMM's `reverse`), light incident from medium
// k = 0 at the (possibly complex) angle th0.  The transfer-matrix product is
// built on the fly, front to back.  NP = 1 evaluates polarisation `pol1`
// (0 = s, 1 = p) into R[0], Tr[0]; NP = 2 evaluates s into [0] and p into
// [1] in one pass: the indices, Snell angles, cosines and phase factors of
// the layers do not depend on the polarisation and are computed once, the
// interface coefficients and the two matrix products per polarisation
// (CoherentTMMMixed, include/AMultilayer.h:114-132, calls CoherentTMM once
// per polarisation and so evaluates them twice).
template <typename T, int NP>
RBG_D void tmm_coherent_n(const DevScene& S, int base, int a, int m, int dir, int pol1, cplxT<T> th0, double lam,
                          double* R, double* Tr) {
  typedef cplxT<T> C;
  auto layer = [&](int k) -> const rbg_layer_desc& { return S.layers[base + a + k * dir]; };
  auto nidx = [&](int k) {
    const rbg_layer_desc& L = layer(k);
    return cx<T>((T)index_n(S, L.index, lam), (T)index_k(S, L.index, lam));
  };
  auto pol_of = [&](int q) { return NP == 2 ? q : pol1; };
  const T pi = T(kPi);
  C n0 = nidx(0);
  C n0s = n0 * csin_(th0);
  // ListSnell (:178-209): the first and the last angle are the forward ones
  C th_first = casin_(cdiv(n0s, n0));
  if (!is_forward_angle(n0, th_first)) th_first = cx<T>(pi) - th_first;
  C a00[NP], a01[NP], a10[NP], a11[NP], r0[NP], t0[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    a00[q] = cx<T>(1);
    a01[q] = cx<T>(0);
    a10[q] = cx<T>(0);
    a11[q] = cx<T>(1);
    r0[q] = cx<T>(0);
    t0[q] = cx<T>(1);
  }
  C n_prev = n0, ct_prev = ccos_(th_first);
  for (int i = 1; i < m; ++i) {
    C ni = nidx(i);
    C thi = casin_(cdiv(n0s, ni));
    if (i == m - 1 && !is_forward_angle(ni, thi)) thi = cx<T>(pi) - thi;
    C cti = ccos_(thi);
    C ii = n_prev * ct_prev;
    // phase of layer i-1 (not for the incidence medium)
    C em = cx<T>(1), ep = cx<T>(1);
    if (i > 1) {
      C kz = (T(2) * pi / (T)lam) * (n_prev * ct_prev);
      C delta = (T)layer(i - 1).thickness * kz;
      if (delta.im > 35) delta.im = 35;
      em = cexp_(C{delta.im, -delta.re});
      ep = cexp_(C{-delta.im, delta.re});
    }
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      // interface (i-1) -> i, interface_rt (:26-56)
      C r, t;
      if (pol_of(q) == 0) {
        C ff = ni * cti;
        r = cdiv(ii - ff, ii + ff);
        t = cdiv(T(2) * ii, ii + ff);
      } else {
        C fi = ni * ct_prev, iff = n_prev * cti;
        r = cdiv(fi - iff, fi + iff);
        t = cdiv(T(2) * ii, fi + iff);
      }
      if (i == 1) {
        r0[q] = r;
        t0[q] = t;
      } else {
        // layer i-1: (1/t) diag(e^{-i delta}, e^{i delta}) [[1, r],[r, 1]]
        C it = cdiv(cx<T>(1), t);
        C m00 = em * it, m01 = em * r * it, m10 = ep * r * it, m11 = ep * it;
        C na = a00[q] * m00 + a01[q] * m10, nb = a00[q] * m01 + a01[q] * m11;
        C nc = a10[q] * m00 + a11[q] * m10, nd = a10[q] * m01 + a11[q] * m11;
        a00[q] = na;
        a01[q] = nb;
        a10[q] = nc;
        a11[q] = nd;
      }
    }
    n_prev = ni;
    ct_prev = cti;
  }
  // transmitted power with the incident angle th0 itself (:466-479)
  C ct0 = ccos_(th0);
  C nf = n_prev, ctf = ct_prev;
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    // prepend the first interface: (1/t0) [[1, r0],[r0, 1]] * Mtilde
    C it0 = cdiv(cx<T>(1), t0[q]);
    C A = (a00[q] + r0[q] * a10[q]) * it0, Cc = (r0[q] * a00[q] + a10[q]) * it0;
    C rr = cdiv(Cc, A), tt = cdiv(cx<T>(1), A);
    T ar = cabs_(rr);
    R[q] = (double)(ar * ar);
    T tt2 = cabs_(tt * tt);
    if (pol_of(q) == 0) Tr[q] = (double)(tt2 * ((nf * ctf).re / (n0 * ct0).re));
    else Tr[q] = (double)(tt2 * ((nf * C{ctf.re, -ctf.im}).re / (n0 * C{ct0.re, -ct0.im}).re));
  }
}

// one polarisation, pol 0 = s, 1 = p
template <typename T>
RBG_D void tmm_coherent(const DevScene& S, int base, int a, int m, int dir, int pol, cplxT<T> th0, double lam,
                        double& R, double& Tr) {
  tmm_coherent_n<T, 1>(S, base, a, m, dir, pol, th0, lam, &R, &Tr);
}

template <typename T>
RBG_D void coherent_tmm(const DevScene& S, int ml, int pol, double th0r, double lam, double& R, double& Tr) {
  const rbg_multilayer_desc& M = S.multilayers[ml];
  tmm_coherent<T>(S, M.layer_offset, 0, M.n_layers, 1, pol, cx<T>((T)th0r), lam, R, Tr);
}

// interface_RT (:93-104): power reflection and transmission of one interface
RBG_D void tmm_interface_RT(int pol, cplxT<double> ni, cplxT<double> nf, cplxT<double> thi, cplxT<double> thf,
                            double& R, double& T) {
  typedef cplxT<double> C;
  const C ci = ccos_(thi), cf = ccos_(thf);
  const C ii = ni * ci;
  C r, t;
  if (pol == 0) {
    const C ff = nf * cf;
    r = cdiv(ii - ff, ii + ff);
    t = cdiv(2.0 * ii, ii + ff);
  } else {
    const C fi = nf * ci, iff = ni * cf;
    r = cdiv(fi - iff, fi + iff);
    t = cdiv(2.0 * ii, fi + iff);
  }
  const double ar = cabs_(r);
  R = ar * ar;
  const double t2 = cabs_(t * t);
  if (pol == 0) T = t2 * ((nf * cf).re / (ni * ci).re);
  else T = t2 * ((nf * C{cf.re, -cf.im}).re / (ni * C{ci.re, -ci.im}).re);
}

// AMultilayer::IncoherentTMM (:555-731), the incoherent / partly coherent
// transfer-matrix method of tmm.inc_tmm: the media flagged incoherent (the
// first and the last always) split the stack into coherent sub-stacks; each
// sub-stack (or bare interface) between two incoherent media contributes its
// forward and backward power R and T; an incoherent medium of thickness d
// passes P = exp(-4 pi d Im(n cos th) / lambda) of the power (at least
// 1e-30); the 2x2 power matrices multiply front to back, T = 1 / L00,
// R = L10 / L00.  FP64, evaluated where the tables are filled.
RBG_D void tmm_incoherent(const DevScene& S, int ml, int pol, cplxT<double> th0, double lam, double& R, double& T) {
  typedef cplxT<double> C;
  const rbg_multilayer_desc& M = S.multilayers[ml];
  const int N = M.n_layers, base = M.layer_offset;
  auto n_of = [&](int k) {
    const rbg_layer_desc& L = S.layers[base + k];
    return cx<double>(index_n(S, L.index, lam), index_k(S, L.index, lam));
  };
  const C n0s = n_of(0) * csin_(th0);
  // ListSnell over all media, forward angles at both ends
  auto th_of = [&](int k) {
    const C nk = n_of(k);
    C th = casin_(cdiv(n0s, nk));
    if ((k == 0 || k == N - 1) && !is_forward_angle(nk, th)) th = cx<double>(kPi) - th;
    return th;
  };
  auto incoherent = [&](int k) { return k == 0 || k == N - 1 || !S.layers[base + k].coherent; };
  // power R/T from incoherent medium p to the next incoherent medium q, both ways
  auto pair = [&](int p, int q, double& Rf, double& Tf, double& Rb, double& Tb) {
    if (q == p + 1) {
      const C np = n_of(p), nq = n_of(q), thp = th_of(p), thq = th_of(q);
      tmm_interface_RT(pol, np, nq, thp, thq, Rf, Tf);
      tmm_interface_RT(pol, nq, np, thq, thp, Rb, Tb);
    } else {
      tmm_coherent<double>(S, base, p, q - p + 1, 1, pol, th_of(p), lam, Rf, Tf);
      tmm_coherent<double>(S, base, q, q - p + 1, -1, pol, th_of(q), lam, Rb, Tb);
    }
  };
  // Ltilde = L(0->1) [ prod_i diag(1/P_i, P_i) L(i->i+1) ]
  int p = 0, q = 1;
  while (!incoherent(q)) ++q;
  double Rf, Tf, Rb, Tb;
  pair(p, q, Rf, Tf, Rb, Tb);
  double l00 = 1 / Tf, l01 = -Rb / Tf, l10 = Rf / Tf, l11 = (Tb * Tf - Rb * Rf) / Tf;
  while (q < N - 1) {
    p = q;
    q = p + 1;
    while (!incoherent(q)) ++q;
    const C np = n_of(p);
    const C thp = th_of(p);
    const C nc = np * ccos_(thp);
    double P = exp(-4 * kPi * S.layers[base + p].thickness * nc.im / lam);
    if (P < 1e-30) P = 1e-30;
    pair(p, q, Rf, Tf, Rb, Tb);
    // L = diag(1/P, P) [[1, -Rb],[Rf, Tb Tf - Rb Rf]] / Tf
    const double b00 = 1 / (P * Tf), b01 = -Rb / (P * Tf), b10 = P * Rf / Tf, b11 = P * (Tb * Tf - Rb * Rf) / Tf;
    const double c00 = l00 * b00 + l01 * b10, c01 = l00 * b01 + l01 * b11;
    const double c10 = l10 * b00 + l11 * b10, c11 = l10 * b01 + l11 * b11;
    l00 = c00;
    l01 = c01;
    l10 = c10;
    l11 = c11;
  }
  T = 1 / l00;
  R = l10 / l00;
}

// TH2::Interpolate on a lam_nbins x th_nbins table (x = lambda, y = theta)
// stored [ix * ny + iy]: bilinear between bin centres, the edge bins held
// constant in their outer half, 0 outside [min, max) of either axis
RBG_D double th2_interpolate(const double* tab, int nx, double xmin, double xmax, int ny, double ymin, double ymax,
                             double x, double y) {
  if (!(x >= xmin && x < xmax && y >= ymin && y < ymax)) return 0.0;
  const double wx = (xmax - xmin) / nx, wy = (ymax - ymin) / ny;
  int bx = 1 + (int)floor((x - xmin) / wx), by = 1 + (int)floor((y - ymin) / wy);
  bx = bx < 1 ? 1 : (bx > nx ? nx : bx);
  by = by < 1 ? 1 : (by > ny ? ny : by);
  const double cxm = xmin + (bx - 0.5) * wx, cym = ymin + (by - 0.5) * wy;
  double x1, x2, y1, y2;
  int bx1, bx2, by1, by2;
  if (x >= cxm) {
    x1 = cxm; x2 = cxm + wx; bx1 = bx; bx2 = bx + 1;
  } else {
    x1 = cxm - wx; x2 = cxm; bx1 = bx - 1; bx2 = bx;
  }
  if (y >= cym) {
    y1 = cym; y2 = cym + wy; by1 = by; by2 = by + 1;
  } else {
    y1 = cym - wy; y2 = cym; by1 = by - 1; by2 = by;
  }
  bx1 = bx1 < 1 ? 1 : bx1;
  bx2 = bx2 > nx ? nx : bx2;
  by1 = by1 < 1 ? 1 : by1;
  by2 = by2 > ny ? ny : by2;
  const double q11 = tab[(bx1 - 1) * ny + by1 - 1], q21 = tab[(bx2 - 1) * ny + by1 - 1];
  const double q12 = tab[(bx1 - 1) * ny + by2 - 1], q22 = tab[(bx2 - 1) * ny + by2 - 1];
  const double d = (x2 - x1) * (y2 - y1);
  return (q11 * (x2 - x) * (y2 - y) + q21 * (x - x1) * (y2 - y) + q12 * (x2 - x) * (y - y1) +
          q22 * (x - x1) * (y - y1)) / d;
}

// CoherentTMMMixed (include/AMultilayer.h:114-132): the precalculated table
// when there is one, else the mean of the p and s evaluations (FP32 in the
// mixed tracer)
template <bool MIXED, unsigned F = kFeatAll>
RBG_D void coherent_tmm_mixed(const DevScene& S, int ml, double th0, double lam, double& R, double& T) {
  const rbg_multilayer_desc& M = S.multilayers[ml];
  if (M.precalc != 0 && S.tmm_off[ml] >= 0) {
    const double* tab = S.tmm_tables + S.tmm_off[ml];
    const int64_t cells = (int64_t)M.lam_nbins * M.th_nbins;
    R = th2_interpolate(tab, M.lam_nbins, M.lam_min, M.lam_max, M.th_nbins, M.th_min, M.th_max, lam, th0);
    T = th2_interpolate(tab + cells, M.lam_nbins, M.lam_min, M.lam_max, M.th_nbins, M.th_min, M.th_max, lam, th0);
    return;
  }
  // [0] = s, [1] = p
  double r[2], t[2];
  if (MIXED) tmm_coherent_n<float, 2>(S, M.layer_offset, 0, M.n_layers, 1, 0, cx<float>((float)th0), lam, r, t);
  else tmm_coherent_n<double, 2>(S, M.layer_offset, 0, M.n_layers, 1, 0, cx<double>(th0), lam, r, t);
  R = (r[1] + r[0]) / 2.;
  T = (t[1] + t[0]) / 2.;
}

// --------------------------------------------------------------------
// ray record and random draws
// --------------------------------------------------------------------
struct Ray {
  d3 x;
  double t;
  d3 d;
  double lambda;
  int status, npoints, last_node;
  RayRng rng;
  unsigned err;
  // history
  int hist_cap;
  double* hist_xyzt;
  int32_t* hist_node;
};

RBG_D double rng_u(Ray& r) {
  Philox4 b = r.rng.next();
  return u53(b.v[0], b.v[1]);
}
RBG_D double rng_gaus(Ray& r, double sigma) {
  Philox4 b = r.rng.next();
  double a = u53(b.v[0], b.v[1]), c = u53(b.v[2], b.v[3]);
  return sigma * sqrt(-2.0 * log(1.0 - a)) * cos(2.0 * kPi * c);
}

RBG_D void add_point(Ray& r, d3 p, double t) {
  r.x = p;
  r.t = t;
  if (r.npoints < r.hist_cap) {
    double* h = r.hist_xyzt + 4 * (size_t)r.npoints;
    h[0] = p.x;
    h[1] = p.y;
    h[2] = p.z;
    h[3] = t;
    r.hist_node[r.npoints] = -2;
  }
  r.npoints++;
}
RBG_D void add_node(Ray& r, int node) {
  r.last_node = node;
  int idx = r.npoints - 1;
  if (idx >= 0 && idx < r.hist_cap) r.hist_node[idx] = node;
}
RBG_D void set_direction(Ray& r, d3 v) {
  double mag = sqrt(dot(v, v));
  if (mag > 0) r.d = mk(v.x / mag, v.y / mag, v.z / mag);
}
// ARay::SetDirection for a vector that is unit to ~1e-8 (a reflected unit
// vector): first-order inverse square root, no FP64 sqrt or division
RBG_D void set_direction_fast(Ray& r, d3 v) {
  double m2 = dot(v, v);
  if (fabs(m2 - 1.0) < 1e-8) {
    double s = 1.5 - 0.5 * m2;
    r.d = mk(v.x * s, v.y * s, v.z * s);
  } else {
    set_direction(r, v);
  }
}

enum { kLens = 0, kObs = 1, kMirror = 2, kFocus = 3, kOpt = 4, kOther = 5, kNull = 6 };
RBG_D int kind_of(const DevScene& S, int node) { return node < 0 ? kNull : S.nodes[node].kind; }

RBG_D int find_border(const DevScene& S, int cur, int next) {
  if (cur < 0) return -1;
  int c1 = S.nodes[cur].volume, c2 = next < 0 ? -1 : S.nodes[next].volume;
  for (int i = 0; i < S.n_borders; ++i)
    if (S.borders[i].component1 == c1 && S.borders[i].component2 == c2) return i;
  return -1;
}

RBG_D double lens_n(const DevScene& S, int node, double lam) {
  return index_n(S, S.volumes[S.nodes[node].volume].index, lam);
}

// TVector3::RotateUz
RBG_D d3 rotate_uz(d3 v, d3 u) {
  double up = u.x * u.x + u.y * u.y;
  if (up > 0) {
    up = sqrt(up);
    return mk((u.x * u.z * v.x - u.y * v.y) / up + u.x * v.z, (u.y * u.z * v.x + u.x * v.y) / up + u.y * v.z,
              -up * v.x + u.z * v.z);
  }
  if (u.z < 0.) return mk(-v.x, v.y, -v.z);
  return v;
}

// GetFacetNormal (:250-301)
// The rejection sampling of GetFacetNormal (src/AOpticsManager.cxx:266-298,
// after G4OpBoundaryProcess): alpha ~ N(0, sigma) accepted when
// U * min(1, 4 sigma) <= sin(alpha) < 1, phi uniform, the facet normal
// rotated onto `normal`, repeated while it faces away from `dir`.  Out of
// line: it runs only on rough reflections, and its FP64 transcendentals
// would otherwise enlarge every trace kernel.  Draws advance `rng`; after
// RBG_ROUGH_MAX_TRIES rejections `normal` is returned with ERR_BIT_CAP.
RBG_NOINLINE d3 sample_facet_normal(d3 normal, d3 dir, double sigma, RayRng& rng, unsigned& err) {
  const double f_max = fmin(1., 4. * sigma);
  int tries = 0;
  for (;;) {
    double alpha;
    for (;;) {
      const Philox4 g = rng.next();
      const double a = u53(g.v[0], g.v[1]), c = u53(g.v[2], g.v[3]);
      alpha = sigma * sqrt(-2.0 * log(1.0 - a)) * cos(2.0 * kPi * c);
      const double u = f_max * rng.uniform();
      if (!(u > sin(alpha) || alpha >= kPi / 2)) break;
      if (++tries > RBG_ROUGH_MAX_TRIES) {
        err |= ERR_BIT_CAP;
        return normal;
      }
    }
    const double phi = 2 * kPi * rng.uniform();
    double sa, ca, sp, cp;
    sincos(alpha, &sa, &ca);
    sincos(phi, &sp, &cp);
    const d3 facet = rotate_uz(mk(sa * cp, sa * sp, ca), normal);
    if (dot(dir, facet) > 0.0) return facet;
    if (++tries > RBG_ROUGH_MAX_TRIES) {
      err |= ERR_BIT_CAP;
      return normal;
    }
  }
}

template <bool MIXED, unsigned F = kFeatAll>
RBG_D d3 get_facet_normal(const DevScene& S, const Nav& nv, Ray& r, int cur, int next) {
  d3 normal = find_normal<MIXED, F>(S, nv);
  if (!(F & kFeatRough)) return normal;
  int bi = find_border(S, cur, next);
  if (bi < 0) return normal;
  const rbg_border_desc B = S.borders[bi];
  if (B.lambertian) return normal;
  if (B.sigma == 0) return normal;
  return sample_facet_normal(normal, nv.d, B.sigma, r.rng, r.err);
}

// TGeoRotation(phi, theta, psi) in degrees applied to v
RBG_D d3 euler_apply(double phi, double theta, double psi, d3 v) {
  double sf, cf, st, ct, sp, cp;
  sincos(phi * kD2R, &sf, &cf);
  sincos(theta * kD2R, &st, &ct);
  sincos(psi * kD2R, &sp, &cp);
  double R0 = cp * cf - ct * sf * sp, R1 = -sp * cf - ct * sf * cp, R2 = st * sf;
  double R3 = cp * sf + ct * cf * sp, R4 = -sp * sf + ct * cf * cp, R5 = -st * cf;
  double R6 = sp * st, R7 = cp * st, R8 = ct;
  return mk(R0 * v.x + R1 * v.y + R2 * v.z, R3 * v.x + R4 * v.y + R5 * v.z, R6 * v.x + R7 * v.y + R8 * v.z);
}

// DoReflection (:170-247); `normal` may be null (computed here)
template <bool MIXED, unsigned F = kFeatAll>
RBG_D void do_reflection(const DevScene& S, Nav& nv, Ray& r, double n1, double step, int cur, int next,
                         const d3* normal) {
  d3 n = normal ? *normal : get_facet_normal<MIXED, F>(S, nv, r, cur, next);
  const d3 d1 = r.d;
  double cos1 = dot(d1, n);
  int bi = (F & (kFeatMultilayer | kFeatRough)) ? find_border(S, cur, next) : -1;
  bool absorbed = false;
  if (kind_of(S, next) == kMirror) {
    const rbg_volume_desc& mv = S.volumes[S.nodes[next].volume];
    // the incidence angle only matters for 2D tables and thin films
    const bool need_angle =
        !MIXED || (bi >= 0 && S.borders[bi].multilayer >= 0) ||
        (mv.refl_table >= 0 && S.tables[mv.refl_table].kind == RBG_TABLE_2D);
    double angle = need_angle ? acos(cos1) : 0.0;
    double ref;
    if ((F & kFeatMultilayer) && bi >= 0 && S.borders[bi].multilayer >= 0) {
      double tr;
      coherent_tmm_mixed<MIXED>(S, S.borders[bi].multilayer, angle, r.lambda, ref, tr);
    } else {
      const rbg_volume_desc& v = S.volumes[S.nodes[next].volume];
      if (v.refl_table >= 0)
        ref = S.tables[v.refl_table].kind == RBG_TABLE_2D ? table2d(S, v.refl_table, r.lambda, angle)
                                                          : table1d(S, v.refl_table, r.lambda);
      else
        ref = v.reflectance;
      ref = ref > 1 ? 1 : ref;
      ref = ref < 0 ? 0 : ref;
    }
    if (ref < rng_u(r)) {
      absorbed = true;
      r.status = RBG_ABSORB;
    }
  }
  d3 d2;
  if ((F & kFeatRough) && bi >= 0 && S.borders[bi].lambertian) {
    double y = 0.5 * rng_u(r);
    double theta = asin(sqrt(2 * y));
    double phi = 2 * kPi * rng_u(r);
    double th_n = (n.x == 0 && n.y == 0 && n.z == 0) ? 0 : atan2(sqrt(n.x * n.x + n.y * n.y), n.z);
    double ph_n = (n.x == 0 && n.y == 0) ? 0 : atan2(n.y, n.x);
    d3 v = mk(sin(theta) * cos(phi), sin(theta) * sin(phi), cos(theta));
    d2 = euler_apply(ph_n / kD2R + 90, th_n / kD2R + 180, 0, v);
  } else {
    d2 = d1 - (2 * cos1) * n;
  }
  if (!absorbed) {
    if (MIXED) set_direction_fast(r, d2);
    else set_direction(r, d2);
  }
  double t = MIXED ? r.t + step * (n1 * (1.0 / RBG_SPEED_OF_LIGHT_CM)) : r.t + step / (RBG_SPEED_OF_LIGHT_CM / n1);
  nv.p = nv.p - RBG_REFLECT_BACKSTEP * d1;
  RBG_EVENT(EV_REFLECT);
  nv.node = MIXED ? locate_from_top_f<F>(S, nv.p) : locate_from_top<F>(S, nv.p);
  nv.d = d2;
  add_point(r, nv.p, t);
  add_node(r, next);
}

// Fresnel reflectance for unpolarised light (:103-136) in precision T
template <typename T>
RBG_D double fresnel_R(T n1, T n2, T k2, T cos1, T sin1, T cos2) {
  T Rs, Rp;
  if (k2 <= T(0)) {
    T eta1S = n1 * cos1, eta2S = n2 * cos2, eta1P = n1 / cos1, eta2P = n2 / cos2;
    T a = (eta1S - eta2S) / (eta1S + eta2S), b = (eta1P - eta2P) / (eta1P + eta2P);
    Rs = a * a;
    Rp = b * b;
  } else {
    T x1S = n1 * cos1, x1P = n1 / cos1;
    T u = n2 * n2 - k2 * k2 - (n1 * sin1) * (n1 * sin1);
    T v = 2 * n2 * k2;
    T tmp = sqrt(u * u + v * v);
    T cosxi2 = sqrt(1 + u / tmp) / sqrt(T(2));
    T sinxi2 = sqrt(1 - u / tmp) / sqrt(T(2));
    T x2S = sqrt(tmp) * cosxi2, y2S = sqrt(tmp) * sinxi2;
    tmp = x2S * x2S + y2S * y2S;
    T x2P = (2 * n2 * k2 * y2S + (n2 * n2 - k2 * k2) * x2S) / tmp;
    T y2P = (2 * n2 * k2 * x2S - (n2 * n2 - k2 * k2) * y2S) / tmp;
    Rs = ((x1S - x2S) * (x1S - x2S) + y2S * y2S) / ((x1S + x2S) * (x1S + x2S) + y2S * y2S);
    Rp = ((x1P - x2P) * (x1P - x2P) + y2P * y2P) / ((x1P + x2P) * (x1P + x2P) + y2P * y2P);
  }
  return (double)((Rs + Rp) / 2);
}

// DoFresnel (:52-167)
template <bool MIXED, unsigned F = kFeatAll>
RBG_D void do_fresnel(const DevScene& S, Nav& nv, Ray& r, double n1, double n2, double k2, double step, int cur,
                      int next, bool disable_fresnel) {
  d3 n = get_facet_normal<MIXED, F>(S, nv, r, cur, next);
  const d3 d1 = r.d;
  double cos1 = dot(d1, n);
  double sin1 = sqrt(1 - cos1 * cos1);
  double sin2 = n1 * sin1 / n2;
  double cos2 = sqrt(1 - sin2 * sin2);
  int bi = find_border(S, cur, next);
  bool absorbed = false;
  bool transmit = false;
  if (bi >= 0 && S.borders[bi].multilayer >= 0) {
    double refl, trans;
    coherent_tmm_mixed<MIXED>(S, S.borders[bi].multilayer, acos(cos1), r.lambda, refl, trans);
    double rnd = rng_u(r);
    if (rnd < refl) {
      do_reflection<MIXED, F>(S, nv, r, n1, step, cur, next, &n);
      return;
    }
    absorbed = !(rnd < refl + trans);
    transmit = true;
  }
  if (!transmit) {
    if (sin2 > 1.) {
      do_reflection<MIXED, F>(S, nv, r, n1, step, cur, next, &n);
      return;
    }
    if (!disable_fresnel) {
      double R = MIXED ? fresnel_R<float>((float)n1, (float)n2, (float)k2, (float)cos1, (float)sin1, (float)cos2)
                       : fresnel_R<double>(n1, n2, k2, cos1, sin1, cos2);
      if (rng_u(r) < R) {
        do_reflection<MIXED, F>(S, nv, r, n1, step, cur, next, &n);
        return;
      }
    }
  }
  d3 d2 = sin1 != 0 ? (sin2 / sin1) * (d1 - cos1 * n) + cos2 * n : d1;
  double t = r.t + step / (RBG_SPEED_OF_LIGHT_CM / n1);
  add_point(r, nv.p, t);
  add_node(r, next);
  if (absorbed) {
    r.status = RBG_ABSORB;
  } else {
    set_direction(r, d2);
    nv.d = d2;
  }
}

// TraceNonSequential(TObjArray*) body for one ray (:346-518), split into
// InitTrack and one iteration of the while (ray->IsRunning()) loop so that
// a persistent kernel can interleave rays
template <bool MIXED = false, unsigned F = kFeatAll>
RBG_D void trace_begin(const DevScene& S, Ray& r, Nav& nv) {
  nv.p = r.x;
  nv.d = r.d;
  nv.node = MIXED ? locate_from_top_f<F>(S, nv.p) : locate_from_top<F>(S, nv.p);
  nv.xnode = -1;
  nv.xn = mk(0, 0, 1);
  nv.xface = 0;
}

template <bool MIXED, unsigned F = kFeatAll>
RBG_D void trace_step(const DevScene& S, Ray& r, Nav& nv, int limit, bool disable_fresnel) {
  const double lambda = r.lambda;
  const d3 x1 = r.x;
  const double t1 = r.t;
  const d3 d1 = r.d;
  const int cur = nv.node;
  double step;
  const int next = MIXED ? find_next_boundary_and_step_f<F>(S, nv, step, r.err)
                         : find_next_boundary_and_step<F>(S, nv, step, r.err);
  const int tc = kind_of(S, cur), tn = kind_of(S, next);

  if ((F & kFeatLens) && tc == kLens) {
    int idx = S.volumes[S.nodes[cur].volume].index;
    double k = index_k(S, idx, lambda);
    double abs_len = k <= 0. ? INFINITY : lambda / (4 * kPi * k);
    if (abs_len > 0 && abs_len != INFINITY) {
      double abs_step = -abs_len * log(1.0 - rng_u(r));
      if (abs_step < step) {
        double n1 = index_n(S, idx, lambda);
        add_point(r, x1 + abs_step * d1, t1 + abs_step / (RBG_SPEED_OF_LIGHT_CM / n1));
        add_node(r, next);
        r.status = RBG_ABSORB;
        return;
      }
    }
  }

  if ((tc == kNull || tc == kOpt || tc == kLens || tc == kOther) && tn == kMirror) {
    double n1 = ((F & kFeatLens) && tc == kLens) ? lens_n(S, cur, lambda) : 1.;
    do_reflection<MIXED, F>(S, nv, r, n1, step, cur, next, nullptr);
  } else if ((F & kFeatLens) && (tc == kNull || tc == kOpt || tc == kOther) && tn == kLens) {
    int idx = S.volumes[S.nodes[next].volume].index;
    do_fresnel<MIXED, F>(S, nv, r, 1, index_n(S, idx, lambda), index_k(S, idx, lambda), step, cur, next,
                      disable_fresnel);
  } else if ((tc == kNull || tc == kLens || tc == kOpt || tc == kOther) && (tn == kObs || tn == kFocus)) {
    double speed = ((F & kFeatLens) && tc == kLens) ? RBG_SPEED_OF_LIGHT_CM / lens_n(S, cur, lambda) : RBG_SPEED_OF_LIGHT_CM;
    add_point(r, nv.p, t1 + step / speed);
    add_node(r, next);
  } else if ((tc == kNull || tc == kOpt || tc == kOther) && (tn == kOther || tn == kOpt)) {
    add_point(r, nv.p, t1 + step / RBG_SPEED_OF_LIGHT_CM);
    add_node(r, next);
  } else if ((F & kFeatLens) && tc == kLens && tn == kLens) {
    int idx = S.volumes[S.nodes[next].volume].index;
    do_fresnel<MIXED, F>(S, nv, r, lens_n(S, cur, lambda), index_n(S, idx, lambda), index_k(S, idx, lambda), step,
                      cur, next, disable_fresnel);
  } else if ((F & kFeatLens) && tc == kLens && (tn == kNull || tn == kOpt || tn == kOther)) {
    do_fresnel<MIXED, F>(S, nv, r, lens_n(S, cur, lambda), 1, 0, step, cur, next, disable_fresnel);
  }

  if (tn == kNull) {
    add_point(r, nv.p, t1 + step / RBG_SPEED_OF_LIGHT_CM);
    add_node(r, next);
    r.status = RBG_EXIT;
  } else if (tc == kFocus || tc == kObs || tc == kMirror || tn == kObs) {
    r.status = RBG_STOP;
  } else if (tn == kFocus) {
    const rbg_volume_desc& v = S.volumes[S.nodes[next].volume];
    double angle = 0.;
    if (v.qe_angle_table >= 0) {
      d3 n = get_facet_normal<MIXED, F>(S, nv, r, cur, next);
      angle = acos(dot(r.d, n));
    }
    double qe = v.qe_lambda_table >= 0 ? table1d(S, v.qe_lambda_table, lambda) : 1.;
    if (v.qe_angle_table >= 0) qe *= table1d(S, v.qe_angle_table, angle);
    if (qe == 1 || rng_u(r) < qe) r.status = RBG_FOCUS;
    else r.status = RBG_STOP;
  }
  if (r.status == RBG_RUN && r.npoints >= limit) r.status = RBG_SUSPEND;
}

template <bool MIXED, unsigned F = kFeatAll>
RBG_D void trace_ray(const DevScene& S, Ray& r, int limit, bool disable_fresnel) {
  Nav nv;
  trace_begin<MIXED, F>(S, r, nv);
  while (r.status == RBG_RUN) trace_step<MIXED, F>(S, r, nv, limit, disable_fresnel);
}

// ---------------------------------------------------------------------
// kernel-side ray I/O (structure of arrays)
// ---------------------------------------------------------------------
struct KernelRays {
  const double *x, *y, *z, *t, *dx, *dy, *dz, *lambda;
  // the mixed tracer's take-up order (ray_order.cu): queue slot q traces
  // ray order[q]; NULL: input order.  With `gathered` set the arrays above
  // hold the rays in queue order (slot q at q) and order[q] is the ray's
  // index for its outputs and random draws.
  const int32_t* order;
  int32_t gathered;
};
struct KernelOut {
  uint8_t* status;
  int32_t *npoints, *last_node;
  double *x, *y, *z, *t, *dx, *dy, *dz;
  int32_t hist_cap;
  double* hist_xyzt;
  int32_t* hist_node;
};

// Read ray i (its inputs at position `src` of `in`), record its start
// point, normalise the direction as ARay::SetDirection does.  Returns false
// (and flags the error) for a ray that cannot be traced: NaN origin or a
// zero/NaN direction.
RBG_D bool load_ray(const KernelRays& in, const KernelOut& out, int64_t src, int64_t i, uint64_t seed,
                    uint64_t id_offset, Ray& r) {
  r.x = mk(in.x[src], in.y[src], in.z[src]);
  r.t = in.t ? in.t[src] : 0.0;
  r.lambda = in.lambda[src];
  d3 dd = mk(in.dx[src], in.dy[src], in.dz[src]);
  r.status = RBG_RUN;
  r.npoints = 0;
  r.last_node = -2;
  r.err = 0;
  r.hist_cap = out.hist_cap;
  r.hist_xyzt = out.hist_cap ? out.hist_xyzt + (size_t)i * out.hist_cap * 4 : nullptr;
  r.hist_node = out.hist_cap ? out.hist_node + (size_t)i * out.hist_cap : nullptr;
  r.rng.init(seed, id_offset + (uint64_t)i, 0);
  add_point(r, r.x, r.t);
  double mag = sqrt(dot(dd, dd));
  bool bad = !(mag > 0) || !isfinite(mag) || !isfinite(r.x.x) || !isfinite(r.x.y) || !isfinite(r.x.z);
  if (bad) {
    r.d = dd;
    r.err |= ERR_BIT_NAN;
    return false;
  }
  set_direction(r, dd);
  return true;
}

// load_ray for the mixed path: the same checks, with the finiteness tests
// on the exponent bits and the direction scaled by a refined reciprocal
// square root instead of three FP64 divisions (the unit vector differs from
// ARay::SetDirection's by at most a few ulp)
RBG_D bool finite_bits(double v) {
  return (__double_as_longlong(v) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}
// Ray i of the batch, its inputs read at position `src` of `in`.
RBG_D bool load_ray_f(const KernelRays& in, const KernelOut& out, int64_t src, int64_t i, uint64_t seed,
                      uint64_t id_offset, Ray& r) {
  r.x = mk(in.x[src], in.y[src], in.z[src]);
  r.t = in.t ? in.t[src] : 0.0;
  r.lambda = in.lambda[src];
  d3 dd = mk(in.dx[src], in.dy[src], in.dz[src]);
  r.status = RBG_RUN;
  r.npoints = 0;
  r.last_node = -2;
  r.err = 0;
  r.hist_cap = out.hist_cap;
  r.hist_xyzt = out.hist_cap ? out.hist_xyzt + (size_t)i * out.hist_cap * 4 : nullptr;
  r.hist_node = out.hist_cap ? out.hist_node + (size_t)i * out.hist_cap : nullptr;
  r.rng.init(seed, id_offset + (uint64_t)i, 0);
  add_point(r, r.x, r.t);
  const double m2 = dot(dd, dd);
  RBG_EVENT(EV_RAY);
  const bool bad = !finite_bits(r.x.x) || !finite_bits(r.x.y) || !finite_bits(r.x.z) || !finite_bits(dd.x) ||
                   !finite_bits(dd.y) || !finite_bits(dd.z) || !(m2 > 0) || !finite_bits(m2);
  if (bad) {
    r.d = dd;
    r.err |= ERR_BIT_NAN;
    return false;
  }
  if (m2 > 1e-30 && m2 < 1e30) {
    const double inv = rsqrt_refined(m2);
    r.d = mk(dd.x * inv, dd.y * inv, dd.z * inv);
  } else {
    set_direction(r, dd);
  }
  return true;
}

RBG_D void store_ray(const KernelOut& out, int64_t i, const Ray& r) {
  if (out.status) out.status[i] = (uint8_t)r.status;
  if (out.npoints) out.npoints[i] = r.npoints;
  if (out.last_node) out.last_node[i] = r.last_node;
  if (out.x) out.x[i] = r.x.x;
  if (out.y) out.y[i] = r.x.y;
  if (out.z) out.z[i] = r.x.z;
  if (out.t) out.t[i] = r.t;
  if (out.dx) out.dx[i] = r.d.x;
  if (out.dy) out.dy[i] = r.d.y;
  if (out.dz) out.dz[i] = r.d.z;
  // history slots the ray did not reach: node -3 and point 0, as the host
  // buffers start, so that no stale device memory reads as a point
  for (int j = r.npoints; j < r.hist_cap; ++j) {
    r.hist_node[j] = -3;
    double* h = r.hist_xyzt + 4 * (size_t)j;
    h[0] = h[1] = h[2] = h[3] = 0.0;
  }
}

}  // namespace rbg
