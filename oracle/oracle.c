/*
 * oracle.c -- CPU FP64 restatement of ROBAST's non-sequential ray tracer.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): the correctness oracle for the
 * GPU tracer.  Plain C99, one ray at a time, written for clarity and for
 * step-by-step agreement with the reference, not for speed.
 *
 * Navigation semantics restated from TGeo's documented behaviour (ROOT is
 * not in the reference tree):
 *  - the current node is the deepest node whose shape contains the point
 *    (daughters tested in placement order);
 *  - FindNextBoundaryAndStep takes the minimum of the distance to leave the
 *    current node and the distances to enter each daughter (ties: leaving
 *    first, then the earliest daughter), moves the point past the boundary
 *    by RBG_BOUNDARY_PUSH and locates it again (down into an entered
 *    daughter, or up from the mother of a left node);
 *  - FindNormal returns the normal of the surface crossed by that step,
 *    oriented along the ray.
 * TGeo primitives are handled as exact solids: all ray/surface roots are
 * sorted and every segment between consecutive roots is classified with the
 * shape's point-containment test; the same code yields CSG booleans.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "robast_gb_layout.h"

#define BIG RBG_BIG
#define PI 3.14159265358979323846
#define D2R (PI / 180.0)

typedef const rbg_flat_scene Scene;

/* ======================================================================
 * Philox4x32-10 (Salmon et al., SC'11)
 * ==================================================================== */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct {
  uint32_t key[2];
  uint32_t id_lo, id_hi, n;
} Rng;

static void rng_block(Rng* r, uint32_t v[4]) {
  uint32_t c[4] = {r->n++, 0u, r->id_lo, r->id_hi};
  orc_philox(c, r->key, v);
}
static double u53(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * (1.0 / 9007199254740992.0);
}
/* uniform in [0, 1) */
static double rng_u(Rng* r) {
  uint32_t v[4];
  rng_block(r, v);
  return u53(v[0], v[1]);
}
/* Gaussian N(0, sigma): Box-Muller on the two halves of one block */
static double rng_gaus(Rng* r, double sigma) {
  uint32_t v[4];
  rng_block(r, v);
  double a = u53(v[0], v[1]), b = u53(v[2], v[3]);
  return sigma * sqrt(-2.0 * log(1.0 - a)) * cos(2.0 * PI * b);
}
/* exponential with mean tau */
static double rng_exp(Rng* r, double tau) { return -tau * log(1.0 - rng_u(r)); }

/* ======================================================================
 * small vector / matrix helpers; matrices: R row-major + t, master = R l + t
 * ==================================================================== */
static void m_to_local(const double* m, const double* p, double* l) {
  double x = p[0] - m[9], y = p[1] - m[10], z = p[2] - m[11];
  l[0] = m[0] * x + m[3] * y + m[6] * z;
  l[1] = m[1] * x + m[4] * y + m[7] * z;
  l[2] = m[2] * x + m[5] * y + m[8] * z;
}
static void m_dir_to_local(const double* m, const double* d, double* l) {
  l[0] = m[0] * d[0] + m[3] * d[1] + m[6] * d[2];
  l[1] = m[1] * d[0] + m[4] * d[1] + m[7] * d[2];
  l[2] = m[2] * d[0] + m[5] * d[1] + m[8] * d[2];
}
static void m_dir_to_master(const double* m, const double* l, double* d) {
  d[0] = m[0] * l[0] + m[1] * l[1] + m[2] * l[2];
  d[1] = m[3] * l[0] + m[4] * l[1] + m[5] * l[2];
  d[2] = m[6] * l[0] + m[7] * l[1] + m[8] * l[2];
}
static void m_mul(const double* a, const double* b, double* c) {
  double r[12];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j)
      r[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
    r[9 + i] = a[i * 3] * b[9] + a[i * 3 + 1] * b[10] + a[i * 3 + 2] * b[11] + a[9 + i];
  }
  memcpy(c, r, sizeof(r));
}
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void normalize3(double* v) {
  double m = sqrt(dot3(v, v));
  if (m > 0) {
    v[0] /= m; v[1] /= m; v[2] /= m;
  }
}
static const double kIdentity[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};

/* cancellation-safe real roots of A t^2 + B t + C = 0 */
static int quad_roots(double A, double B, double C, double* r) {
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

/* ======================================================================
 * tables: TGraph::Eval (linear, extrapolating with the end pairs) and a
 * bilinear rectilinear 2D table (clamped outside the grid)
 * ==================================================================== */
static double table1d(Scene* S, int id, double x) {
  const rbg_table_desc* t = &S->tables[id];
  const double* X = S->params + t->param_offset;
  const double* Y = X + t->nx;
  int n = t->nx;
  if (n == 1) return Y[0];
  for (int i = 0; i < n; ++i)
    if (X[i] == x) return Y[i];
  int lo, hi;
  if (x < X[0]) {
    lo = 0; hi = 1;
  } else if (x > X[n - 1]) {
    lo = n - 2; hi = n - 1;
  } else {
    hi = 1;
    while (hi < n - 1 && X[hi] < x) ++hi;
    lo = hi - 1;
  }
  if (X[hi] == X[lo]) return Y[lo];
  return Y[lo] + (x - X[lo]) * (Y[hi] - Y[lo]) / (X[hi] - X[lo]);
}
static double table2d(Scene* S, int id, double x, double y) {
  const rbg_table_desc* t = &S->tables[id];
  const double* X = S->params + t->param_offset;
  const double* Y = X + t->nx;
  const double* Z = Y + t->ny;
  int nx = t->nx, ny = t->ny;
  int ix = 0, iy = 0;
  double fx = 0, fy = 0;
  if (nx > 1) {
    if (x <= X[0]) { ix = 0; fx = 0; }
    else if (x >= X[nx - 1]) { ix = nx - 2; fx = 1; }
    else { while (ix < nx - 2 && X[ix + 1] < x) ++ix; fx = (x - X[ix]) / (X[ix + 1] - X[ix]); }
  }
  if (ny > 1) {
    if (y <= Y[0]) { iy = 0; fy = 0; }
    else if (y >= Y[ny - 1]) { iy = ny - 2; fy = 1; }
    else { while (iy < ny - 2 && Y[iy + 1] < y) ++iy; fy = (y - Y[iy]) / (Y[iy + 1] - Y[iy]); }
  }
  int ix1 = nx > 1 ? ix + 1 : ix, iy1 = ny > 1 ? iy + 1 : iy;
  double z00 = Z[ix * ny + iy], z01 = Z[ix * ny + iy1], z10 = Z[ix1 * ny + iy], z11 = Z[ix1 * ny + iy1];
  return (1 - fx) * (1 - fy) * z00 + (1 - fx) * fy * z01 + fx * (1 - fy) * z10 + fx * fy * z11;
}
double orc_table_eval(Scene* S, int table, double x, double y) {
  if (table < 0 || table >= S->n_tables) return 0;
  return S->tables[table].kind == RBG_TABLE_1D ? table1d(S, table, x) : table2d(S, table, x, y);
}

/* ======================================================================
 * refractive index models
 * ==================================================================== */
double orc_refractive_index(Scene* S, int id, double lam) {
  if (id < 0) return 1.0;
  const rbg_index_desc* x = &S->indices[id];
  double l = lam / 1e-4; /* cm -> um: lambda / AOpticsManager::um() */
  switch (x->kind) {
    case RBG_INDEX_TABLE:
      return x->n_table >= 0 ? table1d(S, x->n_table, lam) : 1.0;
    case RBG_INDEX_SELLMEIER: { /* src/ASellmeierFormula.cxx:46-54 */
      double l2 = l * l;
      return sqrt(1 + x->coef[0] * l2 / (l2 - x->coef[3]) + x->coef[1] * l2 / (l2 - x->coef[4]) +
                  x->coef[2] * l2 / (l2 - x->coef[5]));
    }
    case RBG_INDEX_CAUCHY: /* src/ACauchyFormula.cxx */
      return x->coef[0] + x->coef[1] * pow(l, -2) + x->coef[2] * pow(l, -4);
    case RBG_INDEX_SCHOTT: /* src/ASchottFormula.cxx */
      return sqrt(x->coef[0] + x->coef[1] * pow(l, 2.) + x->coef[2] * pow(l, -2.) +
                  x->coef[3] * pow(l, -4.) + x->coef[4] * pow(l, -6.) + x->coef[5] * pow(l, -8.));
    case RBG_INDEX_MIXED: /* include/AMixedRefractiveIndex.h */
      return orc_refractive_index(S, x->mix_a, lam) * x->coef[0] +
             orc_refractive_index(S, x->mix_b, lam) * x->coef[1];
  }
  return 1.0;
}
double orc_extinction(Scene* S, int id, double lam) {
  if (id < 0) return 0.0;
  const rbg_index_desc* x = &S->indices[id];
  if (x->kind == RBG_INDEX_MIXED)
    return orc_extinction(S, x->mix_a, lam) * x->coef[0] + orc_extinction(S, x->mix_b, lam) * x->coef[1];
  return x->k_table >= 0 ? table1d(S, x->k_table, lam) : 0.0;
}
/* ALens::GetAbsorptionLength -> ARefractiveIndex::GetAbsorptionLength */
static double absorption_length(Scene* S, int id, double lam) {
  if (id < 0) return INFINITY;
  double k = orc_extinction(S, id, lam);
  return k <= 0. ? INFINITY : lam / (4 * PI * k);
}

/* ======================================================================
 * AMultilayer coherent TMM (tmm.py algorithm as in src/AMultilayer.cxx)
 * ==================================================================== */
static int is_forward_angle(double complex n, double complex th) {
  const double eps = 2.220446049250313e-16;
  double complex nc = n * ccos(th);
  if (fabs(cimag(nc)) > 100 * eps) return cimag(nc) > 0;
  return creal(nc) > 0;
}
/* CoherentTMM over the media ids[0..N-1] (indices into S->layers), light
 * incident from ids[0] at the (possibly complex) angle th0; a reversed
 * stack (CoherentTMM's `reverse`) is the same call with ids reversed. */
static void coh_tmm_seq(Scene* S, const int* ids, int N, int pol, double complex th0, double lam, double* R,
                        double* T) {
  double complex n[64], th[64], ct[64], delta[64], r[64], t[64];
  for (int i = 0; i < N; ++i) {
    const rbg_layer_desc* L = &S->layers[ids[i]];
    n[i] = orc_refractive_index(S, L->index, lam) + I * orc_extinction(S, L->index, lam);
  }
  /* ListSnell (src/AMultilayer.cxx:178-209) */
  double complex n0s = n[0] * csin(th0);
  for (int i = 0; i < N; ++i) th[i] = casin(n0s / n[i]);
  if (!is_forward_angle(n[0], th[0])) th[0] = PI - th[0];
  if (!is_forward_angle(n[N - 1], th[N - 1])) th[N - 1] = PI - th[N - 1];
  for (int i = 0; i < N; ++i) ct[i] = ccos(th[i]);
  for (int i = 1; i < N - 1; ++i) {
    const rbg_layer_desc* L = &S->layers[ids[i]];
    double complex kz = 2 * PI * n[i] * ct[i] / lam;
    delta[i] = kz * L->thickness;
    if (cimag(delta[i]) > 35) delta[i] = creal(delta[i]) + 35 * I; /* opacity clamp */
  }
  /* interface amplitudes (src/AMultilayer.cxx:26-56) */
  for (int i = 0; i < N - 1; ++i) {
    double complex ii = n[i] * ct[i];
    if (pol == 0) {
      double complex ff = n[i + 1] * ct[i + 1];
      r[i] = (ii - ff) / (ii + ff);
      t[i] = 2. * ii / (ii + ff);
    } else {
      double complex fi = n[i + 1] * ct[i];
      double complex iff = n[i] * ct[i + 1];
      r[i] = (fi - iff) / (fi + iff);
      t[i] = 2. * ii / (fi + iff);
    }
  }
  /* Mtilde = prod_i (1/t_i) diag(e^{-i d}, e^{i d}) [[1, r],[r, 1]] */
  double complex a = 1, b = 0, c = 0, d = 1;
  for (int i = 1; i < N - 1; ++i) {
    double complex em = cexp(-I * delta[i]), ep = cexp(I * delta[i]);
    double complex m00 = em / t[i], m01 = em * r[i] / t[i];
    double complex m10 = ep * r[i] / t[i], m11 = ep / t[i];
    double complex na = a * m00 + b * m10, nb = a * m01 + b * m11;
    double complex nc = c * m00 + d * m10, nd = c * m01 + d * m11;
    a = na; b = nb; c = nc; d = nd;
  }
  {
    double complex m00 = 1. / t[0], m01 = r[0] / t[0], m10 = r[0] / t[0], m11 = 1. / t[0];
    double complex na = m00 * a + m01 * c, nb = m00 * b + m01 * d;
    double complex nc = m10 * a + m11 * c, nd = m10 * b + m11 * d;
    a = na; b = nb; c = nc; d = nd;
  }
  double complex rr = c / a, tt = 1. / a;
  *R = cabs(rr) * cabs(rr);
  /* transmitted power with the incident angle th0 itself (:466-479) */
  if (pol == 0)
    *T = cabs(tt * tt) * (creal(n[N - 1] * ct[N - 1]) / creal(n[0] * ccos(th0)));
  else
    *T = cabs(tt * tt) * (creal(n[N - 1] * conj(ct[N - 1])) / creal(n[0] * conj(ccos(th0))));
}

static int ml_ids(Scene* S, int ml, int* ids) {
  const rbg_multilayer_desc* M = &S->multilayers[ml];
  for (int i = 0; i < M->n_layers; ++i) ids[i] = M->layer_offset + i;
  return M->n_layers;
}

int orc_coherent_tmm_c(Scene* S, int ml, int pol, double th_re, double th_im, double lam, double* R, double* T) {
  int ids[64];
  if (ml < 0 || ml >= S->n_multilayers) return RBG_ERR_ARG;
  int N = ml_ids(S, ml, ids);
  coh_tmm_seq(S, ids, N, pol, th_re + I * th_im, lam, R, T);
  return RBG_OK;
}
int orc_coherent_tmm(Scene* S, int ml, int pol, double th0r, double lam, double* R, double* T) {
  return orc_coherent_tmm_c(S, ml, pol, th0r, 0.0, lam, R, T);
}

/* interface_RT (src/AMultilayer.cxx:93-104) */
static void interface_RT(int pol, double complex ni, double complex nf, double complex thi, double complex thf,
                         double* R, double* T) {
  double complex ci = ccos(thi), cf = ccos(thf), ii = ni * ci, r, t;
  if (pol == 0) {
    double complex ff = nf * cf;
    r = (ii - ff) / (ii + ff);
    t = 2. * ii / (ii + ff);
  } else {
    double complex fi = nf * ci, iff = ni * cf;
    r = (fi - iff) / (fi + iff);
    t = 2. * ii / (fi + iff);
  }
  *R = cabs(r) * cabs(r);
  if (pol == 0) *T = cabs(t * t) * (creal(nf * cf) / creal(ni * ci));
  else *T = cabs(t * t) * (creal(nf * conj(cf)) / creal(ni * conj(ci)));
}

/* AMultilayer::IncoherentTMM (src/AMultilayer.cxx:555-731, tmm.inc_tmm):
 * incoherent media (the first and last always) delimit coherent stacks;
 * R/T between consecutive incoherent media come from the bare interface
 * or the stack's forward and reversed CoherentTMM; P_i = exp(-4 pi d
 * Im(n cos th) / lambda) >= 1e-30 per incoherent medium; the power
 * matrices L multiply front to back: T = 1 / L00, R = L10 / L00. */
int orc_incoherent_tmm(Scene* S, int ml, int pol, double th_re, double th_im, double lam, double* R, double* T) {
  int ids[64], inc[64], ninc = 0;
  double complex n[64], th[64];
  double Rl[64][2], Tl[64][2]; /* [i][0]: i -> i+1, [i][1]: i+1 -> i */
  if (ml < 0 || ml >= S->n_multilayers) return RBG_ERR_ARG;
  int N = ml_ids(S, ml, ids);
  for (int i = 0; i < N; ++i) {
    const rbg_layer_desc* L = &S->layers[ids[i]];
    n[i] = orc_refractive_index(S, L->index, lam) + I * orc_extinction(S, L->index, lam);
  }
  double complex th0 = th_re + I * th_im, n0s = n[0] * csin(th0);
  for (int i = 0; i < N; ++i) th[i] = casin(n0s / n[i]);
  if (!is_forward_angle(n[0], th[0])) th[0] = PI - th[0];
  if (!is_forward_angle(n[N - 1], th[N - 1])) th[N - 1] = PI - th[N - 1];
  for (int i = 0; i < N; ++i)
    if (i == 0 || i == N - 1 || !S->layers[ids[i]].coherent) inc[ninc++] = i;
  for (int k = 0; k + 1 < ninc; ++k) {
    int p = inc[k], q = inc[k + 1];
    if (q == p + 1) {
      interface_RT(pol, n[p], n[q], th[p], th[q], &Rl[k][0], &Tl[k][0]);
      interface_RT(pol, n[q], n[p], th[q], th[p], &Rl[k][1], &Tl[k][1]);
    } else {
      int fwd[64], bwd[64], m = q - p + 1;
      for (int j = 0; j < m; ++j) {
        fwd[j] = ids[p + j];
        bwd[j] = ids[q - j];
      }
      coh_tmm_seq(S, fwd, m, pol, th[p], lam, &Rl[k][0], &Tl[k][0]);
      coh_tmm_seq(S, bwd, m, pol, th[q], lam, &Rl[k][1], &Tl[k][1]);
    }
  }
  /* Ltilde = L(0->1) prod_{k>=1} diag(1/P_k, P_k) L(k->k+1) */
  double l00 = 1 / Tl[0][0], l01 = -Rl[0][1] / Tl[0][0], l10 = Rl[0][0] / Tl[0][0];
  double l11 = (Tl[0][1] * Tl[0][0] - Rl[0][1] * Rl[0][0]) / Tl[0][0];
  for (int k = 1; k + 1 < ninc; ++k) {
    int i = inc[k];
    double P = exp(-4 * PI * S->layers[ids[i]].thickness * cimag(n[i] * ccos(th[i])) / lam);
    if (P < 1e-30) P = 1e-30;
    double Tf = Tl[k][0], Rf = Rl[k][0], Tb = Tl[k][1], Rb = Rl[k][1];
    double b00 = 1 / (P * Tf), b01 = -Rb / (P * Tf), b10 = P * Rf / Tf, b11 = P * (Tb * Tf - Rb * Rf) / Tf;
    double c00 = l00 * b00 + l01 * b10, c01 = l00 * b01 + l01 * b11;
    double c10 = l10 * b00 + l11 * b10, c11 = l10 * b01 + l11 * b11;
    l00 = c00; l01 = c01; l10 = c10; l11 = c11;
  }
  *T = 1 / l00;
  *R = l10 / l00;
  return RBG_OK;
}

/* mixed-polarisation value of one stack, coherent or incoherent */
static void stack_mixed(Scene* S, int ml, int incoherent, double th0, double lam, double* R, double* T) {
  double rp, tp, rs, ts;
  if (incoherent) {
    orc_incoherent_tmm(S, ml, 1, th0, 0.0, lam, &rp, &tp);
    orc_incoherent_tmm(S, ml, 0, th0, 0.0, lam, &rs, &ts);
  } else {
    orc_coherent_tmm(S, ml, 1, th0, lam, &rp, &tp);
    orc_coherent_tmm(S, ml, 0, th0, lam, &rs, &ts);
  }
  *R = (rp + rs) / 2.;
  *T = (tp + ts) / 2.;
}

/* TH2::Interpolate of a precalculated table (include/AMultilayer.h:243-282):
 * bilinear between bin centres, edge bins held in their outer half, 0
 * outside [min, max); the four bin contents are evaluated on the spot at
 * their bin centres (the values the table holds) */
static void table_mixed(Scene* S, int ml, double th0, double lam, double* R, double* T) {
  const rbg_multilayer_desc* M = &S->multilayers[ml];
  int nx = M->lam_nbins, ny = M->th_nbins;
  double xmin = M->lam_min, xmax = M->lam_max, ymin = M->th_min, ymax = M->th_max, x = lam, y = th0;
  *R = 0;
  *T = 0;
  if (!(x >= xmin && x < xmax && y >= ymin && y < ymax)) return;
  double wx = (xmax - xmin) / nx, wy = (ymax - ymin) / ny;
  int bx = 1 + (int)floor((x - xmin) / wx), by = 1 + (int)floor((y - ymin) / wy);
  bx = bx < 1 ? 1 : (bx > nx ? nx : bx);
  by = by < 1 ? 1 : (by > ny ? ny : by);
  double cxm = xmin + (bx - 0.5) * wx, cym = ymin + (by - 0.5) * wy, x1, x2, y1, y2;
  int bx1, bx2, by1, by2;
  if (x >= cxm) { x1 = cxm; x2 = cxm + wx; bx1 = bx; bx2 = bx + 1; }
  else { x1 = cxm - wx; x2 = cxm; bx1 = bx - 1; bx2 = bx; }
  if (y >= cym) { y1 = cym; y2 = cym + wy; by1 = by; by2 = by + 1; }
  else { y1 = cym - wy; y2 = cym; by1 = by - 1; by2 = by; }
  if (bx1 < 1) bx1 = 1;
  if (bx2 > nx) bx2 = nx;
  if (by1 < 1) by1 = 1;
  if (by2 > ny) by2 = ny;
  int bxs[2] = {bx1, bx2}, bys[2] = {by1, by2};
  double qr[2][2], qt[2][2];
  for (int u = 0; u < 2; ++u)
    for (int v = 0; v < 2; ++v)
      stack_mixed(S, ml, M->precalc == 2, ymin + (bys[v] - 0.5) * wy, xmin + (bxs[u] - 0.5) * wx, &qr[u][v],
                  &qt[u][v]);
  double dd = (x2 - x1) * (y2 - y1);
  double w11 = (x2 - x) * (y2 - y), w21 = (x - x1) * (y2 - y), w12 = (x2 - x) * (y - y1), w22 = (x - x1) * (y - y1);
  *R = (qr[0][0] * w11 + qr[1][0] * w21 + qr[0][1] * w12 + qr[1][1] * w22) / dd;
  *T = (qt[0][0] * w11 + qt[1][0] * w21 + qt[0][1] * w12 + qt[1][1] * w22) / dd;
}

/* AMultilayer::CoherentTMMMixed (include/AMultilayer.h:114-132) */
int orc_coherent_tmm_mixed(Scene* S, int ml, double th0, double lam, double* R, double* T) {
  if (ml < 0 || ml >= S->n_multilayers) return RBG_ERR_ARG;
  if (S->multilayers[ml].precalc != 0) table_mixed(S, ml, th0, lam, R, T);
  else stack_mixed(S, ml, 0, th0, lam, R, T);
  return RBG_OK;
}

/* AMirror::GetReflectance (src/AMirror.cxx:39-60) */
double orc_mirror_reflectance(Scene* S, int vol, double lam, double angle) {
  const rbg_volume_desc* v = &S->volumes[vol];
  double ret;
  if (v->refl_table >= 0) {
    const rbg_table_desc* t = &S->tables[v->refl_table];
    ret = t->kind == RBG_TABLE_2D ? table2d(S, v->refl_table, lam, angle) : table1d(S, v->refl_table, lam);
  } else {
    ret = v->reflectance;
  }
  ret = ret > 1 ? 1 : ret;
  ret = ret < 0 ? 0 : ret;
  return ret;
}

/* ======================================================================
 * TGeo primitives as exact solids
 * ==================================================================== */
typedef struct {
  double t;
  double n[3]; /* normal of the crossed surface, in the frame of the query */
} Xing;
typedef struct {
  Xing x[RBG_MAX_XINGS];
  int n;
  int overflow;
} XList;

static const double* SP(Scene* S, int shape) { return S->params + S->shapes[shape].param_offset; }

static int phi_in(double x, double y, double phi1, double dphi) {
  if (dphi >= 360.0) return 1;
  double phi = atan2(y, x) / D2R;
  double rel = phi - phi1;
  while (rel < 0) rel += 360.0;
  while (rel >= 360.0) rel -= 360.0;
  return rel <= dphi;
}

/* apothem-type profile radius of a polycone/polygon segment at z */
static int pxcon_contains(const double* P, int pg, double x, double y, double z) {
  int head = pg ? 4 : 3;
  int nz = (int)P[pg ? 3 : 2];
  const double *Z = P + head, *RMIN = Z + nz, *RMAX = RMIN + nz;
  double phi1 = P[0], dphi = P[1];
  if (z < Z[0] || z > Z[nz - 1]) return 0;
  if (!phi_in(x, y, phi1, dphi)) return 0;
  double rho;
  if (pg) {
    int ned = (int)P[2];
    double sector = dphi / ned;
    double phi = atan2(y, x) / D2R;
    double rel = phi - phi1;
    while (rel < 0) rel += 360.0;
    while (rel >= 360.0) rel -= 360.0;
    int e = (int)floor(rel / sector);
    if (e >= ned) e = ned - 1;
    double pe = (phi1 + (e + 0.5) * sector) * D2R;
    rho = x * cos(pe) + y * sin(pe);
  } else {
    rho = sqrt(x * x + y * y);
  }
  for (int k = 0; k < nz - 1; ++k) {
    if (z < Z[k] || z > Z[k + 1]) continue;
    double h = Z[k + 1] - Z[k];
    double f = h > 0 ? (z - Z[k]) / h : 0.0;
    double rmn = RMIN[k] + f * (RMIN[k + 1] - RMIN[k]);
    double rmx = RMAX[k] + f * (RMAX[k + 1] - RMAX[k]);
    if (h == 0) { rmn = fmin(RMIN[k], RMIN[k + 1]); rmx = fmax(RMAX[k], RMAX[k + 1]); }
    if (rho >= rmn && rho <= rmx) return 1;
  }
  return 0;
}

static int prim_contains(Scene* S, int type, const double* P, const double* p) {
  double x = p[0], y = p[1], z = p[2];
  switch (type) {
    case RBG_SHAPE_BOX:
      return fabs(x - P[RBG_BOX_OX]) <= P[RBG_BOX_DX] && fabs(y - P[RBG_BOX_OY]) <= P[RBG_BOX_DY] &&
             fabs(z - P[RBG_BOX_OZ]) <= P[RBG_BOX_DZ];
    case RBG_SHAPE_TUBE: {
      if (fabs(z) > P[RBG_TUBE_DZ]) return 0;
      double r2 = x * x + y * y;
      if (r2 > P[RBG_TUBE_RMAX] * P[RBG_TUBE_RMAX] || r2 < P[RBG_TUBE_RMIN] * P[RBG_TUBE_RMIN]) return 0;
      return phi_in(x, y, P[RBG_TUBE_PHI1], P[RBG_TUBE_DPHI]);
    }
    case RBG_SHAPE_SPHERE: {
      double r2 = x * x + y * y + z * z;
      if (r2 > P[RBG_SPH_RMAX] * P[RBG_SPH_RMAX] || r2 < P[RBG_SPH_RMIN] * P[RBG_SPH_RMIN]) return 0;
      double th = atan2(sqrt(x * x + y * y), z) / D2R;
      if (th < P[RBG_SPH_TH1] || th > P[RBG_SPH_TH2]) return 0;
      return phi_in(x, y, P[RBG_SPH_PHI1], P[RBG_SPH_DPHI]);
    }
    case RBG_SHAPE_PARABOLOID: {
      if (fabs(z) > P[RBG_PARA_DZ]) return 0;
      double f = P[RBG_PARA_A] * (x * x + y * y) + P[RBG_PARA_B];
      return P[RBG_PARA_A] > 0 ? f <= z : f >= z;
    }
    case RBG_SHAPE_PGON:
      return pxcon_contains(P, 1, x, y, z);
    case RBG_SHAPE_PCON:
      return pxcon_contains(P, 0, x, y, z);
  }
  return 0;
}

static void xl_add(XList* L, double t, const double* nl, const double* M) {
  if (!isfinite(t)) return;
  if (L->n >= RBG_MAX_XINGS) {
    L->overflow = 1;
    return;
  }
  Xing* x = &L->x[L->n++];
  x->t = t;
  double n[3] = {nl[0], nl[1], nl[2]};
  normalize3(n);
  m_dir_to_master(M, n, x->n);
}

/* roots of a plane through the z axis at angle phi (deg): -sin x + cos y = 0 */
static void add_phi_planes(XList* L, const double* o, const double* d, double phi1, double dphi,
                           const double* M) {
  if (dphi >= 360.0) return;
  double phis[2] = {phi1 * D2R, (phi1 + dphi) * D2R};
  for (int k = 0; k < 2; ++k) {
    double s = sin(phis[k]), c = cos(phis[k]);
    double den = -s * d[0] + c * d[1];
    if (den == 0) continue;
    double t = -(-s * o[0] + c * o[1]) / den;
    double n[3] = {-s, c, 0};
    xl_add(L, t, n, M);
  }
}

static void add_z_plane(XList* L, const double* o, const double* d, double z0, const double* M) {
  if (d[2] == 0) return;
  double n[3] = {0, 0, 1};
  xl_add(L, (z0 - o[2]) / d[2], n, M);
}

/* x^2 + y^2 = R^2 */
static void add_cylinder(XList* L, const double* o, const double* d, double R, const double* M) {
  double A = d[0] * d[0] + d[1] * d[1];
  double B = 2 * (o[0] * d[0] + o[1] * d[1]);
  double C = o[0] * o[0] + o[1] * o[1] - R * R;
  double r[2];
  int k = quad_roots(A, B, C, r);
  for (int i = 0; i < k; ++i) {
    double p[3] = {o[0] + r[i] * d[0], o[1] + r[i] * d[1], 0};
    xl_add(L, r[i], p, M);
  }
}

static void add_sphere(XList* L, const double* o, const double* d, double R, const double* M) {
  double B = 2 * dot3(o, d);
  double C = dot3(o, o) - R * R;
  double r[2];
  int k = quad_roots(dot3(d, d), B, C, r);
  for (int i = 0; i < k; ++i) {
    double p[3] = {o[0] + r[i] * d[0], o[1] + r[i] * d[1], o[2] + r[i] * d[2]};
    xl_add(L, r[i], p, M);
  }
}

/* double cone about z with half angle theta (deg): z^2 = cos^2(th) |p|^2 */
static void add_theta_cone(XList* L, const double* o, const double* d, double th, const double* M) {
  double c2 = cos(th * D2R);
  c2 *= c2;
  double s2 = 1 - c2;
  double A = d[2] * d[2] * s2 - c2 * (d[0] * d[0] + d[1] * d[1]);
  double B = 2 * (o[2] * d[2] * s2 - c2 * (o[0] * d[0] + o[1] * d[1]));
  double C = o[2] * o[2] * s2 - c2 * (o[0] * o[0] + o[1] * o[1]);
  double r[2];
  int k = quad_roots(A, B, C, r);
  for (int i = 0; i < k; ++i) {
    double p[3] = {o[0] + r[i] * d[0], o[1] + r[i] * d[1], o[2] + r[i] * d[2]};
    double n[3] = {-c2 * p[0], -c2 * p[1], s2 * p[2]};
    xl_add(L, r[i], n, M);
  }
}

/* pgon faces: plane rho_e(x,y) = r0 + s (z - z0) for each edge e */
static void add_pgon_faces(XList* L, const double* P, const double* o, const double* d, const double* M) {
  int ned = (int)P[2], nz = (int)P[3];
  const double *Z = P + 4, *RMIN = Z + nz, *RMAX = RMIN + nz;
  double sector = P[1] / ned;
  for (int k = 0; k < nz - 1; ++k) {
    double h = Z[k + 1] - Z[k];
    if (h <= 0) continue;
    for (int which = 0; which < 2; ++which) {
      const double* R = which ? RMIN : RMAX;
      if (which && R[k] == 0 && R[k + 1] == 0) continue;
      double s = (R[k + 1] - R[k]) / h;
      /* crossings of a face plane outside its section's z range are no
       * boundary points of the solid; they are skipped */
      double tol = 1e-6 * (h + fabs(Z[k]) + fabs(Z[k + 1])) + 1e-9;
      for (int e = 0; e < ned; ++e) {
        double pe = (P[0] + (e + 0.5) * sector) * D2R;
        double n[3] = {cos(pe), sin(pe), -s};
        /* n . p = R[k] - s Z[k] */
        double rhs = R[k] - s * Z[k];
        double den = dot3(n, d);
        if (den == 0) continue;
        double t = (rhs - dot3(n, o)) / den, zt = o[2] + t * d[2];
        if (zt < Z[k] - tol || zt > Z[k + 1] + tol) continue;
        xl_add(L, t, n, M);
      }
    }
  }
}

/* pcon faces: rho = r0 + s (z - z0) for each segment */
static void add_pcon_faces(XList* L, const double* P, const double* o, const double* d, const double* M) {
  int nz = (int)P[2];
  const double *Z = P + 3, *RMIN = Z + nz, *RMAX = RMIN + nz;
  for (int k = 0; k < nz - 1; ++k) {
    double h = Z[k + 1] - Z[k];
    if (h <= 0) continue;
    for (int which = 0; which < 2; ++which) {
      const double* R = which ? RMIN : RMAX;
      if (which && R[k] == 0 && R[k + 1] == 0) continue;
      double s = (R[k + 1] - R[k]) / h;
      double c0 = R[k] - s * Z[k]; /* rho = c0 + s z */
      double A = d[0] * d[0] + d[1] * d[1] - s * s * d[2] * d[2];
      double B = 2 * (o[0] * d[0] + o[1] * d[1] - s * d[2] * (c0 + s * o[2]));
      double C = o[0] * o[0] + o[1] * o[1] - (c0 + s * o[2]) * (c0 + s * o[2]);
      double r[2];
      int m = quad_roots(A, B, C, r);
      double tol = 1e-6 * (h + fabs(Z[k]) + fabs(Z[k + 1])) + 1e-9;
      for (int i = 0; i < m; ++i) {
        double p[3] = {o[0] + r[i] * d[0], o[1] + r[i] * d[1], o[2] + r[i] * d[2]};
        if (p[2] < Z[k] - tol || p[2] > Z[k + 1] + tol) continue; /* not on this section's cone */
        double rz = c0 + s * p[2];
        double n[3] = {p[0], p[1], -s * rz};
        xl_add(L, r[i], n, M);
      }
    }
  }
}

static void prim_collect(Scene* S, int type, const double* P, const double* o, const double* d,
                         const double* M, XList* L) {
  switch (type) {
    case RBG_SHAPE_BOX: {
      for (int k = 0; k < 3; ++k) {
        if (d[k] == 0) continue;
        double n[3] = {0, 0, 0};
        n[k] = 1;
        xl_add(L, (P[3 + k] - P[k] - o[k]) / d[k], n, M);
        xl_add(L, (P[3 + k] + P[k] - o[k]) / d[k], n, M);
      }
      break;
    }
    case RBG_SHAPE_TUBE:
      add_z_plane(L, o, d, -P[RBG_TUBE_DZ], M);
      add_z_plane(L, o, d, P[RBG_TUBE_DZ], M);
      add_cylinder(L, o, d, P[RBG_TUBE_RMAX], M);
      if (P[RBG_TUBE_RMIN] > 0) add_cylinder(L, o, d, P[RBG_TUBE_RMIN], M);
      add_phi_planes(L, o, d, P[RBG_TUBE_PHI1], P[RBG_TUBE_DPHI], M);
      break;
    case RBG_SHAPE_SPHERE:
      add_sphere(L, o, d, P[RBG_SPH_RMAX], M);
      if (P[RBG_SPH_RMIN] > 0) add_sphere(L, o, d, P[RBG_SPH_RMIN], M);
      if (P[RBG_SPH_TH1] > 0) add_theta_cone(L, o, d, P[RBG_SPH_TH1], M);
      if (P[RBG_SPH_TH2] < 180) add_theta_cone(L, o, d, P[RBG_SPH_TH2], M);
      add_phi_planes(L, o, d, P[RBG_SPH_PHI1], P[RBG_SPH_DPHI], M);
      break;
    case RBG_SHAPE_PARABOLOID: {
      add_z_plane(L, o, d, -P[RBG_PARA_DZ], M);
      add_z_plane(L, o, d, P[RBG_PARA_DZ], M);
      double a = P[RBG_PARA_A], b = P[RBG_PARA_B];
      double A = a * (d[0] * d[0] + d[1] * d[1]);
      double B = 2 * a * (o[0] * d[0] + o[1] * d[1]) - d[2];
      double C = a * (o[0] * o[0] + o[1] * o[1]) + b - o[2];
      double r[2];
      int k = quad_roots(A, B, C, r);
      for (int i = 0; i < k; ++i) {
        double p[3] = {o[0] + r[i] * d[0], o[1] + r[i] * d[1], o[2] + r[i] * d[2]};
        double n[3] = {2 * a * p[0], 2 * a * p[1], -1};
        xl_add(L, r[i], n, M);
      }
      break;
    }
    case RBG_SHAPE_PGON: {
      int nz = (int)P[3];
      for (int k = 0; k < nz; ++k) add_z_plane(L, o, d, P[4 + k], M);
      add_pgon_faces(L, P, o, d, M);
      add_phi_planes(L, o, d, P[0], P[1], M);
      break;
    }
    case RBG_SHAPE_PCON: {
      int nz = (int)P[2];
      for (int k = 0; k < nz; ++k) add_z_plane(L, o, d, P[3 + k], M);
      add_pcon_faces(L, P, o, d, M);
      add_phi_planes(L, o, d, P[0], P[1], M);
      break;
    }
  }
  (void)S;
}

/* generic containment of a primitive/composite shape (point in shape frame) */
static int csg_contains(Scene* S, int shape, const double* p) {
  const rbg_shape_desc* sh = &S->shapes[shape];
  if (sh->type != RBG_SHAPE_COMPOSITE) return prim_contains(S, sh->type, SP(S, shape), p);
  const double* P = SP(S, shape);
  double pl[3], pr[3];
  m_to_local(P + RBG_COMP_ML, p, pl);
  m_to_local(P + RBG_COMP_MR, p, pr);
  int a = csg_contains(S, sh->left, pl);
  if (sh->op == RBG_OP_UNION) return a || csg_contains(S, sh->right, pr);
  if (sh->op == RBG_OP_INTERSECTION) return a && csg_contains(S, sh->right, pr);
  return a && !csg_contains(S, sh->right, pr);
}

/* all surface crossings of a shape tree; o, d in frame F, M: shape -> F */
static void csg_collect(Scene* S, int shape, const double* M, const double* o, const double* d, XList* L) {
  const rbg_shape_desc* sh = &S->shapes[shape];
  double ol[3], dl[3];
  m_to_local(M, o, ol);
  m_dir_to_local(M, d, dl);
  if (sh->type != RBG_SHAPE_COMPOSITE) {
    prim_collect(S, sh->type, SP(S, shape), ol, dl, M, L);
    return;
  }
  const double* P = SP(S, shape);
  double ML[12], MR[12];
  m_mul(M, P + RBG_COMP_ML, ML);
  m_mul(M, P + RBG_COMP_MR, MR);
  csg_collect(S, sh->left, ML, o, d, L);
  csg_collect(S, sh->right, MR, o, d, L);
}

static int xing_cmp(const void* a, const void* b) {
  double ta = ((const Xing*)a)->t, tb = ((const Xing*)b)->t;
  return ta < tb ? -1 : ta > tb ? 1 : 0;
}

static int g_cap_flag_dummy;

/* distance to enter (want_exit = 0) or leave (want_exit = 1) the solid */
static double csg_dist(Scene* S, int shape, const double* o, const double* d, int want_exit, double* nrm,
                       int* cap) {
  XList L;
  L.n = 0;
  L.overflow = 0;
  csg_collect(S, shape, kIdentity, o, d, &L);
  if (L.overflow) {
    *cap = 1;
    return BIG;
  }
  qsort(L.x, L.n, sizeof(Xing), xing_cmp);
  int j0 = 0;
  while (j0 < L.n && L.x[j0].t <= 0) ++j0;
  if (j0 == L.n) return BIG;
  int in_prev;
  if (j0 == 0) {
    in_prev = 0;
  } else {
    double tm = 0.5 * (L.x[j0 - 1].t + L.x[j0].t);
    double p[3] = {o[0] + tm * d[0], o[1] + tm * d[1], o[2] + tm * d[2]};
    in_prev = csg_contains(S, shape, p);
  }
  for (int j = j0; j < L.n; ++j) {
    int in_next = 0;
    if (j + 1 < L.n) {
      double tm = 0.5 * (L.x[j].t + L.x[j + 1].t);
      double p[3] = {o[0] + tm * d[0], o[1] + tm * d[1], o[2] + tm * d[2]};
      in_next = csg_contains(S, shape, p);
    }
    if ((!want_exit && !in_prev && in_next) || (want_exit && in_prev && !in_next)) {
      memcpy(nrm, L.x[j].n, 3 * sizeof(double));
      return L.x[j].t;
    }
    in_prev = in_next;
  }
  return BIG;
}

/* ======================================================================
 * AGeoAsphericDisk (src/AGeoAsphericDisk.cxx)
 * ==================================================================== */
typedef struct {
  double z1, z2, c1, c2, k1, k2, rmin, rmax, oz, dz;
  int n1, n2, rseg;
  const double *K1, *K2;
} Asph;

static void asph_load(const double* P, Asph* a) {
  a->z1 = P[RBG_ASPH_Z1]; a->z2 = P[RBG_ASPH_Z2];
  a->c1 = P[RBG_ASPH_C1]; a->c2 = P[RBG_ASPH_C2];
  a->k1 = P[RBG_ASPH_KAPPA1]; a->k2 = P[RBG_ASPH_KAPPA2];
  a->rmin = P[RBG_ASPH_RMIN]; a->rmax = P[RBG_ASPH_RMAX];
  a->n1 = (int)P[RBG_ASPH_NPOL1]; a->n2 = (int)P[RBG_ASPH_NPOL2];
  a->oz = P[RBG_ASPH_ORIGIN_Z]; a->dz = P[RBG_ASPH_DZ];
  a->rseg = P[RBG_ASPH_RSEG] != 0;
  a->K1 = P + RBG_ASPH_K;
  a->K2 = P + RBG_ASPH_K + a->n1;
}
/* CalcF1/CalcF2 (:126-153); returns 0 where the reference throws */
static int asph_F(const Asph* a, int s, double r, double* f) {
  double c = s == 1 ? a->c1 : a->c2, k = s == 1 ? a->k1 : a->k2, z = s == 1 ? a->z1 : a->z2;
  int n = s == 1 ? a->n1 : a->n2;
  const double* K = s == 1 ? a->K1 : a->K2;
  double p = r * r * c * c * k;
  if (1 - p < 0) return 0;
  double ret = z + r * r * c / (1 + sqrt(1 - p));
  for (int i = 0; i < n; ++i) ret += K[i] * pow(r, 2 * (i + 1));
  *f = ret;
  return 1;
}
/* CalcdF1dr/CalcdF2dr (:96-123) */
static int asph_dF(const Asph* a, int s, double r, double* f) {
  double c = s == 1 ? a->c1 : a->c2, k = s == 1 ? a->k1 : a->k2;
  int n = s == 1 ? a->n1 : a->n2;
  const double* K = s == 1 ? a->K1 : a->K2;
  double p = r * r * c * c * k;
  if (1 - p <= 0) return 0;
  double ret = r * c / sqrt(1 - p);
  for (int i = 0; i < n; ++i) ret += 2 * (i + 1) * K[i] * pow(r, 2 * (i + 1) - 1);
  *f = ret;
  return 1;
}
/* Contains (:330-347) */
static int asph_contains(const Asph* a, const double* p) {
  double r = sqrt(p[0] * p[0] + p[1] * p[1]);
  if (r > a->rmax || r < a->rmin) return 0;
  double f1, f2;
  if (!asph_F(a, 1, r, &f1) || !asph_F(a, 2, r, &f2)) return 0;
  if (p[2] < f1 || f2 < p[2]) return 0;
  return 1;
}
/* DistToAsphere (:415-526) */
static double asph_dist_surface(const Asph* a, int n, const double* point, const double* dir) {
  double curve = n == 1 ? a->c1 : a->c2, kappa = n == 1 ? a->k1 : a->k2;
  int npol = n == 1 ? a->n1 : a->n2;
  const double* K = n == 1 ? a->K1 : a->K2;
  double H2 = point[0] * point[0] + point[1] * point[1];
  double d = n == 1 ? a->z1 : a->z2;
  double p = -((point[2] - d) * dir[2] + point[0] * dir[0] + point[1] * dir[1]);
  double M = p * dir[2] + point[2] - d;
  double M2 = (point[2] - d) * (point[2] - d) + H2 - p * p;
  double check = 1 - (M2 * curve - 2 * M) * curve / dir[2] / dir[2];
  if (check < 0) return BIG;
  double q = p + (M2 * curve - 2 * M) / (dir[2] * (1 + sqrt(check)));
  double np[3] = {point[0] + q * dir[0], point[1] + q * dir[1], point[2] + q * dir[2] - d};
  for (int i = 0;; i++) {
    if (i > 100) return BIG;
    H2 = np[0] * np[0] + np[1] * np[1];
    check = 1 - kappa * H2 * curve * curve;
    if (check < 0) return BIG;
    double l = sqrt(check);
    double x = 0;
    if (curve != 0) x += (1 - l) / curve / kappa;
    for (int j = 0; j < npol; j++) x += K[j] * pow(H2, j + 1);
    double v = 0;
    for (int j = 0; j < npol; j++) v += 2 * (j + 1) * K[j] * pow(H2, j);
    v = curve * kappa + l * v;
    double m = -np[0] * v;
    double nn = -np[1] * v;
    double norm = sqrt(l * l + m * m + nn * nn);
    l /= norm;
    m /= norm;
    nn /= norm;
    check = dir[2] * l + dir[0] * m + dir[1] * nn;
    if (check == 0) return BIG;
    double e = l * (x - np[2]) / check;
    for (int j = 0; j < 3; j++) np[j] += e * dir[j];
    if (fabs(e) < 1e-10) break;
  }
  np[2] += d;
  check = dir[0] * (np[0] - point[0]) + dir[1] * (np[1] - point[1]) + dir[2] * (np[2] - point[2]);
  if (check < 0) return BIG;
  double dist_to_zaxis = pow(np[0] * np[0] + np[1] * np[1], 0.5);
  if (dist_to_zaxis < a->rmin || dist_to_zaxis > a->rmax) return BIG;
  return sqrt(pow(np[0] - point[0], 2) + pow(np[1] - point[1], 2) + pow(np[2] - point[2], 2));
}
/* TGeoTube::DistToTube: b = rdotn/nsq, delta = sqrt(b^2 - (rsq - r^2)/nsq) */
static void dist_to_tube(double rsq, double nsq, double rdotn, double radius, double* b, double* delta) {
  double t1 = 1. / nsq;
  double t3 = rsq - radius * radius;
  *b = t1 * rdotn;
  double c = t1 * t3;
  *delta = *b * *b - c;
  if (*delta > 0) *delta = sqrt(*delta);
  else *delta = -1;
}
/* DistToInner / DistToOuter (:529-684) */
static double asph_dist_wall(const Asph* a, int outer, const double* point, const double* dir) {
  if (!outer && !a->rseg) return BIG;
  double rsq = point[0] * point[0] + point[1] * point[1];
  double nsq = dir[0] * dir[0] + dir[1] * dir[1];
  if (sqrt(nsq) < 1e-10) return BIG;
  double rdotn = point[0] * dir[0] + point[1] * dir[1];
  double R = outer ? a->rmax : a->rmin;
  double b, delta;
  dist_to_tube(rsq, nsq, rdotn, R, &b, &delta);
  if (delta < 0) return BIG;
  double t1 = -b + delta, t2 = -b - delta;
  if (t1 < 0 && t2 < 0) return BIG;
  double zmin, zmax;
  /* CalcF1/CalcF2 are called unprotected here; where they would throw the
   * surface does not reach this radius and the wall is never crossed */
  if (!asph_F(a, 1, R, &zmin) || !asph_F(a, 2, R, &zmax)) return BIG;
  if (t2 > 0) {
    if (t1 > 0) {
      double z1 = t1 * dir[2] + point[2];
      double z2 = t2 * dir[2] + point[2];
      if (z1 < zmin || zmax < z1) t1 = BIG;
      if (z2 < zmin || zmax < z2) t2 = BIG;
      return t1 < t2 ? t1 : t2;
    }
  } else if (t2 == 0) {
    if (t1 > 0) {
      if (zmin <= point[2] && point[2] <= zmax) return 0;
      double z1 = t1 * dir[2] + point[2];
      if (zmin <= z1 && z1 <= zmax) return t1;
    } else if (t1 == 0) {
      if (zmin <= point[2] && point[2] <= zmax) return 0;
    }
  } else {
    if (t1 > 0) {
      double z1 = t1 * dir[2] + point[2];
      if (zmin <= z1 && z1 <= zmax) return t1;
    } else if (t1 == 0) {
      if (zmin <= point[2] && point[2] <= zmax) return 0;
    }
  }
  return BIG;
}
static double asph_dist4(const Asph* a, const double* p, const double* d) {
  double v[4] = {asph_dist_surface(a, 1, p, d), asph_dist_surface(a, 2, p, d), asph_dist_wall(a, 0, p, d),
                 asph_dist_wall(a, 1, p, d)};
  int im = 0; /* TMath::LocMin: first minimum */
  for (int i = 1; i < 4; ++i)
    if (v[i] < v[im]) im = i;
  return v[im];
}
/* bounding-tube test of DistFromOutside (:393-395): does the ray meet the
 * hollow tube (rmin, rmax, dz) around the origin at t >= 0 */
static double tube_reach(Scene* S, const double* o, const double* d, double rmin, double rmax, double dz) {
  double P[RBG_TUBE_NP] = {rmin, rmax, dz, 0, 360};
  XList L;
  L.n = 0;
  L.overflow = 0;
  prim_collect(S, RBG_SHAPE_TUBE, P, o, d, kIdentity, &L);
  qsort(L.x, L.n, sizeof(Xing), xing_cmp);
  if (prim_contains(S, RBG_SHAPE_TUBE, P, o)) return 0;
  for (int j = 0; j + 1 < L.n; ++j) {
    if (L.x[j + 1].t <= 0) continue;
    double tm = 0.5 * (L.x[j].t + L.x[j + 1].t);
    double p[3] = {o[0] + tm * d[0], o[1] + tm * d[1], o[2] + tm * d[2]};
    if (prim_contains(S, RBG_SHAPE_TUBE, P, p)) return L.x[j].t > 0 ? L.x[j].t : 0;
  }
  return BIG;
}
static double asph_dist_out(Scene* S, const Asph* a, const double* p, const double* d) {
  double pp[3] = {p[0], p[1], p[2] - a->oz};
  double sdist = tube_reach(S, pp, d, a->rmin, a->rmax, a->dz);
  if (sdist >= BIG) return BIG;
  return asph_dist4(a, p, d);
}
/* ComputeNormal (:246-327) */
static void asph_normal(const Asph* a, const double* point, const double* dir, double* norm) {
  double r = sqrt(point[0] * point[0] + point[1] * point[1]);
  double phi = atan2(point[1], point[0]);
  double saf[4];
  saf[0] = a->rseg ? fabs(r - a->rmin) : BIG;
  saf[1] = fabs(r - a->rmax);
  double f1, f2, df1 = BIG, df2 = BIG;
  if (!asph_F(a, 1, r, &f1)) f1 = -BIG;
  if (f1 == -BIG) {
    saf[2] = BIG;
  } else {
    if (asph_dF(a, 1, r, &df1)) saf[2] = fabs(f1 - point[2]) / sqrt(1 + df1 * df1);
    else saf[2] = BIG;
  }
  if (!asph_F(a, 2, r, &f2)) f2 = BIG;
  if (f2 == BIG) {
    saf[3] = BIG;
  } else {
    if (asph_dF(a, 2, r, &df2)) saf[3] = fabs(f2 - point[2]) / sqrt(1 + df2 * df2);
    else saf[3] = BIG;
  }
  int i = 0;
  for (int k = 1; k < 4; ++k)
    if (saf[k] < saf[i]) i = k;
  double nv[3] = {0, 0, 0};
  if (i == 0 || i == 1) {
    nv[0] = 1;
  } else if (i == 2) {
    if (df1 == 0) nv[2] = 1;
    else { nv[0] = df1 / sqrt(1 + df1 * df1); nv[2] = -1 / sqrt(1 + df1 * df1); }
  } else {
    if (df2 == 0) nv[2] = 1;
    else { nv[0] = df2 / sqrt(1 + df2 * df2); nv[2] = -1 / sqrt(1 + df2 * df2); }
  }
  /* TVector3::RotateZ(phi) */
  double c = cos(phi), s = sin(phi);
  norm[0] = c * nv[0] - s * nv[1];
  norm[1] = s * nv[0] + c * nv[1];
  norm[2] = nv[2];
  if (norm[0] * dir[0] + norm[1] * dir[1] + norm[2] * dir[2] < 0) {
    norm[0] = -norm[0]; norm[1] = -norm[1]; norm[2] = -norm[2];
  }
}

/* ======================================================================
 * AGeoWinstonConePoly (src/AGeoWinstonConePoly.cxx, AGeoWinstonCone2D.cxx)
 * ==================================================================== */
typedef struct {
  double r1, r2, theta, f, dz;
  int n;
} Win;
static void win_load(const double* P, Win* w) {
  w->r1 = P[RBG_WIN_R1]; w->r2 = P[RBG_WIN_R2]; w->n = (int)P[RBG_WIN_N];
  w->theta = P[RBG_WIN_THETA]; w->f = P[RBG_WIN_F]; w->dz = P[RBG_WIN_DZ];
}
/* CalcR (AGeoWinstonCone2D.cxx:82-98) */
static int win_R(const Win* w, double z, double* r) {
  if (fabs(z) > w->dz + 1e-10) return 0;
  double sint = sin(w->theta), cost = cos(w->theta);
  double t = z + w->dz;
  double a0 = t * t * sint * sint - 4. * w->f * (t * cost + w->f);
  double a1 = 2. * t * sint * cost + 4. * w->f * sint;
  double a2 = cost * cost;
  *r = (-a1 + sqrt(a1 * a1 - 4. * a0 * a2)) / (2 * a2) - w->r2;
  return 1;
}
/* CalcdRdZ (:59-79) */
static double win_dRdZ(const Win* w, double z) {
  double sint = sin(w->theta), cost = cos(w->theta);
  double t = z + w->dz;
  double a0 = t * t * sint * sint - 4. * w->f * (t * cost + w->f);
  double a1 = 2. * t * sint * cost + 4. * w->f * sint;
  double a2 = cost * cost;
  double da0dt = 2 * t * sint * sint - 4 * w->f * cost;
  double da1dt = 2 * sint * cost;
  return (-da1dt + (a1 * da1dt - 2 * da0dt * a2) / sqrt(a1 * a1 - 4 * a0 * a2)) / (2 * a2);
}
/* InsidePolygon (ConePoly.cxx:293-309) */
static int win_inside_polygon(const Win* w, double x, double y, double r) {
  double theta = atan2(y, x);
  while (theta > PI / w->n) theta -= 2 * PI / w->n;
  while (theta < -PI / w->n) theta += 2 * PI / w->n;
  if (sqrt(x * x + y * y) * cos(theta) > r) return 0;
  return 1;
}
static int win_contains(const Win* w, const double* p) {
  if (fabs(p[2]) > w->dz) return 0;
  double r;
  if (!win_R(w, p[2], &r)) return 0;
  return win_inside_polygon(w, p[0], p[1], r);
}
/* DistToParabola (Cone2D.cxx:325-428) */
static double win_dist_parabola(const Win* w, const double* point, const double* dir, double phi, double open) {
  double x = cos(phi) * point[0] + sin(phi) * point[1];
  double y = -sin(phi) * point[0] + cos(phi) * point[1];
  double z = point[2];
  double px = cos(phi) * dir[0] + sin(phi) * dir[1];
  double py = -sin(phi) * dir[0] + cos(phi) * dir[1];
  double pz = dir[2];
  if (px == 0 && pz == 0) return BIG;
  double cost = cos(w->theta), sint = sin(w->theta);
  double X = cost * (x + w->r2) + (z + w->dz) * sint;
  double Z = -sint * (x + w->r2) + (z + w->dz) * cost + w->f;
  double alpha = atan2(pz, px);
  double ALPHA = alpha - w->theta;
  double tanA = tan(ALPHA);
  double dist[2];
  double tmp = tanA * tanA - (X * tanA - Z) / w->f;
  if (tmp < 0) {
    dist[0] = BIG;
    dist[1] = BIG;
  } else {
    double Xp, Xm;
    if (w->dz * 2 / fabs(tanA) < 1e-10) {
      Xp = X;
      Xm = X;
    } else {
      Xp = 2 * w->f * (tanA + sqrt(tmp));
      Xm = 2 * w->f * (tanA - sqrt(tmp));
    }
    double Zp = Xp * Xp / 4. / w->f, Zm = Xm * Xm / 4. / w->f;
    double xp = cost * Xp - sint * (Zp - w->f) - w->r2;
    double xm = cost * Xm - sint * (Zm - w->f) - w->r2;
    double zp = sint * Xp + cost * (Zp - w->f) - w->dz;
    double zm = sint * Xm + cost * (Zm - w->f) - w->dz;
    double yp, ym;
    if (fabs(px) <= fabs(pz) && fabs(py) <= fabs(pz)) {
      yp = y + (zp - z) * py / pz;
      ym = y + (zm - z) * py / pz;
    } else if (fabs(py) <= fabs(px) && fabs(pz) <= fabs(px)) {
      yp = y + (xp - x) * py / px;
      ym = y + (xm - x) * py / px;
    } else {
      yp = y + (fabs(px) < 1e-5 ? (zp - z) * py / pz : (xp - x) * py / px);
      ym = y + (fabs(px) < 1e-5 ? (zm - z) * py / pz : (xm - x) * py / px);
    }
    double dx = xp - x, dy = yp - y, dz = zp - z;
    if (xp < w->r2 || w->r1 < xp || zp < -w->dz || w->dz < zp || dx * px + dz * pz < 0) {
      dist[0] = BIG;
    } else {
      dist[0] = fabs(atan2(yp, xp)) <= open / 2. ? sqrt(dx * dx + dy * dy + dz * dz) : BIG;
    }
    dx = xm - x; dy = ym - y; dz = zm - z;
    if (xm < w->r2 || w->r1 < xm || zm < -w->dz || w->dz < zm || dx * px + dz * pz < 0) {
      dist[1] = BIG;
    } else {
      dist[1] = fabs(atan2(ym, xm)) <= open / 2. ? sqrt(dx * dx + dy * dy + dz * dz) : BIG;
    }
  }
  return dist[0] < dist[1] ? dist[0] : dist[1];
}
/* DistFromInside (ConePoly.cxx:150-178) */
static double win_dist_in(const Win* w, const double* p, const double* d) {
  double best = BIG;
  if (d[2] < 0) best = (-p[2] - w->dz) / d[2];
  else if (d[2] > 0) best = (w->dz - p[2]) / d[2];
  for (int i = 0; i < w->n; i++) {
    double v = win_dist_parabola(w, p, d, i * 2 * PI / w->n, PI);
    if (v < best) best = v;
  }
  return best;
}
/* DistFromOutside (ConePoly.cxx:181-226) */
static double win_dist_out(const Win* w, const double* p, const double* d) {
  if (p[2] <= -w->dz) {
    if (d[2] <= 0) return BIG;
    double s = -(w->dz + p[2]) / d[2];
    if (win_inside_polygon(w, p[0] + s * d[0], p[1] + s * d[1], w->r2)) return s;
  } else if (p[2] >= w->dz) {
    if (d[2] >= 0) return BIG;
    double s = (w->dz - p[2]) / d[2];
    if (win_inside_polygon(w, p[0] + s * d[0], p[1] + s * d[1], w->r1)) return s;
  }
  double best = BIG;
  for (int i = 0; i < w->n; i++) {
    double v = win_dist_parabola(w, p, d, i * 2 * PI / w->n, 2 * PI / w->n);
    if (v < best) best = v;
  }
  return best;
}
/* ComputeNormal (ConePoly.cxx:67-122) */
static void win_normal(const Win* w, const double* point, const double* dir, double* norm) {
  double x = point[0], y = point[1], z = point[2];
  double saf[2];
  saf[0] = fabs(fabs(w->dz) - fabs(z));
  double phi = atan2(y, x);
  while (phi > PI / w->n) phi -= 2 * PI / w->n;
  while (phi < -PI / w->n) phi += 2 * PI / w->n;
  double R;
  if (win_R(w, z, &R)) saf[1] = fabs(R - sqrt(x * x + y * y) * cos(phi));
  else saf[1] = BIG;
  if (saf[0] <= saf[1]) {
    norm[0] = 0; norm[1] = 0; norm[2] = 1;
  } else {
    phi = atan2(y, x);
    if (phi < -PI / w->n) phi += 2 * PI;
    int n = (int)floor((phi + PI / w->n) / (2 * PI / w->n));
    norm[0] = cos(n * 2 * PI / w->n);
    norm[1] = sin(n * 2 * PI / w->n);
    norm[2] = -win_dRdZ(w, z);
  }
  normalize3(norm);
  if (norm[0] * dir[0] + norm[1] * dir[1] + norm[2] * dir[2] < 0) {
    norm[0] = -norm[0]; norm[1] = -norm[1]; norm[2] = -norm[2];
  }
}

/* ======================================================================
 * AGeoWinstonCone2D (src/AGeoWinstonCone2D.cxx): the trough of two
 * parabolic walls x = +-R(z), |y| <= dy.  Canonical parameters as the
 * polygonal cone with n = 2 and the half-length in RBG_WIN_DY.
 * ==================================================================== */
/* Contains (:175-190) */
static int win2d_contains(const Win* w, double dy, const double* p) {
  double r;
  if (fabs(p[1]) > dy || fabs(p[2]) > w->dz) return 0;
  if (!win_R(w, p[2], &r)) return 0;
  return !(fabs(p[0]) > r);
}
/* DistFromInside (:203-238) */
static double win2d_dist_in(const Win* w, double dy, const double* p, const double* d) {
  double v[4];
  int i, k = 0;
  v[0] = BIG;
  if (d[2] < 0) v[0] = -(p[2] + w->dz) / d[2];
  else if (d[2] > 0) v[0] = (w->dz - p[2]) / d[2];
  v[1] = BIG;
  if (d[1] < 0) v[1] = -(p[1] + dy) / d[1];
  else if (d[1] > 0) v[1] = (dy - p[1]) / d[1];
  v[2] = win_dist_parabola(w, p, d, 0., PI);
  v[3] = win_dist_parabola(w, p, d, PI, PI);
  for (i = 1; i < 4; ++i)
    if (v[i] < v[k]) k = i;
  return v[k];
}
/* DistFromOutside (:241-322) */
static double win2d_dist_out(const Win* w, double dy, const double* p, const double* d) {
  double s, r, a, b;
  if (p[2] <= -w->dz) {
    if (d[2] <= 0) return BIG;
    s = -(w->dz + p[2]) / d[2];
    if (fabs(p[0] + s * d[0]) <= w->r2 && fabs(p[1] + s * d[1]) <= dy) return s;
  } else if (p[2] >= w->dz) {
    if (d[2] >= 0) return BIG;
    s = (w->dz - p[2]) / d[2];
    if (fabs(p[0] + s * d[0]) <= w->r1 && fabs(p[1] + s * d[1]) <= dy) return s;
  }
  if (p[1] <= -dy) {
    if (d[1] <= 0) return BIG;
    s = -(dy + p[1]) / d[1];
    if (fabs(p[2] + s * d[2]) <= w->dz && win_R(w, p[2] + s * d[2], &r) && fabs(p[0] + s * d[0]) <= r) return s;
  } else if (p[1] >= dy) {
    if (d[1] >= 0) return BIG;
    s = (dy - p[1]) / d[1];
    if (fabs(p[2] + s * d[2]) <= w->dz && win_R(w, p[2] + s * d[2], &r) && fabs(p[0] + s * d[0]) <= r) return s;
  }
  s = win_dist_parabola(w, p, d, 0., PI);
  a = fabs(p[1] + s * d[1]) <= dy ? s : BIG;
  s = win_dist_parabola(w, p, d, PI, PI);
  b = fabs(p[1] + s * d[1]) <= dy ? s : BIG;
  return a < b ? a : b;
}
/* ComputeNormal (:120-172) */
static void win2d_normal(const Win* w, double dy, const double* p, const double* dir, double* n) {
  double saf[3], r, m;
  int i = 0, k;
  saf[0] = fabs(fabs(dy) - fabs(p[1]));
  saf[1] = fabs(fabs(w->dz) - fabs(p[2]));
  saf[2] = win_R(w, p[2], &r) ? fabs(r - fabs(p[0])) : BIG;
  for (k = 1; k < 3; ++k)
    if (saf[k] < saf[i]) i = k;
  if (i == 0) {
    n[0] = 0; n[1] = 1; n[2] = 0;
  } else if (i == 1) {
    n[0] = 0; n[1] = 0; n[2] = 1;
  } else {
    n[0] = 1; n[1] = 0;
    n[2] = p[0] > 0 ? -win_dRdZ(w, p[2]) : win_dRdZ(w, p[2]);
  }
  m = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  n[0] /= m; n[1] /= m; n[2] /= m;
  if (n[0] * dir[0] + n[1] * dir[1] + n[2] * dir[2] < 0) {
    n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2];
  }
}

/* ======================================================================
 * shape dispatch (node-local frame)
 * ==================================================================== */
static int is_ageo(int type) {
  return type == RBG_SHAPE_ASPHERIC_DISK || type == RBG_SHAPE_WINSTON_POLY || type == RBG_SHAPE_WINSTON_2D;
}

static int shape_contains(Scene* S, int shape, const double* p) {
  int type = S->shapes[shape].type;
  if (type == RBG_SHAPE_ASPHERIC_DISK) {
    Asph a;
    asph_load(SP(S, shape), &a);
    return asph_contains(&a, p);
  }
  if (type == RBG_SHAPE_WINSTON_POLY) {
    Win w;
    win_load(SP(S, shape), &w);
    return win_contains(&w, p);
  }
  if (type == RBG_SHAPE_WINSTON_2D) {
    Win w;
    win_load(SP(S, shape), &w);
    return win2d_contains(&w, SP(S, shape)[RBG_WIN_DY], p);
  }
  return csg_contains(S, shape, p);
}
static double shape_dist(Scene* S, int shape, const double* p, const double* d, int exit, double* nrm,
                         int* cap) {
  int type = S->shapes[shape].type;
  if (type == RBG_SHAPE_ASPHERIC_DISK) {
    Asph a;
    asph_load(SP(S, shape), &a);
    return exit ? asph_dist4(&a, p, d) : asph_dist_out(S, &a, p, d);
  }
  if (type == RBG_SHAPE_WINSTON_POLY) {
    Win w;
    win_load(SP(S, shape), &w);
    return exit ? win_dist_in(&w, p, d) : win_dist_out(&w, p, d);
  }
  if (type == RBG_SHAPE_WINSTON_2D) {
    Win w;
    const double dy = SP(S, shape)[RBG_WIN_DY];
    win_load(SP(S, shape), &w);
    return exit ? win2d_dist_in(&w, dy, p, d) : win2d_dist_out(&w, dy, p, d);
  }
  return csg_dist(S, shape, p, d, exit, nrm, cap);
}
double orc_shape_dist_out(Scene* S, int shape, const double* p, const double* d) {
  double n[3];
  int cap = 0;
  return shape_dist(S, shape, p, d, 0, n, &cap);
}
double orc_shape_dist_in(Scene* S, int shape, const double* p, const double* d) {
  double n[3];
  int cap = 0;
  return shape_dist(S, shape, p, d, 1, n, &cap);
}
int orc_shape_contains(Scene* S, int shape, const double* p) { return shape_contains(S, shape, p); }

/* ======================================================================
 * navigator
 * ==================================================================== */
typedef struct {
  int node;        /* current node, -1: outside the top volume */
  double p[3], d[3];
  int xnode;       /* node whose surface the last step crossed */
  double xn[3];    /* its normal (primitive shapes), node-local */
} Nav;

static int node_contains(Scene* S, int k, const double* p) {
  const rbg_node* N = &S->nodes[k];
  for (int a = 0; a < 3; ++a)
    if (p[a] < N->lo[a] || p[a] > N->hi[a]) return 0;
  double l[3];
  m_to_local(N->m, p, l);
  return shape_contains(S, N->shape, l);
}
/* ray segment [0, smax] against an axis-aligned box (conservative cull) */
static int seg_box(const double* o, const double* d, double smax, const double* lo, const double* hi) {
  double t0 = 0, t1 = smax;
  for (int a = 0; a < 3; ++a) {
    if (d[a] == 0) {
      if (o[a] < lo[a] || o[a] > hi[a]) return 0;
      continue;
    }
    double inv = 1.0 / d[a];
    double ta = (lo[a] - o[a]) * inv, tb = (hi[a] - o[a]) * inv;
    if (ta > tb) { double s = ta; ta = tb; tb = s; }
    if (ta > t0) t0 = ta;
    if (tb < t1) t1 = tb;
    if (t0 > t1) return 0;
  }
  return 1;
}
static int locate_down(Scene* S, int k, const double* p) {
  for (;;) {
    const rbg_node* N = &S->nodes[k];
    int found = -1;
    for (int i = 0; i < N->child_count; ++i) {
      int c = S->children[N->child_begin + i];
      if (node_contains(S, c, p)) {
        found = c;
        break;
      }
    }
    if (found < 0) return k;
    k = found;
  }
}
static int locate_from_top(Scene* S, const double* p) {
  if (!node_contains(S, 0, p)) return -1;
  return locate_down(S, 0, p);
}

/* TGeoNavigator::FindNextBoundaryAndStep restated; returns the new node */
static int nav_find_next_boundary_and_step(Scene* S, Nav* nv, double* step, int* cap) {
  int c = nv->node;
  double best = BIG, nbest[3] = {0, 0, 1};
  int xnode = -1, enter = 0;
  if (c < 0) {
    /* outside the top volume: the only boundary is the top's */
    const rbg_node* T = &S->nodes[0];
    double pl[3], dl[3], n[3];
    m_to_local(T->m, nv->p, pl);
    m_dir_to_local(T->m, nv->d, dl);
    best = shape_dist(S, T->shape, pl, dl, 0, n, cap);
    if (best >= BIG) {
      *step = 0;
      nv->xnode = -1;
      return -1;
    }
    memcpy(nbest, n, sizeof(n));
    xnode = 0;
    enter = 1;
  } else {
    const rbg_node* N = &S->nodes[c];
    double pl[3], dl[3], n[3];
    m_to_local(N->m, nv->p, pl);
    m_dir_to_local(N->m, nv->d, dl);
    best = shape_dist(S, N->shape, pl, dl, 1, n, cap);
    memcpy(nbest, n, sizeof(n));
    xnode = c;
    for (int i = 0; i < N->child_count; ++i) {
      int k = S->children[N->child_begin + i];
      const rbg_node* K = &S->nodes[k];
      if (!seg_box(nv->p, nv->d, best, K->lo, K->hi)) continue;
      m_to_local(K->m, nv->p, pl);
      m_dir_to_local(K->m, nv->d, dl);
      double s = shape_dist(S, K->shape, pl, dl, 0, n, cap);
      if (s < best) {
        best = s;
        xnode = k;
        enter = 1;
        memcpy(nbest, n, sizeof(n));
      }
    }
  }
  for (int a = 0; a < 3; ++a) nv->p[a] += (best + RBG_BOUNDARY_PUSH) * nv->d[a];
  nv->xnode = xnode;
  memcpy(nv->xn, nbest, sizeof(nbest));
  int next;
  if (enter) {
    next = locate_down(S, xnode, nv->p);
  } else {
    int q = S->nodes[c].parent;
    while (q >= 0 && !node_contains(S, q, nv->p)) q = S->nodes[q].parent;
    next = q < 0 ? -1 : locate_down(S, q, nv->p);
  }
  nv->node = next;
  *step = best;
  return next;
}

/* TGeoNavigator::FindNormal restated: normal of the crossed surface in the
 * master frame with n . d >= 0 */
static void nav_find_normal(Scene* S, const Nav* nv, double* n) {
  if (nv->xnode < 0) {
    n[0] = 0; n[1] = 0; n[2] = 1;
    return;
  }
  const rbg_node* N = &S->nodes[nv->xnode];
  int type = S->shapes[N->shape].type;
  double nl[3];
  if (is_ageo(type)) {
    double pl[3], dl[3];
    m_to_local(N->m, nv->p, pl);
    m_dir_to_local(N->m, nv->d, dl);
    if (type == RBG_SHAPE_ASPHERIC_DISK) {
      Asph a;
      asph_load(SP(S, N->shape), &a);
      asph_normal(&a, pl, dl, nl);
    } else if (type == RBG_SHAPE_WINSTON_2D) {
      Win w;
      win_load(SP(S, N->shape), &w);
      win2d_normal(&w, SP(S, N->shape)[RBG_WIN_DY], pl, dl, nl);
    } else {
      Win w;
      win_load(SP(S, N->shape), &w);
      win_normal(&w, pl, dl, nl);
    }
  } else {
    memcpy(nl, nv->xn, sizeof(nl));
  }
  m_dir_to_master(N->m, nl, n);
  normalize3(n);
  if (dot3(n, nv->d) < 0) {
    n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2];
  }
}

/* ======================================================================
 * AOpticsManager state machine (src/AOpticsManager.cxx:52-520)
 * ==================================================================== */
typedef struct {
  /* ARay */
  double x[4];     /* last point (x, y, z, t) */
  double d[3];     /* direction */
  double lambda;
  int status;
  int npoints;
  int last_node;
  /* history */
  int hist_cap;
  double* hist_xyzt;
  int32_t* hist_node;
  Rng rng;
  int cap;
} Ray;

static void ray_add_point(Ray* r, const double* p, double t) {
  r->x[0] = p[0]; r->x[1] = p[1]; r->x[2] = p[2]; r->x[3] = t;
  if (r->npoints < r->hist_cap) {
    double* h = r->hist_xyzt + 4 * (size_t)r->npoints;
    h[0] = p[0]; h[1] = p[1]; h[2] = p[2]; h[3] = t;
    r->hist_node[r->npoints] = -2;
  }
  r->npoints++;
}
static void ray_add_node(Ray* r, int node) {
  r->last_node = node;
  int idx = r->npoints - 1;
  if (idx >= 0 && idx < r->hist_cap) r->hist_node[idx] = node;
}
/* ARay::SetDirection: normalise; ignored when the magnitude is not > 0 */
static void ray_set_direction(Ray* r, const double* d) {
  double mag = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (mag > 0) {
    r->d[0] = d[0] / mag; r->d[1] = d[1] / mag; r->d[2] = d[2] / mag;
  }
}

static int kind_of(Scene* S, int node) { return node < 0 ? 6 /* kNull */ : S->nodes[node].kind; }
enum { kLens = 0, kObs = 1, kMirror = 2, kFocus = 3, kOpt = 4, kOther = 5, kNull = 6 };

/* AOpticalComponent::FindBorderSurfaceCondition (src/AOpticalComponent.cxx:51-65) */
static const rbg_border_desc* find_border(Scene* S, int cur, int next) {
  if (cur < 0) return NULL;
  int c1 = S->nodes[cur].volume;
  int c2 = next < 0 ? -1 : S->nodes[next].volume;
  for (int i = 0; i < S->n_borders; ++i)
    if (S->borders[i].component1 == c1 && S->borders[i].component2 == c2) return &S->borders[i];
  return NULL;
}

static double lens_n(Scene* S, int node, double lam) {
  return orc_refractive_index(S, S->volumes[S->nodes[node].volume].index, lam);
}

/* TVector3::RotateUz: rotate v from the frame whose z axis is u */
static void rotate_uz(double* v, const double* u) {
  double u1 = u[0], u2 = u[1], u3 = u[2];
  double up = u1 * u1 + u2 * u2;
  if (up > 0) {
    up = sqrt(up);
    double px = v[0], py = v[1], pz = v[2];
    v[0] = (u1 * u3 * px - u2 * py) / up + u1 * pz;
    v[1] = (u2 * u3 * px + u1 * py) / up + u2 * pz;
    v[2] = -up * px + u3 * pz;
  } else if (u3 < 0.) {
    v[0] = -v[0];
    v[2] = -v[2];
  }
}

/* GetFacetNormal (:250-301) */
static void get_facet_normal(Scene* S, Nav* nv, Ray* r, int cur, int next, double* out) {
  double normal[3];
  nav_find_normal(S, nv, normal);
  const double* momentum = nv->d;
  const rbg_border_desc* cond = find_border(S, cur, next);
  if (cond && cond->lambertian) {
    memcpy(out, normal, sizeof(normal));
    return;
  }
  if (cond && cond->sigma != 0) {
    double sigma = cond->sigma;
    double f_max = fmin(1., 4. * sigma);
    double facet[3];
    int tries = 0;
    for (;;) {
      double alpha;
      for (;;) {
        alpha = rng_gaus(&r->rng, sigma);
        double u = f_max * rng_u(&r->rng);
        if (!(u > sin(alpha) || alpha >= PI / 2)) break;
        if (++tries > RBG_ROUGH_MAX_TRIES) goto capped;
      }
      double phi = 2 * PI * rng_u(&r->rng);
      facet[0] = sin(alpha) * cos(phi);
      facet[1] = sin(alpha) * sin(phi);
      facet[2] = cos(alpha);
      rotate_uz(facet, normal);
      if (dot3(momentum, facet) > 0.0) break;
      if (++tries > RBG_ROUGH_MAX_TRIES) goto capped;
    }
    memcpy(out, facet, sizeof(facet));
    return;
  capped:
    r->cap = 1;
  }
  memcpy(out, normal, sizeof(normal));
}

/* TGeoRotation(phi, theta, psi) (Euler, deg): R = Rz(phi) Rx(theta) Rz(psi) */
static void euler_matrix(double phi, double theta, double psi, double* R) {
  double sf = sin(phi * D2R), cf = cos(phi * D2R);
  double st = sin(theta * D2R), ct = cos(theta * D2R);
  double sp = sin(psi * D2R), cp = cos(psi * D2R);
  R[0] = cp * cf - ct * sf * sp;
  R[1] = -sp * cf - ct * sf * cp;
  R[2] = st * sf;
  R[3] = cp * sf + ct * cf * sp;
  R[4] = -sp * sf + ct * cf * cp;
  R[5] = -st * cf;
  R[6] = sp * st;
  R[7] = cp * st;
  R[8] = ct;
}

/* DoReflection (:170-247) */
static void do_reflection(Scene* S, Nav* nv, Ray* r, double n1, double step, int cur, int next,
                          const double* normal) {
  double n[3];
  if (normal) memcpy(n, normal, sizeof(n));
  else get_facet_normal(S, nv, r, cur, next, n);
  double d1[3] = {r->d[0], r->d[1], r->d[2]};
  double cos1 = dot3(d1, n);
  const rbg_border_desc* cond = find_border(S, cur, next);
  int absorbed = 0;
  if (kind_of(S, next) == kMirror) {
    double angle = acos(cos1);
    double ref, trans;
    if (cond && cond->multilayer >= 0) orc_coherent_tmm_mixed(S, cond->multilayer, angle, r->lambda, &ref, &trans);
    else ref = orc_mirror_reflectance(S, S->nodes[next].volume, r->lambda, angle);
    if (ref < rng_u(&r->rng)) {
      absorbed = 1;
      r->status = RBG_ABSORB;
    }
  }
  double d2[3];
  if (cond && cond->lambertian) {
    double y = 0.5 * rng_u(&r->rng);
    double theta = asin(sqrt(2 * y));
    double phi = 2 * PI * rng_u(&r->rng);
    double th_n = (n[0] == 0 && n[1] == 0 && n[2] == 0) ? 0 : atan2(sqrt(n[0] * n[0] + n[1] * n[1]), n[2]);
    double ph_n = (n[0] == 0 && n[1] == 0) ? 0 : atan2(n[1], n[0]);
    double R[9];
    euler_matrix(ph_n / D2R + 90, th_n / D2R + 180, 0, R);
    double v[3] = {sin(theta) * cos(phi), sin(theta) * sin(phi), cos(theta)};
    d2[0] = R[0] * v[0] + R[1] * v[1] + R[2] * v[2];
    d2[1] = R[3] * v[0] + R[4] * v[1] + R[5] * v[2];
    d2[2] = R[6] * v[0] + R[7] * v[1] + R[8] * v[2];
  } else {
    for (int i = 0; i < 3; i++) d2[i] = d1[i] - 2 * n[i] * cos1;
  }
  if (!absorbed) ray_set_direction(r, d2);
  double speed = RBG_SPEED_OF_LIGHT_CM / n1;
  double t = r->x[3] + step / speed;
  /* step back by kEpsilon along -d1 and relocate, then continue along d2 */
  for (int a = 0; a < 3; ++a) nv->p[a] -= RBG_REFLECT_BACKSTEP * d1[a];
  nv->node = locate_from_top(S, nv->p);
  memcpy(nv->d, d2, sizeof(d2));
  ray_add_point(r, nv->p, t);
  ray_add_node(r, next);
}

/* DoFresnel (:52-167) */
static void do_fresnel(Scene* S, Nav* nv, Ray* r, double n1, double n2, double k2, double step, int cur,
                       int next, int disable_fresnel) {
  double n[3];
  get_facet_normal(S, nv, r, cur, next, n);
  double d1[3] = {r->d[0], r->d[1], r->d[2]};
  double cos1 = dot3(d1, n);
  double sin1 = sqrt(1 - cos1 * cos1);
  double sin2 = n1 * sin1 / n2;
  double cos2 = sqrt(1 - sin2 * sin2);
  const rbg_border_desc* cond = find_border(S, cur, next);
  int absorbed = 0;
  if (cond && cond->multilayer >= 0) {
    double reflectance, transmittance;
    double angle = acos(cos1);
    orc_coherent_tmm_mixed(S, cond->multilayer, angle, r->lambda, &reflectance, &transmittance);
    double rnd = rng_u(&r->rng);
    if (rnd < reflectance) {
      do_reflection(S, nv, r, n1, step, cur, next, n);
      return;
    } else if (rnd < reflectance + transmittance) {
      goto transmission;
    } else {
      absorbed = 1;
      goto transmission;
    }
  }
  if (sin2 > 1.) {
    do_reflection(S, nv, r, n1, step, cur, next, n);
    return;
  }
  if (!disable_fresnel) {
    double Rs, Rp;
#define SQ(v) ((v) * (v))
    if (k2 <= 0.) {
      double eta1S = n1 * cos1, eta2S = n2 * cos2;
      double eta1P = n1 / cos1, eta2P = n2 / cos2;
      Rs = SQ((eta1S - eta2S) / (eta1S + eta2S));
      Rp = SQ((eta1P - eta2P) / (eta1P + eta2P));
    } else {
      double eta1S = n1 * cos1, eta1P = n1 / cos1;
      double x1S = eta1S, x1P = eta1P;
      double u = SQ(n2) - SQ(k2) - SQ(n1 * sin1);
      double v = 2 * n2 * k2;
      double tmp = sqrt(SQ(u) + SQ(v));
      double cosxi2 = sqrt(1 + u / tmp) / sqrt(2.0);
      double sinxi2 = sqrt(1 - u / tmp) / sqrt(2.0);
      double x2S = sqrt(tmp) * cosxi2;
      double y2S = sqrt(tmp) * sinxi2;
      tmp = SQ(x2S) + SQ(y2S);
      double x2P = (2 * n2 * k2 * y2S + (SQ(n2) - SQ(k2)) * x2S) / tmp;
      double y2P = (2 * n2 * k2 * x2S - (SQ(n2) - SQ(k2)) * y2S) / tmp;
      Rs = (SQ(x1S - x2S) + SQ(y2S)) / (SQ(x1S + x2S) + SQ(y2S));
      Rp = (SQ(x1P - x2P) + SQ(y2P)) / (SQ(x1P + x2P) + SQ(y2P));
    }
#undef SQ
    double R = (Rs + Rp) / 2.;
    if (rng_u(&r->rng) < R) {
      do_reflection(S, nv, r, n1, step, cur, next, n);
      return;
    }
  }
transmission: {
  double d2[3];
  for (int i = 0; i < 3; i++) {
    if (sin1 != 0) d2[i] = (d1[i] - cos1 * n[i]) * sin2 / sin1 + n[i] * cos2;
    else d2[i] = d1[i];
  }
  double speed = RBG_SPEED_OF_LIGHT_CM / n1;
  double t = r->x[3] + step / speed;
  ray_add_point(r, nv->p, t);
  ray_add_node(r, next);
  if (absorbed) {
    r->status = RBG_ABSORB;
  } else {
    ray_set_direction(r, d2);
    memcpy(nv->d, d2, sizeof(d2));
  }
}
}

/* TraceNonSequential(TObjArray*) loop body for one ray (:346-518) */
static void trace_ray(Scene* S, Ray* r, const rbg_trace_opts* o) {
  Nav nv;
  memcpy(nv.p, r->x, 3 * sizeof(double));
  memcpy(nv.d, r->d, 3 * sizeof(double));
  nv.node = locate_from_top(S, nv.p); /* InitTrack */
  nv.xnode = -1;
  const double lambda = r->lambda;
  while (r->status == RBG_RUN) {
    double x1[4] = {r->x[0], r->x[1], r->x[2], r->x[3]};
    double d1[3] = {r->d[0], r->d[1], r->d[2]};
    int cur = nv.node;
    double step;
    int next = nav_find_next_boundary_and_step(S, &nv, &step, &r->cap);
    int tc = kind_of(S, cur), tn = kind_of(S, next);

    if (tc == kLens) {
      double abs = absorption_length(S, S->volumes[S->nodes[cur].volume].index, lambda);
      if (abs > 0 && abs != INFINITY) {
        double abs_step = rng_exp(&r->rng, abs);
        if (abs_step < step) {
          double n1 = lens_n(S, cur, lambda);
          double speed = RBG_SPEED_OF_LIGHT_CM / n1;
          double x2[3];
          for (int i = 0; i < 3; i++) x2[i] = x1[i] + abs_step * d1[i];
          ray_add_point(r, x2, x1[3] + abs_step / speed);
          ray_add_node(r, next);
          r->status = RBG_ABSORB;
          continue;
        }
      }
    }

    if ((tc == kNull || tc == kOpt || tc == kLens || tc == kOther) && tn == kMirror) {
      double n1 = tc == kLens ? lens_n(S, cur, lambda) : 1.;
      do_reflection(S, &nv, r, n1, step, cur, next, NULL);
    } else if ((tc == kNull || tc == kOpt || tc == kOther) && tn == kLens) {
      int idx = S->volumes[S->nodes[next].volume].index;
      do_fresnel(S, &nv, r, 1, orc_refractive_index(S, idx, lambda), orc_extinction(S, idx, lambda), step, cur,
                 next, o->disable_fresnel);
    } else if ((tc == kNull || tc == kLens || tc == kOpt || tc == kOther) && (tn == kObs || tn == kFocus)) {
      double speed = tc == kLens ? RBG_SPEED_OF_LIGHT_CM / lens_n(S, cur, lambda) : RBG_SPEED_OF_LIGHT_CM;
      ray_add_point(r, nv.p, x1[3] + step / speed);
      ray_add_node(r, next);
    } else if ((tc == kNull || tc == kOpt || tc == kOther) && (tn == kOther || tn == kOpt)) {
      ray_add_point(r, nv.p, x1[3] + step / RBG_SPEED_OF_LIGHT_CM);
      ray_add_node(r, next);
    } else if (tc == kLens && tn == kLens) {
      int idx = S->volumes[S->nodes[next].volume].index;
      do_fresnel(S, &nv, r, lens_n(S, cur, lambda), orc_refractive_index(S, idx, lambda),
                 orc_extinction(S, idx, lambda), step, cur, next, o->disable_fresnel);
    } else if (tc == kLens && (tn == kNull || tn == kOpt || tn == kOther)) {
      do_fresnel(S, &nv, r, lens_n(S, cur, lambda), 1, 0, step, cur, next, o->disable_fresnel);
    }

    if (tn == kNull) {
      ray_add_point(r, nv.p, x1[3] + step / RBG_SPEED_OF_LIGHT_CM);
      ray_add_node(r, next);
      r->status = RBG_EXIT;
    } else if (tc == kFocus || tc == kObs || tc == kMirror || tn == kObs) {
      r->status = RBG_STOP;
    } else if (tn == kFocus) {
      const rbg_volume_desc* v = &S->volumes[S->nodes[next].volume];
      double angle = 0.;
      if (v->qe_angle_table >= 0) {
        double n[3];
        get_facet_normal(S, &nv, r, cur, next, n);
        angle = acos(dot3(r->d, n));
      }
      double qe = v->qe_lambda_table >= 0 ? table1d(S, v->qe_lambda_table, lambda) : 1.;
      if (v->qe_angle_table >= 0) qe *= table1d(S, v->qe_angle_table, angle);
      if (qe == 1 || rng_u(&r->rng) < qe) r->status = RBG_FOCUS;
      else r->status = RBG_STOP;
    }

    if (r->status == RBG_RUN && r->npoints >= o->limit) r->status = RBG_SUSPEND;
  }
}

/* ======================================================================
 * driver
 * ==================================================================== */
typedef struct {
  Scene* S;
  const rbg_rays* in;
  rbg_result* out;
  const rbg_trace_opts* o;
  int64_t begin, end;
  int bad, cap;
} Job;

static void* run_job(void* arg) {
  Job* j = (Job*)arg;
  Scene* S = j->S;
  for (int64_t i = j->begin; i < j->end; ++i) {
    Ray r;
    memset(&r, 0, sizeof(r));
    r.x[0] = j->in->x[i]; r.x[1] = j->in->y[i]; r.x[2] = j->in->z[i];
    r.x[3] = j->in->t ? j->in->t[i] : 0.0;
    r.lambda = j->in->lambda[i];
    double dd[3] = {j->in->dx[i], j->in->dy[i], j->in->dz[i]};
    r.status = RBG_RUN;
    r.npoints = 0;
    r.last_node = -2;
    r.hist_cap = j->out->hist_cap > 0 && j->out->hist_xyzt && j->out->hist_node ? j->out->hist_cap : 0;
    r.hist_xyzt = r.hist_cap ? j->out->hist_xyzt + (size_t)i * r.hist_cap * 4 : NULL;
    r.hist_node = r.hist_cap ? j->out->hist_node + (size_t)i * r.hist_cap : NULL;
    uint64_t id = j->o->ray_id_offset + (uint64_t)i;
    r.rng.key[0] = (uint32_t)j->o->seed;
    r.rng.key[1] = (uint32_t)(j->o->seed >> 32);
    r.rng.id_lo = (uint32_t)id;
    r.rng.id_hi = (uint32_t)(id >> 32);
    r.rng.n = 0;
    double start[3] = {r.x[0], r.x[1], r.x[2]};
    ray_add_point(&r, start, r.x[3]);
    double mag = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
    int bad = !(mag > 0) || !isfinite(mag) || !isfinite(start[0]) || !isfinite(start[1]) || !isfinite(start[2]);
    if (bad) {
      j->bad = 1;
      r.d[0] = dd[0]; r.d[1] = dd[1]; r.d[2] = dd[2];
    } else {
      ray_set_direction(&r, dd);
      trace_ray(S, &r, j->o);
    }
    if (r.cap) j->cap = 1;
    rbg_result* o = j->out;
    if (o->status) o->status[i] = (uint8_t)r.status;
    if (o->npoints) o->npoints[i] = r.npoints;
    if (o->last_node) o->last_node[i] = r.last_node;
    if (o->x) o->x[i] = r.x[0];
    if (o->y) o->y[i] = r.x[1];
    if (o->z) o->z[i] = r.x[2];
    if (o->t) o->t[i] = r.x[3];
    if (o->dx) o->dx[i] = r.d[0];
    if (o->dy) o->dy[i] = r.d[1];
    if (o->dz) o->dz[i] = r.d[2];
    /* history slots the ray did not reach: node -3, point 0 */
    for (int k = r.npoints; k < r.hist_cap; ++k) {
      r.hist_node[k] = -3;
      for (int c = 0; c < 4; ++c) r.hist_xyzt[4 * k + c] = 0.0;
    }
  }
  return NULL;
}

int orc_trace(Scene* S, const rbg_rays* in, rbg_result* out, const rbg_trace_opts* o, int nthreads) {
  if (!S || !in || !out || !o || in->n < 0) return RBG_ERR_ARG;
  if (in->n > 0 && (!in->x || !in->y || !in->z || !in->dx || !in->dy || !in->dz || !in->lambda))
    return RBG_ERR_ARG;
  if (o->limit <= 0) return RBG_ERR_ARG;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  int64_t n = in->n;
  if (n < nthreads) nthreads = n > 0 ? (int)n : 1;
  Job jobs[256];
  pthread_t th[256];
  /* contiguous chunks as src/AOpticsManager.cxx:533-541 */
  int64_t chunk = n / nthreads;
  for (int i = 0; i < nthreads; ++i) {
    jobs[i].S = S; jobs[i].in = in; jobs[i].out = out; jobs[i].o = o;
    jobs[i].begin = chunk * i;
    jobs[i].end = i == nthreads - 1 ? n : chunk * (i + 1);
    jobs[i].bad = 0;
    jobs[i].cap = 0;
  }
  if (nthreads == 1) {
    run_job(&jobs[0]);
  } else {
    for (int i = 0; i < nthreads; ++i) pthread_create(&th[i], NULL, run_job, &jobs[i]);
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
  }
  int bad = 0, cap = 0;
  for (int i = 0; i < nthreads; ++i) {
    bad |= jobs[i].bad;
    cap |= jobs[i].cap;
  }
  if (bad) return RBG_ERR_NAN;
  if (cap) return RBG_ERR_CAP;
  return RBG_OK;
}

/* ======================================================================
 * AGeoUtil::ContainmentRadius (src/AGeoUtil.cxx:18-42,198-308)
 * ==================================================================== */
typedef struct {
  const double* c;
  int nx, ny;
  double xlo, xw, ylo, yw;
} Hist;
static double sum_in_radius(const Hist* h, double x, double y, double r) {
  double r2 = r * r, total = 0.;
  for (int ix = 0; ix < h->nx; ++ix) {
    double cx = h->xlo + (ix + 0.5) * h->xw;
    for (int iy = 0; iy < h->ny; ++iy) {
      double cy = h->ylo + (iy + 0.5) * h->yw;
      double c = h->c[ix * h->ny + iy];
      if (c <= 0) continue;
      double d2 = (cx - x) * (cx - x) + (cy - y) * (cy - y);
      if (d2 <= r2) total += c;
    }
  }
  return total;
}
void orc_containment_radius(const double* counts, int nx, double xlo, double xhi, int ny, double ylo,
                            double yhi, double fraction, double* pr, double* px, double* py) {
  Hist h = {counts, nx, ny, xlo, (xhi - xlo) / nx, ylo, (yhi - ylo) / ny};
  /* moments from bin centres */
  double sw = 0, sx = 0, sy = 0, sxx = 0, syy = 0;
  for (int ix = 0; ix < nx; ++ix) {
    double cx = xlo + (ix + 0.5) * h.xw;
    for (int iy = 0; iy < ny; ++iy) {
      double cy = ylo + (iy + 0.5) * h.yw;
      double c = counts[ix * ny + iy];
      sw += c; sx += c * cx; sy += c * cy; sxx += c * cx * cx; syy += c * cy * cy;
    }
  }
  double x = sw ? sx / sw : 0, y = sw ? sy / sw : 0;
  double vx = sw ? sxx / sw - x * x : 0, vy = sw ? syy / sw - y * y : 0;
  double sdx = vx > 0 ? sqrt(vx) : 0, sdy = vy > 0 ? sqrt(vy) : 0;
  double r = sqrt(sdx * sdx + sdy * sdy) * 1.5;
  double dr = 0.1 * r;
  double sum_goal = sw * fraction;
  int no_shift = 0, no_stable = 0;
  for (int i = 0; i < 100 && no_shift < 30; i++) {
    int stable_r = 0, stable_x = 1, stable_y = 1;
    double sum0 = sum_in_radius(&h, x, y, r);
    double next_r = r;
    if (sum0 < sum_goal) {
      double sum1 = sum_in_radius(&h, x, y, r + dr);
      if (sum1 == sum0) { dr *= 2.; continue; }
      next_r = r + dr * (sum_goal - sum0) / (sum1 - sum0);
    } else if (sum0 != sum_goal) {
      double sum1 = sum_in_radius(&h, x, y, r - dr);
      if (sum1 == sum0) { dr *= 2.; continue; }
      next_r = r - dr * (sum0 - sum_goal) / (sum0 - sum1);
    }
    if (next_r < 0.) next_r = 0.5 * r;
    if (next_r < 0.5 * r) next_r = 0.5 * r;
    if (next_r > 2. * r) next_r = 2. * r;
    stable_r = fabs(next_r - r) < 0.0001 * r;
    r = next_r;
    {
      double sum1 = sum_in_radius(&h, x, y, r);
      dr *= sum0 != sum_goal ? fabs((sum1 - sum_goal) / (sum0 - sum_goal)) : 0.5;
      if (dr > 0.5 * r) dr = 0.5 * r;
      if (dr < 0.0005 * r) dr = 0.0005 * r;
      no_shift++;
      for (double dx = 0.25 * r; dx > 0.1 * dr; dx *= 0.25) {
        double sx1 = sum_in_radius(&h, x + dx, y, r);
        double sx2 = sum_in_radius(&h, x - dx, y, r);
        while (sx1 > sum1) {
          no_shift = 0; x += dx; sx2 = sum1; sum1 = sx1; sx1 = sum_in_radius(&h, x + dx, y, r); stable_x = 0;
        }
        while (sx2 > sum1) {
          no_shift = 0; x -= dx; sx1 = sum1; sum1 = sx2; sx2 = sum_in_radius(&h, x - dx, y, r); stable_x = 0;
        }
      }
    }
    for (double dy = 0.1 * r; dy > 0.1 * dr; dy *= 0.25) {
      double sum1 = sum_in_radius(&h, x, y, r);
      double sy1 = sum_in_radius(&h, x, y + dy, r);
      double sy2 = sum_in_radius(&h, x, y - dy, r);
      while (sy1 > sum1) {
        no_shift = 0; y += dy; sy2 = sum1; sum1 = sy1; sy1 = sum_in_radius(&h, x, y + dy, r); stable_y = 0;
      }
      while (sy2 > sum1) {
        no_shift = 0; y -= dy; sy1 = sum1; sum1 = sy2; sy2 = sum_in_radius(&h, x, y - dy, r); stable_y = 0;
      }
    }
    if (stable_r && stable_x && stable_y) no_stable++;
    else no_stable = 0;
    if (no_stable >= 4) break;
  }
  *pr = r;
  *px = x;
  *py = y;
}

/* ======================================================================
 * ACorsikaIACTFile::GetRayArray (src/ACorsikaIACTFile.cxx:71-133) for
 * bunches in HOST arrays: ceil(photons) rays per bunch, back-projected to
 * height z over (z - tel_z) / |cz|; a zero wavelength is drawn with
 * 1/lambda uniform in [1/lambda_max, 1/lambda_min] from Philox counter
 * (0, 2, ray index) -- the law the reference meant at :122-125, where it
 * passes its bunch-count limit as the upper wavelength.  Writes at most
 * `capacity` rays and returns their total count.
 * ==================================================================== */
int64_t orc_bunches_to_rays(const rbg_bunches* b, double z, double tel_z, double refractive_index,
                            double lambda_min, double lambda_max, uint64_t seed, double* x, double* y,
                            double* zz, double* t, double* dx, double* dy, double* dz, double* lam,
                            int64_t capacity) {
  const double speed = 2.99792458e10 / refractive_index;
  int64_t r = 0;
  for (int64_t i = 0; i < b->n; ++i) {
    const double cz = b->cz[i];
    const double airmass = -1. / cz;
    const double tel_dist = (z - tel_z) * airmass;
    for (int64_t j = 0; j < b->photons[i]; ++j, ++r) {
      double l = b->lambda[i];
      if (r >= capacity) continue;
      if (l == 0) {
        uint32_t c[4] = {0u, 2u, (uint32_t)r, (uint32_t)((uint64_t)r >> 32)};
        uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)}, v[4];
        orc_philox(c, k, v);
        l = 1. / (1. / lambda_min - u53(v[0], v[1]) * (1. / lambda_min - 1. / lambda_max));
      }
      x[r] = (double)b->x[i] - tel_dist * b->cx[i];
      y[r] = (double)b->y[i] - tel_dist * b->cy[i];
      zz[r] = z;
      t[r] = (double)b->time[i] * 1e-9 - tel_dist / speed;
      dx[r] = b->cx[i];
      dy[r] = b->cy[i];
      dz[r] = cz;
      lam[r] = l * 1e-7;
    }
  }
  return r;
}
