/*
 * oracle.h -- CPU FP64 restatement of ROBAST's non-sequential tracer.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the correctness oracle for the GPU
 * tracer: only the tests, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it, always as the checker, never as the product path.
 *
 * It restates, in plain C99:
 *   AOpticsManager::TraceNonSequential / DoFresnel / DoReflection /
 *     GetFacetNormal                      src/AOpticsManager.cxx:52-520
 *   AGeoAsphericDisk                      src/AGeoAsphericDisk.cxx:96-153,246-347,363-684
 *   AGeoWinstonCone2D / ConePoly          src/AGeoWinstonCone2D.cxx:59-98,325-428
 *                                         src/AGeoWinstonConePoly.cxx:67-226,293-309
 *   AMultilayer::CoherentTMM              src/AMultilayer.cxx:26-104,120-209,240-481
 *   ASellmeierFormula / ARefractiveIndex  src/ASellmeierFormula.cxx:46-54,
 *                                         include/ARefractiveIndex.h:36-65
 *   AMirror / AFocalSurface lookups       src/AMirror.cxx:39-60, src/AFocalSurface.cxx:35-52
 *   AGeoUtil::ContainmentRadius           src/AGeoUtil.cxx:18-42,198-308
 * and, from their documented behaviour (ROOT is not part of the reference
 * tree and is not installed here), TGeo navigation and the TGeo primitive
 * shapes/CSG.  Parity with real ROOT is pinned only by the reference's own
 * unit tests (tutorials/unittest_robast.py), restated in tests/.
 */
#ifndef RBG_ORACLE_H
#define RBG_ORACLE_H

#include <stdint.h>

#include "robast_gb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Trace n rays on `nthreads` host threads (contiguous chunks, as
 * src/AOpticsManager.cxx:533-541).  Same result layout and status codes as
 * rbg_trace_host. */
int orc_trace(const rbg_flat_scene* scene, const rbg_rays* in, rbg_result* out,
              const rbg_trace_opts* opts, int nthreads);

/* AMultilayer::CoherentTMM for one polarisation (0 = s, 1 = p) and the mixed
 * average, for a multilayer of the scene. */
int orc_coherent_tmm(const rbg_flat_scene* scene, int multilayer, int pol,
                     double th0, double lambda, double* R, double* T);
int orc_coherent_tmm_mixed(const rbg_flat_scene* scene, int multilayer,
                           double th0, double lambda, double* R, double* T);
/* The same for a complex incidence angle th_re + i th_im, and
 * AMultilayer::IncoherentTMM (coherent flags of the layers honoured). */
int orc_coherent_tmm_c(const rbg_flat_scene* scene, int multilayer, int pol,
                       double th_re, double th_im, double lambda, double* R, double* T);
int orc_incoherent_tmm(const rbg_flat_scene* scene, int multilayer, int pol,
                       double th_re, double th_im, double lambda, double* R, double* T);
/* Refractive index / extinction of an index entry at lambda (cm). */
double orc_refractive_index(const rbg_flat_scene* scene, int index, double lambda);
double orc_extinction(const rbg_flat_scene* scene, int index, double lambda);
/* AMirror::GetReflectance of a volume. */
double orc_mirror_reflectance(const rbg_flat_scene* scene, int volume, double lambda,
                              double angle);
/* Table evaluation (TGraph::Eval / TH2 interpolation). */
double orc_table_eval(const rbg_flat_scene* scene, int table, double x, double y);

/* Philox4x32-10 block, for known-answer tests. */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* AGeoUtil::ContainmentRadius on a histogram counts[ix*ny+iy]. */
void orc_containment_radius(const double* counts, int nx, double xlo, double xhi,
                            int ny, double ylo, double yhi, double fraction,
                            double* r, double* x, double* y);

/* ACorsikaIACTFile::GetRayArray on host bunch arrays (see oracle.c);
 * returns the number of rays (at most `capacity` are written). */
int64_t orc_bunches_to_rays(const rbg_bunches* b, double z, double tel_z, double refractive_index,
                            double lambda_min, double lambda_max, uint64_t seed, double* x, double* y,
                            double* zz, double* t, double* dx, double* dy, double* dz, double* lam,
                            int64_t capacity);

/* Shape queries in a node's local frame (for unit tests of the shapes). */
double orc_shape_dist_out(const rbg_flat_scene* scene, int shape, const double* p,
                          const double* d);
double orc_shape_dist_in(const rbg_flat_scene* scene, int shape, const double* p,
                         const double* d);
int orc_shape_contains(const rbg_flat_scene* scene, int shape, const double* p);

#ifdef __cplusplus
}
#endif
#endif
