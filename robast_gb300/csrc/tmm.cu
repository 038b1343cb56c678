// tmm.cu -- thin-film stacks on the GPU outside the trace itself:
//  * the precalculated tables of AMultilayer::PreCalculateCoherentTMM /
//    PreCalculateIncoherentTMM (include/AMultilayer.h:243-282): one thread
//    per (lambda, theta) bin centre evaluates the mixed-polarisation R and T
//    in FP64 (the reference fills its TH2Ds in a host loop);
//  * rbg_multilayer_rt: CoherentTMM / IncoherentTMM / CoherentTMMMixed for
//    a batch of (angle, wavelength) pairs, the reference's vector overloads
//    (:157-237).
#include <cuda_runtime.h>

#include "device_state.cuh"
#include "scene_internal.h"
#include "tracer.cuh"

namespace rbg {
namespace {

// one polarisation (0 s, 1 p) or the mean of p and s (2), coherent (mode 0)
// or incoherent (mode 1)
RBG_D void stack_rt(const DevScene& S, int ml, int mode, int pol, cplxT<double> th, double lam, double& R,
                    double& T) {
  const rbg_multilayer_desc& M = S.multilayers[ml];
  if (mode == 0 && pol == 2) {
    // both polarisations in one pass, summed p then s as the loop below
    double r[2], t[2];
    tmm_coherent_n<double, 2>(S, M.layer_offset, 0, M.n_layers, 1, 0, th, lam, r, t);
    R = (r[1] + r[0]) / 2.;
    T = (t[1] + t[0]) / 2.;
    return;
  }
  R = 0;
  T = 0;
  const int first = pol == 2 ? 1 : pol, last = pol == 2 ? 0 : pol;
  for (int q = first;; q = 0) {
    double r, t;
    if (mode == 1) tmm_incoherent(S, ml, q, th, lam, r, t);
    else tmm_coherent<double>(S, M.layer_offset, 0, M.n_layers, 1, q, th, lam, r, t);
    R += r;
    T += t;
    if (q == last) break;
  }
  if (pol == 2) {
    R /= 2.;
    T /= 2.;
  }
}

__global__ void tmm_fill_kernel(DevScene S, int ml, double* tab) {
  const rbg_multilayer_desc M = S.multilayers[ml];
  const int64_t cells = (int64_t)M.lam_nbins * M.th_nbins;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cells) return;
  const int i = (int)(k / M.th_nbins), j = (int)(k % M.th_nbins);
  const double lam = M.lam_min + (i + 0.5) * (M.lam_max - M.lam_min) / M.lam_nbins;
  const double th = M.th_min + (j + 0.5) * (M.th_max - M.th_min) / M.th_nbins;
  double R, T;
  stack_rt(S, ml, M.precalc == 2 ? 1 : 0, 2, cx<double>(th), lam, R, T);
  tab[k] = R;
  tab[cells + k] = T;
}

__global__ void tmm_eval_kernel(DevScene S, int ml, int mode, int pol, int64_t n, const double* th_re,
                                const double* th_im, const double* lam, double* R, double* T) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const cplxT<double> th{th_re[k], th_im ? th_im[k] : 0.0};
  double r, t;
  if (mode == 2 && pol == 2) {
    coherent_tmm_mixed<false>(S, ml, th.re, lam[k], r, t);
  } else {
    stack_rt(S, ml, mode == 1 ? 1 : 0, pol, th, lam[k], r, t);
  }
  if (R) R[k] = r;
  if (T) T[k] = t;
}

}  // namespace

// Fill the precalculated tables of scene s into `tables` (device, laid out
// as s->tmm_tables) on stream st; S must already point at the other tables.
int fill_tmm_tables(const rbg_scene* s, const DevScene& S, double* tables, cudaStream_t st) {
  for (size_t ml = 0; ml < s->multilayers.size(); ++ml) {
    if (s->tmm_off[ml] < 0) continue;
    const int64_t cells = (int64_t)s->multilayers[ml].lam_nbins * s->multilayers[ml].th_nbins;
    const int threads = 128;
    tmm_fill_kernel<<<(unsigned)((cells + threads - 1) / threads), threads, 0, st>>>(S, (int)ml,
                                                                                     tables + s->tmm_off[ml]);
    if (cudaGetLastError() != cudaSuccess) return RBG_ERR_CUDA;
  }
  return RBG_OK;
}

}  // namespace rbg

using namespace rbg;

extern "C" int rbg_multilayer_rt(rbg_scene* s, int32_t ml, int32_t mode, int32_t pol, int64_t n, const double* th_re,
                                 const double* th_im, const double* lambda, double* R, double* T, void* stream) {
  if (!s || n < 0 || ml < 0 || ml >= (int32_t)s->multilayers.size() || mode < 0 || mode > 2 || pol < 0 || pol > 2)
    return RBG_ERR_ARG;
  if (n == 0) return RBG_OK;
  if (!th_re || !lambda) return RBG_ERR_ARG;
  int rc = ensure_device(s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int threads = 128;
  const int64_t blocks = (n + threads - 1) / threads;
  if (blocks > 0x7fffffff) return RBG_ERR_TOO_LARGE;
  tmm_eval_kernel<<<(unsigned)blocks, threads, 0, st>>>(s->dev->view, ml, mode, pol, n, th_re, th_im, lambda, R, T);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) return RBG_ERR_CUDA;
  return RBG_OK;
}
