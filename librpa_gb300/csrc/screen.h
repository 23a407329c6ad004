// Block screening of chi0(I, J, R, tau) contributions and the learned predictor.
//
// LibRI's own filter (LRI.hpp:20-25, applied in LRI-set.hpp:56-61) keeps a tensor block when
// its max-norm exceeds the threshold.  The same rule, applied to the chi0 output blocks with
// LibrpaGB300Options.screen_threshold, is the plain screening: every block is contracted and
// blocks with max |chi0| <= threshold are dropped.  The learned screening predicts
// log10 max |chi0| per block with a small MLP (9 inputs, two hidden layers of 64, GELU, FP16
// weights, FP32 accumulation) and contracts only the blocks predicted above the threshold,
// plus a random audit share of the others; an audited block above the threshold makes the
// whole (tau, spin) fall back to the plain rule.
#pragma once

#include <cuda_fp16.h>

#include <vector>

#include "common.h"
#include "kernels.h"
#include "screen_model.h"

namespace gb {

// ---- block kernels (screen.cu)
// Zero G(sign, cell, I, J) blocks whose max |G| <= thr (LibRI set_Gs_pos / set_Gs_neg filter).
void launch_g_block_filter(double *G, const Geom &g, double thr, cudaStream_t st);
// max |chi0| of every (pair, cell) block -> norm[pair * n_c + cell]
void launch_block_maxnorm(const double *chi0R, const Geom &g, const Pairs &pr, double *norm, cudaStream_t st);
// zero the blocks whose norm <= thr
void launch_block_drop(double *chi0R, const Geom &g, const Pairs &pr, const double *norm, double thr,
                       cudaStream_t st);
// features of every (pair, cell) block at one tau: distance (Bohr), log10 tau,
// log10(cmax_I cmax_J), log10 max |G+_IJ(cell)|, log10 max |G-_IJ(cell)|, log10 of the ABF and
// of the NAO block dimensions (n_abf(I) n_abf(J), n_ao(I) n_ao(J)), and the species (kind) of I
// and of J
void launch_block_features(const double *G, const Geom &g, const Pairs &pr, const float *dist,
                           const float *cmax, const float *kind, double tau, float *feat, cudaStream_t st);

// ---- MLP (screen.cu): predictions, training, and the gradient self-check
// y[n] = model(x[n]) in the target's own units (log10 max |chi0|).
void mlp_predict(const ScreenModel &m, const float *d_x, int n, float *d_y, cudaStream_t st);
// Train on (x, y) host samples with Adam on the GPU; fills m (params, norm, margin).
void mlp_train(ScreenModel &m, const std::vector<float> &x, const std::vector<float> &y, int iterations,
               double lr, unsigned long long seed, cudaStream_t st);
// Loss (mean squared error on normalised targets) and its gradient for given FP32 params
// (rounded to FP16 as the forward pass uses them) and normalisation: the kernels the
// training runs, exposed for the gradient check against the CPU oracle.
double mlp_loss_grad(const float *params, const float *norm, const float *x, const float *y, int n, float *grad,
                     cudaStream_t st);

} // namespace gb
