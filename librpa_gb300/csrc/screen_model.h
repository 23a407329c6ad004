// Host-side state of the learned chi0 block screening (held by a handler).
#pragma once

#include <cstddef>
#include <vector>

namespace gb {

// Block features: distance (Bohr), log10 tau, log10(max|C_I| max|C_J|), log10 max|G+_IJ(R)|,
// log10 max|G-_IJ(R)|, log10(n_abf(I) n_abf(J)), log10(n_ao(I) n_ao(J)), species of I, species of J
constexpr int MLP_IN = 9;
constexpr int MLP_H = 64;
// W1 [H][IN], b1 [H], W2 [H][H], b2 [H], W3 [H], b3
constexpr int MLP_NPARAM = MLP_H * MLP_IN + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1;
// feature means [IN], feature scales [IN], target mean, target scale, decision margin (log10)
constexpr int MLP_NNORM = 2 * MLP_IN + 3;

// Model: FP32 master weights (the FP16 copy the kernels use is made on upload) and the
// feature / target normalisation.
struct ScreenModel
{
    bool trained = false;
    std::vector<float> params;  // MLP_NPARAM
    std::vector<float> norm;    // MLP_NNORM
    double train_rmse = 0.0;    // log10 units, over the training samples
};

// Samples logged by plain-screening calls: features [n][MLP_IN] and the target
// log10 max |chi0| of the block.
struct ScreenLog
{
    std::vector<float> x, y;
    size_t size() const { return y.size(); }
};

} // namespace gb
