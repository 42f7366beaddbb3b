// mlp_view.h — host-visible description of the learned warm-start model shared by the
// model object (mlp.cu), the engine (which runs inference inside the pressure warm
// start) and the kernels (kernels_mlp.cuh). No device code here.
#pragma once
#include <cstdint>

struct dfsph_mlp;

namespace dfsph {

// parameter vector layout (FP32 master copy, gradients, Adam moments)
constexpr int MLP_H = 64;
constexpr int MLP_IN = 4;
constexpr int MLP_OFF_W1 = 0;                            // W1[j][k], 64 x 4
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_IN;  // 256
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;           // 320: W2[o][i], 64 x 64
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;   // 4416
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;           // 4480
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H;           // 4544
constexpr int MLP_NPARAMS = MLP_OFF_B3 + 1;              // 4545
constexpr int MLP_NNORM = 10;                            // x mean[4], x std[4], y mean, y std

// Device view of one model: the weights the kernels use (W1, W2, w3 rounded to BF16 and
// held as FP32; biases FP32), the BF16 image of W2 in the shared-memory tile layout, and
// the feature/target normalisation.
struct MlpView {
  const float *wuse = nullptr;
  const uint16_t *w2img = nullptr;
  float norm[MLP_NNORM] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 1};
  int device = 0;
  // polls allowed to the first tensor-core wait of each inference CTA; -1: the regular limit
  // (a failure-path test hook set by dfsph_mlp_set_wait_limit)
  int first_wait_polls = -1;
};

// Current view of a model (defined in mlp.cu).
MlpView mlp_view(const dfsph_mlp *m);

}  // namespace dfsph
