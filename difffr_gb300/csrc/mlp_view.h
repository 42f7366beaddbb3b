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

// The inference kernel's small weights, a host copy of the BF16-rounded values passed in
// the kernel's parameter block (read from the constant bank: no shared-memory traffic), in
// the order the kernel reads them: W1 in unit pairs (float2 {W1[2p][k], W1[2p+1][k]} at
// 8 p + 2 k), b1, b2, w3, b3. W1, b1 and b2 are stored halved (exact): the kernel carries
// halved pre-activations into its GELUs.
constexpr int MLP_SMALL_W1 = 0, MLP_SMALL_B1 = 256, MLP_SMALL_B2 = 320, MLP_SMALL_W3 = 384, MLP_SMALL_B3 = 448,
              MLP_SMALL_N = 452;

// Device view of one model: the weights the kernels use (W1, W2, w3 rounded to BF16 and
// held as FP32; biases FP32), the BF16 image of W2 in the shared-memory tile layout, the
// feature/target normalisation and the small weights above.
struct MlpView {
  const float *wuse = nullptr;
  const uint16_t *w2img = nullptr;
  float norm[MLP_NNORM] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 1};
  int device = 0;
  // polls allowed to the first tensor-core wait of each inference CTA; -1: the regular limit
  // (a failure-path test hook set by dfsph_mlp_set_wait_limit)
  int first_wait_polls = -1;
  alignas(16) float small[MLP_SMALL_N] = {};
};

// Current view of a model (defined in mlp.cu). The small weights in it are those of the
// last mlp_sync_small.
MlpView mlp_view(const dfsph_mlp *m);
// Brings the host copy of the small weights up to date after a parameter change (one
// synchronous 18 KB read on the model's stream; nothing when they are current).
void mlp_sync_small(dfsph_mlp *m);

}  // namespace dfsph
