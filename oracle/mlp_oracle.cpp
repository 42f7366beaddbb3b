// mlp_oracle.cpp — CPU restatement of the learned warm-start MLP (test infrastructure
// only): forward pass, mean-squared-error loss and its gradient, with the same rounding
// points as the GPU kernels (weights W1, W2, w3 rounded to BF16; the operands of every
// tensor-core product rounded to BF16: h1, dz2, dz1, the normalised features, h2 and the
// output error; everything else FP32, sums over samples in FP64).
//
// There is no reference counterpart (the reference warm start is the formula of
// TimeStepDiffDFSPH.cpp:964-1059); this file checks the GPU training and inference
// kernels, not the reference.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int H = 64, IN = 4;
constexpr int OFF_W1 = 0, OFF_B1 = 256, OFF_W2 = 320, OFF_B2 = 4416, OFF_W3 = 4480, OFF_B3 = 4544, NP = 4545;

float bf16r(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return v;  // inf / nan unchanged
  u += 0x7FFFu + ((u >> 16) & 1u);                  // round to nearest even
  u &= 0xFFFF0000u;
  std::memcpy(&v, &u, 4);
  return v;
}

// GELU of the kernels (tanh form): g = h + h t, h = x / 2, t = tanh(x (c + c a x^2)); d = g'(x).
constexpr float GC = 0.7978845608028654f, GA = 0.044715f, GCA = 0.7978845608028654f * 0.044715f;
float gelu_d(float x, float &d) {
  const float x2 = x * x;
  const float t = std::tanh(x * std::fma(GCA, x2, GC));
  const float h = 0.5f * x;
  d = 0.5f * (1.0f + t) + h * (1.0f - t * t) * GC * (1.0f + 3.0f * GA * x2);
  return std::fma(h, t, h);
}

}  // namespace

extern "C" {

// params[NP], norm[10]; x[n][4], y[n] (y may be NULL: forward only); pred[n] out
// (denormalised); grad[NP] out (may be NULL); returns the mean squared error in
// normalised units (0 when y is NULL).
double orc_mlp_eval(const float *params, const float *norm, const float *x, const float *y, int64_t n, float *pred,
                    double *grad) {
  float W1[H * IN], W2[H * H], w3[H];
  for (int k = 0; k < H * IN; k++) W1[k] = bf16r(params[OFF_W1 + k]);
  for (int k = 0; k < H * H; k++) W2[k] = bf16r(params[OFF_W2 + k]);
  for (int k = 0; k < H; k++) w3[k] = bf16r(params[OFF_W3 + k]);
  const float *b1 = params + OFF_B1, *b2 = params + OFF_B2, b3 = params[OFF_B3];
  float xi[4];
  for (int k = 0; k < 4; k++) xi[k] = 1.0f / norm[4 + k];
  const float yi = 1.0f / norm[9];
  std::vector<double> g(NP, 0.0);
  double loss = 0.0;
  for (int64_t p = 0; p < n; p++) {
    float f[4];
    for (int k = 0; k < 4; k++) f[k] = (x[4 * p + k] - norm[k]) * xi[k];
    float z1d[H], h1b[H];
    for (int j = 0; j < H; j++) {
      const float z = b1[j] + W1[4 * j] * f[0] + W1[4 * j + 1] * f[1] + W1[4 * j + 2] * f[2] + W1[4 * j + 3] * f[3];
      h1b[j] = bf16r(gelu_d(z, z1d[j]));
    }
    float h2[H], g2d[H];
    float out = b3;
    for (int o = 0; o < H; o++) {
      float z = 0.f;
      for (int i = 0; i < H; i++) z += W2[o * H + i] * h1b[i];
      h2[o] = gelu_d(z + b2[o], g2d[o]);
      out += w3[o] * h2[o];
    }
    if (pred) pred[p] = out * norm[9] + norm[8];
    if (!y) continue;
    const float yn = (y[p] - norm[8]) * yi;
    const float e = out - yn;
    loss += (double)e * (double)e;
    if (!grad) continue;
    float dz2b[H];
    for (int o = 0; o < H; o++) dz2b[o] = bf16r(e * w3[o] * g2d[o]);
    const float eb = bf16r(e);
    float fb[4];
    for (int k = 0; k < 4; k++) fb[k] = bf16r(f[k]);
    for (int i = 0; i < H; i++) {
      float dh = 0.f;
      for (int o = 0; o < H; o++) dh += dz2b[o] * W2[o * H + i];
      const float dz1b = bf16r(dh * z1d[i]);
      for (int k = 0; k < 4; k++) g[OFF_W1 + 4 * i + k] += (double)dz1b * fb[k];
      g[OFF_B1 + i] += dz1b;
    }
    for (int o = 0; o < H; o++) {
      for (int i = 0; i < H; i++) g[OFF_W2 + o * H + i] += (double)dz2b[o] * h1b[i];
      g[OFF_B2 + o] += dz2b[o];
      g[OFF_W3 + o] += (double)bf16r(h2[o]) * eb;
    }
    g[OFF_B3] += eb;
  }
  if (grad && n > 0)
    for (int k = 0; k < NP; k++) grad[k] = g[k] * (2.0 / (double)n);
  return n > 0 ? loss / (double)n : 0.0;
}

}  // extern "C"
