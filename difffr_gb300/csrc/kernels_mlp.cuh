// kernels_mlp.cuh — the learned warm start for the DFSPH pressure stiffness: a per-particle
// MLP 4 -> 64 -> 64 -> 1 with GELU activations, BF16 weights and FP32 accumulation.
//
// The 64 x 64 hidden layer (the only dense contraction of the project) runs on the
// tensor cores: tcgen05.mma with BF16 operands staged in shared memory and FP32
// accumulators in TMEM, for the forward product and, in training, for the input
// gradient and for all weight gradients (bias gradients come out of the same products
// through a constant-1 column). The 4-wide input layer and the 64-wide output layer are
// per-thread FP32 arithmetic on BF16-rounded weights.
//
// Features (per particle, at the pressure warm start): the density error rho_adv - 1,
// the neighbour count, the previous step's stiffness kappa (in Jacobi-pass units) and
// |v|. The target is the stiffness the plain solve accumulated in that step. Features
// and target are normalised with per-column mean and standard deviation.
//
// No reference counterpart: the reference warm start is
// TimeStepDiffDFSPH::warmstartPressureSolve (TimeStepDiffDFSPH.cpp:964-1059),
// kappa <- 0.5 max(kappa, -0.00025) / h^2, which is what the learned start replaces.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "f32x2.cuh"
#include "mlp_view.h"
#include "tc.cuh"

namespace dfsph {

constexpr int MLP_TILE = 128;                            // particles per MMA tile (M = 128)
constexpr int MLP_THREADS = 128;
constexpr uint32_t MLP_WAIT_LIMIT = 1u << 21;            // mbarrier polls (x 64 ns sleep) before giving up

// hardware tanh (one MUFU instruction; relative error about 2^-11, below the BF16
// rounding every activation goes through before the tensor-core products)
static __device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// GELU, tanh form: g(x) = h + h t with h = x / 2, t = tanh(x (c + c a x^2)), c = sqrt(2/pi),
// a = 0.044715; d = g'(x).
constexpr float GELU_C = 0.7978845608028654f, GELU_A = 0.044715f, GELU_CA = 0.7978845608028654f * 0.044715f;
static __device__ __forceinline__ float gelu_d(float x, float &d) {
  const float x2 = x * x;
  const float t = tanh_approx(x * fmaf(GELU_CA, x2, GELU_C));
  const float h = 0.5f * x;
  d = 0.5f * (1.0f + t) + h * (1.0f - t * t) * GELU_C * (1.0f + 3.0f * GELU_A * x2);
  return fmaf(h, t, h);
}
static __device__ __forceinline__ float gelu_f(float x) {
  const float t = tanh_approx(x * fmaf(GELU_CA, x * x, GELU_C));
  const float h = 0.5f * x;
  return fmaf(h, t, h);
}

// gelu_f on a pair, from h = x / 2 (the inference kernel carries the halved pre-activations:
// its W1, b1 and b2 are stored halved, which is exact). Every intermediate is a power-of-two
// multiple of gelu_f's, so in exact arithmetic the result is gelu_f(x), with one multiply
// fewer: h^2 = x^2 / 4, 8 c a h^2 + 2 c = 2 (c a x^2 + c), u = h (2 (c + c a x^2)),
// g = h + h t. (The packed operations may round differently from the scalar form in the
// last bit; the tolerance against the oracle covers it.)
static __device__ __forceinline__ float2 gelu2_half(float2 h) {
  const float2 u = mul2(h, fma2(make_float2(8.f * GELU_CA, 8.f * GELU_CA), mul2(h, h),
                                make_float2(2.f * GELU_C, 2.f * GELU_C)));
  const float2 t = make_float2(tanh_approx(u.x), tanh_approx(u.y));
  return fma2(h, t, h);
}

// two round-to-nearest BF16 conversions in one packed instruction (lo in the low half)
static __device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  uint32_t u;
  memcpy(&u, &v, sizeof(u));
  return u;
}
// store 8 consecutive columns (c0 multiple of 8) of row `row` of a core-matrix tile
static __device__ __forceinline__ void st_row8(uint8_t *tile, int row, int c0, int cols, const float *v) {
  uint4 q;
  q.x = pack_bf16x2(v[0], v[1]);
  q.y = pack_bf16x2(v[2], v[3]);
  q.z = pack_bf16x2(v[4], v[5]);
  q.w = pack_bf16x2(v[6], v[7]);
  *reinterpret_cast<uint4 *>(tile + tc::cm_offset(row, c0, cols)) = q;
}

static __device__ __forceinline__ uint8_t *align1024(uint8_t *p) {
  return reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// Small weights of the training kernel in shared memory: W1 (256), b1 (64), b2 (64), w3 (64),
// b3 (1). (The inference kernel reads them from its parameter block, MlpView::small.)
constexpr int MLP_SW_W1 = 0, MLP_SW_B1 = 256, MLP_SW_B2 = 320, MLP_SW_W3 = 384, MLP_SW_B3 = 448, MLP_SW_N = 452;

static __device__ __forceinline__ void mlp_stage_small(const float *wuse, float *sw) {
  for (int k = threadIdx.x; k < MLP_SW_N; k += blockDim.x) {
    float v = 0.f;
    if (k < MLP_SW_B2) v = wuse[k];                                  // W1, b1
    else if (k < MLP_SW_W3) v = wuse[MLP_OFF_B2 + (k - MLP_SW_B2)];  // b2
    else if (k < MLP_SW_B3) v = wuse[MLP_OFF_W3 + (k - MLP_SW_W3)];  // w3
    else if (k == MLP_SW_B3) v = wuse[MLP_OFF_B3];
    sw[k] = v;
  }
}

// hidden layer 1 of the inference kernel, two units per packed operation; the weights come
// from the kernel's parameter block (every index is a compile-time constant after
// unrolling, so each read is a constant-bank operand), W1 and b1 halved, so z holds the
// halved pre-activations gelu2_half takes
static __device__ __forceinline__ void mlp_layer1_paired(const MlpView &mv, const float f[4], uint8_t *tile, int row,
                                                         int cols) {
  const float2 f0 = make_float2(f[0], f[0]), f1 = make_float2(f[1], f[1]), f2 = make_float2(f[2], f[2]),
               f3 = make_float2(f[3], f[3]);
#pragma unroll
  for (int c = 0; c < MLP_H; c += 8) {
    float h[8];
#pragma unroll
    for (int u = 0; u < 8; u += 2) {
      const int p = (c + u) >> 1, w = MLP_SMALL_W1 + 8 * p;
      float2 z = make_float2(mv.small[MLP_SMALL_B1 + c + u], mv.small[MLP_SMALL_B1 + c + u + 1]);
      z = fma2(make_float2(mv.small[w + 0], mv.small[w + 1]), f0, z);
      z = fma2(make_float2(mv.small[w + 2], mv.small[w + 3]), f1, z);
      z = fma2(make_float2(mv.small[w + 4], mv.small[w + 5]), f2, z);
      z = fma2(make_float2(mv.small[w + 6], mv.small[w + 7]), f3, z);
      const float2 g = gelu2_half(z);
      h[u] = g.x;
      h[u + 1] = g.y;
    }
    st_row8(tile, row, c, cols, h);
  }
}

// ------------------------------------------------------------------ inference
// Persistent over tiles of 128 particles: one thread per particle row. Shared memory:
// W2 image 8 KB, the H1 tile 16 KB, one mbarrier; TMEM: 64 columns. The small weights are
// read from the parameter block.
// IO supplies `bool load(int i, float f[4])` (false: no prediction wanted for i) and
// `void store(int i, float y)`.
// 8192 (W2) + 16384 (H1 tile) + 16 (barrier, TMEM address) + 1008 (alignment) bytes, rounded
// up to 27 KB: at most 8 CTAs fit on an SM, and 8 x 64 TMEM columns is exactly the SM's 512,
// so no CTA waits in tcgen05.alloc.
constexpr int MLP_INFER_SMEM = 27 * 1024;
static_assert(8192 + 16384 + 16 + 1008 <= MLP_INFER_SMEM, "inference tile layout fits");
static_assert((228 * 1024) / (MLP_INFER_SMEM + 1024) <= 8, "at most 8 CTAs (512 TMEM columns) per SM");

template <class IO>
static __global__ void __launch_bounds__(MLP_THREADS) k_mlp_infer(MlpView mv, IO io, int n, int *err, int errbit) {
  extern __shared__ uint8_t mlp_smem_raw[];
  uint8_t *base = align1024(mlp_smem_raw);
  uint8_t *sW2 = base;                   // 8192 B
  uint8_t *sH1 = base + 8192;            // 16384 B: 128 rows x 64 cols
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + 8192 + 16384);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;

  {
    static_assert(MLP_THREADS == 128, "staging assumes 128 threads");
    uint4 t[4];
#pragma unroll
    for (int j = 0; j < 4; j++) t[j] = reinterpret_cast<const uint4 *>(mv.w2img)[tid + 128 * j];
#pragma unroll
    for (int j = 0; j < 4; j++) reinterpret_cast<uint4 *>(sW2)[tid + 128 * j] = t[j];
  }
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, 64);
    tc::tmem_relinquish();
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_bf16(128, 64, 0, 0);
  const uint32_t aBase = tc::smem_u32(sH1), bBase = tc::smem_u32(sW2);
  float xm[4], xi[4];
#pragma unroll
  for (int k = 0; k < 4; k++) { xm[k] = mv.norm[k]; xi[k] = 1.0f / mv.norm[4 + k]; }
  const float ym = mv.norm[8], ys = mv.norm[9];
  const int ntiles = (n + MLP_TILE - 1) / MLP_TILE;
  uint32_t phase = 0;
  bool pending = false;
  // the features of the CTA's next tile are loaded while the current tile's product runs
  float fn[4] = {0.f, 0.f, 0.f, 0.f};
  bool wantn = false;
  if (blockIdx.x < ntiles && (int)blockIdx.x * MLP_TILE + tid < n) wantn = io.load(blockIdx.x * MLP_TILE + tid, fn);
  bool first_wait = true;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int i = tile * MLP_TILE + tid;
    float f[4];
    const bool want = wantn;
    if (!__syncthreads_or(want)) {
      // no particle of this tile wants a prediction (in the solver's warm start: none with
      // rho_adv > 1): skip its arithmetic, load the next tile's features
      const int64_t inext = (int64_t)(tile + (int)gridDim.x) * MLP_TILE + tid;
      wantn = false;
#pragma unroll
      for (int k = 0; k < 4; k++) fn[k] = 0.f;
      if (inext < n) wantn = io.load((int)inext, fn);
      continue;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) f[k] = (fn[k] - xm[k]) * xi[k];
    mlp_layer1_paired(mv, f, sH1, tid, 64);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < 4; s++)
        tc::mma_bf16(tmem, tc::sdesc(aBase + 256u * s, 128, 1024), tc::sdesc(bBase + 256u * s, 128, 1024), idesc,
                     s > 0 ? 1u : 0u);
      tc::mma_commit(bar);
    }
    pending = true;
    {
      const int64_t inext = (int64_t)(tile + (int)gridDim.x) * MLP_TILE + tid;
      wantn = false;
#pragma unroll
      for (int k = 0; k < 4; k++) fn[k] = 0.f;
      if (inext < n) wantn = io.load((int)inext, fn);
    }
    // the CTA's first wait may be given fewer polls (a test of the failure path below); the
    // wait for the product still in flight after a failure always has the regular limit
    const uint32_t lim = (first_wait && mv.first_wait_polls >= 0) ? (uint32_t)mv.first_wait_polls : MLP_WAIT_LIMIT;
    first_wait = false;
    // one thread polls the barrier (every poll is a shared-memory access), the block follows
    const bool ok = __syncthreads_and(tid == 0 ? tc::mbar_wait(bar, phase, lim) : true) != 0;
    if (!ok) break;
    pending = false;
    phase ^= 1u;
    tc::fence_after_sync();
    // output layer: the even and odd hidden units summed in two packed partial sums
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 64; c += 16) {
      float z[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, z);
#pragma unroll
      for (int u = 0; u < 16; u += 2) {
        const int j = c + u;
        // (z + b2) / 2 in one rounding: fma(1/2, z, b2 / 2) with b2 stored halved
        const float2 b = make_float2(mv.small[MLP_SMALL_B2 + j], mv.small[MLP_SMALL_B2 + j + 1]);
        const float2 w = make_float2(mv.small[MLP_SMALL_W3 + j], mv.small[MLP_SMALL_W3 + j + 1]);
        acc = fma2(w, gelu2_half(fma2(make_float2(0.5f, 0.5f), make_float2(z[u], z[u + 1]), b)), acc);
      }
    }
    const float out = mv.small[MLP_SMALL_B3] + (acc.x + acc.y);
    if (want) io.store(i, out * ys + ym);
    tc::fence_before_sync();
  }
  if (pending) {
    // an MMA may still be in flight: record the failure, give it a bounded wait, then free TMEM
    if (tid == 0) {
      atomicOr(err, errbit);
      tc::mbar_wait(bar, phase, MLP_WAIT_LIMIT);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// Plain device arrays: x[n][4] -> y[n].
struct MlpArrayIO {
  const float *x;
  float *y;
  __device__ bool load(int i, float f[4]) const {
    const float4 v = reinterpret_cast<const float4 *>(x)[i];
    f[0] = v.x; f[1] = v.y; f[2] = v.z; f[3] = v.w;
    return true;
  }
  __device__ void store(int i, float v) const { y[i] = v; }
};

// ------------------------------------------------------------------ training
// One CTA of 1024 threads per SM, persistent over the batch's tiles of 128 samples. Warp w
// reaches TMEM lanes 32 (w % 4) .. + 31, so the sample row is r = 32 (w % 4) + lane and the
// CTA's 32 warps form 8 column groups g = w / 4: the 8 threads of a row each take 8 of the
// 64 hidden units, [8 g, 8 g + 8). Per tile:
//   forward:   z1 = W1 f + b1, h1 = gelu(z1)           (per thread, its 8 units, FP32)
//              Z2 = H1 W2^T                             (MMA1, M=128 N=64 K=64)
//              h2 = gelu(z2 + b2), y = w3 . h2 + b3     (per thread its 8 units; the 8
//                                                        partial dot products summed per row
//                                                        through shared memory, fixed order)
//   backward:  e = y - target, dz2 = e w3 gelu'(z2)
//              DH1 = DZ2 W2                             (MMA2, M=128 N=64 K=64)
//              GW2 += DZ2^T [H1 | 1]                    (MMA3, M=128 N=80 K=128: dW2 and db2)
//              GW3 += [H2 | 1]^T e                      (MMA5, M=128 N=16 K=128: dw3 and db3)
//              dz1 = dh1 gelu'(z1)
//              GW1 += DZ1^T [F | 1]                     (MMA4, M=128 N=16 K=128: dW1 and db1)
// The weight-gradient products read the per-sample tiles as MN-major operands, so every
// thread writes only its own row segment. Rows 64..127 of the M dimension are zero padding
// (M = 128 keeps row r of D in TMEM lane r). At the end the CTA writes its gradient
// partial sums (unscaled) and its loss partial; k_mlp_adam reduces them in fixed order.
constexpr int MLP_TRAIN_THREADS = 1024;
constexpr int MLP_TRAIN_GROUPS = MLP_TRAIN_THREADS / MLP_TILE;  // 8 column groups of 8 units
static_assert(MLP_TRAIN_GROUPS * 8 == MLP_H, "8 units per column group");
namespace mlptrain {
constexpr int SW2 = 0;                      // W2 image, 64 x 64
constexpr int SH1 = SW2 + 8192;             // 128 x 80  (col 64 = 1)
constexpr int SDZ2 = SH1 + 128 * 80 * 2;    // 128 x 128 (cols 64.. = 0)
constexpr int SH2 = SDZ2 + 128 * 128 * 2;   // 128 x 128 (col 64 = 1)
constexpr int SDZ1 = SH2 + 128 * 128 * 2;   // 128 x 128 (cols 64.. = 0)
constexpr int SFX = SDZ1 + 128 * 128 * 2;   // 128 x 16  (cols 0..3 features, col 4 = 1)
constexpr int SDO = SFX + 128 * 16 * 2;     // 128 x 16  (col 0 = error)
constexpr int SSW = SDO + 128 * 16 * 2;     // small weights
constexpr int SRED = SSW + MLP_SW_N * 4;    // output-layer partial sums [group][row], FP32
constexpr int SBAR = SRED + MLP_TRAIN_GROUPS * MLP_TILE * 4;  // mbarrier, TMEM address
constexpr int SEND = SBAR + 16;
// The dynamic allocation is padded far beyond SEND so that every operand read of every
// MMA stays inside it even if the descriptor's two byte offsets were read the other way
// round (largest such read: a 128-column tile read with 2048-B M/N stride from SDZ1).
constexpr int SMEM = 225 * 1024;
static_assert(SDZ1 + 15 * 2048 + 7 * 4096 + 128 * 2 + 128 < SMEM - 1024, "operand reads stay in the allocation");
static_assert(SEND < SMEM - 1024, "layout fits");
static_assert(SRED % 16 == 0 && SBAR % 8 == 0, "aligned regions");
// TMEM columns
constexpr uint32_t TZ2 = 0, TDH1 = 64, TGW2 = 128, TGW1 = 208, TGW3 = 224, TCOLS = 256;
}  // namespace mlptrain

// hidden layer 1 for one sample row, units [c0, c0 + 8): h1 to the tile row as BF16,
// gelu'(z1) into g1d
static __device__ __forceinline__ void mlp_layer1_cols8(const float *sw, const float f[4], uint8_t *tile, int row,
                                                        int cols, int c0, float g1d[8]) {
  float h[8];
#pragma unroll
  for (int u = 0; u < 8; u++) {
    const int j = c0 + u;
    const float *w = sw + MLP_SW_W1 + 4 * j;
    const float z = sw[MLP_SW_B1 + j] + w[0] * f[0] + w[1] * f[1] + w[2] * f[2] + w[3] * f[3];
    float d;
    h[u] = gelu_d(z, d);
    g1d[u] = d;
  }
  st_row8(tile, row, c0, cols, h);
}

static __global__ void __launch_bounds__(MLP_TRAIN_THREADS, 1)
    k_mlp_train(MlpView mv, const float *__restrict__ x, const float *__restrict__ y, const int *__restrict__ idx, int n,
                int nsrc, float *__restrict__ gpart, double *__restrict__ lpart, int *err) {
  using namespace mlptrain;
  extern __shared__ uint8_t mlp_smem_raw[];
  uint8_t *base = align1024(mlp_smem_raw);
  float *sw = reinterpret_cast<float *>(base + SSW);
  float *red = reinterpret_cast<float *>(base + SRED);
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + SBAR);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(base + SBAR + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = 32 * (warp & 3) + lane;  // the sample row (TMEM lane) of this thread
  const int grp = warp >> 2, c0 = 8 * grp;  // its column group and first hidden unit

  // constant parts of the tiles: zeros, and the constant-1 columns
  for (int k = tid; k < (SSW - SH1) / 16; k += MLP_TRAIN_THREADS)
    reinterpret_cast<uint4 *>(base + SH1)[k] = make_uint4(0, 0, 0, 0);
  for (int k = tid; k < 8192 / 16; k += MLP_TRAIN_THREADS)
    reinterpret_cast<uint4 *>(base + SW2)[k] = reinterpret_cast<const uint4 *>(mv.w2img)[k];
  mlp_stage_small(mv.wuse, sw);
  __syncthreads();
  if (grp == 0) {
    const uint16_t one = __bfloat16_as_ushort(__float2bfloat16_rn(1.0f));
    *reinterpret_cast<uint16_t *>(base + SH1 + tc::cm_offset(row, 64, 80)) = one;
    *reinterpret_cast<uint16_t *>(base + SH2 + tc::cm_offset(row, 64, 128)) = one;
    *reinterpret_cast<uint16_t *>(base + SFX + tc::cm_offset(row, 4, 16)) = one;
  }
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, TCOLS);
    tc::tmem_relinquish();
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t lane_off = (uint32_t)(32 * (warp & 3)) << 16;
  const uint32_t sb = tc::smem_u32(base);
  float xm[4], xi[4];
#pragma unroll
  for (int k = 0; k < 4; k++) { xm[k] = mv.norm[k]; xi[k] = 1.0f / mv.norm[4 + k]; }
  const float ym = mv.norm[8], yi = 1.0f / mv.norm[9];

  const int ntiles = (n + MLP_TILE - 1) / MLP_TILE;
  uint32_t phase = 0;
  bool pending = false, failed = false;
  int it = 0;
  double loss = 0.0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int r = tile * MLP_TILE + row;
    bool valid = r < n;
    float f[4] = {0.f, 0.f, 0.f, 0.f}, yn = 0.f;
    int s = r;
    if (valid && idx) {
      s = idx[r];
      if (s < 0 || s >= nsrc) {  // an index outside the sample arrays: flag it, skip the sample
        if (grp == 0) atomicOr(err, 2);
        valid = false;
      }
    }
    if (valid) {
      const float4 v = reinterpret_cast<const float4 *>(x)[s];
      f[0] = (v.x - xm[0]) * xi[0]; f[1] = (v.y - xm[1]) * xi[1];
      f[2] = (v.z - xm[2]) * xi[2]; f[3] = (v.w - xm[3]) * xi[3];
      yn = (y[s] - ym) * yi;
    }
    float g1d[8];
    mlp_layer1_cols8(sw, f, base + SH1, row, 80, c0, g1d);
    if (grp == 0) {
      const float fr[8] = {f[0], f[1], f[2], f[3], 1.0f, 0.f, 0.f, 0.f};
      st_row8(base + SFX, row, 0, 16, fr);
    }
    // ---- MMA1: Z2 = H1 W2^T
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t id1 = tc::idesc_bf16(128, 64, 0, 0);
#pragma unroll
      for (int s = 0; s < 4; s++)
        tc::mma_bf16(tmem + TZ2, tc::sdesc(sb + SH1 + 256u * s, 128, 1280), tc::sdesc(sb + SW2 + 256u * s, 128, 1024),
                     id1, s > 0 ? 1u : 0u);
      tc::mma_commit(bar);
    }
    pending = true;
    if (!__syncthreads_and(tid == 0 ? tc::mbar_wait(bar, phase, MLP_WAIT_LIMIT) : true)) { failed = true; break; }
    pending = false;
    phase ^= 1u;
    tc::fence_after_sync();
    // ---- output layer (this thread's 8 units), error, dz2
    float d2[8];
    {
      float t[8];
      tc::tmem_ld8(tmem + lane_off + TZ2 + (uint32_t)c0, t);
      float h[8], part = 0.f;
#pragma unroll
      for (int u = 0; u < 8; u++) {
        h[u] = gelu_d(t[u] + sw[MLP_SW_B2 + c0 + u], d2[u]);
        part += sw[MLP_SW_W3 + c0 + u] * h[u];
      }
      st_row8(base + SH2, row, c0, 128, h);
      red[grp * MLP_TILE + row] = part;
    }
    __syncthreads();
    float out = sw[MLP_SW_B3];
#pragma unroll
    for (int g = 0; g < MLP_TRAIN_GROUPS; g++) out += red[g * MLP_TILE + row];
    const float e = valid ? out - yn : 0.f;
    if (grp == 0) {
      loss += (double)e * (double)e;
      const float er[8] = {e, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      st_row8(base + SDO, row, 0, 16, er);
    }
    {
      float d[8];
#pragma unroll
      for (int u = 0; u < 8; u++) d[u] = e * sw[MLP_SW_W3 + c0 + u] * d2[u];
      st_row8(base + SDZ2, row, c0, 128, d);
    }
    // ---- MMA2 (DH1 = DZ2 W2), MMA3 (GW2 += DZ2^T [H1|1]), MMA5 (GW3 += [H2|1]^T e)
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t id2 = tc::idesc_bf16(128, 64, 0, 1);
#pragma unroll
      for (int s = 0; s < 4; s++)
        tc::mma_bf16(tmem + TDH1, tc::sdesc(sb + SDZ2 + 256u * s, 128, 2048),
                     tc::sdesc(sb + SW2 + 2048u * s, 1024, 128), id2, s > 0 ? 1u : 0u);
      const uint32_t id3 = tc::idesc_bf16(128, 80, 1, 1);
      const uint32_t id5 = tc::idesc_bf16(128, 16, 1, 1);
#pragma unroll
      for (int s = 0; s < 8; s++) {
        const uint32_t acc = (it > 0 || s > 0) ? 1u : 0u;
        tc::mma_bf16(tmem + TGW2, tc::sdesc(sb + SDZ2 + 4096u * s, 2048, 128),
                     tc::sdesc(sb + SH1 + 2560u * s, 1280, 128), id3, acc);
        tc::mma_bf16(tmem + TGW3, tc::sdesc(sb + SH2 + 4096u * s, 2048, 128),
                     tc::sdesc(sb + SDO + 512u * s, 256, 128), id5, acc);
      }
      tc::mma_commit(bar);
    }
    pending = true;
    if (!__syncthreads_and(tid == 0 ? tc::mbar_wait(bar, phase, MLP_WAIT_LIMIT) : true)) { failed = true; break; }
    pending = false;
    phase ^= 1u;
    tc::fence_after_sync();
    // ---- dz1 = dh1 gelu'(z1) (this thread's 8 units)
    {
      float t[8], a[8];
      tc::tmem_ld8(tmem + lane_off + TDH1 + (uint32_t)c0, t);
#pragma unroll
      for (int u = 0; u < 8; u++) a[u] = valid ? t[u] * g1d[u] : 0.f;
      st_row8(base + SDZ1, row, c0, 128, a);
    }
    // ---- MMA4: GW1 += DZ1^T [F|1]
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t id4 = tc::idesc_bf16(128, 16, 1, 1);
#pragma unroll
      for (int s = 0; s < 8; s++)
        tc::mma_bf16(tmem + TGW1, tc::sdesc(sb + SDZ1 + 4096u * s, 2048, 128),
                     tc::sdesc(sb + SFX + 512u * s, 256, 128), id4, (it > 0 || s > 0) ? 1u : 0u);
      tc::mma_commit(bar);
    }
    pending = true;
    if (!__syncthreads_and(tid == 0 ? tc::mbar_wait(bar, phase, MLP_WAIT_LIMIT) : true)) { failed = true; break; }
    pending = false;
    phase ^= 1u;
    tc::fence_after_sync();
  }
  if (failed) {
    if (tid == 0) atomicOr(err, 1);
    if (pending && tid == 0) tc::mbar_wait(bar, phase, MLP_WAIT_LIMIT);
  }
  // ---- gradient partials of this CTA: D rows 0..64 sit in TMEM lanes 0..64 (warps with
  // w % 4 = 0, 1 and lane 0 of w % 4 = 2); the column groups split the columns
  float *gp = gpart + (size_t)blockIdx.x * MLP_NPARAMS;
  const int q = warp & 3;
  if (it == 0 || failed) {
    for (int k = tid; k < MLP_NPARAMS; k += MLP_TRAIN_THREADS) gp[k] = 0.f;
  } else if (q < 2 && grp < 5) {
    // GW2: 80 columns (W2 row `row`, then b2 in column 64), 16 per group
    float t[16];
    tc::tmem_ld16(tmem + lane_off + TGW2 + (uint32_t)(16 * grp), t);
#pragma unroll
    for (int u = 0; u < 16; u++) {
      const int col = 16 * grp + u;
      if (col < 64) gp[MLP_OFF_W2 + row * 64 + col] = t[u];
      else if (col == 64) gp[MLP_OFF_B2 + row] = t[u];
    }
  } else if (q < 2 && grp == 5) {
    float t[8];
    tc::tmem_ld8(tmem + lane_off + TGW1, t);
#pragma unroll
    for (int k = 0; k < 4; k++) gp[MLP_OFF_W1 + row * 4 + k] = t[k];
    gp[MLP_OFF_B1 + row] = t[4];
  } else if (q < 3 && grp == 6) {
    float t[8];
    tc::tmem_ld8(tmem + lane_off + TGW3, t);
    if (row < 64) gp[MLP_OFF_W3 + row] = t[0];
    else if (row == 64) gp[MLP_OFF_B3] = t[0];
  }
  // ---- loss partial (fixed order; only column group 0 holds the rows' losses)
  __shared__ double lred[MLP_TRAIN_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if (lane == 0) lred[warp] = loss;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < MLP_TRAIN_THREADS / 32; w++) s += lred[w];
    lpart[blockIdx.x] = s;
  }
  if (warp == 0) tc::tmem_dealloc(tmem, TCOLS);
}

// Sums the CTA partials in fixed order, scales (2/n: gradient of the mean squared error),
// writes the gradient, and (lr > 0) takes one Adam step on the FP32 master weights; then
// refreshes the weights the kernels use (BF16-rounded W1, W2, w3) and the W2 image.
static __global__ void k_mlp_adam(int nparts, const float *__restrict__ gpart, float scale, float *__restrict__ grad,
                                  float *__restrict__ master, float *__restrict__ m1, float *__restrict__ m2,
                                  float *__restrict__ wuse, uint16_t *__restrict__ w2img, float lr, float b1c,
                                  float b2c) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= MLP_NPARAMS) return;
  float g = 0.f;
  for (int c = 0; c < nparts; c++) g += gpart[(size_t)c * MLP_NPARAMS + p];
  g *= scale;
  if (grad) grad[p] = g;
  float w = master[p];
  if (lr > 0.f) {
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float a = beta1 * m1[p] + (1.f - beta1) * g;
    const float b = beta2 * m2[p] + (1.f - beta2) * g * g;
    m1[p] = a;
    m2[p] = b;
    w -= lr * (a / b1c) / (sqrtf(b / b2c) + eps);
    master[p] = w;
  }
  const bool is_w = (p < MLP_OFF_B1) || (p >= MLP_OFF_W2 && p < MLP_OFF_B2) || (p >= MLP_OFF_W3 && p < MLP_OFF_B3);
  const __nv_bfloat16 wb = __float2bfloat16_rn(w);
  wuse[p] = is_w ? __bfloat162float(wb) : w;
  if (p >= MLP_OFF_W2 && p < MLP_OFF_B2) {
    const int o = (p - MLP_OFF_W2) / 64, i = (p - MLP_OFF_W2) % 64;
    w2img[tc::cm_offset(o, i, 64) / 2] = __bfloat16_as_ushort(wb);
  }
}

// Feature/target statistics: per block partial sums (double) of x, x^2 (4 columns) and y, y^2.
static __global__ void k_mlp_stats(const float *__restrict__ x, const float *__restrict__ y, int n,
                                   double *__restrict__ part) {
  double s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 v = reinterpret_cast<const float4 *>(x)[i];
    const double a[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; k++) { s[k] += a[k]; s[4 + k] += a[k] * a[k]; }
    s[8] += (double)y[i];
    s[9] += (double)y[i] * (double)y[i];
  }
  __shared__ double red[8][10];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 10; k++) {
    double t = s[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[w][k] = t;
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q][threadIdx.x];
    part[blockIdx.x * 10 + threadIdx.x] = t;
  }
}

}  // namespace dfsph
