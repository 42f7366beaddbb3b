// mlp.cu — the learned warm-start model object behind the dfsph_mlp_* entry points:
// parameter storage (FP32 master, Adam moments, BF16-rounded working copy, W2 image),
// normalisation, training steps, gradients and batch prediction. All data arguments are
// device pointers; every call is synchronous with respect to the host.
#include <cuda_runtime.h>

#include <cmath>
#include <climits>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/dfsph.h"
#include "engine_api.h"
#include "kernels_mlp.cuh"

struct dfsph_mlp {
  int device = 0;
  int nparts = 0;
  cudaStream_t stream = nullptr;
  float *master = nullptr, *m1 = nullptr, *m2 = nullptr, *wuse = nullptr, *grad = nullptr, *gpart = nullptr;
  uint16_t *w2img = nullptr;
  double *lpart = nullptr, *spart = nullptr;
  int *err = nullptr;
  float norm[dfsph::MLP_NNORM] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 1};
  int64_t adam_t = 0;
  int first_wait_polls = -1;
  float small[dfsph::MLP_SMALL_N] = {};  // host copy of the inference kernel's small weights
  bool small_stale = true;               // set whenever the device weights change
};

namespace dfsph {

MlpView mlp_view(const dfsph_mlp *m) {
  MlpView v;
  v.wuse = m->wuse;
  v.w2img = m->w2img;
  std::memcpy(v.norm, m->norm, sizeof(v.norm));
  v.device = m->device;
  v.first_wait_polls = m->first_wait_polls;
  std::memcpy(v.small, m->small, sizeof(v.small));
  return v;
}

namespace {

constexpr int STATS_BLOCKS = 512;

template <class F>
int guard_mlp(F &&f) {
  set_last_error("");
  try {
    return f();
  } catch (const DfsphException &e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return DFSPH_ERR_CUDA;
  }
}

void check_device_ptr(const void *p, const char *what) {
  if (!p) throw DfsphException(DFSPH_ERR_INVALID_ARG, std::string(what) + " is NULL");
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess || (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)) {
    cudaGetLastError();
    throw DfsphException(DFSPH_ERR_INVALID_ARG, std::string(what) + " must be a device pointer");
  }
}

struct DeviceScope {
  int prev = 0;
  explicit DeviceScope(int dev) {
    DF_CK(cudaGetDevice(&prev));
    DF_CK(cudaSetDevice(dev));
  }
  ~DeviceScope() { cudaSetDevice(prev); }
};

// splitmix64 -> uniform [0, 1)
uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

void refresh(dfsph_mlp *m, float lr, bool with_grad, float scale, int nparts) {
  float b1c = 1.f, b2c = 1.f;
  if (lr > 0.f) {
    m->adam_t++;
    b1c = 1.f - std::pow(0.9f, (float)m->adam_t);
    b2c = 1.f - std::pow(0.999f, (float)m->adam_t);
  }
  k_mlp_adam<<<(MLP_NPARAMS + 255) / 256, 256, 0, m->stream>>>(nparts, m->gpart, scale, with_grad ? m->grad : nullptr,
                                                              m->master, m->m1, m->m2, m->wuse, m->w2img, lr, b1c, b2c);
  DF_CK(cudaGetLastError());
  m->small_stale = true;
}

void upload_params(dfsph_mlp *m, const float *params) {
  DF_CK(cudaMemcpyAsync(m->master, params, MLP_NPARAMS * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  DF_CK(cudaMemsetAsync(m->m1, 0, MLP_NPARAMS * sizeof(float), m->stream));
  DF_CK(cudaMemsetAsync(m->m2, 0, MLP_NPARAMS * sizeof(float), m->stream));
  m->adam_t = 0;
  refresh(m, 0.f, false, 0.f, 0);
  DF_CK(cudaStreamSynchronize(m->stream));
}

// One pass of the training kernel over n samples: gradient partials and loss; returns
// the mean loss (normalised units).
double run_train_kernel(dfsph_mlp *m, const float *x, const float *y, const int *idx, int64_t n, int64_t nsrc) {
  if (n <= 0) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n must be positive");
  if (n > (int64_t)1 << 30) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n too large");
  if (nsrc > INT32_MAX) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n_samples too large");
  if (!idx && nsrc < n) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n exceeds n_samples");
  const int ntiles = (int)((n + MLP_TILE - 1) / MLP_TILE);
  const int grid = std::min(ntiles, m->nparts);
  DF_CK(cudaMemsetAsync(m->err, 0, sizeof(int), m->stream));
  k_mlp_train<<<grid, MLP_TRAIN_THREADS, mlptrain::SMEM, m->stream>>>(mlp_view(m), x, y, idx, (int)n, (int)nsrc, m->gpart,
                                                                 m->lpart, m->err);
  DF_CK(cudaGetLastError());
  std::vector<double> lp(grid);
  DF_CK(cudaMemcpyAsync(lp.data(), m->lpart, grid * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  int e = 0;
  DF_CK(cudaMemcpyAsync(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  DF_CK(cudaStreamSynchronize(m->stream));
  if (e & 2) throw DfsphException(DFSPH_ERR_INVALID_ARG, "a sample index is outside [0, n_samples)");
  if (e) throw DfsphException(DFSPH_ERR_DEVICE, "tensor-core MMA wait timed out in the training kernel");
  double s = 0.0;
  for (double v : lp) s += v;
  return s / (double)n;
}

}  // namespace

void mlp_sync_small(dfsph_mlp *m) {
  if (!m->small_stale) return;
  DeviceScope ds(m->device);
  std::vector<float> w(MLP_NPARAMS);
  DF_CK(cudaMemcpyAsync(w.data(), m->wuse, MLP_NPARAMS * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  DF_CK(cudaStreamSynchronize(m->stream));
  for (int p = 0; p < MLP_H / 2; p++)
    for (int k = 0; k < MLP_IN; k++)
      for (int odd = 0; odd < 2; odd++)
        m->small[MLP_SMALL_W1 + 8 * p + 2 * k + odd] = 0.5f * w[MLP_OFF_W1 + MLP_IN * (2 * p + odd) + k];
  for (int j = 0; j < MLP_H; j++) {
    m->small[MLP_SMALL_B1 + j] = 0.5f * w[MLP_OFF_B1 + j];
    m->small[MLP_SMALL_B2 + j] = 0.5f * w[MLP_OFF_B2 + j];
    m->small[MLP_SMALL_W3 + j] = w[MLP_OFF_W3 + j];
  }
  m->small[MLP_SMALL_B3] = w[MLP_OFF_B3];
  m->small_stale = false;
}

}  // namespace dfsph

using namespace dfsph;

extern "C" {

int dfsph_mlp_create(int32_t device, uint64_t seed, dfsph_mlp **out) {
  return guard_mlp([&] {
    if (!out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    DF_CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) throw DfsphException(DFSPH_ERR_INVALID_ARG, "device index");
    DeviceScope ds(device);
    cudaDeviceProp prop;
    DF_CK(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) throw DfsphException(DFSPH_ERR_UNSUPPORTED, "the warm-start model needs a Blackwell GPU (tcgen05)");
    std::unique_ptr<dfsph_mlp> m(new dfsph_mlp());
    m->device = device;
    m->nparts = prop.multiProcessorCount;
    DF_CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    const size_t P = MLP_NPARAMS * sizeof(float);
    DF_CK(cudaMalloc(&m->master, P));
    DF_CK(cudaMalloc(&m->m1, P));
    DF_CK(cudaMalloc(&m->m2, P));
    DF_CK(cudaMalloc(&m->wuse, P));
    DF_CK(cudaMalloc(&m->grad, P));
    DF_CK(cudaMalloc(&m->gpart, P * m->nparts));
    DF_CK(cudaMalloc(&m->w2img, MLP_H * MLP_H * sizeof(uint16_t)));
    DF_CK(cudaMalloc(&m->lpart, m->nparts * sizeof(double)));
    DF_CK(cudaMalloc(&m->spart, STATS_BLOCKS * 10 * sizeof(double)));
    DF_CK(cudaMalloc(&m->err, sizeof(int)));
    DF_CK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, mlptrain::SMEM));
    DF_CK(cudaFuncSetAttribute(k_mlp_infer<MlpArrayIO>, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_INFER_SMEM));
    // Xavier-uniform weights from the seed, zero biases
    std::vector<float> p(MLP_NPARAMS, 0.f);
    uint64_t s = seed;
    auto fill = [&](int off, int count, int fan_in, int fan_out) {
      const double a = std::sqrt(6.0 / (fan_in + fan_out));
      for (int k = 0; k < count; k++) p[off + k] = (float)((2.0 * uniform01(s) - 1.0) * a);
    };
    fill(MLP_OFF_W1, MLP_H * MLP_IN, MLP_IN, MLP_H);
    fill(MLP_OFF_W2, MLP_H * MLP_H, MLP_H, MLP_H);
    fill(MLP_OFF_W3, MLP_H, MLP_H, 1);
    upload_params(m.get(), p.data());
    *out = m.release();
    return DFSPH_OK;
  });
}

int dfsph_mlp_destroy(dfsph_mlp *m) {
  if (!m) return DFSPH_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(m->device);
  cudaStreamSynchronize(m->stream);
  for (void *p : {(void *)m->master, (void *)m->m1, (void *)m->m2, (void *)m->wuse, (void *)m->grad, (void *)m->gpart,
                  (void *)m->w2img, (void *)m->lpart, (void *)m->spart, (void *)m->err})
    if (p) cudaFree(p);
  cudaStreamDestroy(m->stream);
  cudaSetDevice(prev);
  delete m;
  return DFSPH_OK;
}

int dfsph_mlp_get_params(dfsph_mlp *m, float *params, float *norm) {
  return guard_mlp([&] {
    if (!m) throw DfsphException(DFSPH_ERR_INVALID_ARG, "model is NULL");
    DeviceScope ds(m->device);
    if (params) {
      DF_CK(cudaMemcpyAsync(params, m->master, MLP_NPARAMS * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
      DF_CK(cudaStreamSynchronize(m->stream));
    }
    if (norm) std::memcpy(norm, m->norm, sizeof(m->norm));
    return DFSPH_OK;
  });
}

int dfsph_mlp_set_params(dfsph_mlp *m, const float *params, const float *norm) {
  return guard_mlp([&] {
    if (!m) throw DfsphException(DFSPH_ERR_INVALID_ARG, "model is NULL");
    DeviceScope ds(m->device);
    if (norm) {
      for (int k = 0; k < 4; k++)
        if (!(norm[4 + k] > 0.f)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "feature scales must be positive");
      if (!(norm[9] > 0.f)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "target scale must be positive");
      std::memcpy(m->norm, norm, sizeof(m->norm));
    }
    if (params) upload_params(m, params);
    return DFSPH_OK;
  });
}

int dfsph_mlp_fit_normalization(dfsph_mlp *m, const float *x, const float *y, int64_t n) {
  return guard_mlp([&] {
    if (!m) throw DfsphException(DFSPH_ERR_INVALID_ARG, "model is NULL");
    if (n <= 1 || n > (int64_t)1 << 31) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n");
    DeviceScope ds(m->device);
    check_device_ptr(x, "x");
    check_device_ptr(y, "y");
    k_mlp_stats<<<STATS_BLOCKS, 256, 0, m->stream>>>(x, y, (int)n, m->spart);
    DF_CK(cudaGetLastError());
    std::vector<double> part(STATS_BLOCKS * 10);
    DF_CK(cudaMemcpyAsync(part.data(), m->spart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    DF_CK(cudaStreamSynchronize(m->stream));
    double s[10] = {0};
    for (int b = 0; b < STATS_BLOCKS; b++)
      for (int k = 0; k < 10; k++) s[k] += part[b * 10 + k];
    for (int k = 0; k < 4; k++) {
      const double mean = s[k] / n, var = std::max(s[4 + k] / n - mean * mean, 0.0);
      m->norm[k] = (float)mean;
      m->norm[4 + k] = var > 1e-30 ? (float)std::sqrt(var) : 1.f;
    }
    const double ym = s[8] / n, yv = std::max(s[9] / n - ym * ym, 0.0);
    m->norm[8] = (float)ym;
    m->norm[9] = yv > 1e-30 ? (float)std::sqrt(yv) : 1.f;
    return DFSPH_OK;
  });
}

int dfsph_mlp_train_step(dfsph_mlp *m, const float *x, const float *y, int64_t n_samples, const int32_t *idx,
                         int64_t n, float lr, double *loss) {
  return guard_mlp([&] {
    if (!m) throw DfsphException(DFSPH_ERR_INVALID_ARG, "model is NULL");
    if (!(lr > 0.f)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "lr must be positive");
    DeviceScope ds(m->device);
    check_device_ptr(x, "x");
    check_device_ptr(y, "y");
    if (idx) check_device_ptr(idx, "idx");
    if (n_samples <= 0) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n_samples must be positive");
    const double l = run_train_kernel(m, x, y, idx, n, n_samples);
    const int grid = std::min((int)((n + MLP_TILE - 1) / MLP_TILE), m->nparts);
    refresh(m, lr, false, 2.0f / (float)n, grid);
    DF_CK(cudaStreamSynchronize(m->stream));
    if (loss) *loss = l;
    return DFSPH_OK;
  });
}

int dfsph_mlp_gradient(dfsph_mlp *m, const float *x, const float *y, int64_t n, double *grad, double *loss) {
  return guard_mlp([&] {
    if (!m || !grad) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL argument");
    DeviceScope ds(m->device);
    check_device_ptr(x, "x");
    check_device_ptr(y, "y");
    const double l = run_train_kernel(m, x, y, nullptr, n, n);
    const int grid = std::min((int)((n + MLP_TILE - 1) / MLP_TILE), m->nparts);
    refresh(m, 0.f, true, 2.0f / (float)n, grid);
    std::vector<float> g(MLP_NPARAMS);
    DF_CK(cudaMemcpyAsync(g.data(), m->grad, MLP_NPARAMS * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    DF_CK(cudaStreamSynchronize(m->stream));
    for (int k = 0; k < MLP_NPARAMS; k++) grad[k] = g[k];
    if (loss) *loss = l;
    return DFSPH_OK;
  });
}

int dfsph_mlp_predict(dfsph_mlp *m, const float *x, float *y, int64_t n) {
  return guard_mlp([&] {
    if (!m) throw DfsphException(DFSPH_ERR_INVALID_ARG, "model is NULL");
    if (n < 0 || n > (int64_t)INT32_MAX - MLP_TILE) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n");
    if (n == 0) return DFSPH_OK;
    DeviceScope ds(m->device);
    check_device_ptr(x, "x");
    check_device_ptr(y, "y");
    {
      // the kernel reads the next tile's features before it writes the current tile's outputs
      const auto xb = reinterpret_cast<uintptr_t>(x), yb = reinterpret_cast<uintptr_t>(y);
      const auto xe = xb + (uintptr_t)n * 4 * sizeof(float), ye = yb + (uintptr_t)n * sizeof(float);
      if (xb < ye && yb < xe) throw DfsphException(DFSPH_ERR_INVALID_ARG, "x and y overlap");
    }
    mlp_sync_small(m);
    const int ntiles = (int)((n + MLP_TILE - 1) / MLP_TILE);
    const int grid = std::min(ntiles, m->nparts * 8);
    DF_CK(cudaMemsetAsync(m->err, 0, sizeof(int), m->stream));
    k_mlp_infer<MlpArrayIO><<<grid, MLP_THREADS, MLP_INFER_SMEM, m->stream>>>(mlp_view(m), MlpArrayIO{x, y}, (int)n,
                                                                             m->err, 1);
    DF_CK(cudaGetLastError());
    int e = 0;
    DF_CK(cudaMemcpyAsync(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    DF_CK(cudaStreamSynchronize(m->stream));
    if (e) throw DfsphException(DFSPH_ERR_DEVICE, "tensor-core MMA wait timed out in the inference kernel");
    return DFSPH_OK;
  });
}

int dfsph_mlp_set_wait_limit(dfsph_mlp *m, int32_t polls) {
  return guard_mlp([&] {
    if (!m) throw DfsphException(DFSPH_ERR_INVALID_ARG, "model is NULL");
    if (polls < -1) throw DfsphException(DFSPH_ERR_INVALID_ARG, "polls must be -1 (default) or >= 0");
    m->first_wait_polls = polls;
    return DFSPH_OK;
  });
}

}  // extern "C"
