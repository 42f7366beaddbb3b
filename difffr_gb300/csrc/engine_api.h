// engine_api.h — the host-side interface between the C ABI (abi.cu) and the
// precision-specific engines (engine_fp32.cu, engine_fp64.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/dfsph.h"
#include "mlp_view.h"

namespace dfsph {

struct DfsphException : std::runtime_error {
  int code;
  DfsphException(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define DF_CK(call)                                                                               \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      throw ::dfsph::DfsphException(e_ == cudaErrorMemoryAllocation ? DFSPH_ERR_OUT_OF_MEMORY     \
                                                                    : DFSPH_ERR_CUDA,             \
                                    std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)

class EngineBase {
 public:
  virtual ~EngineBase() {}
  virtual int step(int nsteps, dfsph_step_stats *st) = 0;
  virtual void reset() = 0;
  virtual void reset_gradient() = 0;
  virtual void set_rigid_init(int b, const double *v, const double *w) = 0;
  virtual void get_rigid_init(int b, double *v, double *w) = 0;
  virtual void get_rigid_state(int b, double *x, double *q, double *v, double *w) = 0;
  virtual void set_rigid_velocity(int b, const double *v, const double *w) = 0;
  virtual void get_rigid_force(int b, double *F, double *T) = 0;
  virtual void get_rigid_mass(int b, double *m, double *I) = 0;
  virtual void get_rigid_grad(int b, double *out) = 0;
  virtual void get_net_jacobians(int b, double *out) = 0;
  virtual void backward(const double *dL, double *out) = 0;
  virtual int64_t tape_length() = 0;
  virtual void copy_field(int f, double *dst, int64_t n) = 0;
  virtual void set_field(int f, const double *src, int64_t n) = 0;
  virtual void counts(int64_t *nf, int64_t *nb) = 0;
  virtual void neighbors(int which, int64_t *start, int32_t *idx, int64_t *total) = 0;
  virtual void get_time(double *t, int64_t *sc) = 0;
  virtual void synchronize() = 0;
  virtual int64_t launches() = 0;
  virtual void record_event(int slot) = 0;
  virtual double event_elapsed(int a, int b) = 0;
  virtual void profile_enable(bool on) = 0;
  virtual void profile_read(int k, int64_t *launches, double *ms, int64_t *units) = 0;
  virtual void set_time(double t, int64_t sc) = 0;
  virtual void set_rigid_state(int b, const double *x, const double *q, const double *v, const double *w) = 0;
  virtual void set_gradient_enabled(bool on) = 0;
  virtual int checkpoint_save() = 0;
  virtual void checkpoint_restore(int slot) = 0;
  virtual void checkpoint_free(int slot) = 0;
  virtual void adjoint_sweep(const double *lam_in, double *lam_out) = 0;
  virtual void set_warmstart_model(const MlpView *v) = 0;
  virtual void ml_record(bool on) = 0;
  virtual int64_t ml_capture(float *x, float *y, int64_t cap) = 0;
  virtual void get_manager_grad(int b, int b2, double *out) = 0;
  virtual void get_manager_jacobians(int b, int b2, double *out) = 0;
  virtual void contact_count(int64_t *nc, int64_t *na) = 0;
};

EngineBase *make_engine_fp32(const dfsph_scene *sc);
// Sets the calling thread's message returned by dfsph_last_error (defined in abi.cu).
void set_last_error(const std::string &msg);
EngineBase *make_engine_fp64(const dfsph_scene *sc);

}  // namespace dfsph
