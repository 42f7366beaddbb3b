// abi.cu — the extern "C" entry points of include/dfsph.h. Every call catches the
// engine's exceptions and returns a status code; the message is kept per thread.
#include <cstring>
#include <new>
#include <string>

#include "../../include/dfsph.h"
#include "engine_api.h"

using dfsph::DfsphException;
using dfsph::EngineBase;
using dfsph::MlpView;
using dfsph::mlp_view;
using dfsph::mlp_sync_small;

struct dfsph_ctx {
  EngineBase *engine;
  int device;
  dfsph_mlp *mlp = nullptr;  // learned warm-start model in use (not owned)
};

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

template <class F>
int guard(F &&f) {
  try {
    g_last_error.clear();
    return f();
  } catch (const DfsphException &e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc &) {
    return fail(DFSPH_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(DFSPH_ERR_CUDA, e.what());
  } catch (...) {
    return fail(DFSPH_ERR_CUDA, "unknown error");
  }
}

int valid(dfsph_ctx *c) {
  if (!c || !c->engine) throw DfsphException(DFSPH_ERR_INVALID_ARG, "context is NULL");
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) throw DfsphException(DFSPH_ERR_CUDA, cudaGetErrorString(e));
  return 0;
}
}  // namespace

namespace dfsph {
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace dfsph

extern "C" {

int dfsph_abi_version(void) { return DFSPH_ABI_VERSION; }

const char *dfsph_last_error(void) { return g_last_error.c_str(); }

int dfsph_default_params(dfsph_params *p) {
  if (!p) return fail(DFSPH_ERR_INVALID_ARG, "params is NULL");
  std::memset(p, 0, sizeof(*p));
  p->struct_size = sizeof(dfsph_params);
  p->fluid_precision = DFSPH_FP32;
  p->particle_radius = 0.025;
  p->density0 = 1000.0;
  p->viscosity = 0.01;
  p->gravity[0] = 0.0; p->gravity[1] = -9.81; p->gravity[2] = 0.0;
  p->time_step = 0.001;
  p->min_iterations = 2;
  p->max_iterations = 100;
  p->max_error = 0.01;
  p->max_iterations_v = 100;
  p->max_error_v = 0.1;
  p->enable_divergence_solver = 1;
  p->use_pressure_warmstart = 1;
  p->use_divergence_warmstart = 1;
  p->gradient_mode = DFSPH_GRAD_INCOMPLETE;
  p->rigid_body_mode = DFSPH_RB_GYROSCOPIC;
  p->optimize_rotation = 1;
  p->enable_gradient = 1;
  p->truncate_gradient_coeff = 1;
  p->release_rigid_body_mode = 0;
  p->uniform_accelerate_rb_time = 0.0;
  p->target_time = 0.8;
  p->surface_tension_method = 0;
  p->surface_tension = 0.05;
  p->surface_tension_boundary = 0.01;
  p->cfl_method = 0;
  p->cfl_factor = 0.5;
  p->cfl_min_time_step = 0.0001;
  p->cfl_max_time_step = 0.005;
  p->use_rigid_contact_solver = 0;
  p->use_rigid_gradient_manager = 0;
  p->rigid_contact_gamma = 0.7;
  p->rigid_contact_beta = 1.0;
  p->rigid_contact_support_radius_factor = 4.0;
  p->rigid_contact_friction_coeff = 0.0;
  p->viscosity_boundary = 0.0;
  return DFSPH_OK;
}

int dfsph_set_device(int32_t device) {
  return guard([&] {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) throw DfsphException(DFSPH_ERR_CUDA, cudaGetErrorString(e));
    if (device < 0 || device >= n) throw DfsphException(DFSPH_ERR_INVALID_ARG, "device index out of range");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) throw DfsphException(DFSPH_ERR_CUDA, cudaGetErrorString(e));
    return DFSPH_OK;
  });
}

int dfsph_create(const dfsph_scene *scene, dfsph_ctx **out) {
  return guard([&] {
    if (!out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!scene) throw DfsphException(DFSPH_ERR_INVALID_ARG, "scene is NULL");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw DfsphException(DFSPH_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    EngineBase *eng = nullptr;
    if (scene->params.fluid_precision == DFSPH_FP64) eng = dfsph::make_engine_fp64(scene);
    else if (scene->params.fluid_precision == DFSPH_FP32) eng = dfsph::make_engine_fp32(scene);
    else throw DfsphException(DFSPH_ERR_INVALID_ARG, "fluid_precision");
    *out = new dfsph_ctx{eng, dev};
    return DFSPH_OK;
  });
}

int dfsph_destroy(dfsph_ctx *ctx) {
  return guard([&] {
    if (!ctx) return DFSPH_OK;
    cudaSetDevice(ctx->device);
    delete ctx->engine;
    delete ctx;
    return DFSPH_OK;
  });
}

int dfsph_reset(dfsph_ctx *ctx) {
  return guard([&] { valid(ctx); ctx->engine->reset(); return DFSPH_OK; });
}

int dfsph_step(dfsph_ctx *ctx, int32_t nsteps, dfsph_step_stats *stats) {
  return guard([&] {
    valid(ctx);
    if (ctx->mlp) {
      mlp_sync_small(ctx->mlp);
      const MlpView v = mlp_view(ctx->mlp);  // the model's current weights and normalisation
      ctx->engine->set_warmstart_model(&v);
    }
    const int rc = ctx->engine->step(nsteps, stats);
    if (rc == DFSPH_ERR_NOT_CONVERGED) g_last_error = "a solve reached its iteration cap";
    return rc;
  });
}

int dfsph_set_rigid_init(dfsph_ctx *ctx, int32_t body, const double v[3], const double omega[3]) {
  return guard([&] {
    valid(ctx);
    if (!v || !omega) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL vector");
    ctx->engine->set_rigid_init(body, v, omega);
    return DFSPH_OK;
  });
}

int dfsph_get_rigid_init(dfsph_ctx *ctx, int32_t body, double v[3], double omega[3]) {
  return guard([&] {
    valid(ctx);
    if (!v || !omega) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL vector");
    ctx->engine->get_rigid_init(body, v, omega);
    return DFSPH_OK;
  });
}

int dfsph_get_rigid_state(dfsph_ctx *ctx, int32_t body, double x[3], double q[4], double v[3], double omega[3]) {
  return guard([&] { valid(ctx); ctx->engine->get_rigid_state(body, x, q, v, omega); return DFSPH_OK; });
}

int dfsph_set_rigid_velocity(dfsph_ctx *ctx, int32_t body, const double v[3], const double omega[3]) {
  return guard([&] {
    valid(ctx);
    if (!v || !omega) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL vector");
    ctx->engine->set_rigid_velocity(body, v, omega);
    return DFSPH_OK;
  });
}

int dfsph_get_rigid_force(dfsph_ctx *ctx, int32_t body, double force[3], double torque[3]) {
  return guard([&] {
    valid(ctx);
    if (!force || !torque) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL vector");
    ctx->engine->get_rigid_force(body, force, torque);
    return DFSPH_OK;
  });
}

int dfsph_get_rigid_mass(dfsph_ctx *ctx, int32_t body, double *mass, double inertia[9]) {
  return guard([&] {
    valid(ctx);
    if (!mass || !inertia) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->get_rigid_mass(body, mass, inertia);
    return DFSPH_OK;
  });
}

int dfsph_get_rigid_grad(dfsph_ctx *ctx, int32_t body, double out[78]) {
  return guard([&] {
    valid(ctx);
    if (!out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->get_rigid_grad(body, out);
    return DFSPH_OK;
  });
}

int dfsph_get_net_jacobians(dfsph_ctx *ctx, int32_t body, double out[78]) {
  return guard([&] {
    valid(ctx);
    if (!out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->get_net_jacobians(body, out);
    return DFSPH_OK;
  });
}

int dfsph_get_manager_grad(dfsph_ctx *ctx, int32_t body, int32_t body2, double out[78]) {
  return guard([&] {
    valid(ctx);
    if (!out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->get_manager_grad(body, body2, out);
    return DFSPH_OK;
  });
}

int dfsph_get_manager_jacobians(dfsph_ctx *ctx, int32_t body, int32_t body2, double out[78]) {
  return guard([&] {
    valid(ctx);
    if (!out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->get_manager_jacobians(body, body2, out);
    return DFSPH_OK;
  });
}

int dfsph_get_contact_count(dfsph_ctx *ctx, int64_t *n_contact, int64_t *n_active) {
  return guard([&] {
    valid(ctx);
    if (!n_contact || !n_active) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->contact_count(n_contact, n_active);
    return DFSPH_OK;
  });
}

int dfsph_reset_gradient(dfsph_ctx *ctx) {
  return guard([&] { valid(ctx); ctx->engine->reset_gradient(); return DFSPH_OK; });
}

int dfsph_backward(dfsph_ctx *ctx, const double *dL_dstate, double *dL_dinit) {
  return guard([&] { valid(ctx); ctx->engine->backward(dL_dstate, dL_dinit); return DFSPH_OK; });
}

int dfsph_tape_length(dfsph_ctx *ctx, int64_t *n_steps) {
  return guard([&] {
    valid(ctx);
    if (!n_steps) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    *n_steps = ctx->engine->tape_length();
    return DFSPH_OK;
  });
}

int dfsph_copy_field(dfsph_ctx *ctx, int32_t field, double *dst, int64_t n) {
  return guard([&] {
    valid(ctx);
    if (!dst && n > 0) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->copy_field(field, dst, n);
    return DFSPH_OK;
  });
}

int dfsph_set_field(dfsph_ctx *ctx, int32_t field, const double *src, int64_t n) {
  return guard([&] {
    valid(ctx);
    if (!src && n > 0) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL input");
    ctx->engine->set_field(field, src, n);
    return DFSPH_OK;
  });
}

int dfsph_num_particles(dfsph_ctx *ctx, int64_t *n_fluid, int64_t *n_boundary) {
  return guard([&] {
    valid(ctx);
    if (!n_fluid || !n_boundary) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    ctx->engine->counts(n_fluid, n_boundary);
    return DFSPH_OK;
  });
}

int dfsph_get_neighbors(dfsph_ctx *ctx, int32_t which, int64_t *start, int32_t *idx, int64_t *total) {
  return guard([&] {
    valid(ctx);
    if (!total) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL total");
    ctx->engine->neighbors(which, start, idx, total);
    return DFSPH_OK;
  });
}

int dfsph_get_time(dfsph_ctx *ctx, double *t, int64_t *step_count) {
  return guard([&] {
    valid(ctx);
    double tt;
    int64_t sc;
    ctx->engine->get_time(&tt, &sc);
    if (t) *t = tt;
    if (step_count) *step_count = sc;
    return DFSPH_OK;
  });
}

int dfsph_synchronize(dfsph_ctx *ctx) {
  return guard([&] { valid(ctx); ctx->engine->synchronize(); return DFSPH_OK; });
}

int dfsph_launch_count(dfsph_ctx *ctx, int64_t *count) {
  return guard([&] {
    valid(ctx);
    if (!count) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    *count = ctx->engine->launches();
    return DFSPH_OK;
  });
}

int dfsph_record_event(dfsph_ctx *ctx, int32_t slot) {
  return guard([&] { valid(ctx); ctx->engine->record_event(slot); return DFSPH_OK; });
}

int dfsph_event_elapsed(dfsph_ctx *ctx, int32_t slot_a, int32_t slot_b, double *ms) {
  return guard([&] {
    valid(ctx);
    if (!ms) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    *ms = ctx->engine->event_elapsed(slot_a, slot_b);
    return DFSPH_OK;
  });
}

int dfsph_profile_enable(dfsph_ctx *ctx, int32_t on) {
  return guard([&] { valid(ctx); ctx->engine->profile_enable(on != 0); return DFSPH_OK; });
}

int dfsph_profile_read(dfsph_ctx *ctx, int32_t kernel_class, int64_t *launches, double *total_ms, int64_t *units) {
  return guard([&] { valid(ctx); ctx->engine->profile_read(kernel_class, launches, total_ms, units); return DFSPH_OK; });
}

const char *dfsph_kernel_class_name(int32_t k) {
  static const char *names[DFSPH_PROFILE_COUNT] = {
      "sort",        "lists_density_factor", "bf_lists", "density_pass", "velocity_pass",    "xsph_advect",
      "integrate",   "pairs",                "rigid",    "mlp",          "divergence_solve", "pressure_solve"};
  return (k >= 0 && k < DFSPH_PROFILE_COUNT) ? names[k] : "";
}

int dfsph_set_time(dfsph_ctx *ctx, double t, int64_t step_count) {
  return guard([&] { valid(ctx); ctx->engine->set_time(t, step_count); return DFSPH_OK; });
}

int dfsph_set_rigid_state(dfsph_ctx *ctx, int32_t body, const double x[3], const double q[4], const double v[3],
                          const double omega[3]) {
  return guard([&] { valid(ctx); ctx->engine->set_rigid_state(body, x, q, v, omega); return DFSPH_OK; });
}

int dfsph_set_gradient_enabled(dfsph_ctx *ctx, int32_t on) {
  return guard([&] { valid(ctx); ctx->engine->set_gradient_enabled(on != 0); return DFSPH_OK; });
}

int dfsph_checkpoint_save(dfsph_ctx *ctx, int32_t *slot) {
  return guard([&] {
    valid(ctx);
    if (!slot) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL output");
    *slot = ctx->engine->checkpoint_save();
    return DFSPH_OK;
  });
}

int dfsph_checkpoint_restore(dfsph_ctx *ctx, int32_t slot) {
  return guard([&] { valid(ctx); ctx->engine->checkpoint_restore(slot); return DFSPH_OK; });
}

int dfsph_checkpoint_free(dfsph_ctx *ctx, int32_t slot) {
  return guard([&] { valid(ctx); ctx->engine->checkpoint_free(slot); return DFSPH_OK; });
}

int dfsph_adjoint_sweep(dfsph_ctx *ctx, const double *lam_in, double *lam_out) {
  return guard([&] { valid(ctx); ctx->engine->adjoint_sweep(lam_in, lam_out); return DFSPH_OK; });
}

int dfsph_set_warmstart_model(dfsph_ctx *ctx, dfsph_mlp *m) {
  return guard([&] {
    valid(ctx);
    if (m) {
      mlp_sync_small(m);
      const MlpView v = mlp_view(m);
      ctx->engine->set_warmstart_model(&v);
    } else {
      ctx->engine->set_warmstart_model(nullptr);
    }
    ctx->mlp = m;
    return DFSPH_OK;
  });
}

int dfsph_ml_record(dfsph_ctx *ctx, int32_t on) {
  return guard([&] { valid(ctx); ctx->engine->ml_record(on != 0); return DFSPH_OK; });
}

int dfsph_ml_capture(dfsph_ctx *ctx, float *x, float *y, int64_t capacity, int64_t *count) {
  return guard([&] {
    valid(ctx);
    if (!x || !y || !count) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL argument");
    if (capacity < 0) throw DfsphException(DFSPH_ERR_INVALID_ARG, "capacity < 0");
    cudaPointerAttributes a;
    for (const void *p : {(const void *)x, (const void *)y}) {
      if (cudaPointerGetAttributes(&a, p) != cudaSuccess ||
          (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)) {
        cudaGetLastError();
        throw DfsphException(DFSPH_ERR_INVALID_ARG, "x and y must be device pointers");
      }
    }
    *count = ctx->engine->ml_capture(x, y, capacity);
    return DFSPH_OK;
  });
}

}  // extern "C"
