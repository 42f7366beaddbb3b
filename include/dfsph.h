/*
 * dfsph.h — C ABI of libdfsph, a GB300 (sm_103a) implementation of DiffFR's
 * differentiable DFSPH fluid–rigid time step (method "DiffDFSPH", Akinci2012
 * boundary coupling, forward-mode rigid gradient chain plus a reverse-mode
 * adjoint over the same chain).
 *
 * Conventions
 *  - Every function returns an int status: DFSPH_OK (0) or a positive error
 *    code. No C++ exception crosses this boundary. dfsph_last_error() gives a
 *    human-readable message for the last failing call on the calling thread.
 *  - A context owns all device memory and its CUDA streams (the fluid stream,
 *    the rigid-body stream and the per-body chain-rule stream). Calls on one
 *    context are not thread-safe; distinct contexts are independent.
 *  - Host buffers are owned by the caller. Positions and velocities cross the
 *    boundary as row-major double[n][3] in the caller's (original) particle
 *    order, whatever order the device keeps internally.
 *  - Quaternions are (w, x, y, z), as the reference's get_quaternion_rb_vec4.
 *  - Matrices are row-major doubles.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the DiffFR repository root).
 */
#ifndef DFSPH_H
#define DFSPH_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DFSPH_ABI_VERSION 1

/* status codes */
#define DFSPH_OK                  0
#define DFSPH_ERR_INVALID_ARG     1
#define DFSPH_ERR_CUDA            2
#define DFSPH_ERR_NOT_CONVERGED   3  /* solver hit max iterations (informational; state is valid) */
#define DFSPH_ERR_DEVICE          4  /* device error word set (e.g. neighbour list overflow) */
#define DFSPH_ERR_OUT_OF_MEMORY   5
#define DFSPH_ERR_UNSUPPORTED     6
#define DFSPH_ERR_STATE           7  /* call not valid in the current state */

/* fluid arithmetic precision */
#define DFSPH_FP32 0
#define DFSPH_FP64 1

/* reference enum SPH::GradientMode (SPlisHSPlasH/Simulation.h:173) */
#define DFSPH_GRAD_COMPLETE        0
#define DFSPH_GRAD_INCOMPLETE      1
#define DFSPH_GRAD_RIGID_ONLY      2

/* reference enum SPH::RigidBodyMode (SPlisHSPlasH/Simulation.h:174) */
#define DFSPH_RB_GYROSCOPIC        0
#define DFSPH_RB_NO_GYROSCOPIC     1

#define DFSPH_MAX_BODIES 16

/*
 * Scene parameters. Field meanings and defaults follow the reference's
 * scene "Configuration" keys (SPlisHSPlasH/Utilities/SceneLoader.cpp:41-200)
 * and the DiffDFSPH parameters (SPlisHSPlasH/DiffDFSPH/TimeStepDiffDFSPH.cpp:90-134,
 * SPlisHSPlasH/TimeStep.cpp:24-30). dfsph_default_params() fills the defaults.
 */
typedef struct dfsph_params {
  int32_t struct_size;                 /* = sizeof(dfsph_params) */
  int32_t fluid_precision;             /* DFSPH_FP32 | DFSPH_FP64; rigid state is always FP64 */
  double  particle_radius;             /* r; kernel support h = 4 r (Simulation.cpp:382-387) */
  double  density0;                    /* fluid rest density */
  double  viscosity;                   /* XSPH coefficient, fluid-fluid (Viscosity_XSPH.cpp:66) */
  double  gravity[3];
  double  time_step;                   /* fixed dt (cflMethod 0) */
  int32_t min_iterations;              /* pressure solve, default 2 */
  int32_t max_iterations;              /* pressure solve, default 100 */
  double  max_error;                   /* pressure solve, percent, default 0.01 */
  int32_t max_iterations_v;            /* divergence solve, default 100 */
  double  max_error_v;                 /* divergence solve, percent, default 0.1 */
  int32_t enable_divergence_solver;    /* default 1 */
  int32_t use_pressure_warmstart;      /* default 1 */
  int32_t use_divergence_warmstart;    /* default 1 */
  int32_t gradient_mode;               /* DFSPH_GRAD_*, default Incomplete */
  int32_t rigid_body_mode;             /* DFSPH_RB_*, default gyroscopic */
  int32_t optimize_rotation;           /* default 1 (TimeStepDiffDFSPH.cpp:108) */
  int32_t enable_gradient;             /* accumulate pair Jacobians each solver sweep (reference BACKWARD build) */
  int32_t truncate_gradient_coeff;     /* reproduce the unsigned 1/h^2, 1/h coefficient of
                                          TimeStepDiffDFSPH.cpp:1266; default 1 */
  int32_t release_rigid_body_mode;     /* useReleaseRigidBodyMode, default 0 */
  double  uniform_accelerate_rb_time;  /* uniformAccelerateRBTime, default 0 */
  double  target_time;                 /* targetTime, default 0.8 */
  int32_t max_fluid_neighbors;         /* capacity of each fluid particle's fluid list (0 = default 96) */
  int32_t max_boundary_neighbors;      /* capacity of each fluid particle's boundary list (0 = default 96) */
  int32_t surface_tension_method;      /* 0 none, 2 Akinci2013 (SurfaceTension_Akinci2013.cpp:28-148);
                                          scene "surfaceTensionMethod"; default 0 */
  double  surface_tension;             /* "surfaceTension", default 0.05 (SurfaceTensionBase.cpp:12) */
  double  surface_tension_boundary;    /* "surfaceTensionBoundary", default 0.01 (SurfaceTensionBase.cpp:13) */
  int32_t cfl_method;                  /* 0 fixed time_step, 1 CFL (Simulation.cpp:524-616); "cflMethod";
                                          default 0 */
  double  cfl_factor;                  /* "cflFactor", default 0.5 */
  double  cfl_min_time_step;           /* "cflMinTimeStepSize", default 0.0001 */
  double  cfl_max_time_step;           /* "cflMaxTimeStepSize", default 0.005 */
  /* Rigid-rigid contact (InterlinkedSPH RigidContactSolver, penalty form,
     RigidContactSolver.cpp:307-555, RigidBody3dBoundarySimulator.cpp:278-320; scene keys of SceneLoader.cpp:54-71) */
  int32_t use_rigid_contact_solver;    /* "useRigidContactSolver", default 0 */
  int32_t use_rigid_gradient_manager;  /* "useRigidGradientManager": the multi-body chain of
                                          RigidBodyGradientManager.cpp:96-468 instead of the
                                          per-body chain; default 0 */
  double  rigid_contact_gamma;         /* "rigidContactGamma", default 0.7 */
  double  rigid_contact_beta;          /* "rigidContactBeta" (penalty stiffness), default 1.0 */
  double  rigid_contact_support_radius_factor; /* "rigidContactSupportRadiusFactor", default 4.0 */
  double  rigid_contact_friction_coeff; /* "rigidContactFrictionCoeff", default 0.0 */
  double  viscosity_boundary;          /* XSPH coefficient against boundary samples, with the
                                          reaction on dynamic bodies (Viscosity_XSPH.cpp:72-82);
                                          material "viscosityBoundary", default 0 */
} dfsph_params;

/*
 * One rigid body with Akinci2012 boundary samples (reference: a "RigidBodies"
 * scene entry, SceneLoader.cpp:95-200; Dynamic3dRigidBody, BoundaryModel_Akinci2012).
 * Samples are in the body's local frame; world = R(q) sample + translation
 * (SimulatorBase.cpp:1827-1857). Mass and inertia follow the reference's shell
 * model (Dynamic3dRigidBody.h:184-213): every sample carries (4/3) pi r^3 * density.
 */
typedef struct dfsph_body_desc {
  int32_t       is_dynamic;
  int32_t       is_animated;
  int64_t       n_samples;
  const double *samples;               /* [n_samples][3] local coordinates */
  double        translation[3];
  double        rotation[4];           /* (w, x, y, z) */
  double        density;
  double        init_velocity[3];      /* "initVelocity" -> set_init_v_rb */
  double        init_angular_velocity[3];
  double        target_x[3];
} dfsph_body_desc;

typedef struct dfsph_scene {
  int32_t                struct_size;  /* = sizeof(dfsph_scene) */
  dfsph_params           params;
  int64_t                n_fluid;
  const double          *fluid_x;      /* [n_fluid][3] */
  const double          *fluid_v;      /* [n_fluid][3] or NULL for zero */
  int32_t                n_bodies;
  const dfsph_body_desc *bodies;
} dfsph_scene;

/* Per-step statistics (reference counters "DFSPH - iterations",
   "DFSPH - iterationsV", TimeStepDiffDFSPH.cpp:750,863). */
typedef struct dfsph_step_stats {
  int32_t steps_done;
  int32_t pressure_iterations;         /* last step */
  int32_t divergence_iterations;       /* last step */
  int32_t trajectory_finished;         /* is_trajectory_finish_callback() after the last step */
  double  pressure_avg_error;          /* last step, kg/m^3 (rho0 * (rho_adv - 1) averaged) */
  double  divergence_avg_error;        /* last step */
  int64_t total_pressure_iterations;   /* summed over the steps of this call */
  int64_t total_divergence_iterations;
  double  time;                        /* simulated time after the call */
  double  time_step;                   /* time step size after the call (changes under CFL) */
} dfsph_step_stats;

/* Fluid fields for dfsph_copy_field (reference FluidModel / SimulationDataDiffDFSPH
   accessors, SimulationDataDiffDFSPH.h:254-266). Vector fields have 3 components. */
#define DFSPH_FIELD_X          0  /* position, 3 */
#define DFSPH_FIELD_V          1  /* velocity, 3 */
#define DFSPH_FIELD_DENSITY    2
#define DFSPH_FIELD_FACTOR     3  /* alpha */
#define DFSPH_FIELD_KAPPA      4
#define DFSPH_FIELD_KAPPA_V    5
#define DFSPH_FIELD_DENSITY_ADV 6
#define DFSPH_FIELD_SUM_GRAD_P 7  /* sum_grad_p_k, 3 */
#define DFSPH_FIELD_BOUNDARY_X   8   /* boundary positions, 3, body-concatenated order */
#define DFSPH_FIELD_BOUNDARY_V   9   /* boundary velocities, 3 */
#define DFSPH_FIELD_BOUNDARY_PSI 10  /* boundary psi volume */

/* Neighbour sets for dfsph_get_neighbors (reference Simulation::numberOfNeighbors /
   getNeighbor, Simulation.h:526-534). Indices are in the caller's particle order. */
#define DFSPH_NB_FLUID_FLUID     0   /* fluid i -> fluid j (j != i) */
#define DFSPH_NB_FLUID_BOUNDARY  1   /* fluid i -> boundary k (all bodies) */
#define DFSPH_NB_BOUNDARY_FLUID  2   /* dynamic boundary k -> fluid i (rows for static k are empty) */

/* Library */
int         dfsph_abi_version(void);
const char *dfsph_last_error(void);
/* Fills defaults of the reference (see dfsph_params). */
int         dfsph_default_params(dfsph_params *out);

typedef struct dfsph_ctx dfsph_ctx;

/* Selects the CUDA device that the next dfsph_create uses (the library keeps its own
   current device; default 0). One process per GPU: call once at start-up. */
int dfsph_set_device(int32_t device);

/* Replaces SimulatorBase::init + initSimulation + deferredInit for a DiffDFSPH scene
   (Simulator/SimulatorBase.cpp:494-588, Simulation::setSimulationMethod(5)
   SPlisHSPlasH/Simulation.cpp:714-719, RigidBody3dBoundarySimulator::initBoundaryData /
   deferredInit Simulator/RigidBody3dBoundarySimulator.cpp:68-270,
   Simulation::updateBoundaryVolume Simulation.cpp:831-900). Uses the current CUDA device. */
int dfsph_create(const dfsph_scene *scene, dfsph_ctx **out);
int dfsph_destroy(dfsph_ctx *ctx);

/* Replaces SimulatorBase::reset (SimulatorBase.cpp:887-934): fluid back to the
   scene state, bodies to their initial pose, psi recomputed, gradients reset,
   time 0. Initial rigid velocities set by dfsph_set_rigid_init are kept. */
int dfsph_reset(dfsph_ctx *ctx);

/* Replaces nsteps iterations of SimulatorBase::timeStep's inner loop
   (SimulatorBase.cpp:999-1016): TimeStepDiffDFSPH::step (TimeStepDiffDFSPH.cpp:526-652)
   followed by RigidBody3dBoundarySimulator::velocityTimeStep and positionTimeStep
   (RigidBody3dBoundarySimulator.cpp:278-344). stats may be NULL. Returns
   DFSPH_ERR_NOT_CONVERGED (state valid) if a solve hit its iteration cap.
   Returns once the fluid and the bodies are updated; the last step's per-body chain
   rule may still run on the device, and every call that reads it (dfsph_get_rigid_grad,
   dfsph_backward, dfsph_adjoint_sweep, checkpoints, dfsph_synchronize) waits for it. */
int dfsph_step(dfsph_ctx *ctx, int32_t nsteps, dfsph_step_stats *stats);

/* Replaces TimeStepDiffDFSPH::set_init_v_rb / set_init_omega_rb
   (pySPlisHSPlasH/DiffDFSPHModule.cpp:63-64). */
int dfsph_set_rigid_init(dfsph_ctx *ctx, int32_t body, const double v[3], const double omega[3]);
int dfsph_get_rigid_init(dfsph_ctx *ctx, int32_t body, double v[3], double omega[3]);

/* Replaces BoundaryModel_Akinci2012::get_position_rb / get_quaternion_rb_vec4 /
   get_velocity_rb / get_angular_velocity_rb (pySPlisHSPlasH/BoundaryModelModule.cpp:68-71).
   Any output pointer may be NULL. */
int dfsph_get_rigid_state(dfsph_ctx *ctx, int32_t body, double x[3], double q[4],
                          double v[3], double omega[3]);
/* Overwrites a body's current velocity and angular velocity and refreshes its boundary
   particle velocities, as Dynamic3dRigidBody::setVelocity / setAngularVelocity followed by
   SimulatorBase::updateBoundaryParticles (SimulatorBase.cpp:1827-1857). */
int dfsph_set_rigid_velocity(dfsph_ctx *ctx, int32_t body, const double v[3], const double omega[3]);

/* Replaces BoundaryModel::getForce / getTorque (SPlisHSPlasH/BoundaryModel.cpp:56-75):
   net fluid force and torque on the body from the last step. */
int dfsph_get_rigid_force(dfsph_ctx *ctx, int32_t body, double force[3], double torque[3]);

/* Body mass and world inertia (Dynamic3dRigidBody::getMass / getInertiaTensorWorld). */
int dfsph_get_rigid_mass(dfsph_ctx *ctx, int32_t body, double *mass, double inertia[9]);

/* Forward-mode chain state of one body (BoundaryModel_Akinci2012 get_grad_x_to_v0,
   get_grad_x_to_omega0, get_grad_quaternion_to_v0, get_grad_quaternion_to_omega0,
   get_grad_v_to_v0, get_grad_v_to_omega0, get_grad_omega_to_v0, get_grad_omega_to_omega0,
   BoundaryModelModule.cpp:73-80). out[78] = x_v0(3x3) x_w0(3x3) q_v0(4x3) q_w0(4x3)
   v_v0(3x3) v_w0(3x3) w_v0(3x3) w_w0(3x3), all row-major. */
int dfsph_get_rigid_grad(dfsph_ctx *ctx, int32_t body, double out[78]);

/* Per-step net Jacobians of the last step (BoundaryModel_Akinci2012 grad_net_force_to_* /
   grad_net_torque_to_*, BoundaryModel_Akinci2012.cpp:453-497; also what
   RigidBodyGradientManager::get_grad_net_force_to_vn(R,R) returns, SimulationModule.cpp:406-415).
   out[78] = F_v F_x F_w (3x3 each) F_q (3x4) T_w T_v T_x (3x3 each) T_q (3x4). */
int dfsph_get_net_jacobians(dfsph_ctx *ctx, int32_t body, double out[78]);

/* Multi-body chain state of the gradient manager (use_rigid_gradient_manager):
   RigidBodyGradientManager get_grad_x_to_v0(R, RR), get_grad_x_to_omega0, get_grad_q_to_v0,
   get_grad_q_to_omega0 and the v / omega blocks (SimulationModule.cpp:406-415) — the
   derivative of body R's state with respect to body RR's initial (v, omega). out[78] in the
   layout of dfsph_get_rigid_grad. DFSPH_ERR_UNSUPPORTED when the manager is off. */
int dfsph_get_manager_grad(dfsph_ctx *ctx, int32_t body, int32_t body2, double out[78]);

/* The manager's current force / torque Jacobian blocks [R][RR] (get_grad_net_force_to_vn(R, RR),
   get_grad_net_torque_to_omega_n(R, RR), ...): the fluid's blocks on the diagonal after a fluid
   step, overwritten by the contact solver's blocks for every dynamic pair when it runs
   (RigidContactSolver.cpp:1341-1369). out[78] in the layout of dfsph_get_net_jacobians. */
int dfsph_get_manager_jacobians(dfsph_ctx *ctx, int32_t body, int32_t body2, double out[78]);

/* Rigid contact of the last step: samples of dynamic bodies with a boundary neighbour of
   another body (num_contacts, RigidContactSolver.cpp:307-345) and, of those, the samples whose
   contact density exceeded their rest density and so carried a penalty force. */
int dfsph_get_contact_count(dfsph_ctx *ctx, int64_t *n_contact, int64_t *n_active);

/* Replaces TimeStepDiffDFSPH::reset_gradient (DiffDFSPHModule.cpp:91): chain state to
   identity/zero and the recorded per-step adjoint tape cleared. With the gradient manager
   on, its chain state is reset too (RigidBodyGradientManager::reset); its Jacobian blocks
   stay, because the next step's fluid stage reads the last contact blocks (dfsph_reset
   clears them). */
int dfsph_reset_gradient(dfsph_ctx *ctx);

/* Reverse-mode adjoint over the per-step chain matrices recorded since the last
   dfsph_reset / dfsph_reset_gradient. dL_dstate has 13 doubles per body
   (dL/dx[3], dL/dq[4] (w,x,y,z), dL/dv[3], dL/domega[3]) for the current state;
   dL_dinit receives 6 doubles per body (dL/dv0[3], dL/domega0[3]). Equal to
   contracting dL_dstate with the forward-mode chain state. No reference counterpart:
   the reference only propagates forward-mode tangents. With the gradient manager on the
   step maps couple the bodies, and dL_dinit of body RR collects every body's dL_dstate. */
int dfsph_backward(dfsph_ctx *ctx, const double *dL_dstate, double *dL_dinit);
int dfsph_tape_length(dfsph_ctx *ctx, int64_t *n_steps);

/* Field export/import in the caller's particle order (FluidModel::getPosition etc.).
   dst/src are host buffers of n*components doubles. */
int dfsph_copy_field(dfsph_ctx *ctx, int32_t field, double *dst, int64_t n);
int dfsph_set_field(dfsph_ctx *ctx, int32_t field, const double *src, int64_t n);
int dfsph_num_particles(dfsph_ctx *ctx, int64_t *n_fluid, int64_t *n_boundary);

/* Neighbour sets of the last neighbour search as CSR in the caller's order, each row
   sorted ascending. Call once with idx == NULL to get total; then with buffers.
   start has n_rows+1 entries. */
int dfsph_get_neighbors(dfsph_ctx *ctx, int32_t which, int64_t *start, int32_t *idx,
                        int64_t *total);

/* Simulated time (TimeManager::getTime) and steps since reset (get_step_count). */
int dfsph_get_time(dfsph_ctx *ctx, double *t, int64_t *step_count);
/* Sets the simulated time and step counter (TimeManager::setTime; used when a saved
   state is restored, SimulatorBase::loadState SimulatorBase.cpp:2046-2203). */
int dfsph_set_time(dfsph_ctx *ctx, double t, int64_t step_count);

/* Overwrites a body's pose and velocities (Dynamic3dRigidBody::setPosition / setRotation /
   setVelocity / setAngularVelocity, Dynamic3dRigidBody.h:67-96) and refreshes its boundary
   samples (SimulatorBase::updateBoundaryParticles). q is (w, x, y, z) and is normalised. */
int dfsph_set_rigid_state(dfsph_ctx *ctx, int32_t body, const double x[3], const double q[4],
                          const double v[3], const double omega[3]);

/* Switches the per-sweep pair-Jacobian accumulation and the per-step chain/tape on or off
   (the reference always accumulates in its BACKWARD build). */
int dfsph_set_gradient_enabled(dfsph_ctx *ctx, int32_t on);

/* Device-resident snapshots of the full simulation state (fluid records, kappa, kappaV,
   particle order, rigid states, dynamic samples, time) for checkpointed recomputation
   (the reference keeps no in-memory checkpoints; it writes state files,
   SimulatorBase::saveState SimulatorBase.cpp:1899-2005). A snapshot lives in HBM until
   dfsph_checkpoint_free. */
int dfsph_checkpoint_save(dfsph_ctx *ctx, int32_t *slot);
int dfsph_checkpoint_restore(dfsph_ctx *ctx, int32_t slot);
int dfsph_checkpoint_free(dfsph_ctx *ctx, int32_t slot);

/* Reverse sweep of the recorded step matrices on full 13-component adjoints: lam_out =
   A_1^T ... A_N^T lam_in, per body (x, q, v, omega). Lets a caller chain the adjoint across
   recomputed segments; dfsph_backward is this sweep followed by taking the (v, omega) part.
   With the gradient manager on, the maps of the v0 columns and of the omega0 columns differ
   (RigidBodyGradientManager.cpp:196-205 drops the q term of the v0 columns), so lam_in and
   lam_out hold 26 doubles per body: 13 per body for the v0 sweep, then 13 per body for the
   omega0 sweep. */
int dfsph_adjoint_sweep(dfsph_ctx *ctx, const double *lam_in, double *lam_out);

/* Synchronises all of the context's streams (for timing from the caller). */
int dfsph_synchronize(dfsph_ctx *ctx);

/* Kernel launches issued by this context since creation (for launch accounting). */
int dfsph_launch_count(dfsph_ctx *ctx, int64_t *count);

/* Timing on the context's stream (no reference counterpart; the reference times with
   host clocks, Utilities/Timing.h:22-37). dfsph_record_event records CUDA event `slot`
   (0..7) on the fluid stream, which has joined the rigid-body stream at the end of each
   dfsph_step call and joins the chain-rule stream at the calls listed under dfsph_step;
   dfsph_event_elapsed gives milliseconds between two recorded slots (synchronises on the
   second). */
int dfsph_record_event(dfsph_ctx *ctx, int32_t slot);
int dfsph_event_elapsed(dfsph_ctx *ctx, int32_t slot_a, int32_t slot_b, double *ms);

/* Per-kernel-class device timing with CUDA events around each launch (replaces the
   reference's START_TIMING/STOP_TIMING_AVG phases, TimeStepDiffDFSPH.cpp:528-651).
   dfsph_profile_read resolves and returns the totals since profiling was enabled:
   launches, summed device milliseconds and summed work units (particles, or samples
   for the boundary kernels). Kernel classes are DFSPH_K_*. */
#define DFSPH_K_SORT           0
#define DFSPH_K_LISTS_DENSITY  1
#define DFSPH_K_BF_LISTS       2
#define DFSPH_K_DENSITY_PASS   3
#define DFSPH_K_VELOCITY_PASS  4
#define DFSPH_K_XSPH           5
#define DFSPH_K_INTEGRATE      6
#define DFSPH_K_PAIRS          7
#define DFSPH_K_RIGID          8
#define DFSPH_K_MLP            9   /* learned warm-start inference */
#define DFSPH_K_COUNT          10
/* Phases (read with dfsph_profile_read like kernel classes): whole solves, from their
   first launch to their last, including the host's residual checks in between. */
#define DFSPH_PHASE_DIVERGENCE_SOLVE 10
#define DFSPH_PHASE_PRESSURE_SOLVE   11
#define DFSPH_PROFILE_COUNT          12
int dfsph_profile_enable(dfsph_ctx *ctx, int32_t on);
int dfsph_profile_read(dfsph_ctx *ctx, int32_t kernel_class, int64_t *launches, double *total_ms,
                       int64_t *units);
const char *dfsph_kernel_class_name(int32_t kernel_class);

/* ---- Learned warm start for the pressure stiffness.
   No reference counterpart: it replaces the stiffness formula of
   TimeStepDiffDFSPH::warmstartPressureSolve (TimeStepDiffDFSPH.cpp:964-1059),
   kappa <- 0.5 max(kappa, -0.00025) / h^2 (where rho_adv > 1), with a per-particle MLP
   4 -> 64 -> 64 -> 1 (GELU, BF16 weights, FP32 accumulation; the hidden layer on the
   tensor cores). The Jacobi solve then runs to the same tolerance from that start.
   Features (float[4] per sample): rho_adv - 1 at the warm start, neighbour count,
   previous step's stiffness in pass units, |v|; target: the stiffness the solve
   accumulated in that step (pass units). Data pointers of the dfsph_mlp_* calls are
   DEVICE pointers (x: float[n][4], y: float[n], idx: int32[n]); the calls are synchronous
   with the host but not ordered against other streams: the caller finishes writing its
   buffers (synchronises its stream) before the call.
   Parameter vector (DFSPH_MLP_NPARAMS floats): W1[64][4], b1[64], W2[64][64] (row =
   output), b2[64], w3[64], b3. Normalisation (10 floats): feature means[4], feature
   standard deviations[4], target mean, target standard deviation. */
#define DFSPH_MLP_NPARAMS 4545
typedef struct dfsph_mlp dfsph_mlp;
int dfsph_mlp_create(int32_t device, uint64_t seed, dfsph_mlp **out);
int dfsph_mlp_destroy(dfsph_mlp *m);
int dfsph_mlp_get_params(dfsph_mlp *m, float *params, float *norm);
/* Either pointer may be NULL (left unchanged); new parameters reset the Adam state. */
int dfsph_mlp_set_params(dfsph_mlp *m, const float *params, const float *norm);
/* Sets the normalisation from the mean and standard deviation of n samples. */
int dfsph_mlp_fit_normalization(dfsph_mlp *m, const float *x, const float *y, int64_t n);
/* One Adam step (beta 0.9/0.999) on the mean squared error (normalised units) over the
   samples idx[0..n) of the n_samples rows of x and y (idx NULL: rows 0..n); *loss = that
   error before the step. An index outside [0, n_samples) is an error (the sample is not
   read). */
int dfsph_mlp_train_step(dfsph_mlp *m, const float *x, const float *y, int64_t n_samples, const int32_t *idx,
                         int64_t n, float lr, double *loss);
/* Gradient of that loss over samples 0..n (DFSPH_MLP_NPARAMS doubles, host) without
   updating the parameters. */
int dfsph_mlp_gradient(dfsph_mlp *m, const float *x, const float *y, int64_t n, double *grad, double *loss);
/* Predicted targets (denormalised) for n samples: x[n][4] -> y[n] (device pointers; the
   two ranges may not overlap). */
int dfsph_mlp_predict(dfsph_mlp *m, const float *x, float *y, int64_t n);
/* Failure-path test hook (no counterpart in the reference, whose CPU path has no device
   waits): the number of polls the first tensor-core wait of each inference CTA may take
   before it gives up (-1: the regular limit). With 0 that wait gives up while the product
   is still in flight; the kernel then sets its error bit, waits for the product with the
   regular limit, frees its tensor memory and returns, and the call (dfsph_mlp_predict, or
   the dfsph_step whose warm start used the model) returns DFSPH_ERR_DEVICE. A context takes
   the model's setting when dfsph_set_warmstart_model is called. */
int dfsph_mlp_set_wait_limit(dfsph_mlp *m, int32_t polls);
/* Use model m for the pressure warm start of ctx (NULL: the reference formula). The
   context keeps the pointer: detach before destroying the model. Needs
   use_pressure_warmstart. */
int dfsph_set_warmstart_model(dfsph_ctx *ctx, dfsph_mlp *m);
/* Recording of training samples: while on, each step keeps its warm-start features and
   final stiffness; dfsph_ml_capture copies the last step's samples with rho_adv > 1
   (at most `capacity`) to device buffers and returns how many it wrote. */
int dfsph_ml_record(dfsph_ctx *ctx, int32_t on);
int dfsph_ml_capture(dfsph_ctx *ctx, float *x, float *y, int64_t capacity, int64_t *count);

/* Allocation-free average density error, for callers that cannot allocate GPU memory
   where they need it (an embedding that gives its whole device budget to its own pool,
   or a real-time loop that forbids allocations after start-up). No counterpart in the
   reference. Computes mean(rho0 * rho_adv - rho0) (pressure_mode != 0) or
   mean(rho0 * rho_adv) (pressure_mode == 0) over n device values (float or double per
   fluid_precision) into *out (device pointer, one double), by a fixed-order FP64
   reduction (deterministic for a given input order; equal to the solver's own average up
   to FP64 rounding, since the solver sums in cell-sorted order), on `stream` (a
   cudaStream_t; NULL = default stream). Its only scratch is a static device array in the
   library: n is limited to 4,194,304; calls on one device share that array, so calls that
   overlap on the GPU race; the first call on each device resolves the array's address
   (make it before any stream capture). That address is kept for the life of the process:
   resetting a device's primary context (cudaDeviceReset) while the library is loaded is
   not supported by this entry point. */
int dfsph_density_error_noalloc(const void *rho_adv, int32_t fluid_precision, int64_t n, double density0,
                                int32_t pressure_mode, double *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* DFSPH_H */
