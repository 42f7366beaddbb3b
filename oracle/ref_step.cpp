// ref_step.cpp — runs the reference's own DiffDFSPH time step on a scene read from a file
// and writes what each step produced. Test infrastructure only: built by
// oracle/build_ref_step.sh from the reference's sources (TimeStepDiffDFSPH.cpp,
// BoundaryModel_Akinci2012.cpp, Simulation.cpp, ...) against the stand-ins for its three
// fetched dependencies in oracle/refshim/, and run by tests/golden/make_ref_step_golden.py
// to make the fixtures the CPU oracle is pinned to.
//
// The reference's arithmetic all stays in its own code. This file only does what the
// reference's simulator shell does around it, in the same order, with the reference's own
// classes and methods:
//   - set-up as SimulatorBase::initSimulation, buildModel, readParameters and deferredInit
//     do (Simulator/SimulatorBase.cpp:494-647,860-885,1321-1508) and
//     RigidBody3dBoundarySimulator::initBoundaryData / deferredInit
//     (Simulator/RigidBody3dBoundarySimulator.cpp:68-270) for bodies given as body-frame
//     samples: Dynamic3dRigidBody, determineMassProperties, BoundaryModel_Akinci2012::initModel,
//     updateBoundaryParticles(true), Simulation::updateBoundaryVolume;
//   - each step as SimulatorBase::timeStep (SimulatorBase.cpp:969-1016): the method's
//     step() (which runs beginStep, the solves, the chain rule and endStep), then
//     RigidBody3dBoundarySimulator::velocityTimeStep (BoundarySimulator::updateBoundaryForces,
//     BoundarySimulator.cpp:10-35, then gravity) and positionTimeStep (animate, then
//     SimulatorBase::updateBoundaryParticles, SimulatorBase.cpp:1827-1857).
// Simulation::registerNonpressureForces (NonPressureForceRegistration.cpp) is defined here
// with the viscosity models at their reference positions (0 None, 1 Standard, 2 XSPH); only
// XSPH is built, and Standard, which FluidModel::init selects before the scene's choice, is
// created as no model.
//
// Input (all values float64, little-endian; counts stored as float64):
//   version (=1), r, dt, rho0, viscosity, g[3], max_error, max_error_v, min_iterations,
//   max_iterations, max_iterations_v, gradient_mode, enable_divergence_solver,
//   use_pressure_warmstart, use_divergence_warmstart, release_rigid_body_mode,
//   uniform_accelerate_rb_time, target_time, optimize_rotation, steps, n_fluid, n_bodies,
//   x[n][3], v[n][3], then per body: dynamic, animated, density, translation[3],
//   q[4] (w x y z), init_v[3], init_omega[3], n_samples, samples[n_samples][3] (body frame).
// Output (float64): per step: pressure sweeps, divergence sweeps, then per body x[3],
//   q[4] (w x y z), v[3], omega[3], the step's fluid force[3] and torque[3], and the chain
//   state (78 numbers: dx/dv0, dx/domega0, dq/dv0, dq/domega0, dv/dv0, dv/domega0,
//   domega/dv0, domega/domega0, row-major); after the last step, per fluid particle
//   x[3], v[3], density, factor, kappa, kappa_v, advected density, sum_grad_p_k[3], and per
//   boundary sample its volume psi.
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "SPlisHSPlasH/BoundaryModel_Akinci2012.h"
#include "SPlisHSPlasH/DiffDFSPH/TimeStepDiffDFSPH.h"
#include "SPlisHSPlasH/Dynamic3dRigidBody.h"
#include "SPlisHSPlasH/FluidModel.h"
#include "SPlisHSPlasH/Simulation.h"
#include "SPlisHSPlasH/TimeManager.h"
#include "SPlisHSPlasH/Viscosity/ViscosityBase.h"
#include "SPlisHSPlasH/Viscosity/Viscosity_XSPH.h"
#include "Simulator/SceneConfiguration.h"
#include "Utilities/Counting.h"
#include "Utilities/Logger.h"
#include "Utilities/Timing.h"

INIT_TIMING
INIT_LOGGING
INIT_COUNTING

using namespace SPH;

void Simulation::registerNonpressureForces() {
  auto none = [](FluidModel *) -> NonPressureForceBase * { return nullptr; };
  addDragMethod("None", none);
  addElasticityMethod("None", none);
  addSurfaceTensionMethod("None", none);
  addViscosityMethod("None", none);
  addViscosityMethod("Standard", none);
  addViscosityMethod("XSPH", Viscosity_XSPH::creator);
  addVorticityMethod("None", none);
}

namespace {

bool g_trace = false;
void trace(const char *m) {
  if (g_trace) fprintf(stderr, "ref_step: %s\n", m);
}

// Read access to the method's per-particle solver fields (protected in the reference).
struct DataAccess : TimeStepDiffDFSPH {
  static SimulationDataDiffDFSPH &of(TimeStepDiffDFSPH *t) { return t->*(&DataAccess::m_simulationData); }
};

struct In {
  std::vector<double> d;
  size_t k = 0;
  double next() {
    if (k >= d.size()) throw std::runtime_error("input too short");
    return d[k++];
  }
  Vector3r v3() {
    const double a = next(), b = next(), c = next();
    return Vector3r((Real)a, (Real)b, (Real)c);
  }
};

struct Out {
  FILE *f;
  void put(double x) { fwrite(&x, sizeof(double), 1, f); }
  void put3(const Vector3r &v) { for (int c = 0; c < 3; c++) put((double)v[c]); }
  template <class M> void putm(const M &m) {
    for (int r = 0; r < (int)m.rows(); r++)
      for (int c = 0; c < (int)m.cols(); c++) put((double)m(r, c));
  }
};

// SimulatorBase::updateBoundaryParticles (SimulatorBase.cpp:1827-1857)
void update_boundary_particles(bool force) {
  Simulation *sim = Simulation::getCurrent();
  for (unsigned int i = 0; i < sim->numberOfBoundaryModels(); i++) {
    auto *bm = static_cast<BoundaryModel_Akinci2012 *>(sim->getBoundaryModel(i));
    RigidBodyObject *rbo = bm->getRigidBodyObject();
    if (!(rbo->isDynamic() || rbo->isAnimated() || force)) continue;
    for (int j = 0; j < (int)bm->numberOfParticles(); j++) {
      bm->getPosition(j) = rbo->getRotation() * bm->getPosition0(j) + rbo->getPosition();
      if (rbo->isDynamic() || rbo->isAnimated())
        bm->getVelocity(j) = rbo->getAngularVelocity().cross(bm->getPosition(j) - rbo->getPosition()) + rbo->getVelocity();
      else
        bm->getVelocity(j).setZero();
    }
  }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s scene.bin out.bin\n", argv[0]);
    return 2;
  }
  g_trace = getenv("REF_STEP_TRACE") != nullptr;
  In in;
  {
    FILE *f = fopen(argv[1], "rb");
    if (!f) { perror(argv[1]); return 2; }
    double x;
    while (fread(&x, sizeof(double), 1, f) == 1) in.d.push_back(x);
    fclose(f);
  }
  if ((int)in.next() != 1) { fprintf(stderr, "input version\n"); return 2; }
  const Real r = (Real)in.next(), dt = (Real)in.next(), rho0 = (Real)in.next(), visc = (Real)in.next();
  Vector3r g = in.v3();
  const Real maxError = (Real)in.next(), maxErrorV = (Real)in.next();
  const unsigned int minIt = (unsigned int)in.next(), maxIt = (unsigned int)in.next(), maxItV = (unsigned int)in.next();
  const int gradMode = (int)in.next();
  const bool enableDiv = in.next() != 0, usePW = in.next() != 0, useDW = in.next() != 0, release = in.next() != 0;
  const Real uat = (Real)in.next(), targetTime = (Real)in.next();
  const bool optRot = in.next() != 0;
  const int steps = (int)in.next();
  const size_t n = (size_t)in.next();
  const int nb = (int)in.next();
  std::vector<Vector3r> fx(n), fv(n);
  for (size_t i = 0; i < n; i++) fx[i] = in.v3();
  for (size_t i = 0; i < n; i++) fv[i] = in.v3();

  // the bodies as the scene loader would hold them (SceneLoader.h:29-57); the simulation's
  // and the method's constructors read these (Simulation.cpp:113-126,
  // SimulationDataDiffDFSPH.cpp:14-60)
  struct BodyIn {
    bool dyn, anim;
    Real density;
    Vector3r t, v0, w0;
    Quaternionr q;
    std::vector<Vector3r> samples;
  };
  std::vector<BodyIn> bodies(nb);
  for (int b = 0; b < nb; b++) {
    BodyIn &B = bodies[b];
    B.dyn = in.next() != 0;
    B.anim = in.next() != 0;
    B.density = (Real)in.next();
    B.t = in.v3();
    const double qw = in.next(), qx = in.next(), qy = in.next(), qz = in.next();
    B.q = Quaternionr((Real)qw, (Real)qx, (Real)qy, (Real)qz);
    B.v0 = in.v3();
    B.w0 = in.v3();
    B.samples.resize((size_t)in.next());
    for (auto &p : B.samples) p = in.v3();
  }
  trace("input read");
  Utilities::SceneLoader::Scene &scene = SceneConfiguration::getCurrent()->getScene();
  scene.particleRadius = r;
  scene.sim2D = false;
  scene.timeStepSize = dt;
  scene.useRigidContactSolver = false;
  scene.useRigidGradientManager = false;
  scene.useReleaseRigidBodyMode = release;
  scene.rigidContactGamma = 0.7;
  scene.rigidContactFrictionCoeff = 0;
  scene.rigidContactBeta = 1;
  scene.rigidContactSupportRadiusFactor = 4;
  scene.targetTime = targetTime;
  scene.uniformAccelerateRBTime = uat;
  scene.gradientMode = (unsigned int)gradMode;
  for (int b = 0; b < nb; b++) {
    auto *bd = new Utilities::SceneLoader::BoundaryData();
    bd->translation = bodies[b].t;
    bd->rotation = bodies[b].q.toRotationMatrix();
    bd->scale = Vector3r(1, 1, 1);
    bd->density = bodies[b].density;
    bd->dynamic = bodies[b].dyn;
    bd->isWall = false;
    bd->isAnimated = bodies[b].anim;
    bd->samplingMode = 0;
    bd->target_x.setZero();
    bd->target_angle_in_degree.setZero();
    bd->init_velocity = bodies[b].v0;
    bd->init_angular_velocity = bodies[b].w0;
    scene.boundaryModels.push_back(bd);
  }

  // SimulatorBase::initSimulation: Simulation::init, then buildModel (SimulatorBase.cpp:860-885)
  TimeManager::getCurrent()->setTimeStepSize(dt);
  Simulation *sim = Simulation::getCurrent();
  sim->init(r, false);
  std::vector<unsigned int> ids(n, 0);
  trace("simulation initialised");
  sim->addFluidModel("Fluid", (unsigned int)n, fx.data(), fv.data(), ids.data(), 0);
  sim->setValue(Simulation::KERNEL_METHOD, Simulation::ENUM_KERNEL_PRECOMPUTED_CUBIC);
  sim->setValue(Simulation::GRAD_KERNEL_METHOD, Simulation::ENUM_GRADKERNEL_PRECOMPUTED_CUBIC);
  // readParameters: the scene's "Configuration" into the simulation, then into the method
  sim->setValue<int>(Simulation::SIMULATION_METHOD, 5);  // DiffDFSPH (Simulation.h:171)
  sim->setValue<int>(Simulation::CFL_METHOD, 0);
  sim->setValue<bool>(Simulation::ENABLE_Z_SORT, false);
  sim->setValue<int>(Simulation::BOUNDARY_HANDLING_METHOD, 0);  // Akinci2012
  sim->setValue<int>(Simulation::GRADIENT_MODE, gradMode);
  sim->setValue<int>(Simulation::RIGIDBODY_MODE, 0);  // gyroscopic
  sim->setValue<bool>(Simulation::IS_RELEASE_RIGID_BODY_MODE, release);
  sim->setVecValue<Real>(Simulation::GRAVITATION, g.data());
  trace("simulation parameters set");
  auto *ts = static_cast<TimeStepDiffDFSPH *>(sim->getTimeStep());
  ts->setValue<Real>(TimeStep::MAX_ERROR, maxError);
  ts->setValue<unsigned int>(TimeStep::MIN_ITERATIONS, minIt);
  ts->setValue<unsigned int>(TimeStep::MAX_ITERATIONS, maxIt);
  ts->setValue<Real>(TimeStepDiffDFSPH::MAX_ERROR_V, maxErrorV);
  ts->setValue<unsigned int>(TimeStepDiffDFSPH::MAX_ITERATIONS_V, maxItV);
  ts->setValue<bool>(TimeStepDiffDFSPH::USE_DIVERGENCE_SOLVER, enableDiv);
  ts->setValue<bool>(TimeStepDiffDFSPH::USE_PRESSURE_WARMSTART, usePW);
  ts->setValue<bool>(TimeStepDiffDFSPH::USE_DIV_WARMSTART, useDW);
  ts->setValue<bool>(TimeStepDiffDFSPH::OPTIMIZE_ROTATION, optRot);
  ts->setValue<Real>(TimeStepDiffDFSPH::UNIFORM_ACC_RB_TIME, uat);
  ts->setValue<Real>(TimeStepDiffDFSPH::TARGET_TIME, targetTime);
  // the fluid's material: density0 and XSPH viscosity (viscosityMethod 2)
  FluidModel *fm = sim->getFluidModel(0);
  fm->setValue<Real>(FluidModel::DENSITY0, rho0);
  fm->setValue<int>(FluidModel::VISCOSITY_METHOD, 2);
  fm->getViscosityBase()->setValue<Real>(ViscosityBase::VISCOSITY_COEFFICIENT, visc);

  trace("method parameters set");
  // deferredInit: RigidBody3dBoundarySimulator::initBoundaryData for sampled bodies
  std::vector<Vector3r> initV(nb), initW(nb);
  for (int b = 0; b < nb; b++) {
    BodyIn &B = bodies[b];
    initV[b] = B.v0;
    initW[b] = B.w0;
    Dynamic3dRigidBody *rb = new Dynamic3dRigidBody();
    rb->setIsAnimated(B.anim);
    rb->setIsDynamic(B.dyn);
    rb->setPosition0(B.t);
    rb->setPosition(B.t);
    rb->setRotation0(B.q);
    rb->setRotation(B.q);
    rb->determineMassProperties(B.density, r, B.samples);
    BoundaryModel_Akinci2012 *bm = new BoundaryModel_Akinci2012();
    bm->initModel(rb, (unsigned int)B.samples.size(), B.samples.data());
    sim->addBoundaryModel(bm);
    rb->updateMeshTransformation();
  }
  trace("bodies created");
  sim->setSimulationInitialized(true);
  // RigidBody3dBoundarySimulator::deferredInit (z-sort off)
  update_boundary_particles(true);
  sim->updateBoundaryVolume();
  for (int b = 0; b < nb; b++) {
    ts->set_init_v_rb(b, initV[b]);
    ts->set_init_omega_rb(b, initW[b]);
  }

  FILE *of = fopen(argv[2], "wb");
  if (!of) { perror(argv[2]); return 2; }
  Out out{of};
  trace("boundary volumes computed");
  for (int s = 0; s < steps; s++) {
    ts->step();
    trace("method step done");
    const unsigned int ip = ts->getValue<unsigned int>(TimeStep::SOLVER_ITERATIONS);
    const unsigned int iv = ts->getValue<unsigned int>(TimeStepDiffDFSPH::SOLVER_ITERATIONS_V);
    // RigidBody3dBoundarySimulator::velocityTimeStep without the contact solver:
    // BoundarySimulator::updateBoundaryForces, then gravity
    std::vector<Vector3r> F(nb, Vector3r::Zero()), T(nb, Vector3r::Zero());
    for (int b = 0; b < nb; b++) {
      BoundaryModel *bm = sim->getBoundaryModel(b);
      RigidBodyObject *rbo = bm->getRigidBodyObject();
      if (rbo->isDynamic()) {
        bm->getForceAndTorque(F[b], T[b]);
        if (!rbo->isAnimated()) {
          rbo->addForce(F[b]);
          rbo->addTorque(T[b]);
        }
        bm->clearForceAndTorque();
      }
    }
    for (int b = 0; b < nb; b++) {
      RigidBodyObject *rbo = sim->getBoundaryModel(b)->getRigidBodyObject();
      auto *d3 = dynamic_cast<Dynamic3dRigidBody *>(rbo);
      if (d3 && rbo->isDynamic() && !rbo->isAnimated()) d3->addGravity();
    }
    // positionTimeStep
    for (int b = 0; b < nb; b++) {
      RigidBodyObject *rbo = sim->getBoundaryModel(b)->getRigidBodyObject();
      auto *d3 = dynamic_cast<Dynamic3dRigidBody *>(rbo);
      if (d3 && rbo->isDynamic()) d3->animate();
    }
    update_boundary_particles(false);

    out.put(ip);
    out.put(iv);
    for (int b = 0; b < nb; b++) {
      auto *bm = static_cast<BoundaryModel_Akinci2012 *>(sim->getBoundaryModel(b));
      RigidBodyObject *rbo = bm->getRigidBodyObject();
      out.put3(rbo->getPosition());
      const Quaternionr q = rbo->getRotation();
      out.put(q.w()); out.put(q.x()); out.put(q.y()); out.put(q.z());
      out.put3(rbo->getVelocity());
      out.put3(rbo->getAngularVelocity());
      out.put3(F[b]);
      out.put3(T[b]);
      out.putm(bm->get_grad_x_to_v0());
      out.putm(bm->get_grad_x_to_omega0());
      out.putm(bm->get_grad_quaternion_to_v0());
      out.putm(bm->get_grad_quaternion_to_omega0());
      out.putm(bm->get_grad_v_to_v0());
      out.putm(bm->get_grad_v_to_omega0());
      out.putm(bm->get_grad_omega_to_v0());
      out.putm(bm->get_grad_omega_to_omega0());
    }
  }
  SimulationDataDiffDFSPH &sd = DataAccess::of(ts);
  for (size_t i = 0; i < n; i++) {
    out.put3(fm->getPosition((unsigned int)i));
    out.put3(fm->getVelocity((unsigned int)i));
    out.put(fm->getDensity((unsigned int)i));
    out.put(sd.getFactor(0, (unsigned int)i));
    out.put(sd.getKappa(0, (unsigned int)i));
    out.put(sd.getKappaV(0, (unsigned int)i));
    out.put(sd.getDensityAdv(0, (unsigned int)i));
    out.put3(sd.get_sum_grad_p_k(0, (unsigned int)i));
  }
  for (int b = 0; b < nb; b++) {
    auto *bm = static_cast<BoundaryModel_Akinci2012 *>(sim->getBoundaryModel(b));
    for (unsigned int j = 0; j < bm->numberOfParticles(); j++) out.put(bm->getVolume(j));
  }
  fclose(of);
  return 0;
}
