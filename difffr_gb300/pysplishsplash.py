"""A `pysplishsplash`-compatible Python surface over libdfsph.

The reference exposes its simulator to the optimisation scripts through the pybind11
module `pysplishsplash` (pySPlisHSPlasH/main.cpp:47-76; DiffDFSPHModule.cpp:45-102,
BoundaryModelModule.cpp:43-91, SimulationModule.cpp:95-415). This module provides the
subset those scripts call, with the same names, argument meanings and return types
(numpy arrays for vectors and matrices), so that a script written as

    import difffr_gb300.pysplishsplash as sph
    base = sph.Exec.SimulatorBase()
    base.init(sceneFile=..., useGui=False, stopAt=...)
    base.initSimulation()
    sim = sph.Simulation.getCurrent()
    timestep = sim.getTimeStep()
    ...
    base.setTimeStepCB(callback)
    base.runSimulation()

drives the GPU implementation. Scenes come from the JSON subset read by
difffr_gb300.scene_json (or a difffr_gb300.scene.Scene passed as `scene=`). There is no
GUI: sph.GUI.Simulator_GUI_imgui is accepted and does nothing.
"""
from __future__ import annotations

import math
import os
import types

import numpy as np

from . import _abi
from .sim import DiffDFSPH

_state = {"base": None}


def _quat_mul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 + y1 * w2 + z1 * x2 - x1 * z2, w1 * z2 + z1 * w2 + x1 * y2 - y1 * x2])


def _axis_angle(axis, a):
    h = 0.5 * a
    v = np.zeros(3)
    v[axis] = math.sin(h)
    return np.array([math.cos(h), *v])


class TimeManager:
    """TimeManager::getCurrent()->getTime() / getTimeStepSize()."""

    @staticmethod
    def getCurrent():
        return TimeManager()

    def getTime(self):
        b = _state["base"]
        return b._sim.time()[0] if b and b._sim else 0.0

    def getTimeStepSize(self):
        b = _state["base"]
        return b._scene.params.time_step if b else 0.0


class RigidBodyObject:
    """Dynamic3dRigidBody accessors (SPlisHSPlasH/Dynamic3dRigidBody.h)."""

    def __init__(self, base, index):
        self._base, self._i = base, index

    def _st(self):
        return self._base._sim.rigid_state(self._i)

    def getPosition(self):
        return self._st()[0]

    def getRotation(self):
        return self._st()[1]

    def getVelocity(self):
        return self._st()[2]

    def getAngularVelocity(self):
        return self._st()[3]

    def setVelocity(self, v):
        x, q, _, w = self._st()
        self._base._sim.set_rigid_velocity(self._i, v, w)

    def setAngularVelocity(self, w):
        x, q, v, _ = self._st()
        self._base._sim.set_rigid_velocity(self._i, v, w)

    def getMass(self):
        return self._base._sim.rigid_mass(self._i)[0]

    def getInertiaTensorWorld(self):
        return self._base._sim.rigid_mass(self._i)[1]

    def isDynamic(self):
        return bool(self._base._scene.bodies[self._i].is_dynamic)

    def isAnimated(self):
        return bool(self._base._scene.bodies[self._i].is_animated)


class BoundaryModelAkinci2012:
    """BoundaryModel_Akinci2012 accessors (pySPlisHSPlasH/BoundaryModelModule.cpp:43-91)."""

    def __init__(self, base, index):
        self._base, self._i = base, index

    def _g(self):
        return self._base._sim.rigid_grad_blocks(self._i)

    def numberOfParticles(self):
        return int(self._base._scene.bodies[self._i].samples.shape[0])

    def getPointSetIndex(self):
        return 1 + self._i

    def get_position_rb(self):
        return self._base._sim.rigid_state(self._i)[0]

    def get_quaternion_rb_vec4(self):
        return self._base._sim.rigid_state(self._i)[1]

    def get_velocity_rb(self):
        return self._base._sim.rigid_state(self._i)[2]

    def get_angular_velocity_rb(self):
        return self._base._sim.rigid_state(self._i)[3]

    def set_velocity_rb(self, v):
        self.getRigidBodyObject().setVelocity(v)

    def set_angular_velocity_rb(self, w):
        self.getRigidBodyObject().setAngularVelocity(w)

    def get_grad_x_to_v0(self):
        return self._g()["x_v0"]

    def get_grad_x_to_omega0(self):
        return self._g()["x_w0"]

    def get_grad_quaternion_to_v0(self):
        return self._g()["q_v0"]

    def get_grad_quaternion_to_omega0(self):
        return self._g()["q_w0"]

    def get_grad_v_to_v0(self):
        return self._g()["v_v0"]

    def get_grad_v_to_omega0(self):
        return self._g()["v_w0"]

    def get_grad_omega_to_v0(self):
        return self._g()["w_v0"]

    def get_grad_omega_to_omega0(self):
        return self._g()["w_w0"]

    def getForce(self):
        return self._base._sim.rigid_force(self._i)[0]

    def getTorque(self):
        return self._base._sim.rigid_force(self._i)[1]

    def getRigidBodyObject(self):
        return RigidBodyObject(self._base, self._i)


def _split_nets(o):
    return {"Fv": o[0:9].reshape(3, 3), "Fx": o[9:18].reshape(3, 3), "Fw": o[18:27].reshape(3, 3),
            "Fq": o[27:39].reshape(3, 4), "Tw": o[39:48].reshape(3, 3), "Tv": o[48:57].reshape(3, 3),
            "Tx": o[57:66].reshape(3, 3), "Tq": o[66:78].reshape(3, 4)}


def _nets(base, R):
    return _split_nets(base._sim.net_jacobians(R))


class RigidBodyGradientManager:
    """RigidBodyGradientManager accessors (SimulationModule.cpp:406-415). With
    useRigidGradientManager the library runs the manager's own chain over body pairs
    (RigidBodyGradientManager.cpp:96-468), coupled through the rigid contact solver's blocks,
    and [R][RR] is that chain's state. Without it the manager is not stepped in the reference
    either; these accessors then return body R's own chain state on the diagonal and zero
    elsewhere."""

    def __init__(self, base):
        self._base = base

    def _blk(self, R, RR, key, shape):
        sim = self._base._sim
        if sim.uses_manager:
            return sim.manager_grad_blocks(R, RR)[key]
        if R != RR:
            return np.zeros(shape)
        return sim.rigid_grad_blocks(R)[key]

    def _jac(self, R, RR, key):
        sim = self._base._sim
        if sim.uses_manager:
            return _split_nets(sim.manager_jacobians(R, RR))[key]
        return _nets(self._base, R)[key] if R == RR else np.zeros((3, 4) if key in ("Fq", "Tq") else (3, 3))

    def get_grad_x_to_v0(self, R, RR):
        return self._blk(R, RR, "x_v0", (3, 3))

    def get_grad_x_to_omega0(self, R, RR):
        return self._blk(R, RR, "x_w0", (3, 3))

    def get_grad_q_to_v0(self, R, RR):
        return self._blk(R, RR, "q_v0", (4, 3))

    def get_grad_q_to_omega0(self, R, RR):
        return self._blk(R, RR, "q_w0", (4, 3))

    def get_grad_v_to_v0(self, R, RR):
        return self._blk(R, RR, "v_v0", (3, 3))

    def get_grad_v_to_omega0(self, R, RR):
        return self._blk(R, RR, "v_w0", (3, 3))

    def get_grad_omega_to_v0(self, R, RR):
        return self._blk(R, RR, "w_v0", (3, 3))

    def get_grad_omega_to_omega0(self, R, RR):
        return self._blk(R, RR, "w_w0", (3, 3))

    def get_grad_net_force_to_vn(self, R, RR):
        return self._jac(R, RR, "Fv")

    def get_grad_net_force_to_xn(self, R, RR):
        return self._jac(R, RR, "Fx")

    def get_grad_net_force_to_omega_n(self, R, RR):
        return self._jac(R, RR, "Fw")

    def get_grad_net_force_to_qn(self, R, RR):
        return self._jac(R, RR, "Fq")

    def get_grad_net_torque_to_vn(self, R, RR):
        return self._jac(R, RR, "Tv")

    def get_grad_net_torque_to_xn(self, R, RR):
        return self._jac(R, RR, "Tx")

    def get_grad_net_torque_to_omega_n(self, R, RR):
        return self._jac(R, RR, "Tw")

    def get_grad_net_torque_to_qn(self, R, RR):
        return self._jac(R, RR, "Tq")

    def reset(self):
        self._base._sim.reset_gradient()


class TimeStepDiffDFSPH:
    """TimeStepDiffDFSPH accessors (pySPlisHSPlasH/DiffDFSPHModule.cpp:45-102)."""

    def __init__(self, base):
        self._base = base
        self._loss = self._loss_x = self._loss_rot = 0.0
        self._lr = 1.0
        self._finished = False

    def get_boundary_model(self, i):
        return BoundaryModelAkinci2012(self._base, i)

    def set_init_v_rb(self, i, v):
        _, w = self._base._sim.rigid_init(i)
        self._base._sim.set_rigid_init(i, np.asarray(v, dtype=np.float64), w)

    def set_init_omega_rb(self, i, w):
        v, _ = self._base._sim.rigid_init(i)
        self._base._sim.set_rigid_init(i, v, np.asarray(w, dtype=np.float64))

    def get_init_v_rb(self, i):
        return self._base._sim.rigid_init(i)[0]

    def get_init_omega_rb(self, i):
        return self._base._sim.rigid_init(i)[1]

    def get_target_x(self, i):
        return np.asarray(self._base._scene.bodies[i].target_x, dtype=np.float64)

    def set_target_x(self, i, x):
        self._base._scene.bodies[i].target_x = tuple(float(v) for v in x)

    def get_target_angle_in_radian(self, i):
        a = getattr(self._base._scene.bodies[i], "target_angle_in_degree", (0.0, 0.0, 0.0))
        return np.radians(np.asarray(a, dtype=np.float64))

    def get_target_quaternion_vec4(self, i):
        """AngleAxis(a0, X) * AngleAxis(a1, Y) * AngleAxis(a2, Z) as (w, x, y, z)
        (SimulationDataDiffDFSPH.h:169-183)."""
        a = self.get_target_angle_in_radian(i)
        return _quat_mul(_quat_mul(_axis_angle(0, a[0]), _axis_angle(1, a[1])), _axis_angle(2, a[2]))

    def get_loss(self):
        return self._loss

    def set_loss(self, v):
        self._loss = float(v)

    def get_loss_x(self):
        return self._loss_x

    def set_loss_x(self, v):
        self._loss_x = float(v)

    def get_loss_rotation(self):
        return self._loss_rot

    def set_loss_rotation(self, v):
        self._loss_rot = float(v)

    def get_lr(self):
        return self._lr

    def set_lr(self, v):
        self._lr = float(v)

    def is_trajectory_finish_callback(self):
        return self._finished

    def clear_all_callbacks(self):
        self._finished = False

    def get_step_count(self):
        return self._base._sim.time()[1]

    def reset_gradient(self):
        self._base._sim.reset_gradient()

    def add_log(self, msg):
        print(msg, flush=True)

    def get_num_1ring_fluid_particle(self):
        """Fluid particles with at least one dynamic or animated boundary neighbour
        (TimeStepDiffDFSPH::countNeighborDOF, :283-350)."""
        sc = self._base._scene
        movable = np.zeros(sum(b.samples.shape[0] for b in sc.bodies), dtype=bool)
        o = 0
        for b in sc.bodies:
            n = b.samples.shape[0]
            movable[o:o + n] = b.is_dynamic or b.is_animated
            o += n
        start, idx = self._base._sim.neighbors(_abi.NB_FLUID_BOUNDARY)
        hit = movable[idx] if idx.size else np.zeros(0, dtype=bool)
        row = np.repeat(np.arange(len(start) - 1), np.diff(start))
        return int(np.unique(row[hit]).size)


class RigidContactSolver:
    """BoundarySimulator::getRigidContactSolver() (SimulationModule.cpp:383-397): the
    penalty-form contact solver runs inside each step; reset() has nothing to clear between
    trajectories beyond what SimulatorBase.reset() restores, and the last step's contact
    counts are exposed for inspection."""

    def __init__(self, base):
        self._base = base

    def reset(self):
        pass

    def num_contacts(self):
        return self._base._sim.contact_count()[0]


class _BoundarySimulator:
    def __init__(self, base):
        self._base = base

    def getRigidContactSolver(self):
        return RigidContactSolver(self._base) if self._base._scene.params.use_rigid_contact_solver else None


class Simulation:
    """Simulation::getCurrent() and the accessors the scripts use
    (SimulationModule.cpp:95-211)."""

    @staticmethod
    def getCurrent():
        b = _state["base"]
        if b is None or b._simulation is None:
            raise RuntimeError("no simulation: call SimulatorBase.init() and initSimulation() first")
        return b._simulation

    def __init__(self, base):
        self._base = base

    def getTimeStep(self):
        return self._base._timestep

    def getBoundaryModel(self, i):
        return BoundaryModelAkinci2012(self._base, i)

    def numberOfBoundaryModels(self):
        return len(self._base._scene.bodies)

    def numberOfFluidModels(self):
        return 1 if self._base._scene.n_fluid else 0

    def getGradientMode(self):
        return int(self._base._scene.params.gradient_mode)

    def setGradientMode(self, m):
        self._base._set_param(gradient_mode=int(m))

    def useRigidGradientManager(self):
        return bool(self._base._scene.params.use_rigid_gradient_manager)

    def useRigidContactSolver(self):
        return bool(self._base._scene.params.use_rigid_contact_solver)

    def getParticleRadius(self):
        return self._base._scene.params.particle_radius


class _SimulatorBase:
    """SimulatorBase (SimulationModule.cpp:237-362): scene set-up, the time-step loop with
    its per-step callback, reset, and in-memory state save/restore."""

    STATE_EXPORT, STATE_EXPORT_FPS, PAUSE, STOP_AT = "state_export", "state_export_fps", "pause", "stop_at"

    def __init__(self):
        self._scene = None
        self._sim = None
        self._simulation = None
        self._timestep = None
        self._cb = None
        self._stop_at = -1.0
        self._values = {}
        self._output = os.getcwd()
        self._stop = False
        self._saved = {}
        _state["base"] = self

    def init(self, sceneFile="", useGui=False, initialPause=False, useCache=True, stopAt=-1.0, stateFile="",
             loadFluidPos=False, loadFluidPosAndVel=False, outputDir="", param="", scene=None, precision=0):
        from .scene_json import load_scene
        self._scene = scene if scene is not None else load_scene(sceneFile, precision=precision)
        if stateFile and (loadFluidPos or loadFluidPosAndVel):
            # initial fluid from a saved state (SimulatorBase::init with loadFluidPos[AndVel]):
            # the state's particles replace the scene's fluid
            import dataclasses
            from .partio_bgeo import read_bgeo
            st = read_bgeo(stateFile)
            x = st["position"].astype(np.float64)
            v = st["velocity"].astype(np.float64) if (loadFluidPosAndVel and "velocity" in st) else np.zeros_like(x)
            self._scene = dataclasses.replace(self._scene, fluid_x=x, fluid_v=v)
        self._stop_at = float(stopAt)
        if outputDir:
            self._output = outputDir
        return True

    def setGui(self, gui):
        return None

    def initSimulation(self):
        self._create()

    def initSimulationWithDeferredInit(self):
        self._create()

    def _create(self):
        if self._sim is not None:
            self._sim.close()
        self._sim = DiffDFSPH(self._scene)
        self._simulation = Simulation(self)
        if self._timestep is None:
            self._timestep = TimeStepDiffDFSPH(self)
        self._timestep._base = self

    def _set_param(self, **kw):
        import dataclasses
        t, sc = self._sim.time() if self._sim else (0.0, 0)
        if sc != 0:
            raise RuntimeError("simulation parameters can only change before the first step or after reset()")
        inits = [self._sim.rigid_init(b) for b in range(self._sim.n_bodies)] if self._sim else None
        self._scene = dataclasses.replace(self._scene, params=dataclasses.replace(self._scene.params, **kw))
        self._create()
        if inits:
            for b, (v, w) in enumerate(inits):
                self._sim.set_rigid_init(b, v, w)

    def setTimeStepCB(self, cb):
        self._cb = cb

    def singleTimeStep(self):
        st = self._sim.step(1)
        self._timestep._finished = bool(st["trajectory_finished"])
        if self._cb:
            self._cb()
        return st

    def forwardFixedSteps(self, n):
        for _ in range(int(n)):
            self.singleTimeStep()

    def runSimulation(self, max_steps=None):
        """Steps until the stop-at time (if set), stop(), or max_steps."""
        self._stop = False
        k = 0
        while not self._stop:
            if self._stop_at > 0 and self._sim.time()[0] >= self._stop_at:
                break
            if max_steps is not None and k >= max_steps:
                break
            self.singleTimeStep()
            k += 1

    def runNewTrajectory(self):
        self.reset()
        while True:
            self.singleTimeStep()
            if self._timestep._finished:
                break

    def stop(self):
        self._stop = True

    def reset(self):
        self._sim.reset()
        self._timestep._finished = False

    def getRigidBodyGradientManager(self):
        return RigidBodyGradientManager(self)

    def getBoundarySimulator(self):
        return _BoundarySimulator(self)

    def getOutputPath(self):
        return self._output

    def setStateExportPath(self, p):
        self._values["state_export_path"] = p

    def setValueBool(self, key, v):
        self._values[key] = bool(v)

    def setValueFloat(self, key, v):
        self._values[key] = float(v)

    def setValueInt(self, key, v):
        self._values[key] = int(v)

    def getValueFloat(self, key):
        return self._values.get(key, 0.0)

    def _moving_bodies(self):
        return [k for k, b in enumerate(self._scene.bodies) if b.is_dynamic or b.is_animated]

    def saveState(self, path=""):
        """Snapshot of the full state kept on the device; returns a handle string usable
        with loadStateWithRigidExisted. When `path` is given, the reference's state-export
        files are written there too (SimulatorBase::saveState): the fluid particles
        (position, velocity, kappa, kappa_v, id) as state_<n>_particle_Fluid.bgeo and the
        dynamic and animated bodies' records as state_<n>_dynamicRB.bin, n the step count."""
        from . import _abi
        slot = self._sim.checkpoint_save()
        name = os.path.join(path or self._output, f"state_{slot}")
        self._saved[name] = slot
        self._saved[name + ".bin"] = slot
        if path:
            from .partio_bgeo import write_bgeo
            from .state_bin import write_dynamic_rb
            os.makedirs(path, exist_ok=True)
            prefix = os.path.join(path, f"state_{self._sim.time()[1]}")
            fn = prefix + "_particle_Fluid.bgeo"
            write_bgeo(fn, self._sim.field(_abi.FIELD_X), velocity=self._sim.field(_abi.FIELD_V),
                       kappa=self._sim.field(_abi.FIELD_KAPPA), kappa_v=self._sim.field(_abi.FIELD_KAPPA_V),
                       id=np.arange(self._sim.n_fluid, dtype=np.int32))
            real = np.float64 if self._scene.params.fluid_precision == _abi.DFSPH_FP64 else np.float32
            write_dynamic_rb(prefix + "_dynamicRB.bin", [self._sim.rigid_state(b) for b in self._moving_bodies()],
                             real=real)
        return name

    def loadStateWithRigidExisted(self, name):
        """Restores a state saved in this session. From files: a state .bin (the reference's
        state_<n>.bin or state_<n>_dynamicRB.bin) sets the dynamic and animated bodies' pose
        and velocities from its rigid records and the fluid from the state_<n>_particle_Fluid.bgeo
        beside it when present; a .bgeo file sets the fluid's positions and velocities (and
        kappa fields when present) and keeps the rigid bodies."""
        from . import _abi
        if name in self._saved:
            self._sim.checkpoint_restore(self._saved[name])
            return
        if name.endswith(".bin"):
            from .state_bin import read_rigid_records
            moving = self._moving_bodies()
            recs, _ = read_rigid_records(name, len(moving))
            for b, (x, q, v, w) in zip(moving, recs):
                self._sim.set_rigid_state(b, x, q, v, w)
            stem = name[:-4]
            if stem.endswith("_dynamicRB"):
                stem = stem[: -len("_dynamicRB")]
            fluid = stem + "_particle_Fluid.bgeo"
            if os.path.exists(fluid):
                self.loadStateWithRigidExisted(fluid)
            return
        from .partio_bgeo import read_bgeo
        st = read_bgeo(name)
        if st["position"].shape[0] != self._sim.n_fluid:
            raise ValueError(f"{name}: {st['position'].shape[0]} particles, the simulation has {self._sim.n_fluid}")
        self._sim.set_field(_abi.FIELD_X, st["position"].astype(np.float64))
        if "velocity" in st:
            self._sim.set_field(_abi.FIELD_V, st["velocity"].astype(np.float64))
        for key, fid in (("kappa", _abi.FIELD_KAPPA), ("kappa_v", _abi.FIELD_KAPPA_V)):
            if key in st:
                self._sim.set_field(fid, st[key].astype(np.float64).ravel())

    def cleanup(self):
        if self._sim is not None:
            self._sim.close()
            self._sim = None


Exec = types.SimpleNamespace(SimulatorBase=_SimulatorBase)


class _NoGui:
    def __init__(self, base=None):
        pass


GUI = types.SimpleNamespace(Simulator_GUI_imgui=_NoGui)


class _Timing:
    """Utilities.Timing (Utilities/Timing.h, bound in pySPlisHSPlasH/UtilitiesModule.cpp):
    the reference prints its CPU timers' sums and averages; the GPU path's per-kernel device
    times come from DiffDFSPH.profile(), so these print a short note instead."""

    @staticmethod
    def printAverageTimes():
        print("timing: per-kernel device times are available from DiffDFSPH.profile()")

    @staticmethod
    def printTimeSums():
        print("timing: per-kernel device times are available from DiffDFSPH.profile()")


Utilities = types.SimpleNamespace(Timing=_Timing)
