"""Scene JSON reader for the subset of the reference's scene format this library covers.

Rigid bodies whose "geometryFile" is an OBJ file that exists are sampled from the mesh
(difffr_gb300/mesh_sampling.py, regular triangle pattern at 1.5 r).

Keys follow SPlisHSPlasH/Utilities/SceneLoader.cpp:41-200 (see the Params docstring for
the Configuration keys). Fluid blocks are sampled as SimulatorBase::createFluidBlocks does
for mode 0 (SimulatorBase.cpp:1638-1720: lattice at 2r starting at min + 2r,
round(extent / 2r) - 1 points per axis). Rigid bodies need boundary samples: the reference
samples OBJ meshes; here a body is either
  - "particleFile": a .npy or .txt file of body-frame samples (n x 3), or
  - "geometryFile" naming an analytic shape: a file name containing "box" (the reference's
    UnitBox.obj, a unit cube centred at the origin, scaled by "scale"; "isWall": true
    samples its faces as a container) or "sphere" (unit-radius sphere scaled by "scale"),
    or "ellipsoid" (semi-axes = "scale"), sampled at spacing 2r.
Rotation: "rotationAxis" + "rotationAngle" (degrees), as the reference.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from . import scene as scn

CONFIG_KEYS = {
    "particleRadius": "particle_radius", "density0": "density0", "timeStepSize": "time_step",
    "maxIterations": "max_iterations", "minIterations": "min_iterations", "maxError": "max_error",
    "maxIterationsV": "max_iterations_v", "maxErrorV": "max_error_v",
    "enableDivergenceSolver": "enable_divergence_solver", "gradientMode": "gradient_mode",
    "useReleaseRigidBodyMode": "release_rigid_body_mode", "targetTime": "target_time",
    "uniformAccelerateRBTime": "uniform_accelerate_rb_time",
    "surfaceTensionMethod": "surface_tension_method", "surfaceTension": "surface_tension",
    "surfaceTensionBoundary": "surface_tension_boundary", "viscosity": "viscosity",
    "cflMethod": "cfl_method", "cflFactor": "cfl_factor", "cflMinTimeStepSize": "cfl_min_time_step",
    "cflMaxTimeStepSize": "cfl_max_time_step",
    "useRigidContactSolver": "use_rigid_contact_solver", "useRigidGradientManager": "use_rigid_gradient_manager",
    "rigidContactGamma": "rigid_contact_gamma", "rigidContactBeta": "rigid_contact_beta",
    "rigidContactSupportRadiusFactor": "rigid_contact_support_radius_factor",
    "rigidContactFrictionCoeff": "rigid_contact_friction_coeff", "viscosityBoundary": "viscosity_boundary",
}


def quat_from_axis_angle(axis, angle_deg):
    a = np.asarray(axis, dtype=np.float64)
    n = np.linalg.norm(a)
    if n == 0 or angle_deg == 0:
        return (1.0, 0.0, 0.0, 0.0)
    a = a / n
    h = 0.5 * math.radians(angle_deg)
    return (math.cos(h), *(math.sin(h) * a))


def _quat_matrix(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _body_samples(b, base_dir, r, seed=0):
    sp = 2.0 * r
    scale = np.asarray(b.get("scale", [1.0, 1.0, 1.0]), dtype=np.float64)
    pf = b.get("particleFile", "")
    if pf:
        path = pf if os.path.isabs(pf) else os.path.join(base_dir, pf)
        pts = np.load(path) if path.endswith(".npy") else np.loadtxt(path)
        return np.asarray(pts, dtype=np.float64).reshape(-1, 3) * scale[0]
    gf = b.get("geometryFile", "")
    gpath = gf if os.path.isabs(gf) else os.path.join(base_dir, gf)
    if gf.lower().endswith(".obj") and os.path.exists(gpath):
        from .mesh_sampling import sample_obj
        # "samplingMode" (SceneLoader.cpp:147-148): 0 Poisson disk (the default), 1 regular triangle
        return sample_obj(gpath, scale, r, mode=int(b.get("samplingMode", 0)), seed=seed)
    g = os.path.basename(gf).lower()
    if "box" in g:
        half = 0.5 * scale
        return scn.box_surface(-half, half, sp)
    if "ellipsoid" in g:
        return scn.ellipsoid_surface(*scale, sp)
    if "sphere" in g:
        return scn.sphere_surface(float(scale[0]), sp)
    raise ValueError(f"unsupported rigid body geometry {b.get('geometryFile')!r}: give a particleFile or a "
                     "box/sphere/ellipsoid geometry")


def load_scene(path_or_dict, precision=0, seed=0):
    if isinstance(path_or_dict, dict):
        data, base_dir = path_or_dict, os.getcwd()
    else:
        with open(path_or_dict) as f:
            data = json.load(f)
        base_dir = os.path.dirname(os.path.abspath(path_or_dict))
    if "synthetic" in data:
        name = data["synthetic"]
        fn = {"config0": scn.config0, "config1": scn.config1, "config2": scn.config2, "config4": scn.config4,
              "small_contact": scn.small_contact_scene}[name]
        return fn(seed=data.get("seed", seed), **data.get("overrides", {}))
    cfg = dict(data.get("Configuration", {}))
    # fluid material keys ("Materials" entries, SceneLoader.cpp) apply to the one fluid
    for mat in data.get("Materials", []):
        for k in ("surfaceTensionMethod", "surfaceTension", "surfaceTensionBoundary", "viscosity",
                  "viscosityBoundary"):
            if k in mat:
                cfg[k] = mat[k]
    kw = {}
    for k, v in CONFIG_KEYS.items():
        if k in cfg:
            kw[v] = type(getattr(scn.Params(), v))(cfg[k])
    if "gravitation" in cfg:
        kw["gravity"] = tuple(float(x) for x in cfg["gravitation"])
    kw["fluid_precision"] = precision
    params = scn.Params(**kw)
    r = params.particle_radius
    rng = np.random.default_rng(seed)
    fluid = []
    for fb in data.get("FluidBlocks", []):
        lo = np.asarray(fb["start"], dtype=np.float64)
        hi = np.asarray(fb["end"], dtype=np.float64)
        diam = 2.0 * r
        steps = [int(round((hi[c] - lo[c]) / diam)) - 1 for c in range(3)]
        pts = scn.fluid_lattice(steps, diam, lo + diam, r, rng, jitter=bool(fb.get("jitter", False)))
        fluid.append(pts)
    fvel = [np.zeros_like(b) for b in fluid]
    for fm in data.get("FluidModels", []):
        # particle files: the reference's readParticles (PartioReaderWriter.cpp) with the
        # model's scale, rotation and translation
        pf = fm.get("particleFile", "")
        path = pf if os.path.isabs(pf) else os.path.join(base_dir, pf)
        if path.endswith(".bgeo"):
            from .partio_bgeo import read_bgeo
            st = read_bgeo(path)
            pos = st["position"].astype(np.float64)
            vel = st["velocity"].astype(np.float64) if "velocity" in st else np.zeros_like(pos)
        else:
            pos = np.asarray(np.load(path) if path.endswith(".npy") else np.loadtxt(path), dtype=np.float64).reshape(-1, 3)
            vel = np.zeros_like(pos)
        sc_ = np.asarray(fm.get("scale", [1.0, 1.0, 1.0]), dtype=np.float64)
        q = quat_from_axis_angle(fm.get("rotationAxis", [1, 0, 0]), float(fm.get("rotationAngle", 0.0)))
        Rm = _quat_matrix(q)
        pos = (pos * sc_) @ Rm.T + np.asarray(fm.get("translation", [0, 0, 0]), dtype=np.float64)
        vel = vel @ Rm.T
        if "initialVelocity" in fm:
            vel = vel + np.asarray(fm["initialVelocity"], dtype=np.float64)
        fluid.append(pos)
        fvel.append(vel)
    fx = np.vstack(fluid) if fluid else np.zeros((0, 3))
    fv = np.vstack(fvel) if fluid else np.zeros((0, 3))
    bodies = []
    for k, b in enumerate(data.get("RigidBodies", [])):
        q = quat_from_axis_angle(b.get("rotationAxis", [1, 0, 0]), float(b.get("rotationAngle", 0.0)))
        bodies.append(scn.Body(
            samples=_body_samples(b, base_dir, r, seed=seed + 101 * k), translation=tuple(b.get("translation", [0, 0, 0])), rotation=q,
            density=float(b.get("density", 1000.0)), is_dynamic=bool(b.get("isDynamic", False)),
            is_animated=bool(b.get("isAnimated", False)), init_velocity=tuple(b.get("initVelocity", [0, 0, 0])),
            init_angular_velocity=tuple(b.get("initAngularVelocity", [0, 0, 0])),
            target_x=tuple(b.get("targetX", [0.8, 2.0, 0.0]))))
        bodies[-1].target_angle_in_degree = tuple(b.get("targetAngleInDegree", [0, 0, 0]))
    sc = scn.Scene(params=params, fluid_x=fx, fluid_v=fv, bodies=bodies,
                   name=os.path.basename(str(path_or_dict)))
    return sc
