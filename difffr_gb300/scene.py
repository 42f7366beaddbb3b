"""Scene description and seeded synthetic scenes.

A scene is what the reference reads from its JSON "Configuration", "FluidBlocks" and
"RigidBodies" sections (SPlisHSPlasH/Utilities/SceneLoader.cpp:41-200) after sampling:
fluid particle positions and velocities, and per rigid body its boundary samples in
the body frame, pose, density and initial velocities.

The synthetic scenes stand in for the reference's OBJ-mesh scenes. Fluid blocks are
cubic lattices at spacing 2r starting one spacing inside the container, as
SimulatorBase::createFluidBlocks does (Simulator/SimulatorBase.cpp:1638-1720), with a
seeded per-axis jitter U(-0.01 r, 0.01 r). Containers are single-layer grids of
boundary samples at spacing 2r; spheres and ellipsoids are Fibonacci-lattice surface
samples with one sample per (2r)^2 of area.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import _abi


@dataclass
class Params:
    """dfsph_params (include/dfsph.h) with the reference's defaults."""
    fluid_precision: int = _abi.DFSPH_FP32
    particle_radius: float = 0.025
    density0: float = 1000.0
    viscosity: float = 0.01
    gravity: tuple = (0.0, -9.81, 0.0)
    time_step: float = 0.001
    min_iterations: int = 2
    max_iterations: int = 100
    max_error: float = 0.01
    max_iterations_v: int = 100
    max_error_v: float = 0.1
    enable_divergence_solver: int = 1
    use_pressure_warmstart: int = 1
    use_divergence_warmstart: int = 1
    gradient_mode: int = _abi.GRAD_INCOMPLETE
    rigid_body_mode: int = _abi.RB_GYROSCOPIC
    optimize_rotation: int = 1
    enable_gradient: int = 1
    truncate_gradient_coeff: int = 1
    release_rigid_body_mode: int = 0
    uniform_accelerate_rb_time: float = 0.0
    target_time: float = 0.8
    max_fluid_neighbors: int = 0
    max_boundary_neighbors: int = 0
    surface_tension_method: int = 0
    surface_tension: float = 0.05
    surface_tension_boundary: float = 0.01
    cfl_method: int = 0
    cfl_factor: float = 0.5
    cfl_min_time_step: float = 0.0001
    cfl_max_time_step: float = 0.005
    use_rigid_contact_solver: int = 0
    use_rigid_gradient_manager: int = 0
    rigid_contact_gamma: float = 0.7
    rigid_contact_beta: float = 1.0
    rigid_contact_support_radius_factor: float = 4.0
    rigid_contact_friction_coeff: float = 0.0
    viscosity_boundary: float = 0.0


@dataclass
class Body:
    samples: np.ndarray
    translation: tuple = (0.0, 0.0, 0.0)
    rotation: tuple = (1.0, 0.0, 0.0, 0.0)
    density: float = 1000.0
    is_dynamic: bool = False
    is_animated: bool = False
    init_velocity: tuple = (0.0, 0.0, 0.0)
    init_angular_velocity: tuple = (0.0, 0.0, 0.0)
    target_x: tuple = (0.0, 0.0, 0.0)


@dataclass
class Scene:
    params: Params
    fluid_x: np.ndarray
    fluid_v: np.ndarray
    bodies: List[Body] = field(default_factory=list)
    name: str = "scene"
    steps: int = 1

    @property
    def n_fluid(self):
        return int(self.fluid_x.shape[0])

    @property
    def n_boundary(self):
        return int(sum(b.samples.shape[0] for b in self.bodies))

    def n_dynamic_boundary(self):
        return int(sum(b.samples.shape[0] for b in self.bodies if b.is_dynamic))

    def replace_params(self, **kw):
        return dataclasses.replace(self, params=dataclasses.replace(self.params, **kw))


# ----------------------------------------------------------------------------- samplers

def fluid_lattice(counts, spacing, origin, r, rng, jitter=True):
    """Cubic lattice of counts[0] x counts[1] x counts[2] points at `spacing` from `origin`,
    jittered per axis by U(-0.01 r, 0.01 r)."""
    nx, ny, nz = counts
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pts = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64) * spacing
    pts += np.asarray(origin, dtype=np.float64)
    if jitter:
        pts += rng.uniform(-0.01 * r, 0.01 * r, size=pts.shape)
    return pts


def box_surface(lo, hi, spacing, open_top=False, up_axis=1):
    """Grid samples on the faces of an axis-aligned box, spacing close to `spacing`."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    n = np.maximum(np.round((hi - lo) / spacing).astype(int), 1)
    axes = [np.linspace(lo[c], hi[c], n[c] + 1) for c in range(3)]
    ii, jj, kk = np.meshgrid(np.arange(n[0] + 1), np.arange(n[1] + 1), np.arange(n[2] + 1), indexing="ij")
    idx = [ii, jj, kk]
    on = np.zeros(ii.shape, dtype=bool)
    for c in range(3):
        on |= (idx[c] == 0) | (idx[c] == n[c])
    if open_top:
        top = idx[up_axis] == n[up_axis]
        side = np.zeros(ii.shape, dtype=bool)
        for c in range(3):
            if c != up_axis:
                side |= (idx[c] == 0) | (idx[c] == n[c])
        on &= ~(top & ~side)
    pts = np.stack([axes[0][ii[on]], axes[1][jj[on]], axes[2][kk[on]]], axis=1)
    return pts


def fibonacci_sphere(n):
    k = np.arange(n, dtype=np.float64) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / n)
    theta = math.pi * (1.0 + 5.0 ** 0.5) * k
    return np.stack([np.cos(theta) * np.sin(phi), np.cos(phi), np.sin(theta) * np.sin(phi)], axis=1)


def sphere_surface(radius, spacing):
    n = max(int(round(4.0 * math.pi * radius * radius / (spacing * spacing))), 4)
    return radius * fibonacci_sphere(n)


def ellipsoid_surface(a, b, c, spacing):
    p = 1.6075  # Knud Thomsen's surface-area approximation
    area = 4.0 * math.pi * (((a * b) ** p + (a * c) ** p + (b * c) ** p) / 3.0) ** (1.0 / p)
    n = max(int(round(area / (spacing * spacing))), 4)
    return fibonacci_sphere(n) * np.array([a, b, c])


def quat_random(rng):
    q = rng.normal(size=4)
    return tuple(q / np.linalg.norm(q))


# ----------------------------------------------------------------------------- scenes

def tank_sphere(n=(20, 20, 20), r=0.025, box=None, sphere_radius=0.1, sphere_density=500.0,
                drop_gap=0.3, sphere_v=(0.5, 0.0, 0.0), sphere_w=(0.0, 1.0, 0.0), dt=0.001,
                seed=0, fluid_origin=None, sphere_xz=None, precision=_abi.DFSPH_FP32, steps=200,
                open_top=False, **param_kw):
    """Fluid lattice in a closed box with one dynamic sphere released `drop_gap` above
    the fluid surface (gap measured from the top fluid layer to the sphere's lowest point)."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * r
    if fluid_origin is None:
        fluid_origin = (sp, sp, sp)
    fx = fluid_lattice(n, sp, fluid_origin, r, rng)
    top = fluid_origin[1] + (n[1] - 1) * sp
    if box is None:
        box = (fluid_origin[0] + n[0] * sp, top + drop_gap + 2 * sphere_radius + 2 * sp,
               fluid_origin[2] + n[2] * sp)
    walls = box_surface((0.0, 0.0, 0.0), box, sp, open_top=open_top)
    if sphere_xz is None:
        sphere_xz = (fluid_origin[0] + 0.5 * (n[0] - 1) * sp, fluid_origin[2] + 0.5 * (n[2] - 1) * sp)
    center = (sphere_xz[0], top + drop_gap + sphere_radius, sphere_xz[1])
    # no fluid inside (or touching) the body's volume
    fx = fx[np.linalg.norm(fx - np.asarray(center), axis=1) > sphere_radius + r]
    bodies = [
        Body(samples=walls, density=1000.0, is_dynamic=False),
        Body(samples=sphere_surface(sphere_radius, sp), translation=center, density=sphere_density,
             is_dynamic=True, init_velocity=tuple(sphere_v), init_angular_velocity=tuple(sphere_w),
             target_x=center),
    ]
    params = Params(fluid_precision=precision, particle_radius=r, time_step=dt, **param_kw)
    return Scene(params=params, fluid_x=fx, fluid_v=np.zeros_like(fx), bodies=bodies,
                 name=f"tank_sphere_{fx.shape[0]}", steps=steps)


def config0(precision=_abi.DFSPH_FP64, seed=0, **kw):
    """8,000-particle lattice (r = 0.025) in a closed box with a dynamic sphere (R 0.1,
    density 500) released 0.3 m above the fluid with v = (0.5, 0, 0), omega = (0, 1, 0);
    dt 1 ms, 200 steps. The stated closed 1 m box cannot hold a 1 m lattice plus the sphere,
    so the box is 1.05 m wide (one spacing of clearance) and tall enough for the drop."""
    return tank_sphere(n=(20, 20, 20), r=0.025, sphere_radius=0.1, sphere_density=500.0, drop_gap=0.3,
                       sphere_v=(0.5, 0.0, 0.0), sphere_w=(0.0, 1.0, 0.0), dt=0.001, seed=seed,
                       precision=precision, steps=200, **kw)


def dam_break_sphere(n=(100, 100, 100), r=0.005, box=(2.4, 1.2, 1.2), seed=0, dt=0.0005, steps=500,
                     precision=_abi.DFSPH_FP32, sphere_radius=0.05, sphere_density=500.0, **kw):
    """1,000,000-particle dam break (r = 0.005) in a 2.4 x 1.2 x 1.2 m box with one sphere
    (R 0.05, density 500) dropped just above the fluid with v, omega ~ U(-1, 1) (seeded)."""
    rng = np.random.default_rng(seed + 1000)
    v = tuple(rng.uniform(-1.0, 1.0, 3))
    w = tuple(rng.uniform(-1.0, 1.0, 3))
    sp = 2.0 * r
    zoff = 0.5 * (box[2] - (n[2] - 1) * sp)
    sc = tank_sphere(n=n, r=r, box=box, sphere_radius=sphere_radius, sphere_density=sphere_density,
                     drop_gap=0.02, sphere_v=v, sphere_w=w, dt=dt, seed=seed,
                     fluid_origin=(sp, sp, zoff), sphere_xz=(0.5 * n[0] * sp, zoff + 0.5 * (n[2] - 1) * sp),
                     precision=precision, steps=steps, **kw)
    sc.name = f"dam_break_sphere_{sc.n_fluid}"
    return sc


def config1(seed=0, **kw):
    return dam_break_sphere(seed=seed, **kw)


def dam_break_two_spheres(seed=0, gap=0.01, speed=0.5, beta=2000.0, **kw):
    """The 1M dam break with a second sphere beside the first, `gap` apart surface to
    surface (within one support radius) and the two moving towards each other along x, with
    the rigid contact solver and the gradient manager on."""
    sc = dam_break_sphere(seed=seed, use_rigid_contact_solver=1, use_rigid_gradient_manager=1,
                          rigid_contact_beta=beta, **kw)
    first = sc.bodies[1]
    R = float(np.linalg.norm(first.samples, axis=1).max())
    cx, cy, cz = first.translation
    first.translation = (cx - (R + 0.5 * gap), cy, cz)
    first.init_velocity = (speed, 0.0, 0.0)
    second = Body(samples=first.samples.copy(), translation=(cx + R + 0.5 * gap, cy, cz),
                  density=first.density, is_dynamic=True, init_velocity=(-speed, 0.0, 0.0),
                  init_angular_velocity=tuple(-np.asarray(first.init_angular_velocity)),
                  target_x=first.target_x)
    sc.bodies.append(second)
    sc.name = f"dam_break_two_spheres_{sc.n_fluid}"
    return sc


def pool_ellipsoid(n=(125, 16, 125), r=0.004, pool=(1.0, 0.5, 1.0), seed=0, dt=0.0005, steps=1000,
                   precision=_abi.DFSPH_FP32, **kw):
    """250,000-particle layer (125 x 16 x 125 at r = 0.004) in an open 1.0 x 0.5 x 1.0 m pool
    with a dynamic ellipsoid (semi-axes 0.15, 0.08, 0.10; density 600), v ~ U(-2,2)^3,
    omega ~ U(-5,5)^3 (seeded)."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * r
    fx = fluid_lattice(n, sp, (sp, sp, sp), r, rng)
    top = sp + (n[1] - 1) * sp
    walls = box_surface((0.0, 0.0, 0.0), pool, sp, open_top=True)
    rng2 = np.random.default_rng(seed + 2000)
    v = tuple(rng2.uniform(-2.0, 2.0, 3))
    w = tuple(rng2.uniform(-5.0, 5.0, 3))
    center = (0.5 * pool[0], top + 0.08 + 0.02, 0.5 * pool[2])
    target = tuple(np.asarray(center) + rng2.uniform(-0.1, 0.1, 3) * np.array([1.0, 0.0, 1.0]))
    bodies = [Body(samples=walls, density=1000.0),
              Body(samples=ellipsoid_surface(0.15, 0.08, 0.10, sp), translation=center, density=600.0,
                   is_dynamic=True, init_velocity=v, init_angular_velocity=w, target_x=target)]
    params = Params(fluid_precision=precision, particle_radius=r, time_step=dt, **kw)
    return Scene(params=params, fluid_x=fx, fluid_v=np.zeros_like(fx), bodies=bodies,
                 name=f"pool_ellipsoid_{fx.shape[0]}", steps=steps)


def config2(seed=0, **kw):
    return pool_ellipsoid(seed=seed, **kw)


def billiards_on_water(n=(200, 100, 200), r=0.0025, box=(1.2, 0.8, 1.2), seed=0, dt=0.0005, steps=300,
                       precision=_abi.DFSPH_FP32, **kw):
    """4,000,000-particle basin (200 x 100 x 200 at r = 0.0025) in a 1.2 x 0.8 x 1.2 m box
    with two dynamic spheres (R 0.03, density 700, seeded v and omega) and a static box obstacle."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * r
    fx = fluid_lattice(n, sp, (sp, sp, sp), r, rng)
    top = sp + (n[1] - 1) * sp
    walls = box_surface((0.0, 0.0, 0.0), box, sp)
    obstacle = box_surface((-0.05, -0.05, -0.05), (0.05, 0.05, 0.05), sp)
    rng2 = np.random.default_rng(seed + 3000)
    bodies = [Body(samples=walls, density=1000.0),
              Body(samples=obstacle, translation=(1.1, 0.05 + sp, 0.6), density=1000.0)]
    for cx in (0.3, 0.7):
        v = tuple(rng2.uniform(-1.0, 1.0, 3))
        w = tuple(rng2.uniform(-1.0, 1.0, 3))
        c = (cx, top + 0.03 + 0.01, 0.6)
        bodies.append(Body(samples=sphere_surface(0.03, sp), translation=c, density=700.0, is_dynamic=True,
                           init_velocity=v, init_angular_velocity=w, target_x=c))
    params = Params(fluid_precision=precision, particle_radius=r, time_step=dt, **kw)
    return Scene(params=params, fluid_x=fx, fluid_v=np.zeros_like(fx), bodies=bodies,
                 name=f"billiards_on_water_{fx.shape[0]}", steps=steps)


def config4(seed=0, **kw):
    return billiards_on_water(seed=seed, **kw)


def small_contact_scene(n=(12, 10, 12), r=0.025, seed=0, precision=_abi.DFSPH_FP64, drop_gap=-0.05,
                        sphere_radius=0.1, **kw):
    """A small tank whose sphere starts slightly immersed, so that coupling and the gradient
    pair terms are active from the first step (used by parity tests)."""
    return tank_sphere(n=n, r=r, sphere_radius=sphere_radius, drop_gap=drop_gap, seed=seed, precision=precision,
                       steps=20, **kw)


def two_sphere_contact(n=(20, 6, 10), r=0.025, seed=0, precision=_abi.DFSPH_FP64, sphere_radius=0.1,
                       gap=0.02, speed=0.5, beta=20000.0, friction=0.0, release=False, uat=0.0, **kw):
    """Two dynamic spheres, half immersed in a shallow tank, moving towards each other along
    x with seeded spins; they start `gap` apart (surface to surface), so their boundary samples
    are within one support radius and the rigid contact solver acts from the first step. The
    gradient manager is on (the reference's two-ball billiards setup: useRigidContactSolver,
    useRigidGradientManager, rigidContactBeta)."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * r
    fx = fluid_lattice(n, sp, (sp, sp, sp), r, rng)
    box = ((n[0] + 1) * sp, (n[1] + 8) * sp, (n[2] + 1) * sp)
    walls = box_surface((0.0, 0.0, 0.0), box, sp)
    top = sp + (n[1] - 1) * sp
    cz = 0.5 * box[2]
    cx0 = 0.5 * box[0] - sphere_radius - 0.5 * gap
    cx1 = 0.5 * box[0] + sphere_radius + 0.5 * gap
    for cx in (cx0, cx1):  # no fluid inside the spheres
        fx = fx[np.linalg.norm(fx - np.array([cx, top, cz]), axis=1) > sphere_radius + r]
    rng2 = np.random.default_rng(seed + 5000)
    bodies = [Body(samples=walls, density=1000.0)]
    for cx, sgn in ((cx0, 1.0), (cx1, -1.0)):
        w = tuple(rng2.uniform(-1.0, 1.0, 3))
        c = (cx, top, cz)
        bodies.append(Body(samples=sphere_surface(sphere_radius, sp), translation=c, density=500.0,
                           is_dynamic=True, init_velocity=(sgn * speed, 0.0, 0.0), init_angular_velocity=w,
                           target_x=c))
    kw.setdefault("time_step", 0.001)
    params = Params(fluid_precision=precision, particle_radius=r, use_rigid_contact_solver=1,
                    use_rigid_gradient_manager=1, rigid_contact_beta=beta, rigid_contact_friction_coeff=friction,
                    release_rigid_body_mode=int(release), uniform_accelerate_rb_time=uat, **kw)
    return Scene(params=params, fluid_x=fx, fluid_v=np.zeros_like(fx), bodies=bodies,
                 name=f"two_sphere_contact_{fx.shape[0]}", steps=40)


def sphere_on_floor(r=0.0125, precision=_abi.DFSPH_FP64, radius=0.8, gap=0.01, beta=5000.0, **kw):
    """A large dynamic sphere resting `gap` above the floor of an empty container: several
    hundred of its samples are in contact with the floor's at once (no fluid)."""
    sp = 2.0 * r
    box = (2.0 * radius + 0.4, 2.0 * radius + 0.4, 2.0 * radius + 0.4)
    walls = box_surface((0.0, 0.0, 0.0), box, sp)
    c = (0.5 * box[0], radius + gap, 0.5 * box[2])
    bodies = [Body(samples=walls, density=1000.0),
              Body(samples=sphere_surface(radius, sp), translation=c, density=800.0, is_dynamic=True,
                   init_velocity=(0.1, 0.0, 0.0), init_angular_velocity=(0.0, 0.3, 0.2))]
    kw.setdefault("time_step", 0.001)
    params = Params(fluid_precision=precision, particle_radius=r, use_rigid_contact_solver=1,
                    use_rigid_gradient_manager=1, rigid_contact_beta=beta, **kw)
    return Scene(params=params, fluid_x=np.zeros((0, 3)), fluid_v=np.zeros((0, 3)), bodies=bodies,
                 name="sphere_on_floor", steps=20)


CONFIGS = {0: config0, 1: config1, 2: config2, 4: config4}
