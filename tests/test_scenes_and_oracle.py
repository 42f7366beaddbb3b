"""Scene generators, the scene-JSON reader, and oracle-level checks (CPU only)."""
import json
import os

import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn
from difffr_gb300.scene_json import load_scene
from oracle import reference_root

REF = reference_root()


def test_benchmark_scene_sizes():
    sc = scn.config1()
    assert sc.n_fluid == 1_000_000
    assert 140_000 < sc.n_boundary - sc.n_dynamic_boundary() < 150_000
    assert sc.n_dynamic_boundary() == 314
    assert sc.params.time_step == 0.0005 and sc.params.particle_radius == 0.005
    sc0 = scn.config0()
    assert sc0.n_fluid == 8000 and sc0.n_dynamic_boundary() == 50
    sc2 = scn.config2()
    assert sc2.n_fluid == 250_000 and 2000 < sc2.n_dynamic_boundary() < 2500


def test_lattice_jitter_bounds():
    rng = np.random.default_rng(0)
    r = 0.01
    p = scn.fluid_lattice((4, 5, 6), 2 * r, (0, 0, 0), r, rng)
    base = scn.fluid_lattice((4, 5, 6), 2 * r, (0, 0, 0), r, rng, jitter=False)
    assert p.shape == (120, 3)
    assert np.all(np.abs(p - base) <= 0.01 * r)


def test_scene_json_fluid_block_and_bodies(tmp_path):
    data = {
        "Configuration": {"particleRadius": 0.025, "timeStepSize": 0.002, "maxError": 0.05, "gradientMode": 0,
                          "targetTime": 0.5, "gravitation": [0, -9.8, 0]},
        "FluidBlocks": [{"start": [0, 0, 0], "end": [0.5, 0.5, 0.5]}],
        "RigidBodies": [
            {"geometryFile": "../models/UnitBox.obj", "scale": [1, 1, 1], "translation": [0.5, 0.5, 0.5],
             "isDynamic": False, "isWall": True},
            {"geometryFile": "sphere.obj", "scale": [0.1, 0.1, 0.1], "translation": [0.25, 0.8, 0.25],
             "isDynamic": True, "density": 500, "initVelocity": [1, 0, 0], "targetX": [0.3, 0.2, 0.1],
             "rotationAxis": [0, 0, 1], "rotationAngle": 90},
        ],
    }
    f = tmp_path / "s.json"
    f.write_text(json.dumps(data))
    sc = load_scene(str(f))
    # createFluidBlocks: round(0.5 / 0.05) - 1 = 9 points per axis, starting at min + 2r
    assert sc.n_fluid == 9 ** 3
    assert np.allclose(sc.fluid_x.min(0), 0.05)
    assert sc.params.gradient_mode == 0 and sc.params.max_error == 0.05 and sc.params.time_step == 0.002
    assert sc.params.gravity == (0.0, -9.8, 0.0)
    s = sc.bodies[1]
    assert s.is_dynamic and s.init_velocity == (1, 0, 0)
    assert np.allclose(np.linalg.norm(s.samples, axis=1), 0.1)
    assert np.allclose(s.rotation, (np.cos(np.pi / 4), 0, 0, np.sin(np.pi / 4)))


def test_synthetic_scene_reference_in_json():
    sc = load_scene({"synthetic": "small_contact", "overrides": {"n": (6, 6, 6)}})
    assert sc.n_fluid > 0 and len(sc.bodies) == 2


def _oracle_pair(oracle_lib, sc, steps):
    a = oracle_lib.Oracle(sc)
    for _ in range(steps):
        a.step(1)
    return a


def test_oracle_step_force_jacobian_against_finite_differences(oracle_lib):
    """The per-step dF/dv_n of the reference's formulation against central differences of
    the net fluid force, the check of experiments/others/python/finite-difference.py:78-126.
    The formulation drops the fluid's coupled response to the boundary velocity, so only the
    direction is expected to agree (cosine of the flattened 3x3 blocks)."""
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64)
    ref = _oracle_pair(oracle_lib, sc, 3)
    x, q, v, w = ref.rigid_state(1)
    eps = 1e-4
    J = np.zeros((3, 3))
    for c in range(3):
        p, m = _oracle_pair(oracle_lib, sc, 3), _oracle_pair(oracle_lib, sc, 3)
        vp, vm = v.copy(), v.copy()
        vp[c] += eps
        vm[c] -= eps
        p.set_rigid_velocity(1, vp, w)
        m.set_rigid_velocity(1, vm, w)
        p.step(1)
        m.step(1)
        J[:, c] = (p.rigid_force(1)[0] - m.rigid_force(1)[0]) / (2 * eps)
    ref.step(1)
    Fv = ref.net_jacobians(1)[0:9].reshape(3, 3)
    cos = float(np.sum(Fv * J) / (np.linalg.norm(Fv) * np.linalg.norm(J)))
    assert cos > 0.9, (cos, Fv, J)


def test_oracle_free_flight_chain_matches_finite_differences(oracle_lib):
    """Without fluid contact the chain rule is exact rigid-body dynamics: its dx_T/dv0 and
    dx_T/domega0 must match central differences of full trajectories."""
    sc = scn.tank_sphere(n=(4, 4, 4), r=0.025, drop_gap=0.6, sphere_v=(0.3, 0.1, -0.2),
                         sphere_w=(0.5, 1.0, -0.3), precision=_abi.DFSPH_FP64, steps=20,
                         gradient_mode=_abi.GRAD_COMPLETE)
    steps = 20
    base = _oracle_pair(oracle_lib, sc, steps)
    G = base.rigid_grad(1)
    Gx_v, Gx_w = G[0:9].reshape(3, 3), G[9:18].reshape(3, 3)
    eps = 1e-6
    v0 = np.array(sc.bodies[1].init_velocity)
    w0 = np.array(sc.bodies[1].init_angular_velocity)
    fd_v, fd_w = np.zeros((3, 3)), np.zeros((3, 3))
    for c in range(3):
        xs = []
        for sgn in (1, -1):
            o = oracle_lib.Oracle(sc)
            dv = np.zeros(3)
            dv[c] = sgn * eps
            o.set_rigid_init(1, v0 + dv, w0)
            for _ in range(steps):
                o.step(1)
            xs.append(o.rigid_state(1)[0])
        fd_v[:, c] = (xs[0] - xs[1]) / (2 * eps)
        xs = []
        for sgn in (1, -1):
            o = oracle_lib.Oracle(sc)
            dw = np.zeros(3)
            dw[c] = sgn * eps
            o.set_rigid_init(1, v0, w0 + dw)
            for _ in range(steps):
                o.step(1)
            xs.append(o.rigid_state(1)[0])
        fd_w[:, c] = (xs[0] - xs[1]) / (2 * eps)
    assert np.allclose(Gx_v, fd_v, rtol=1e-4, atol=1e-7), (Gx_v, fd_v)
    assert np.allclose(Gx_w, fd_w, rtol=1e-4, atol=1e-7), (Gx_w, fd_w)


def test_oracle_hydrostatic_column_settles(oracle_lib):
    """A fluid block at rest in a closed box: densities stay near rest, velocities small."""
    sc = scn.tank_sphere(n=(8, 8, 8), r=0.025, drop_gap=0.5, precision=_abi.DFSPH_FP64, steps=30)
    o = oracle_lib.Oracle(sc)
    for _ in range(30):
        o.step(1)
    rho = o.field(_abi.FIELD_DENSITY)
    v = o.field(_abi.FIELD_V)
    assert rho.max() < 1.05 * 1000.0
    assert np.abs(v).max() < 0.5
    q = o.rigid_state(1)[1]
    assert abs(np.linalg.norm(q) - 1.0) < 1e-12


def test_scene_json_material_keys():
    sc = load_scene({"Configuration": {"particleRadius": 0.02},
                     "Materials": [{"id": "Fluid", "surfaceTension": 0.5, "surfaceTensionBoundary": 0.0,
                                    "surfaceTensionMethod": 2, "viscosity": 0.02}],
                     "FluidBlocks": [{"start": [0, 0, 0], "end": [0.2, 0.2, 0.2]}]})
    p = sc.params
    assert p.surface_tension_method == 2 and p.surface_tension == 0.5 and p.surface_tension_boundary == 0.0
    assert p.viscosity == 0.02


def test_oracle_surface_tension_conserves_fluid_momentum(oracle_lib):
    """Without boundary adhesion the fluid-fluid surface-tension accelerations are pairwise
    antisymmetric (K_ij symmetric, cohesion along x_ij, curvature n_i - n_j), as are the
    DFSPH pressure and divergence corrections: in a fluid block without gravity, walls or
    XSPH viscosity (whose m_j / rho_j weights are not symmetric) the total momentum stays zero."""
    rng = np.random.default_rng(5)
    r = 0.025
    fx = scn.fluid_lattice((8, 8, 8), 2 * r, (0, 0, 0), r, rng)
    params = scn.Params(fluid_precision=_abi.DFSPH_FP64, particle_radius=r, gravity=(0.0, 0.0, 0.0),
                        viscosity=0.0, surface_tension_method=2, surface_tension=0.5, surface_tension_boundary=0.0,
                        enable_gradient=0)
    sc = scn.Scene(params=params, fluid_x=fx, fluid_v=np.zeros_like(fx), bodies=[])
    o = oracle_lib.Oracle(sc)
    o.step(3)
    v = o.field(_abi.FIELD_V)
    assert np.abs(v).max() > 1e-6  # the blob moves (surface tension acts)
    assert np.abs(v.sum(axis=0)).max() < 1e-9 * np.abs(v).sum()


def _write_cube_obj(path):
    v = [(-0.5, -0.5, 0.5), (0.5, -0.5, 0.5), (-0.5, 0.5, 0.5), (0.5, 0.5, 0.5),
         (-0.5, 0.5, -0.5), (0.5, 0.5, -0.5), (-0.5, -0.5, -0.5), (0.5, -0.5, -0.5)]
    quads = [(1, 2, 4, 3), (3, 4, 6, 5), (5, 6, 8, 7), (7, 8, 2, 1), (2, 8, 6, 4), (7, 1, 3, 5)]
    with open(path, "w") as f:
        f.write("# unit cube\n")
        for p in v:
            f.write("v %f %f %f\n" % p)
        for q in quads:
            f.write("f %d/1 %d/2 %d/3 %d/4\n" % q)


def test_obj_regular_triangle_sampling(tmp_path):
    from difffr_gb300.mesh_sampling import load_obj, regular_triangle_samples
    path = tmp_path / "cube.obj"
    _write_cube_obj(path)
    v, f = load_obj(str(path), scale=(2.0, 1.0, 1.0))
    assert v.shape == (8, 3) and f.shape == (12, 3)
    assert np.allclose(v.min(0), (-1.0, -0.5, -0.5)) and np.allclose(v.max(0), (1.0, 0.5, 0.5))
    d = 0.1
    s = regular_triangle_samples(v, f, d)
    # every sample lies on the box surface
    on = np.isclose(np.abs(s[:, 0]), 1.0) | np.isclose(np.abs(s[:, 1]), 0.5) | np.isclose(np.abs(s[:, 2]), 0.5)
    assert on.all()
    inside = (np.abs(s[:, 0]) <= 1.0 + 1e-12) & (np.abs(s[:, 1]) <= 0.5 + 1e-12) & (np.abs(s[:, 2]) <= 0.5 + 1e-12)
    assert inside.all()
    # no point of the surface is farther than about d from a sample (probe a random set)
    rng = np.random.default_rng(0)
    probes = rng.uniform(-1, 1, size=(500, 3)) * np.array([1.0, 0.5, 0.5])
    ax = rng.integers(0, 3, size=500)
    probes[np.arange(500), ax] = np.sign(probes[np.arange(500), ax]) * np.array([1.0, 0.5, 0.5])[ax]
    dist = np.min(np.linalg.norm(probes[:, None, :] - s[None, :, :], axis=2), axis=1)
    assert dist.max() < d
    # edges: 18 unique edges of the triangulated cube, vertices once
    assert np.unique(np.round(s, 9), axis=0).shape[0] <= s.shape[0]


def test_scene_json_obj_body(tmp_path):
    path = tmp_path / "UnitBox.obj"
    _write_cube_obj(path)
    scene = {"Configuration": {"particleRadius": 0.02},
             "RigidBodies": [{"geometryFile": "UnitBox.obj", "scale": [1, 1, 1], "isWall": True, "isDynamic": False}],
             "FluidBlocks": [{"start": [-0.3, -0.3, -0.3], "end": [0.3, 0.3, 0.3]}]}
    f = tmp_path / "s.json"
    f.write_text(json.dumps(scene))
    sc = load_scene(str(f))
    b = sc.bodies[0].samples
    assert np.all(np.max(np.abs(b), axis=1) > 0.5 - 1e-9)


@pytest.mark.skipif(REF is None, reason="reference checkout not present")
def test_reference_scene_files_load():
    """The reference's own scene files (read-only checkout, when present) load with their OBJ
    bodies sampled from the meshes."""
    base = os.path.join(REF, "experiments", "rigid_body_trajectory_optimization", "scene")
    sc = load_scene(os.path.join(base, "diff-stone-skipping.json"))
    assert sc.params.surface_tension_method == 2 and sc.params.particle_radius == 0.015
    assert sc.n_fluid > 100000 and len(sc.bodies) == 2
    assert sc.bodies[1].is_dynamic and sc.bodies[1].samples.shape[0] > 100


def test_bgeo_round_trip(tmp_path):
    from difffr_gb300.partio_bgeo import read_bgeo, write_bgeo
    rng = np.random.default_rng(1)
    x = rng.normal(size=(1000, 3)).astype(np.float32)
    v = rng.normal(size=(1000, 3)).astype(np.float32)
    k = rng.normal(size=1000).astype(np.float32)
    ids = np.arange(1000, dtype=np.int32)
    p = tmp_path / "s.bgeo"
    write_bgeo(str(p), x, velocity=v, kappa=k, id=ids)
    d = read_bgeo(str(p))
    assert np.array_equal(d["position"], x) and np.array_equal(d["velocity"], v)
    assert np.array_equal(d["kappa"].ravel(), k) and np.array_equal(d["id"].ravel(), ids)


def test_scene_json_fluid_model_from_bgeo(tmp_path):
    from difffr_gb300.partio_bgeo import write_bgeo
    x = np.array([[0.1, 0.2, 0.3], [0.15, 0.2, 0.3]], np.float32)
    v = np.array([[1.0, 0.0, 0.0], [0.0, 2.0, 0.0]], np.float32)
    write_bgeo(str(tmp_path / "fluid.bgeo"), x, velocity=v)
    sc = load_scene({"Configuration": {"particleRadius": 0.025},
                     "FluidModels": [{"particleFile": str(tmp_path / "fluid.bgeo"), "translation": [1, 0, 0],
                                      "rotationAxis": [0, 0, 1], "rotationAngle": 90}]})
    assert sc.n_fluid == 2
    assert np.allclose(sc.fluid_x[0], [1 - 0.2, 0.1, 0.3], atol=1e-6)
    assert np.allclose(sc.fluid_v[1], [-2.0, 0.0, 0.0], atol=1e-6)


@pytest.mark.skipif(REF is None, reason="reference checkout not present")
def test_reference_state_file_reads():
    from difffr_gb300.partio_bgeo import read_bgeo
    d = read_bgeo(os.path.join(REF, "experiments", "rigid_body_trajectory_optimization", "state", "billiards",
                               "state_17_particle_Fluid.bgeo"))
    assert d["position"].shape == (87374, 3) and d["velocity"].shape == (87374, 3)
    assert {"id", "kappa", "kappa_v"} <= set(d)
    assert np.all(np.isfinite(d["position"])) and np.abs(d["position"]).max() < 2.0


@pytest.mark.skipif(REF is None, reason="reference checkout not present")
def test_reference_contact_scene_loads():
    """The reference's two-ball billiards scene turns on the rigid contact solver and the
    gradient manager (its Configuration keys reach dfsph_params)."""
    base = os.path.join(REF, "experiments", "rigid_body_trajectory_optimization", "scene")
    sc = load_scene(os.path.join(base, "billiards-on-water-2balls.json"))
    p = sc.params
    assert p.use_rigid_contact_solver == 1 and p.use_rigid_gradient_manager == 1
    assert p.rigid_contact_beta == 20000.0 and p.release_rigid_body_mode == 1
    assert [b.is_dynamic for b in sc.bodies] == [False, True, True]


def test_scene_json_contact_keys():
    cfg = {"Configuration": {"particleRadius": 0.02, "useRigidContactSolver": True, "useRigidGradientManager": True,
                             "rigidContactBeta": 500.0, "rigidContactGamma": 0.6,
                             "rigidContactSupportRadiusFactor": 3.5, "rigidContactFrictionCoeff": 0.1},
           "FluidBlocks": [{"start": [0, 0, 0], "end": [0.2, 0.2, 0.2]}]}
    p = load_scene(cfg).params
    assert (p.use_rigid_contact_solver, p.use_rigid_gradient_manager) == (1, 1)
    assert (p.rigid_contact_beta, p.rigid_contact_gamma) == (500.0, 0.6)
    assert (p.rigid_contact_support_radius_factor, p.rigid_contact_friction_coeff) == (3.5, 0.1)
    d = load_scene({"Configuration": {}, "FluidBlocks": []}).params
    assert (d.use_rigid_contact_solver, d.rigid_contact_gamma, d.rigid_contact_beta) == (0, 0.7, 1.0)
    assert d.rigid_contact_support_radius_factor == 4.0 and d.rigid_contact_friction_coeff == 0.0


def test_oracle_contact_penalty_and_manager_blocks():
    """Oracle restatement of the penalty contact (RigidContactSolver.cpp:307-555) and the
    manager chain (RigidBodyGradientManager.cpp:96-468): the spheres, pushed together, are
    driven apart; the samples in contact carry forces; the cross blocks [R][RR] and the
    cross chain state are non-zero and finite."""
    import oracle
    sc = scn.two_sphere_contact(speed=0.5)
    o = oracle.Oracle(sc, mode=oracle.MODE_F64)
    o.step(1)
    nc, na = o.contact_count()
    assert 0 < na <= nc
    o.step(2)
    assert o.rigid_state(1)[2][0] < 0.0 < o.rigid_state(2)[2][0]
    Fx12 = o.manager_jacobians(1, 2)[9:18]
    assert np.linalg.norm(Fx12) > 0 and np.all(np.isfinite(o.manager_jacobians(2, 1)))
    g21 = o.manager_grad(2, 1)
    assert np.linalg.norm(g21) > 0 and np.all(np.isfinite(g21))
    # without contact the cross terms stay exactly zero
    far = scn.two_sphere_contact(gap=0.3, speed=0.0)  # clear of each other and of the walls
    o2 = oracle.Oracle(far, mode=oracle.MODE_F64)
    o2.step(3)
    assert o2.contact_count() == (0, 0)
    assert np.all(o2.manager_grad(2, 1) == 0.0) and np.all(o2.manager_jacobians(1, 2) == 0.0)


def test_oracle_manager_reset_gradient_keeps_blocks():
    """reset_gradient restarts the manager's chain state but keeps its blocks (the next
    step's fluid stage reads the last contact blocks); reset clears both."""
    import oracle
    o = oracle.Oracle(scn.two_sphere_contact(), mode=oracle.MODE_F64)
    o.step(3)
    jac = o.manager_jacobians(1, 2).copy()
    o.reset_gradient()
    assert np.array_equal(o.manager_jacobians(1, 2), jac)
    g = oracle.grad_blocks(o.manager_grad(1, 1))
    assert np.array_equal(g["v_v0"], np.eye(3)) and not g["x_v0"].any()
    o.reset()
    assert not o.manager_jacobians(1, 2).any()


@pytest.mark.parametrize("real", [np.float32, np.float64])
def test_state_bin_rigid_records_round_trip(tmp_path, real):
    """state_<n>_dynamicRB.bin (SimulatorBase.cpp:1985-2000): raw (x, q as x y z w, v, omega)
    per moving body; read back from the end of the file with the scalar type detected."""
    from difffr_gb300.state_bin import read_rigid_records, write_dynamic_rb
    rng = np.random.default_rng(0)
    recs = []
    for _ in range(3):
        q = rng.normal(size=4)
        recs.append((rng.normal(size=3), q / np.linalg.norm(q), rng.normal(size=3), rng.normal(size=3)))
    f = tmp_path / "state_7_dynamicRB.bin"
    write_dynamic_rb(str(f), recs, real=real)
    assert f.stat().st_size == 3 * 13 * np.dtype(real).itemsize
    got, dt = read_rigid_records(str(f), 3)
    assert dt == np.dtype(real)
    tol = 1e-6 if real == np.float32 else 0.0
    for a, b in zip(got, recs):
        for u, w in zip(a, b):
            np.testing.assert_allclose(u, w, atol=tol, rtol=tol)
    # a main state file: arbitrary header bytes, then the same records
    g = tmp_path / "state_7.bin"
    g.write_bytes(b"\x20\x00\x00\x00" + bytes(range(200)) + f.read_bytes())
    got2, _ = read_rigid_records(str(g), 3)
    np.testing.assert_array_equal(got2[1][0], got[1][0])


@pytest.mark.skipif(REF is None, reason="reference checkout not present")
def test_reference_state_file_rigid_records():
    """The reference's billiards state (state/billiards/state_17.bin, two moving balls):
    float records with unit quaternions at the end of the file."""
    from difffr_gb300.state_bin import read_rigid_records
    f = os.path.join(REF, "experiments", "rigid_body_trajectory_optimization", "state", "billiards", "state_17.bin")
    recs, dt = read_rigid_records(f, 2)
    assert dt == np.dtype(np.float32)
    np.testing.assert_allclose(recs[0][0], [-0.95, 0.7864, 0.0], atol=1e-4)
    np.testing.assert_allclose(recs[1][0], [-0.1, 0.4316, -0.0001], atol=1e-4)
    for x, q, v, w in recs:
        assert abs(np.linalg.norm(q) - 1.0) < 1e-6


def test_poisson_disk_sampling_flat_and_cube(tmp_path):
    """Poisson-disk surface sampling (PoissonDiskSampling.cpp, minimum distance r): on a flat
    square every pair of samples is at least r apart and the density is that of a maximal
    Poisson-disk set (0.5-0.8 samples per r^2); on a cube all samples lie on the faces; the
    sampling is deterministic for a seed; the scene loader uses it by default (samplingMode 0)
    and the regular triangle pattern for samplingMode 1."""
    from scipy.spatial import cKDTree
    from difffr_gb300.mesh_sampling import poisson_disk_samples
    r = 0.02
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], dtype=np.float64)
    f = np.array([[0, 1, 2], [0, 2, 3]])
    s = poisson_disk_samples(v, f, r, seed=1)
    d, _ = cKDTree(s).query(s, k=2)
    assert d[:, 1].min() >= r
    assert 0.5 < s.shape[0] * r * r < 0.8
    assert np.all(np.abs(s[:, 2]) < 1e-12) and s[:, :2].min() >= 0 and s[:, :2].max() <= 1
    assert np.array_equal(s, poisson_disk_samples(v, f, r, seed=1))
    path = tmp_path / "UnitBox.obj"
    _write_cube_obj(path)
    body = {"geometryFile": "UnitBox.obj", "scale": [1, 1, 1], "isDynamic": True}
    cfg = {"Configuration": {"particleRadius": 0.02}, "RigidBodies": [body], "FluidBlocks": []}
    (tmp_path / "a.json").write_text(json.dumps(cfg))
    pd = load_scene(str(tmp_path / "a.json")).bodies[0].samples
    assert np.allclose(np.max(np.abs(pd), axis=1), 0.5)
    assert 0.5 < pd.shape[0] * 0.02 ** 2 / 6.0 < 0.8
    body["samplingMode"] = 1
    (tmp_path / "b.json").write_text(json.dumps(cfg))
    rt = load_scene(str(tmp_path / "b.json")).bodies[0].samples
    assert rt.shape[0] != pd.shape[0]
