"""Parity of the GPU library (through the C ABI) with the CPU oracle.

Tolerances:
  FP64 fluid: fields and rigid state within 1e-9 relative after one step (summation
  order differs), neighbour sets identical.
  FP32 fluid: densities within 1e-4 relative, rigid state within 1e-4, neighbour sets
  identical (same FP32 predicate on identical positions).
"""
import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn

pytestmark = pytest.mark.gpu


def make(sc):
    from difffr_gb300.sim import DiffDFSPH
    return DiffDFSPH(sc)


def rows(start, idx):
    return [idx[start[i]:start[i + 1]] for i in range(len(start) - 1)]


def assert_same_neighbors(gpu, ref, which):
    sg, ig = gpu.neighbors(which)
    sr, ir = ref.neighbors(which)
    assert np.array_equal(sg, sr), f"set {which}: row lengths differ"
    assert np.array_equal(ig, ir), f"set {which}: indices differ"


@pytest.mark.parametrize("precision", [_abi.DFSPH_FP32, _abi.DFSPH_FP64])
def test_neighbor_sets_bit_exact(gpu_lib, oracle_lib, precision):
    sc = scn.small_contact_scene(precision=precision)
    gpu, ref = make(sc), oracle_lib.Oracle(sc)
    gpu.step(1)
    ref.step(1)
    for which in (_abi.NB_FLUID_FLUID, _abi.NB_FLUID_BOUNDARY, _abi.NB_BOUNDARY_FLUID):
        assert_same_neighbors(gpu, ref, which)
    # identical arbitrary positions in both: a jittered, compressed cloud
    rng = np.random.default_rng(7)
    x = gpu.positions() + rng.normal(scale=0.3 * sc.params.particle_radius, size=(gpu.n_fluid, 3))
    gpu.set_field(_abi.FIELD_X, x)
    ref.set_field(_abi.FIELD_X, gpu.positions())
    gpu.step(1)
    ref.step(1)
    for which in (_abi.NB_FLUID_FLUID, _abi.NB_FLUID_BOUNDARY, _abi.NB_BOUNDARY_FLUID):
        assert_same_neighbors(gpu, ref, which)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)


FIELDS = [_abi.FIELD_DENSITY, _abi.FIELD_FACTOR, _abi.FIELD_SUM_GRAD_P, _abi.FIELD_V, _abi.FIELD_X,
          _abi.FIELD_KAPPA, _abi.FIELD_KAPPA_V, _abi.FIELD_DENSITY_ADV, _abi.FIELD_BOUNDARY_PSI,
          _abi.FIELD_BOUNDARY_X, _abi.FIELD_BOUNDARY_V]


def test_fp64_single_step_fields(gpu_lib, oracle_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64)
    gpu, ref = make(sc), oracle_lib.Oracle(sc)
    sg, sr = gpu.step(1), ref.step(1)
    assert sg["pressure_iterations"] == sr["pressure_iterations"]
    assert sg["divergence_iterations"] == sr["divergence_iterations"]
    for f in FIELDS:
        assert rel(gpu.field(f), ref.field(f)) < 1e-9, f
    for b in range(len(sc.bodies)):
        for a, c in zip(gpu.rigid_state(b), ref.rigid_state(b)):
            assert np.allclose(a, c, rtol=1e-9, atol=1e-12)
    Fg, Tg = gpu.rigid_force(1)
    Fr, Tr = ref.rigid_force(1)
    assert rel(Fg, Fr) < 1e-9 and rel(Tg, Tr) < 1e-9
    assert rel(gpu.net_jacobians(1), ref.net_jacobians(1)) < 1e-8
    assert rel(gpu.rigid_grad(1), ref.rigid_grad(1)) < 1e-9
    mg, Ig = gpu.rigid_mass(1)
    mr, Ir = ref.rigid_mass(1)
    assert mg == pytest.approx(mr, rel=1e-14) and np.allclose(Ig, Ir, rtol=1e-12)


@pytest.mark.parametrize("mode", [_abi.GRAD_COMPLETE, _abi.GRAD_INCOMPLETE, _abi.GRAD_RIGID_ONLY])
def test_fp64_multistep_chain_all_gradient_modes(gpu_lib, oracle_lib, mode):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64, gradient_mode=mode)
    gpu, ref = make(sc), oracle_lib.Oracle(sc)
    for _ in range(6):
        sg, sr = gpu.step(1), ref.step(1)
        assert sg["pressure_iterations"] == sr["pressure_iterations"]
    for a, c in zip(gpu.rigid_state(1), ref.rigid_state(1)):
        assert np.allclose(a, c, rtol=1e-8, atol=1e-11)
    assert rel(gpu.rigid_grad(1), ref.rigid_grad(1)) < 1e-7
    assert rel(gpu.field(_abi.FIELD_X), ref.field(_abi.FIELD_X)) < 1e-9


def test_fp32_against_mixed_oracle(gpu_lib, oracle_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32)
    gpu, ref = make(sc), oracle_lib.Oracle(sc, mode=oracle_lib.MODE_MIXED)
    gpu.step(1)
    ref.step(1)
    assert rel(gpu.field(_abi.FIELD_DENSITY), ref.field(_abi.FIELD_DENSITY)) < 1e-5
    assert rel(gpu.field(_abi.FIELD_FACTOR), ref.field(_abi.FIELD_FACTOR)) < 1e-4
    assert rel(gpu.field(_abi.FIELD_V), ref.field(_abi.FIELD_V)) < 1e-4
    Fg, _ = gpu.rigid_force(1)
    Fr, _ = ref.rigid_force(1)
    assert rel(Fg, Fr) < 1e-3
    for _ in range(4):
        gpu.step(1)
        ref.step(1)
    xg, qg, vg, wg = gpu.rigid_state(1)
    xr, qr, vr, wr = ref.rigid_state(1)
    assert np.allclose(xg, xr, atol=1e-5) and np.allclose(qg, qr, atol=1e-4)
    assert np.allclose(vg, vr, rtol=2e-3, atol=2e-3)
    assert rel(gpu.rigid_grad(1), ref.rigid_grad(1)) < 2e-2


def test_backward_equals_forward_chain_contraction(gpu_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64, gradient_mode=_abi.GRAD_COMPLETE)
    gpu = make(sc)
    gpu.step(8)
    assert gpu.tape_length() == 8
    rng = np.random.default_rng(3)
    dL = rng.normal(size=(gpu.n_bodies, 13))
    g = gpu.backward(dL)
    blk = gpu.rigid_grad_blocks(1)
    Gv = np.vstack([blk["x_v0"], blk["q_v0"], blk["v_v0"], blk["w_v0"]])
    Gw = np.vstack([blk["x_w0"], blk["q_w0"], blk["v_w0"], blk["w_w0"]])
    fwd = np.concatenate([dL[1] @ Gv, dL[1] @ Gw])
    assert np.allclose(g[1], fwd, rtol=1e-10, atol=1e-13)


def test_deterministic_replay(gpu_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32)
    a, b = make(sc), make(sc)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.rigid_grad(1), b.rigid_grad(1))
    a.reset()
    a.step(5)
    assert np.array_equal(a.positions(), b.positions())
    # five single-step calls (each ends with both streams synchronised) equal one call of
    # five steps (the rigid stream overlapping the next step's fluid work)
    c = make(sc)
    for _ in range(5):
        c.step(1)
    assert np.array_equal(c.positions(), b.positions())
    assert np.array_equal(c.rigid_grad(1), b.rigid_grad(1))


def test_edge_cases_empty_and_no_bodies(gpu_lib, oracle_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64)
    only_fluid = scn.Scene(params=sc.params, fluid_x=sc.fluid_x, fluid_v=sc.fluid_v, bodies=[])
    g, r = make(only_fluid), oracle_lib.Oracle(only_fluid)
    g.step(2)
    r.step(2)
    assert rel(g.positions(), r.field(_abi.FIELD_X)) < 1e-9
    no_fluid = scn.Scene(params=sc.params, fluid_x=np.zeros((0, 3)), fluid_v=np.zeros((0, 3)), bodies=sc.bodies)
    g2 = make(no_fluid)
    g2.step(3)
    x, q, v, w = g2.rigid_state(1)
    assert np.all(np.isfinite(x))


@pytest.mark.parametrize("precision", [_abi.DFSPH_FP64, _abi.DFSPH_FP32])
def test_edge_cases_lone_particles(gpu_lib, oracle_lib, precision):
    """One fluid particle, then three far apart (empty neighbour lists: density from the
    particle itself, a zero DFSPH factor, fewer than 20 neighbours), falling in the scene's
    container beside its bodies; every field and the rigid state against the oracle."""
    sc = scn.small_contact_scene(precision=precision)
    lo, hi = sc.fluid_x.min(axis=0), sc.fluid_x.max(axis=0)
    mid = 0.5 * (lo + hi)
    for pts in ([mid], [lo, mid, hi]):
        x = np.asarray(pts, np.float64).reshape(-1, 3)
        lone = scn.Scene(params=sc.params, fluid_x=x, fluid_v=np.zeros_like(x), bodies=sc.bodies)
        g, r = make(lone), oracle_lib.Oracle(lone)
        g.step(3)
        r.step(3)
        tol = 1e-9 if precision == _abi.DFSPH_FP64 else 1e-5
        for f in (_abi.FIELD_X, _abi.FIELD_V, _abi.FIELD_DENSITY, _abi.FIELD_FACTOR):
            assert rel(g.field(f), r.field(f)) < tol, (len(pts), f)
        assert np.allclose(g.rigid_state(1)[0], r.rigid_state(1)[0], rtol=tol, atol=1e-12)
        assert g.neighbor_total(_abi.NB_FLUID_FLUID) == 0


def test_neighbor_overflow_reports_device_error(gpu_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32, max_fluid_neighbors=4)
    g = make(sc)
    with pytest.raises(_abi.DfsphError) as e:
        g.step(1)
    assert e.value.code == _abi.DFSPH_ERR_DEVICE


@pytest.mark.parametrize("precision", [_abi.DFSPH_FP64, _abi.DFSPH_FP32])
def test_surface_tension_akinci2013_matches_oracle(gpu_lib, oracle_lib, precision):
    """Akinci2013 surface tension (cohesion, curvature, boundary adhesion) with the
    reference scenes' coefficient 0.5 and a boundary coefficient 0.1, against the oracle:
    FP64 over 4 steps, FP32 over 3 steps, every field and the rigid state within 1e-9 (FP64)
    or 1e-4 (FP32, max norm). The reference's cohesion kernel is discontinuous at |r| = h/2
    (SPHKernels.h:471-473 subtracts h^6/64 unscaled by k), which is the lattice spacing of
    these scenes: once FP32 positions differ in their last bits, a pair sitting within that
    distance of h/2 takes the other branch, and its ~8 m/s^2 jump spreads through the next
    pressure solve. FP32 runs are compared before that happens."""
    sc = scn.small_contact_scene(precision=precision, surface_tension_method=2, surface_tension=0.5,
                                 surface_tension_boundary=0.1)
    gpu, ref = make(sc), oracle_lib.Oracle(sc)
    steps = 4 if precision == _abi.DFSPH_FP64 else 3
    gpu.step(steps)
    ref.step(steps)
    tol = 1e-9 if precision == _abi.DFSPH_FP64 else 1e-4
    for f in (_abi.FIELD_X, _abi.FIELD_DENSITY, _abi.FIELD_V):
        assert rel(gpu.field(f), ref.field(f)) < tol, f
    assert rel(gpu.rigid_state(1)[0], ref.rigid_state(1)[0]) < tol
    # the surface tension changes the flow (not a no-op)
    plain = scn.small_contact_scene(precision=precision)
    g2 = make(plain)
    g2.step(steps)
    assert rel(g2.field(_abi.FIELD_V), gpu.field(_abi.FIELD_V)) > 10 * tol


@pytest.mark.parametrize("precision", [_abi.DFSPH_FP64, _abi.DFSPH_FP32])
def test_boundary_viscosity_matches_oracle(gpu_lib, oracle_lib, precision):
    """XSPH viscosity against the boundary samples with the bodies' reaction
    (Viscosity_XSPH.cpp:72-82, viscosityBoundary 0.5), against the oracle: fields, the
    rigid state and the body's fluid force within 1e-9 (FP64) or 1e-4 (FP32) after 6 steps;
    the term changes both the flow and the force on the sphere."""
    sc = scn.small_contact_scene(precision=precision, viscosity_boundary=0.5, sphere_v=(1.0, -0.5, 0.0))
    gpu, ref = make(sc), oracle_lib.Oracle(sc)
    gpu.step(6)
    ref.step(6)
    tol = 1e-9 if precision == _abi.DFSPH_FP64 else 1e-4
    for f in (_abi.FIELD_X, _abi.FIELD_DENSITY, _abi.FIELD_V):
        assert rel(gpu.field(f), ref.field(f)) < tol, f
    for a, b in zip(gpu.rigid_state(1), ref.rigid_state(1)):
        assert rel(a, b) < tol
    assert rel(gpu.rigid_force(1)[0], ref.rigid_force(1)[0]) < 10 * tol
    plain = make(scn.small_contact_scene(precision=precision, sphere_v=(1.0, -0.5, 0.0)))
    plain.step(6)
    assert rel(plain.field(_abi.FIELD_V), gpu.field(_abi.FIELD_V)) > 10 * tol
    assert rel(plain.rigid_force(1)[0], gpu.rigid_force(1)[0]) > 10 * tol


def test_cfl_time_stepping_matches_oracle(gpu_lib, oracle_lib):
    """Adaptive CFL step size (Simulation::updateTimeStepSizeCFL): from 1 ms the size goes to
    the 5 ms cap while the boundary samples are still at rest, then drops below it once the
    sphere's 2.2 m/s reaches its samples; GPU (FP64) and oracle agree on the simulated time
    (the sum of the sizes), the fields and the rigid state within 1e-9."""
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64, cfl_method=1, cfl_factor=0.5, cfl_max_time_step=0.005,
                                 sphere_v=(2.0, -1.0, 0.0))
    gpu, ref = make(sc), oracle_lib.Oracle(sc)
    sizes = []
    for _ in range(6):
        st = gpu.step(1)
        ref.step(1)
        sizes.append(st["time_step"])
    assert max(sizes) == sc.params.cfl_max_time_step and min(sizes) < 0.6 * sc.params.cfl_max_time_step
    assert abs(gpu.time()[0] - ref.time()) <= 1e-12 * ref.time()
    for f in (_abi.FIELD_X, _abi.FIELD_V, _abi.FIELD_DENSITY):
        assert rel(gpu.field(f), ref.field(f)) < 1e-9, f
    assert rel(gpu.rigid_state(1)[0], ref.rigid_state(1)[0]) < 1e-9
