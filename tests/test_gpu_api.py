"""The user-facing layers over the C ABI on the GPU: device checkpoints, state control,
the autograd rollout (direct and checkpointed schedules), finite-difference checks of the
gradient, and the pysplishsplash-style module driving an optimisation loop."""
import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn

pytestmark = pytest.mark.gpu


def make(sc):
    from difffr_gb300.sim import DiffDFSPH
    return DiffDFSPH(sc)


def test_checkpoint_restore_replays_bit_exact(gpu_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32)
    g = make(sc)
    g.step(3)
    slot = g.checkpoint_save()
    g.step(4)
    x1, s1 = g.positions(), g.rigid_state_vector(1)
    t1 = g.time()
    g.checkpoint_restore(slot)
    assert g.time()[1] == 3
    g.step(4)
    assert np.array_equal(g.positions(), x1)
    assert np.array_equal(g.rigid_state_vector(1), s1)
    assert g.time() == t1
    g.checkpoint_free(slot)
    with pytest.raises(_abi.DfsphError):
        g.checkpoint_restore(slot)


def test_gradient_switch_leaves_forward_trajectory_unchanged(gpu_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32)
    a, b = make(sc), make(sc)
    b.set_gradient_enabled(False)
    a.step(6)
    b.step(6)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.rigid_state_vector(1), b.rigid_state_vector(1))


def test_set_rigid_state_round_trip(gpu_lib):
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64)
    g = make(sc)
    x = np.array([0.1, 0.35, 0.12])
    q = np.array([0.9, 0.1, -0.2, 0.3])
    v = np.array([0.2, -0.1, 0.05])
    w = np.array([1.0, 0.5, -0.25])
    g.set_rigid_state(1, x, q, v, w)
    xs, qs, vs, ws = g.rigid_state(1)
    assert np.allclose(xs, x) and np.allclose(qs, q / np.linalg.norm(q)) and np.allclose(vs, v) and np.allclose(ws, w)
    bx = g.field(_abi.FIELD_BOUNDARY_X)
    assert np.all(np.isfinite(bx))


def _rollout_grad(sim, p0, steps, k):
    import torch
    from difffr_gb300.autograd import rollout
    p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    out = rollout(sim, p, steps, checkpoint_every=k)
    rng = np.random.default_rng(11)
    wts = torch.tensor(rng.normal(size=out.shape), dtype=torch.float64)
    loss = (out * wts).sum()
    loss.backward()
    return out.detach().numpy(), p.grad.numpy()


@pytest.mark.parametrize("precision", [_abi.DFSPH_FP32, _abi.DFSPH_FP64])
def test_autograd_checkpointed_equals_direct(gpu_lib, precision):
    sc = scn.small_contact_scene(precision=precision, gradient_mode=_abi.GRAD_COMPLETE)
    sim = make(sc)
    p0 = np.zeros((sim.n_bodies, 6))
    p0[1] = [0.3, -0.2, 0.1, 0.5, -1.0, 0.25]
    out_d, g_d = _rollout_grad(sim, p0, 12, None)
    out_c, g_c = _rollout_grad(sim, p0, 12, 5)
    assert np.array_equal(out_d, out_c)
    assert np.allclose(g_c, g_d, rtol=1e-12, atol=1e-15)
    assert np.any(g_d[1] != 0)


def test_autograd_matches_oracle_forward_chain(gpu_lib, oracle_lib):
    """Gradient of a weighted sum of the final rigid state with respect to (v0, omega0):
    GPU reverse sweep (FP32 fluid, FP64 rigid) against the oracle's forward-mode chain with
    FP32 fluid / FP64 rigid arithmetic, and against the FP64 oracle."""
    for precision, mode, tol in ((_abi.DFSPH_FP64, oracle_lib.MODE_F64, 1e-9),
                                 (_abi.DFSPH_FP32, oracle_lib.MODE_MIXED, None)):
        sc = scn.small_contact_scene(precision=precision, gradient_mode=_abi.GRAD_COMPLETE)
        sim = make(sc)
        p0 = np.zeros((sim.n_bodies, 6))
        p0[1] = [0.3, -0.2, 0.1, 0.5, -1.0, 0.25]
        steps = 20
        _, g = _rollout_grad(sim, p0, steps, 7)
        ref = oracle_lib.Oracle(sc, mode=mode)
        ref.set_rigid_init(1, p0[1, :3], p0[1, 3:])
        for _ in range(steps):
            ref.step(1)
        blk = ref.rigid_grad_blocks(1)
        Gv = np.vstack([blk["x_v0"], blk["q_v0"], blk["v_v0"], blk["w_v0"]])
        Gw = np.vstack([blk["x_w0"], blk["q_w0"], blk["v_w0"], blk["w_w0"]])
        rng = np.random.default_rng(11)
        wts = rng.normal(size=(sim.n_bodies, 13))
        ref_g = np.concatenate([wts[1] @ Gv, wts[1] @ Gw])
        cos = float(ref_g @ g[1] / (np.linalg.norm(ref_g) * np.linalg.norm(g[1])))
        assert cos >= 0.999, (precision, cos)
        if tol is not None:
            assert np.max(np.abs(g[1] - ref_g)) <= tol * np.max(np.abs(ref_g)), (g[1], ref_g)


def test_free_flight_gradient_matches_central_differences(gpu_lib):
    """A body that never meets fluid or walls: the chain is exact rigid dynamics, so the
    autograd gradient equals central differences (eps = 1e-4) of the rollout."""
    import torch
    from difffr_gb300.autograd import rollout
    sc = scn.tank_sphere(n=(4, 4, 4), r=0.025, drop_gap=0.6, precision=_abi.DFSPH_FP64, steps=30,
                         gradient_mode=_abi.GRAD_COMPLETE)
    sim = make(sc)
    p0 = np.zeros((sim.n_bodies, 6))
    p0[1] = [0.3, 0.1, -0.2, 0.5, 1.0, -0.3]
    steps = 30
    out, g = _rollout_grad(sim, p0, steps, 10)
    rng = np.random.default_rng(11)
    wts = rng.normal(size=out.shape)

    def loss(p):
        with torch.no_grad():
            o = rollout(sim, torch.tensor(p, dtype=torch.float64), steps).numpy()
        return float((o * wts).sum())

    eps = 1e-4
    fd = np.zeros(6)
    for c in range(6):
        pp, pm = p0.copy(), p0.copy()
        pp[1, c] += eps
        pm[1, c] -= eps
        fd[c] = (loss(pp) - loss(pm)) / (2 * eps)
    assert np.allclose(g[1], fd, rtol=1e-5, atol=1e-7), (g[1], fd)


def test_pysplishsplash_optimisation_loop(gpu_lib):
    """The reference's optimisation scripts' call pattern: init from a scene, set initial
    velocities, run a trajectory with a per-step callback, read the gradient blocks, update,
    reset and run again; save/restore of the state."""
    from difffr_gb300.pysplishsplash import Exec, Simulation, TimeManager
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32, target_time=0.01)
    base = Exec.SimulatorBase()
    base.init(scene=sc, useGui=False)
    base.initSimulation()
    sim = Simulation.getCurrent()
    ts = sim.getTimeStep()
    bm = sim.getBoundaryModel(1)
    assert bm.getRigidBodyObject().isDynamic()
    seen = []
    base.setTimeStepCB(lambda: seen.append(TimeManager.getCurrent().getTime()))
    ts.set_init_v_rb(1, np.array([0.2, 0.0, 0.0]))
    ts.set_init_omega_rb(1, np.array([0.0, 1.0, 0.0]))
    losses = []
    for it in range(3):
        base.runNewTrajectory()
        assert ts.is_trajectory_finish_callback()
        x = np.asarray(bm.get_position_rb())
        tgt = np.asarray(ts.get_target_x(1))
        losses.append(float(np.sum((x - tgt) ** 2)))
        dxdv = np.asarray(bm.get_grad_x_to_v0())
        assert dxdv.shape == (3, 3) and np.all(np.isfinite(dxdv))
        grad_v = 2 * (x - tgt) @ dxdv
        ts.set_init_v_rb(1, np.asarray(ts.get_init_v_rb(1)) - 0.5 * grad_v)
    assert len(seen) >= 3 * 10
    assert np.all(np.isfinite(losses))
    base.reset()
    base.singleTimeStep()
    name = base.saveState()
    base.singleTimeStep()
    s1 = np.asarray(bm.get_position_rb()).copy()
    base.loadStateWithRigidExisted(name)
    base.singleTimeStep()
    assert np.array_equal(np.asarray(bm.get_position_rb()), s1)
    base.cleanup()


def test_pysplishsplash_state_files(gpu_lib, tmp_path):
    """saveState(path) writes the fluid as the reference's state_<t>_particle_Fluid.bgeo;
    loadStateWithRigidExisted(file) sets the fluid back from it."""
    import glob
    from difffr_gb300.pysplishsplash import Exec
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32)
    base = Exec.SimulatorBase()
    base.init(scene=sc)
    base.initSimulation()
    base.singleTimeStep()
    base.saveState(str(tmp_path))
    files = glob.glob(str(tmp_path / "state_*_particle_Fluid.bgeo"))
    assert len(files) == 1
    x1 = base._sim.positions().copy()
    v1 = base._sim.velocities().copy()
    rigid1 = [np.asarray(a).copy() for a in base._sim.rigid_state(1)]
    base.cleanup()
    # a fresh simulator of the same scene takes the fluid from the file
    other = Exec.SimulatorBase()
    other.init(scene=sc)
    other.initSimulation()
    assert not np.allclose(other._sim.positions(), x1)
    other.loadStateWithRigidExisted(files[0])
    assert np.allclose(other._sim.positions(), x1, atol=1e-6)
    assert np.allclose(other._sim.velocities(), v1, atol=1e-6)
    other.cleanup()
    # the rigid records (state_<n>_dynamicRB.bin) set the body's pose and velocities, and the
    # fluid file beside them is read too
    rb = glob.glob(str(tmp_path / "state_*_dynamicRB.bin"))
    assert len(rb) == 1
    third = Exec.SimulatorBase()
    third.init(scene=sc)
    third.initSimulation()
    third.loadStateWithRigidExisted(rb[0])
    for a, b in zip(third._sim.rigid_state(1), rigid1):
        assert np.allclose(a, b, rtol=1e-6, atol=1e-6)
    assert np.allclose(third._sim.positions(), x1, atol=1e-6)
    third.cleanup()
