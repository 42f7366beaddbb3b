"""Rigid-rigid contact (penalty form of the InterlinkedSPH RigidContactSolver) and the
gradient manager's multi-body chain on the GPU, against the CPU oracle through the C ABI.

The scene is two half-immersed spheres pushed towards each other in a shallow tank
(``scene.two_sphere_contact``): their boundary samples are within one support radius
from the first step, so the penalty force, its Jacobian blocks and the manager's cross
blocks [R][RR] are active at once. Tolerances:

* FP64 fluid: rigid states to 1e-8 relative; the manager's chain state and blocks to 1e-6
  relative per [R][RR] pair (the GPU sums neighbours in cell order, the oracle in index
  order, and the penalty stiffness amplifies the last bits);
* FP32 fluid: rigid velocities to 2e-3 absolute over 8 steps (FP32 fluid forces);
* the reverse sweep equals the forward-mode contraction to 1e-9 relative, and the
  checkpointed replay equals the direct schedule to 1e-12 relative.
"""
import numpy as np
import pytest
import torch

import oracle
from difffr_gb300 import scene as scn
from difffr_gb300.autograd import rollout
from difffr_gb300.sim import DiffDFSPH

pytestmark = pytest.mark.gpu

DYN = (1, 2)


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _chain_matrix(blocks):
    """13 x 6 derivative of (x, q, v, omega) with respect to (v0, omega0)."""
    rows = [np.hstack([blocks[f"{k}_v0"], blocks[f"{k}_w0"]]) for k in ("x", "q", "v", "w")]
    return np.vstack(rows)


def test_contact_forward_fp64_matches_oracle():
    sc = scn.two_sphere_contact()
    g, o = DiffDFSPH(sc), oracle.Oracle(sc, mode=oracle.MODE_F64)
    seen_force = False
    for _ in range(20):
        g.step(1)
        o.step(1)
        assert g.contact_count() == o.contact_count()
        seen_force |= g.contact_count()[1] > 0
        for b in DYN:
            for a, c in zip(g.rigid_state(b), o.rigid_state(b)):
                np.testing.assert_allclose(a, c, rtol=1e-8, atol=1e-10)
    assert seen_force


def test_contact_pushes_the_spheres_apart():
    sc = scn.two_sphere_contact(speed=0.5)
    g = DiffDFSPH(sc)
    g.step(3)
    v1, v2 = g.rigid_state(1)[2], g.rigid_state(2)[2]
    assert v1[0] < 0.0 < v2[0]  # they started towards each other at 0.5 m/s


def test_manager_chain_and_blocks_match_oracle():
    sc = scn.two_sphere_contact()
    g, o = DiffDFSPH(sc), oracle.Oracle(sc, mode=oracle.MODE_F64)
    g.step(12)
    o.step(12)
    for R in DYN:
        for RR in DYN:
            a, b = g.manager_grad(R, RR), o.manager_grad(R, RR)
            assert np.all(np.isfinite(a))
            assert _rel(a, b) < 1e-6, (R, RR, _rel(a, b))
            ja, jb = g.manager_jacobians(R, RR), o.manager_jacobians(R, RR)
            assert _rel(ja, jb) < 1e-6, (R, RR, _rel(ja, jb))
    # the cross blocks are what couples the bodies
    assert np.linalg.norm(g.manager_grad(2, 1)[0:9]) > 0.0


def test_manager_without_contact_matches_oracle():
    sc = scn.small_contact_scene().replace_params(use_rigid_gradient_manager=1)
    g, o = DiffDFSPH(sc), oracle.Oracle(sc, mode=oracle.MODE_F64)
    g.step(10)
    o.step(10)
    assert _rel(g.manager_grad(1, 1), o.manager_grad(1, 1)) < 1e-7
    assert g.contact_count() == (0, 0)


def test_release_mode_with_contact_matches_oracle():
    # body 1 is held (animated, zero velocity) for the first 5 ms, then released with its
    # initial velocities; the contact solver still adds gravity and contact forces to it
    sc = scn.two_sphere_contact(release=True, uat=0.005)
    g, o = DiffDFSPH(sc), oracle.Oracle(sc, mode=oracle.MODE_F64)
    for _ in range(12):
        g.step(1)
        o.step(1)
        for b in DYN:
            for a, c in zip(g.rigid_state(b), o.rigid_state(b)):
                np.testing.assert_allclose(a, c, rtol=1e-8, atol=1e-10)
    for R in DYN:
        for RR in DYN:
            assert _rel(g.manager_grad(R, RR), o.manager_grad(R, RR)) < 1e-6


def test_contact_fp32_fluid_matches_mixed_oracle():
    sc = scn.two_sphere_contact(precision=scn._abi.DFSPH_FP32)
    g, o = DiffDFSPH(sc), oracle.Oracle(sc, mode=oracle.MODE_MIXED)
    for _ in range(8):
        g.step(1)
        o.step(1)
        for b in DYN:
            np.testing.assert_allclose(g.rigid_state(b)[2], o.rigid_state(b)[2], atol=2e-3)
            np.testing.assert_allclose(g.rigid_state(b)[0], o.rigid_state(b)[0], atol=1e-5)


def test_manager_adjoint_equals_forward_contraction():
    sc = scn.two_sphere_contact()
    g = DiffDFSPH(sc)
    g.step(15)
    rng = np.random.default_rng(7)
    dL = rng.normal(size=(3, 13))
    dL[0] = 0.0
    got = g.backward(dL)
    want = np.zeros((3, 6))
    for RR in DYN:
        for R in DYN:
            want[RR] += _chain_matrix(g.manager_grad_blocks(R, RR)).T @ dL[R]
    assert _rel(got[1:], want[1:]) < 1e-9


def test_manager_checkpointed_rollout_equals_direct():
    sc = scn.two_sphere_contact()
    sim = DiffDFSPH(sc)
    p0 = np.zeros((3, 6))
    for b in DYN:
        p0[b, :3] = sc.bodies[b].init_velocity
        p0[b, 3:] = sc.bodies[b].init_angular_velocity
    w = np.random.default_rng(3).normal(size=(3, 13))
    w[:2] = 0.0  # a loss on body 2 only: its gradient with respect to body 1 is the cross term
    w = torch.tensor(w)
    grads, finals = [], []
    for ck in (None, 5):
        p = torch.tensor(p0, requires_grad=True)
        out = rollout(sim, p, 15, checkpoint_every=ck)
        (out * w).sum().backward()
        grads.append(p.grad.numpy().copy())
        finals.append(out.detach().numpy().copy())
    np.testing.assert_array_equal(finals[0], finals[1])
    assert _rel(grads[1], grads[0]) < 1e-12
    assert np.abs(grads[0][1, :3]).max() > 0.0


def test_many_contact_samples_without_fluid_matches_oracle():
    """A large sphere on the floor of an empty container: several hundred force-carrying
    samples on one body (the sequential application is staged in chunks), no fluid stage in
    the manager chain; rigid state and the manager's chain state against the oracle."""
    sc = scn.sphere_on_floor()
    g, o = DiffDFSPH(sc), oracle.Oracle(sc, mode=oracle.MODE_F64)
    for _ in range(10):
        g.step(1)
        o.step(1)
        assert g.contact_count() == o.contact_count()
        for a, c in zip(g.rigid_state(1), o.rigid_state(1)):
            np.testing.assert_allclose(a, c, rtol=1e-8, atol=1e-10)
    assert g.contact_count()[1] > 256
    assert _rel(g.manager_grad(1, 1), o.manager_grad(1, 1)) < 1e-6


def test_manager_and_contact_api_errors():
    """The manager getters answer DFSPH_ERR_UNSUPPORTED when the manager is off and
    DFSPH_ERR_INVALID_ARG for a body index out of range or a NULL output; without the
    contact solver the contact counts are zero."""
    import ctypes
    from difffr_gb300 import _abi
    plain = DiffDFSPH(scn.small_contact_scene())
    plain.step(1)
    out = (ctypes.c_double * 78)()
    assert plain.lib.dfsph_get_manager_grad(plain.h, 1, 1, out) == _abi.DFSPH_ERR_UNSUPPORTED
    assert plain.lib.dfsph_get_manager_jacobians(plain.h, 1, 1, out) == _abi.DFSPH_ERR_UNSUPPORTED
    assert plain.contact_count() == (0, 0)
    g = DiffDFSPH(scn.two_sphere_contact())
    g.step(1)
    assert g.lib.dfsph_get_manager_grad(g.h, 3, 1, out) == _abi.DFSPH_ERR_INVALID_ARG
    assert g.lib.dfsph_get_manager_grad(g.h, 1, -1, out) == _abi.DFSPH_ERR_INVALID_ARG
    assert g.lib.dfsph_get_manager_jacobians(g.h, 1, 1, None) == _abi.DFSPH_ERR_INVALID_ARG
    assert g.lib.dfsph_get_contact_count(g.h, None, None) == _abi.DFSPH_ERR_INVALID_ARG


def test_overlapped_steps_equal_single_steps():
    """One call of 12 steps (the contact pass beside the pressure solve, the manager's
    kernels beside the next step's fluid work) equals 12 calls of one step (each ending with
    both streams synchronised): rigid states, contact counts and the manager's chain state
    and blocks, bit for bit."""
    sc = scn.two_sphere_contact()
    a, b = DiffDFSPH(sc), DiffDFSPH(sc)
    a.step(12)
    for _ in range(12):
        b.step(1)
    assert a.contact_count() == b.contact_count()
    for body in DYN:
        for u, v in zip(a.rigid_state(body), b.rigid_state(body)):
            np.testing.assert_array_equal(u, v)
        for RR in DYN:
            np.testing.assert_array_equal(a.manager_grad(body, RR), b.manager_grad(body, RR))
            np.testing.assert_array_equal(a.manager_jacobians(body, RR), b.manager_jacobians(body, RR))
