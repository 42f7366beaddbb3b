"""Validation at the benchmark scenes' sizes on the GPU (a few seconds each).

- the 4M-particle basin scene scaled to 256k particles: gradient of a fixed weighting of
  the final rigid states with respect to the 12 initial velocities, GPU autograd against
  the oracle's forward chain (FP32 fluid / FP64 rigid in both): cosine >= 0.999 per body;
  rigid positions within 1e-3 relative after 20 steps;
- the 250k pool with the ellipsoid: a 1000-step adjoint with a device checkpoint every 50
  steps equals the direct schedule (bit-identical forward states, gradients to 1e-12).
"""
import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn

pytestmark = pytest.mark.gpu


def test_billiards_downscaled_gradient_matches_oracle(gpu_lib, oracle_lib):
    import torch
    from difffr_gb300.autograd import rollout
    from difffr_gb300.sim import DiffDFSPH
    from difffr_gb300.validate import _init_params
    steps = 20
    sc = scn.billiards_on_water(n=(80, 40, 80), r=0.00625, enable_gradient=1, gradient_mode=_abi.GRAD_COMPLETE)
    sim = DiffDFSPH(sc)
    p0 = _init_params(sim)
    p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    out = rollout(sim, p, steps)
    rng = np.random.default_rng(11)
    wts = rng.normal(size=(sim.n_bodies, 13))
    (out * torch.as_tensor(wts)).sum().backward()
    g = p.grad.numpy()
    ref = oracle_lib.Oracle(sc, mode=oracle_lib.MODE_MIXED)
    for b in range(sim.n_bodies):
        ref.set_rigid_init(b, p0[b, :3], p0[b, 3:])
    ref.step(steps)
    for b in (2, 3):
        blk = ref.rigid_grad_blocks(b)
        Gv = np.vstack([blk["x_v0"], blk["q_v0"], blk["v_v0"], blk["w_v0"]])
        Gw = np.vstack([blk["x_w0"], blk["q_w0"], blk["v_w0"], blk["w_w0"]])
        rg = np.concatenate([wts[b] @ Gv, wts[b] @ Gw])
        cos = float(rg @ g[b] / (np.linalg.norm(rg) * np.linalg.norm(g[b])))
        assert cos >= 0.999, (b, cos)
        sx = sim.rigid_state(b)[0]
        ox = ref.rigid_state(b)[0]
        assert np.linalg.norm(sx - ox) <= 1e-3 * np.linalg.norm(ox)
    sim.close()


def test_pool_thousand_step_checkpointed_adjoint():
    pytest.importorskip("torch")
    from difffr_gb300.validate import pool_adjoint
    r = pool_adjoint(steps=1000, every=50, fd=False)
    assert r["forward_identical"]
    assert r["max_rel_grad_diff_checkpointed_vs_direct"] <= 1e-12
    assert np.all(np.isfinite(r["grad"]))


def test_config0_fp64_trajectory_matches_oracle(gpu_lib, oracle_lib):
    """The reference's CPU-runnable configuration (8k particles, FP64, sphere dropped into
    the tank with v = (0.5, 0, 0), omega = (0, 1, 0)), 200 steps: rigid state within 1e-6
    relative of the FP64 oracle and the gradient blocks (forward chain) with cosine
    >= 0.9999 per block; the same pressure and divergence sweep counts."""
    from difffr_gb300.sim import DiffDFSPH
    sc = scn.config0(precision=_abi.DFSPH_FP64, enable_gradient=1)
    steps = 200
    gpu, ref = DiffDFSPH(sc), oracle_lib.Oracle(sc)
    tot_g = tot_r = 0
    for _ in range(steps):
        sg = gpu.step(1)
        sr = ref.step(1)
        tot_g += sg["pressure_iterations"] + sg["divergence_iterations"]
        tot_r += sr["pressure_iterations"] + sr["divergence_iterations"]
    assert tot_g == tot_r
    for a, r in zip(gpu.rigid_state(1), ref.rigid_state(1)):
        assert np.max(np.abs(a - r)) <= 1e-6 * max(np.max(np.abs(r)), 1e-3), (a, r)
    bg, br = gpu.rigid_grad_blocks(1), ref.rigid_grad_blocks(1)
    for k in bg:
        u, v = bg[k].ravel(), br[k].ravel()
        if np.linalg.norm(v) < 1e-12:  # a block the gradient mode leaves at zero
            assert np.linalg.norm(u) < 1e-12, (k, u)
            continue
        cos = float(u @ v / (np.linalg.norm(u) * np.linalg.norm(v)))
        assert cos >= 0.9999, (k, cos)
    gpu.close()
