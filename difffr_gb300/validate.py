"""Validation runs at the benchmark scenes' sizes (GPU), each returning a JSON-able dict.

    python -m difffr_gb300.validate [--out PATH] [--only NAME ...]

- ``pool_adjoint``: the 250k-particle pool with the ellipsoid, 1000 steps, loss =
  |x_T - x*|^2 + (geodesic angle between q_T and q*)^2, gradient with respect to the 6
  initial velocities through the autograd rollout with a device checkpoint every 50 steps,
  against the direct schedule (must agree) and central finite differences (eps = 1e-4).
- ``rollout_1M``: a 1000-step checkpointed adjoint rollout of the 1M dam break and the
  device memory it takes.
- ``billiards_4M``: the 4M-particle basin with two spheres and a static box: forward +
  adjoint steps per second and the gradient with respect to the 12 initial velocities.

The comparison of the 4M scene's gradient with the CPU oracle on a 256k-particle copy of
the scene is a test (tests/test_gpu_scale.py), since the oracle is test infrastructure.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np


def _init_params(sim):
    p = np.zeros((sim.n_bodies, 6))
    for b in range(sim.n_bodies):
        v, w = sim.rigid_init(b)
        p[b, :3], p[b, 3:] = v, w
    return p


def _loss_torch(final, body, x_t, q_t):
    import torch
    x = final[body, 0:3]
    q = final[body, 3:7]
    qt = torch.as_tensor(q_t, dtype=final.dtype)
    d = torch.clamp(torch.abs(torch.dot(q, qt)), max=1.0 - 1e-12)
    ang = 2.0 * torch.acos(d)
    return torch.sum((x - torch.as_tensor(x_t, dtype=final.dtype)) ** 2) + ang ** 2


def _forward_only(sim, p, steps):
    for b in range(sim.n_bodies):
        sim.set_rigid_init(b, p[b, :3], p[b, 3:])
    sim.set_gradient_enabled(False)
    sim.reset()
    sim.step(steps)
    return np.stack([sim.rigid_state_vector(b) for b in range(sim.n_bodies)])


def _seeded_target_quaternion(seed):
    rng = np.random.default_rng(seed)
    q = rng.normal(size=4)
    return q / np.linalg.norm(q)


def pool_adjoint(steps=1000, every=50, eps=1e-4, fd=True):
    import torch
    from . import scene as scn
    from .autograd import rollout
    from .sim import DiffDFSPH
    sc = scn.config2(enable_gradient=1)
    sim = DiffDFSPH(sc)
    body = 1
    x_t = np.asarray(sc.bodies[body].target_x)
    q_t = _seeded_target_quaternion(2024)
    p0 = _init_params(sim)
    res = {"scene": sc.name, "n_fluid": sim.n_fluid, "steps": steps, "checkpoint_every": every}
    grads = {}
    for name, k in (("checkpointed", every), ("direct", None)):
        p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
        t0 = time.perf_counter()
        out = rollout(sim, p, steps, checkpoint_every=k)
        loss = _loss_torch(out, body, x_t, q_t)
        loss.backward()
        res[f"{name}_s"] = time.perf_counter() - t0
        grads[name] = (out.detach().numpy(), p.grad.numpy()[body].copy(), float(loss.detach()))
    (oc, gc, lc), (od, gd, ld) = grads["checkpointed"], grads["direct"]
    res["forward_identical"] = bool(np.array_equal(oc, od))
    res["max_rel_grad_diff_checkpointed_vs_direct"] = float(np.max(np.abs(gc - gd)) / max(np.max(np.abs(gd)), 1e-300))
    res["loss"] = lc
    res["grad"] = gc.tolist()
    if fd:
        fdg = np.zeros(6)
        t0 = time.perf_counter()
        for c in range(6):
            vals = []
            for sgn in (1.0, -1.0):
                p = p0.copy()
                p[body, c] += sgn * eps
                out = torch.as_tensor(_forward_only(sim, p, steps))
                vals.append(float(_loss_torch(out, body, x_t, q_t)))
            fdg[c] = (vals[0] - vals[1]) / (2 * eps)
        res["fd_s"] = time.perf_counter() - t0
        res["fd_grad"] = fdg.tolist()
        res["cosine_vs_fd"] = float(gc @ fdg / (np.linalg.norm(gc) * np.linalg.norm(fdg) + 1e-300))
        res["cosine_vs_fd_velocity_block"] = float(gc[:3] @ fdg[:3] / (np.linalg.norm(gc[:3]) * np.linalg.norm(fdg[:3]) + 1e-300))
    sim.close()
    return res


def rollout_1M(steps=1000, every=50):
    import torch
    from . import scene as scn
    from .autograd import rollout
    from .sim import DiffDFSPH
    free0, total = torch.cuda.mem_get_info()
    sc = scn.config1(enable_gradient=1)
    sim = DiffDFSPH(sc)
    free1, _ = torch.cuda.mem_get_info()
    p = torch.tensor(_init_params(sim), dtype=torch.float64, requires_grad=True)
    t0 = time.perf_counter()
    out = rollout(sim, p, steps, checkpoint_every=every)
    free2, _ = torch.cuda.mem_get_info()
    out[1, 0:3].sum().backward()
    t1 = time.perf_counter()
    res = {"scene": sc.name, "n_fluid": sim.n_fluid, "steps": steps, "checkpoint_every": every,
           "context_bytes": int(free0 - free1), "checkpoint_bytes": int(free1 - free2),
           "device_total_bytes": int(total), "wall_s": t1 - t0,
           "grad_finite": bool(np.all(np.isfinite(p.grad.numpy()))), "grad_dx_dv0": p.grad.numpy()[1].tolist()}
    sim.close()
    return res


def billiards_4M(steps=20):
    import torch
    from . import scene as scn
    from .autograd import rollout
    from .sim import DiffDFSPH
    sc = scn.config4(enable_gradient=1)
    sim = DiffDFSPH(sc)
    sim.step(3)
    sim.reset()
    p = torch.tensor(_init_params(sim), dtype=torch.float64, requires_grad=True)
    sim.synchronize()
    t0 = time.perf_counter()
    out = rollout(sim, p, steps)
    out[2:, 0:3].sum().backward()
    sim.synchronize()
    dt = time.perf_counter() - t0
    g = p.grad.numpy()
    res = {"scene": sc.name, "n_fluid": sim.n_fluid, "n_boundary": sim.n_boundary, "steps": steps,
           "fwd_adjoint_steps_per_s_wall": steps / dt, "grad_finite": bool(np.all(np.isfinite(g))),
           "grad_bodies_2_3": g[2:].tolist()}
    sim.close()
    return res


RUNS = {"pool_adjoint": pool_adjoint, "rollout_1M": rollout_1M, "billiards_4M": billiards_4M}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="")
    ap.add_argument("--only", nargs="*", default=list(RUNS))
    args = ap.parse_args()
    res = {}
    for name in args.only:
        t0 = time.perf_counter()
        res[name] = RUNS[name]()
        res[name]["wall_total_s"] = time.perf_counter() - t0
        print(name, json.dumps(res[name])[:2000], flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
