"""Trains the learned pressure warm start on the 1M-particle dam break and evaluates it.

    python -m difffr_gb300.train_warmstart [--out PATH] [--eval-seeds 1 2 3 4] [--summary PATH]

Protocol: the seed-0 scene runs `--start` plain steps (the reference warm start) to reach
the collapse phase, then `--record` more plain steps whose (features, final stiffness)
samples form the training set. The model (MLP 4 -> 64 -> 64 -> 1) is trained with the
library's tensor-core kernels (Adam, shuffled minibatches). Evaluation: each evaluation
seed runs `--start` plain steps, saves a device checkpoint, then runs `--eval-steps` steps
with the reference warm start and, from the same checkpoint, with the learned one; both
solve to the same tolerance. Reported per seed: pressure iterations per step,
pressure-solve device time per step, step time and the final average density error.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(HERE, "data", "warmstart_dam_break_1M.npz")


def run_window(sim, steps, model=None):
    """`steps` steps from the current state with the given warm start; device timings."""
    sim.set_warmstart_model(model)
    sim.profile_enable(True)
    its, errs = [], []
    sim.synchronize()
    sim.record_event(0)
    for _ in range(steps):
        st = sim.step(1)
        its.append(st["pressure_iterations"])
        errs.append(st["pressure_avg_error"])
    sim.record_event(1)
    ms = sim.event_elapsed_ms(0, 1)
    prof = sim.profile()
    sim.profile_enable(False)
    sim.set_warmstart_model(None)
    return {
        "pressure_iterations_per_step": float(np.mean(its)),
        "pressure_solve_ms_per_step": prof["pressure_solve"]["ms"] / steps,
        "step_ms": ms / steps,
        "avg_density_error": float(np.mean(errs)),
        "max_density_error": float(np.max(errs)),
        "mlp_ms_per_step": prof["mlp"]["ms"] / steps,
    }


def evaluate(model, seed, start, steps, n=(100, 100, 100)):
    from . import scene as scn
    from .sim import DiffDFSPH
    sim = DiffDFSPH(scn.dam_break_sphere(n=n, seed=seed, enable_gradient=0))
    sim.step(start)
    slot = sim.checkpoint_save()
    plain = run_window(sim, steps, None)
    sim.checkpoint_restore(slot)
    learned = run_window(sim, steps, model)
    sim.checkpoint_free(slot)
    sim.close()
    cut = 1.0 - learned["pressure_solve_ms_per_step"] / plain["pressure_solve_ms_per_step"]
    return {"seed": seed, "plain": plain, "learned": learned, "pressure_solve_time_cut": cut}


def train_model(seed=0, start=300, record=200, epochs=3, batch=65536, lr=2e-3, lr_final=1e-4, n=(100, 100, 100)):
    from . import scene as scn
    from .sim import DiffDFSPH
    from .warmstart import WarmStartModel, collect_samples, train
    sim = DiffDFSPH(scn.dam_break_sphere(n=n, seed=seed, enable_gradient=0))
    sim.step(start)
    x, y = collect_samples(sim, record)
    sim.close()
    model = WarmStartModel(seed=seed)
    t0 = time.perf_counter()
    losses = train(model, x, y, epochs=epochs, batch=batch, lr=lr, lr_final=lr_final, seed=seed)
    info = {"samples": int(x.shape[0]), "epochs": epochs, "batch": batch, "losses": losses,
            "train_s": time.perf_counter() - t0}
    return model, info


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_MODEL)
    ap.add_argument("--start", type=int, default=300)
    ap.add_argument("--record", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--eval-seeds", type=int, nargs="*", default=[1, 2, 3, 4])
    ap.add_argument("--eval-steps", type=int, default=200)
    ap.add_argument("--summary", default="")
    args = ap.parse_args()
    model, info = train_model(start=args.start, record=args.record, epochs=args.epochs)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    model.save(args.out)
    res = {"training": info, "model": os.path.basename(args.out), "evaluation": []}
    for s in args.eval_seeds:
        r = evaluate(model, s, args.start, args.eval_steps)
        res["evaluation"].append(r)
        print(json.dumps(r), flush=True)
    if args.eval_seeds:
        res["mean_pressure_solve_time_cut"] = float(np.mean([r["pressure_solve_time_cut"] for r in res["evaluation"]]))
    print(json.dumps({k: v for k, v in res.items() if k != "evaluation"}), flush=True)
    if args.summary:
        with open(args.summary, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
