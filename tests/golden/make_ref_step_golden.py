"""Generates the step-level golden vectors from the reference's own DiffDFSPH step.

oracle/build_ref_step.sh compiles the reference's TimeStepDiffDFSPH, BoundaryModel_Akinci2012,
Simulation, FluidModel, kernel and viscosity sources (where they lie in a DiffFR checkout)
together with oracle/ref_step.cpp into oracle/_ref/ref_step_{double,float}. This script runs
them on small seeded scenes and stores, per step, the sweep counts and every dynamic body's
state, fluid force and torque and gradient chain state, and after the last step the fluid
fields and the boundary volumes, in tests/golden/reference_step.npz. Run in a container that
has the reference checkout:

    sh oracle/build_ref_step.sh /path/to/DiffFR && python tests/golden/make_ref_step_golden.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from difffr_gb300 import _abi  # noqa: E402
from difffr_gb300 import scene as scn  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
OUT = os.path.join(HERE, "reference_step.npz")
PER_BODY = 3 + 4 + 3 + 3 + 3 + 3 + 78  # x, q, v, omega, force, torque, chain state
FLUID_COLS = 14                        # x[3], v[3], rho, factor, kappa, kappa_v, rho_adv, sum_grad_p_k[3]

# name -> (scene constructor keyword arguments, parameter overrides, steps, build); the fluid
# fields after the last step are kept for the cases in FLUID_CASES
FLUID_CASES = ("contact_complete_fp64", "contact_incomplete_fp32")
CASES = {
    "contact_complete_fp64": (dict(precision=_abi.DFSPH_FP64, gradient_mode=_abi.GRAD_COMPLETE), {}, 10, "double"),
    "contact_incomplete_fp64": (dict(precision=_abi.DFSPH_FP64, gradient_mode=_abi.GRAD_INCOMPLETE), {}, 10, "double"),
    "contact_rigid_only_fp64": (dict(precision=_abi.DFSPH_FP64, gradient_mode=_abi.GRAD_RIGID_ONLY), {}, 10, "double"),
    "contact_release_fp64": (dict(precision=_abi.DFSPH_FP64, gradient_mode=_abi.GRAD_COMPLETE),
                             dict(release_rigid_body_mode=1, uniform_accelerate_rb_time=0.003), 10, "double"),
    "contact_incomplete_fp32": (dict(precision=_abi.DFSPH_FP32, gradient_mode=_abi.GRAD_INCOMPLETE), {}, 10, "float"),
}


def make_scene(kw, overrides):
    sc = scn.small_contact_scene(**kw)
    return sc.replace_params(**overrides) if overrides else sc


def write_input(sc, steps, path):
    p = sc.params
    head = [1, p.particle_radius, p.time_step, p.density0, p.viscosity, *p.gravity, p.max_error, p.max_error_v,
            p.min_iterations, p.max_iterations, p.max_iterations_v, p.gradient_mode, p.enable_divergence_solver,
            p.use_pressure_warmstart, p.use_divergence_warmstart, p.release_rigid_body_mode,
            p.uniform_accelerate_rb_time, p.target_time, p.optimize_rotation, steps, sc.n_fluid, len(sc.bodies)]
    parts = [np.array(head, np.float64), np.asarray(sc.fluid_x, np.float64).ravel(),
             np.asarray(sc.fluid_v, np.float64).ravel()]
    for b in sc.bodies:
        parts.append(np.array([int(b.is_dynamic), int(b.is_animated), b.density, *b.translation, *b.rotation,
                               *b.init_velocity, *b.init_angular_velocity, b.samples.shape[0]], np.float64))
        parts.append(np.asarray(b.samples, np.float64).ravel())
    np.concatenate(parts).tofile(path)


def run_reference(sc, steps, build):
    """Runs the reference step; returns (per-step rows, fluid fields, boundary volumes)."""
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_input(sc, steps, fin)
        subprocess.run([os.path.join(REF, f"ref_step_{build}"), fin, fout], check=True, stdout=subprocess.DEVNULL)
        d = np.fromfile(fout, np.float64)
    nb = len(sc.bodies)
    per = 2 + nb * PER_BODY
    n = sc.n_fluid
    expected = steps * per + n * FLUID_COLS + sc.n_boundary
    if d.size != expected:
        raise RuntimeError(f"reference run wrote {d.size} values, expected {expected}")
    rows = d[:steps * per].reshape(steps, per)
    fluid = d[steps * per:steps * per + n * FLUID_COLS].reshape(n, FLUID_COLS)
    psi = d[steps * per + n * FLUID_COLS:]
    return rows, fluid, psi


def main():
    out = {}
    meta = {}
    for name, (kw, ov, steps, build) in CASES.items():
        sc = make_scene(kw, ov)
        rows, fluid, psi = run_reference(sc, steps, build)
        out[name + "/rows"] = rows
        if name in FLUID_CASES:
            out[name + "/fluid"] = fluid
            out[name + "/psi"] = psi
        meta[name] = {"scene": "small_contact_scene", "kwargs": kw, "overrides": ov, "steps": steps, "build": build,
                      "n_bodies": len(sc.bodies)}
        print(name, rows.shape, fluid.shape, psi.shape)
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT))


if __name__ == "__main__":
    main()
