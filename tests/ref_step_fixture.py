"""Reading tests/golden/reference_step.npz, the per-step outputs of the reference's own
DiffDFSPH step (tests/golden/make_ref_step_golden.py), and comparing a simulation with it.

Used by the oracle's pin (CPU) and by the GPU library's direct pin. A simulation is anything
with step(), rigid_state(b), rigid_force(b), rigid_grad(b) and field(f) (the oracle and
DiffDFSPH both are).
"""
import json
import os

import numpy as np

from difffr_gb300 import _abi

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_step.npz")
PER_BODY = 97
FLUID_FIELDS = ((_abi.FIELD_X, slice(0, 3)), (_abi.FIELD_V, slice(3, 6)), (_abi.FIELD_DENSITY, 6),
                (_abi.FIELD_FACTOR, 7), (_abi.FIELD_KAPPA, 8), (_abi.FIELD_KAPPA_V, 9),
                (_abi.FIELD_DENSITY_ADV, 10), (_abi.FIELD_SUM_GRAD_P, slice(11, 14)))


def load():
    g = np.load(GOLD)
    meta = json.loads(bytes(g["meta"]).decode())
    return g, meta


def scene_of(meta_case):
    from difffr_gb300 import scene as scn
    sc = scn.small_contact_scene(**meta_case["kwargs"])
    return sc.replace_params(**meta_case["overrides"]) if meta_case["overrides"] else sc


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def compare(sim, sc, g, name, steps):
    """Steps `sim` through the case and returns the largest relative difference from the
    reference per quantity, and whether every step's sweep counts were equal."""
    rows = g[name + "/rows"]
    worst = {}
    iters_equal = True
    for s in range(steps):
        st = sim.step(1)
        row = rows[s]
        iters_equal &= (st["pressure_iterations"], st["divergence_iterations"]) == (int(row[0]), int(row[1]))
        for b, body in enumerate(sc.bodies):
            if not body.is_dynamic:
                continue
            o = 2 + b * PER_BODY
            x, q, v, w = sim.rigid_state(b)
            F, T = sim.rigid_force(b)
            for k, mine, ref in (("x", x, row[o:o + 3]), ("q", q, row[o + 3:o + 7]), ("v", v, row[o + 7:o + 10]),
                                 ("omega", w, row[o + 10:o + 13]), ("force", F, row[o + 13:o + 16]),
                                 ("torque", T, row[o + 16:o + 19]), ("grad", sim.rigid_grad(b), row[o + 19:o + 97])):
                worst[k] = max(worst.get(k, 0.0), rel(mine, ref))
    if name + "/fluid" in g:
        fl = g[name + "/fluid"]
        for f, col in FLUID_FIELDS:
            ref = fl[:, col]
            worst[f"field{f}"] = rel(np.asarray(sim.field(f)).reshape(ref.shape), ref)
        worst["psi"] = rel(sim.field(_abi.FIELD_BOUNDARY_PSI), g[name + "/psi"])
    return worst, iters_equal
