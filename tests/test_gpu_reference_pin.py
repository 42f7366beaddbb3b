"""The GPU library against the reference's own DiffDFSPH step, directly.

tests/golden/reference_step.npz holds what the reference's step (its sources compiled by
oracle/build_ref_step.sh, the fixtures made by tests/golden/make_ref_step_golden.py)
produced on small contact scenes, in all three gradient modes and in release mode. Through
the C ABI, the GPU library's FP64 build reproduces it within 1e-9 relative per step (rigid
state, fluid force and torque, gradient chain state) and in the fluid fields, with the same
sweep counts. Against the reference's float build, the GPU's FP32 fluid / FP64 rigid split
agrees within FP32 tolerances (fields 1e-4 of their maximum, rigid state 1e-4, force and
chain state 2e-2 after 10 steps: the reference integrates the bodies in FP32 as well).
The same FP32 / FP64 split against the reference's FP64 build states the split's own error
(what running the fluid in FP32 costs) on every double-build case.
"""
import pytest

import ref_step_fixture as rsf

pytestmark = pytest.mark.gpu

_GOLD, _META = rsf.load()


@pytest.mark.parametrize("case", sorted(_META))
def test_gpu_step_matches_reference_step(gpu_lib, case):
    from difffr_gb300.sim import DiffDFSPH
    m = _META[case]
    sc = rsf.scene_of(m)
    sim = DiffDFSPH(sc)
    worst, iters_equal = rsf.compare(sim, sc, _GOLD, case, m["steps"])
    print(case, {k: f"{v:.2e}" for k, v in worst.items()})
    assert iters_equal
    if m["build"] == "double":
        bad = {k: v for k, v in worst.items() if v > 1e-9}
    else:
        tol = {"x": 1e-4, "q": 1e-4, "v": 1e-3, "omega": 1e-3, "force": 2e-2, "torque": 2e-2, "grad": 2e-2}
        bad = {k: v for k, v in worst.items() if v > tol.get(k, 1e-4)}
    assert not bad, (case, bad)
    sim.close()


_DOUBLE_CASES = sorted(c for c, m in _META.items() if m["build"] == "double")


@pytest.mark.parametrize("case", _DOUBLE_CASES)
def test_fp32_split_against_reference_fp64_build(gpu_lib, case):
    """The GPU's FP32 fluid / FP64 rigid build on the double-build cases: the error against
    the reference's FP64 run, printed per quantity and bounded at FP32 tolerances (sweep
    counts may differ by a sweep where the FP32 residual crosses the tolerance)."""
    from difffr_gb300 import _abi
    from difffr_gb300 import scene as scn
    from difffr_gb300.sim import DiffDFSPH
    m = _META[case]
    kw = dict(m["kwargs"], precision=_abi.DFSPH_FP32)
    sc = scn.small_contact_scene(**kw)
    sc = sc.replace_params(**m["overrides"]) if m["overrides"] else sc
    sim = DiffDFSPH(sc)
    worst, iters_equal = rsf.compare(sim, sc, _GOLD, case, m["steps"])
    print("fp32 split vs reference fp64", case, "sweeps equal" if iters_equal else "sweeps differ",
          {k: f"{v:.2e}" for k, v in worst.items()})
    tol = {"x": 1e-4, "q": 1e-4, "v": 1e-3, "omega": 1e-3, "force": 2e-2, "torque": 2e-2, "grad": 2e-2}
    bad = {k: v for k, v in worst.items() if v > tol.get(k, 1e-3)}
    assert not bad, (case, bad)
    sim.close()

