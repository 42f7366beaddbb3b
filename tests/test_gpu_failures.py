"""Failure detection without a GPU fault: each failure is made on the host or by a bounded
wait that a test hook lets run out, and the call reports it through its status code while
the context stays usable.

- A non-finite particle position uploaded from the host: the sort kernel sets the
  non-finite bit of the device error word, the step returns DFSPH_ERR_DEVICE, and a reset
  (which restores the initial state and clears the word) runs clean.
- A solve capped at one sweep (max_iterations = 1): DFSPH_ERR_NOT_CONVERGED with a finite,
  valid state, and the context keeps stepping.
- The learned warm start's tensor-core wait given no polls (dfsph_mlp_set_wait_limit): the
  kernel records the timeout, waits for its product with the regular limit, frees its
  tensor memory and returns; prediction and the solver's warm start report
  DFSPH_ERR_DEVICE, and with the regular limit restored both run again with the same
  results as before.
"""
import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn

pytestmark = pytest.mark.gpu


def test_nonfinite_position_reports_device_error(gpu_lib):
    from difffr_gb300.sim import DiffDFSPH
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32)
    sim = DiffDFSPH(sc)
    sim.step(2)
    x = sim.positions()
    x[5] = np.nan
    sim.set_field(_abi.FIELD_X, x)
    with pytest.raises(_abi.DfsphError) as e:
        sim.step(1)
    assert e.value.code == _abi.DFSPH_ERR_DEVICE and "non-finite" in str(e.value)
    sim.reset()
    st = sim.step(3)
    assert st["rc"] == 0 and np.all(np.isfinite(sim.positions()))
    ref = DiffDFSPH(sc)
    ref.step(3)
    assert np.array_equal(sim.positions(), ref.positions())
    sim.close()
    ref.close()


def test_nonfinite_initial_state_reports_device_error(gpu_lib):
    from difffr_gb300.sim import DiffDFSPH
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64)
    sc.fluid_x = sc.fluid_x.copy()
    sc.fluid_x[0, 1] = np.inf
    sim = DiffDFSPH(sc)
    with pytest.raises(_abi.DfsphError) as e:
        sim.step(1)
    assert e.value.code == _abi.DFSPH_ERR_DEVICE and "non-finite" in str(e.value)
    sim.close()


def test_iteration_cap_reports_not_converged_with_valid_state(gpu_lib):
    from difffr_gb300.sim import DiffDFSPH
    sc = scn.small_contact_scene(precision=_abi.DFSPH_FP32).replace_params(max_iterations=1, min_iterations=1)
    sim = DiffDFSPH(sc)
    sim.step(3)
    with pytest.raises(_abi.DfsphError) as e:
        sim.step(1, allow_not_converged=False)
    assert e.value.code == _abi.DFSPH_ERR_NOT_CONVERGED
    st = sim.step(1)
    assert st["rc"] == _abi.DFSPH_ERR_NOT_CONVERGED and st["pressure_iterations"] == 1
    assert np.all(np.isfinite(sim.positions())) and np.all(np.isfinite(sim.velocities()))
    for a in sim.rigid_state(1):
        assert np.all(np.isfinite(a))
    sim.close()


def test_mlp_wait_timeout_is_reported_and_recovers(gpu_lib):
    import torch
    from difffr_gb300.sim import DiffDFSPH
    from difffr_gb300.warmstart import WarmStartModel
    lib = gpu_lib
    m = WarmStartModel(seed=3)
    rng = np.random.default_rng(0)
    x = torch.tensor(rng.normal(size=(5000, 4)).astype(np.float32), device="cuda")
    y0 = m.predict(x).clone()
    _abi.check(lib, lib.dfsph_mlp_set_wait_limit(m.h, 0))
    with pytest.raises(_abi.DfsphError) as e:
        m.predict(x)
    assert e.value.code == _abi.DFSPH_ERR_DEVICE and "timed out" in str(e.value)
    _abi.check(lib, lib.dfsph_mlp_set_wait_limit(m.h, -1))
    assert torch.equal(m.predict(x), y0)

    # the same wait inside the solver's warm start, in the collapse phase (the kernel skips
    # tiles in which no particle has rho_adv > 1, so some must)
    sc = scn.dam_break_sphere(n=(16, 16, 16), r=0.01, box=(0.7, 0.45, 0.45), dt=0.001)
    sim = DiffDFSPH(sc)
    sim.step(100)
    _abi.check(lib, lib.dfsph_mlp_set_wait_limit(m.h, 0))
    sim.set_warmstart_model(m)
    with pytest.raises(_abi.DfsphError) as e:
        sim.step(1)
    assert e.value.code == _abi.DFSPH_ERR_DEVICE and "timed out" in str(e.value)
    _abi.check(lib, lib.dfsph_mlp_set_wait_limit(m.h, -1))
    sim.set_warmstart_model(m)
    sim.reset()
    sim.step(5)
    st = sim.step(2)
    assert st["rc"] in (0, _abi.DFSPH_ERR_NOT_CONVERGED)
    assert np.all(np.isfinite(sim.positions()))
    sim.set_warmstart_model(None)
    sim.close()
    m.close()
