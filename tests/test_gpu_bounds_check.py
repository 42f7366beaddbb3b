"""The bounds-checked build (-DDFSPH_BOUNDS_CHECK, difffr_gb300/libdfsph_boundscheck.so) on
small scenes against the oracle: every neighbour index the kernels read from a list, and
every cell range they walk, is checked before use, and a bad one would end the step with
DFSPH_ERR_DEVICE. On these scenes no check fires and the results equal the oracle's as the
regular build's do (FP64 fields and rigid state within 1e-9 relative, equal sweep counts)."""
import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bounds_lib(gpu_lib):
    from difffr_gb300 import build
    return build.build(bounds_check=True)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)


@pytest.mark.parametrize("name", ["contact_complete", "two_sphere_contact", "surface_tension"])
def test_bounds_checked_build_matches_oracle(bounds_lib, oracle_lib, name):
    from difffr_gb300.sim import DiffDFSPH
    if name == "contact_complete":
        sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64, gradient_mode=_abi.GRAD_COMPLETE)
    elif name == "two_sphere_contact":
        sc = scn.two_sphere_contact(precision=_abi.DFSPH_FP64)
    else:
        sc = scn.small_contact_scene(precision=_abi.DFSPH_FP64).replace_params(surface_tension_method=2,
                                                                                surface_tension=0.5)
    assert sc.n_fluid + sc.n_boundary <= 8192
    sim = DiffDFSPH(sc, lib_path=bounds_lib)
    ref = oracle_lib.Oracle(sc)
    for _ in range(8):
        sg, sr = sim.step(1), ref.step(1)
        assert sg["pressure_iterations"] == sr["pressure_iterations"]
        assert sg["divergence_iterations"] == sr["divergence_iterations"]
    for f in (_abi.FIELD_X, _abi.FIELD_V, _abi.FIELD_DENSITY, _abi.FIELD_KAPPA):
        assert rel(sim.field(f), ref.field(f)) < 1e-9, f
    for b, body in enumerate(sc.bodies):
        if body.is_dynamic:
            for a, c in zip(sim.rigid_state(b), ref.rigid_state(b)):
                assert np.allclose(a, c, rtol=1e-8, atol=1e-11)
    sim.close()
