"""dfsph_density_error_noalloc: the allocation-free density-error reduction.

Callers that cannot allocate GPU memory at the point of use pass their own input and
output buffers; the entry point's only scratch is a static device array. This checks,
through the C ABI and on two calls in a row, that it returns the same average density
error the solver reports for the same rho_adv values (relative tolerance 1e-9: the
library reduces in cell-sorted order, this test passes the field in particle order).
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn

pytestmark = pytest.mark.gpu


def compressed_block():
    """A fluid block packed at 0.9 of the rest spacing, so the pressure solve has work."""
    rng = np.random.default_rng(5)
    r = 0.025
    n = (12, 12, 12)
    fx = scn.fluid_lattice(n, 1.8 * r, (2 * r, 2 * r, 2 * r), r, rng)
    walls = scn.box_surface((0.0, 0.0, 0.0), (0.7, 0.7, 0.7), 2 * r)
    params = scn.Params(fluid_precision=_abi.DFSPH_FP32, particle_radius=r, time_step=0.001)
    return scn.Scene(params=params, fluid_x=fx, fluid_v=np.zeros_like(fx), bodies=[scn.Body(samples=walls)])


def test_noalloc_density_error_matches_solver(gpu_lib):
    import torch
    from difffr_gb300.sim import DiffDFSPH

    sim = DiffDFSPH(compressed_block())
    lib = _abi.load_library()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for call in range(2):
        st = sim.step(1)
        rho_adv = sim.field(_abi.FIELD_DENSITY_ADV)
        d_ra = torch.tensor(rho_adv, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.dfsph_density_error_noalloc(ctypes.c_void_p(d_ra.data_ptr()), _abi.DFSPH_FP32, d_ra.numel(),
                                             1000.0, 1, ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.dfsph_last_error()
        torch.cuda.synchronize()
        got = float(out.item())
        want = st["pressure_avg_error"]
        assert abs(want) > 1e-6, "the scene should leave a nonzero density error"
        assert got == pytest.approx(want, rel=1e-9, abs=1e-12), (call, got, want)


def test_noalloc_rejects_oversized_input(gpu_lib):
    lib = _abi.load_library()
    rc = lib.dfsph_density_error_noalloc(ctypes.c_void_p(16), _abi.DFSPH_FP32, 4_194_305, 1000.0, 1,
                                         ctypes.c_void_p(16), None)
    assert rc == _abi.DFSPH_ERR_INVALID_ARG
    assert b"4,194,304" in lib.dfsph_last_error()
