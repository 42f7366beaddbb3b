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


def _noalloc(lib, d, precision, n, pressure_mode, out):
    rc = lib.dfsph_density_error_noalloc(ctypes.c_void_p(d.data_ptr()), precision, n, 1000.0, pressure_mode,
                                         ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.dfsph_last_error()


@pytest.mark.parametrize("precision", [_abi.DFSPH_FP32, _abi.DFSPH_FP64])
@pytest.mark.parametrize("pressure_mode", [1, 0])
@pytest.mark.parametrize("n", [1_000_003, 4_194_304])
def test_noalloc_many_blocks_against_float64_mean(gpu_lib, precision, pressure_mode, n):
    """More partials than the final block has threads (its strided loop), up to the largest
    accepted size, in both precisions and both modes, against numpy's float64 mean of the
    same per-value terms formed in the input's precision; twice in a row on the shared
    scratch. Tolerance: 1e-9 relative in FP64; 1e-6 in FP32, where the compiler may form
    rho0 * r - rho0 with one rounding (a fused multiply-add) or two, a difference of up to
    half an FP32 ulp of 1000 per value."""
    import torch
    lib = _abi.load_library()
    rng = np.random.default_rng(n + 7 * pressure_mode + precision)
    ra = 1.0 + 0.01 * rng.random(n)
    dt = np.float32 if precision == _abi.DFSPH_FP32 else np.float64
    ra = ra.astype(dt)
    rho0 = dt(1000.0)
    terms = (rho0 * ra - rho0) if pressure_mode else (rho0 * ra)
    want = float(np.mean(terms.astype(np.float64)))
    d = torch.tensor(ra, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        out.fill_(0.0)
        torch.cuda.synchronize()
        _noalloc(lib, d, precision, n, pressure_mode, out)
        torch.cuda.synchronize()
        tol = 1e-6 if precision == _abi.DFSPH_FP32 else 1e-9
        assert float(out.item()) == pytest.approx(want, rel=tol, abs=1e-12)
