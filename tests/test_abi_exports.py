"""libdfsph.so loads and exports every entry point declared in include/dfsph.h (no GPU calls)."""
import ctypes
import os
import re

from difffr_gb300 import _abi, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "dfsph.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dfsph_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_all_declared_symbols():
    build.build()
    lib = ctypes.CDLL(_abi.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(_abi.EXPORTED_SYMBOLS)


def test_struct_layouts_match_header():
    lib = _abi.load_library()
    p = _abi.DfsphParams()
    assert lib.dfsph_default_params(ctypes.byref(p)) == 0
    assert p.struct_size == ctypes.sizeof(_abi.DfsphParams)
    assert p.min_iterations == 2 and p.max_iterations == 100
    assert abs(p.max_error - 0.01) < 1e-15 and abs(p.max_error_v - 0.1) < 1e-15
    assert p.gradient_mode == _abi.GRAD_INCOMPLETE and p.optimize_rotation == 1
    assert lib.dfsph_abi_version() == 1


def test_defaults_match_python_params():
    from difffr_gb300.scene import Params
    lib = _abi.load_library()
    p = _abi.DfsphParams()
    lib.dfsph_default_params(ctypes.byref(p))
    q = Params()
    for name, _ in _abi.DfsphParams._fields_:
        if name in ("struct_size", "gravity", "max_fluid_neighbors", "max_boundary_neighbors"):
            continue
        assert abs(getattr(p, name) - getattr(q, name)) < 1e-12, name


def test_null_arguments_are_rejected_without_device_work():
    lib = _abi.load_library()
    assert lib.dfsph_default_params(None) == _abi.DFSPH_ERR_INVALID_ARG
    assert lib.dfsph_step(None, 1, None) == _abi.DFSPH_ERR_INVALID_ARG
    out = (ctypes.c_double * 78)()
    assert lib.dfsph_get_manager_grad(None, 0, 0, out) == _abi.DFSPH_ERR_INVALID_ARG
    assert lib.dfsph_get_manager_jacobians(None, 0, 0, out) == _abi.DFSPH_ERR_INVALID_ARG
    nc, na = ctypes.c_int64(), ctypes.c_int64()
    assert lib.dfsph_get_contact_count(None, ctypes.byref(nc), ctypes.byref(na)) == _abi.DFSPH_ERR_INVALID_ARG
    assert b"NULL" in lib.dfsph_last_error()
    assert lib.dfsph_destroy(None) == 0
