"""ctypes mirror of include/dfsph.h and the loader of the CUDA library.

The library is built in-tree (``difffr_gb300/libdfsph.so``). Loading fails loudly
when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int32, c_int64, c_uint64, c_void_p

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdfsph.so")

DFSPH_OK = 0
DFSPH_ERR_INVALID_ARG = 1
DFSPH_ERR_CUDA = 2
DFSPH_ERR_NOT_CONVERGED = 3
DFSPH_ERR_DEVICE = 4
DFSPH_ERR_OUT_OF_MEMORY = 5
DFSPH_ERR_UNSUPPORTED = 6
DFSPH_ERR_STATE = 7

DFSPH_FP32 = 0
DFSPH_FP64 = 1
GRAD_COMPLETE, GRAD_INCOMPLETE, GRAD_RIGID_ONLY = 0, 1, 2
RB_GYROSCOPIC, RB_NO_GYROSCOPIC = 0, 1

FIELD_X, FIELD_V, FIELD_DENSITY, FIELD_FACTOR, FIELD_KAPPA, FIELD_KAPPA_V = 0, 1, 2, 3, 4, 5
FIELD_DENSITY_ADV, FIELD_SUM_GRAD_P = 6, 7
FIELD_BOUNDARY_X, FIELD_BOUNDARY_V, FIELD_BOUNDARY_PSI = 8, 9, 10
FIELD_COMPONENTS = {FIELD_X: 3, FIELD_V: 3, FIELD_SUM_GRAD_P: 3, FIELD_BOUNDARY_X: 3, FIELD_BOUNDARY_V: 3}
BOUNDARY_FIELDS = (FIELD_BOUNDARY_X, FIELD_BOUNDARY_V, FIELD_BOUNDARY_PSI)

NB_FLUID_FLUID, NB_FLUID_BOUNDARY, NB_BOUNDARY_FLUID = 0, 1, 2

MAX_BODIES = 16


class DfsphParams(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_int32),
        ("fluid_precision", c_int32),
        ("particle_radius", c_double),
        ("density0", c_double),
        ("viscosity", c_double),
        ("gravity", c_double * 3),
        ("time_step", c_double),
        ("min_iterations", c_int32),
        ("max_iterations", c_int32),
        ("max_error", c_double),
        ("max_iterations_v", c_int32),
        ("max_error_v", c_double),
        ("enable_divergence_solver", c_int32),
        ("use_pressure_warmstart", c_int32),
        ("use_divergence_warmstart", c_int32),
        ("gradient_mode", c_int32),
        ("rigid_body_mode", c_int32),
        ("optimize_rotation", c_int32),
        ("enable_gradient", c_int32),
        ("truncate_gradient_coeff", c_int32),
        ("release_rigid_body_mode", c_int32),
        ("uniform_accelerate_rb_time", c_double),
        ("target_time", c_double),
        ("max_fluid_neighbors", c_int32),
        ("max_boundary_neighbors", c_int32),
        ("surface_tension_method", c_int32),
        ("surface_tension", c_double),
        ("surface_tension_boundary", c_double),
        ("cfl_method", c_int32),
        ("cfl_factor", c_double),
        ("cfl_min_time_step", c_double),
        ("cfl_max_time_step", c_double),
        ("use_rigid_contact_solver", c_int32),
        ("use_rigid_gradient_manager", c_int32),
        ("rigid_contact_gamma", c_double),
        ("rigid_contact_beta", c_double),
        ("rigid_contact_support_radius_factor", c_double),
        ("rigid_contact_friction_coeff", c_double),
        ("viscosity_boundary", c_double),
    ]


class DfsphBodyDesc(ctypes.Structure):
    _fields_ = [
        ("is_dynamic", c_int32),
        ("is_animated", c_int32),
        ("n_samples", c_int64),
        ("samples", POINTER(c_double)),
        ("translation", c_double * 3),
        ("rotation", c_double * 4),
        ("density", c_double),
        ("init_velocity", c_double * 3),
        ("init_angular_velocity", c_double * 3),
        ("target_x", c_double * 3),
    ]


class DfsphScene(ctypes.Structure):
    _fields_ = [
        ("struct_size", c_int32),
        ("params", DfsphParams),
        ("n_fluid", c_int64),
        ("fluid_x", POINTER(c_double)),
        ("fluid_v", POINTER(c_double)),
        ("n_bodies", c_int32),
        ("bodies", POINTER(DfsphBodyDesc)),
    ]


class DfsphStepStats(ctypes.Structure):
    _fields_ = [
        ("steps_done", c_int32),
        ("pressure_iterations", c_int32),
        ("divergence_iterations", c_int32),
        ("trajectory_finished", c_int32),
        ("pressure_avg_error", c_double),
        ("divergence_avg_error", c_double),
        ("total_pressure_iterations", c_int64),
        ("total_divergence_iterations", c_int64),
        ("time", c_double),
        ("time_step", c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def dptr(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_double))


class CScene:
    """Holds a DfsphScene and the numpy buffers it points into (keep alive)."""

    def __init__(self, scene):
        p = scene.params
        self._keep = []
        cp = DfsphParams()
        cp.struct_size = ctypes.sizeof(DfsphParams)
        for name, _ in DfsphParams._fields_:
            if name == "struct_size":
                continue
            val = getattr(p, name)
            if name == "gravity":
                cp.gravity = (c_double * 3)(*[float(g) for g in val])
            else:
                setattr(cp, name, val)
        fx = np.ascontiguousarray(scene.fluid_x, dtype=np.float64).reshape(-1, 3)
        fv = np.ascontiguousarray(scene.fluid_v, dtype=np.float64).reshape(-1, 3)
        self._keep += [fx, fv]
        nb = len(scene.bodies)
        arr = (DfsphBodyDesc * max(nb, 1))()
        for k, b in enumerate(scene.bodies):
            s = np.ascontiguousarray(b.samples, dtype=np.float64).reshape(-1, 3)
            self._keep.append(s)
            d = arr[k]
            d.is_dynamic = int(b.is_dynamic)
            d.is_animated = int(b.is_animated)
            d.n_samples = s.shape[0]
            d.samples = dptr(s)
            d.translation = (c_double * 3)(*[float(t) for t in b.translation])
            d.rotation = (c_double * 4)(*[float(t) for t in b.rotation])
            d.density = float(b.density)
            d.init_velocity = (c_double * 3)(*[float(t) for t in b.init_velocity])
            d.init_angular_velocity = (c_double * 3)(*[float(t) for t in b.init_angular_velocity])
            d.target_x = (c_double * 3)(*[float(t) for t in b.target_x])
        self._keep.append(arr)
        sc = DfsphScene()
        sc.struct_size = ctypes.sizeof(DfsphScene)
        sc.params = cp
        sc.n_fluid = fx.shape[0]
        sc.fluid_x = dptr(fx)
        sc.fluid_v = dptr(fv)
        sc.n_bodies = nb
        sc.bodies = ctypes.cast(arr, POINTER(DfsphBodyDesc))
        self.c = sc

    def ref(self):
        return ctypes.byref(self.c)


class DfsphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"dfsph error {code}: {msg}")
        self.code = code


_lib = None


def load_library(path: str | None = None):
    """Loads libdfsph.so (built by ``__graft_entry__.build()``). Raises when absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            f"libdfsph.so not found at {p}: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            " (the CUDA library is required; there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    vp = c_void_p
    sig = {
        "dfsph_abi_version": ([], c_int32),
        "dfsph_last_error": ([], c_char_p),
        "dfsph_default_params": ([POINTER(DfsphParams)], c_int32),
        "dfsph_create": ([POINTER(DfsphScene), POINTER(vp)], c_int32),
        "dfsph_destroy": ([vp], c_int32),
        "dfsph_reset": ([vp], c_int32),
        "dfsph_step": ([vp, c_int32, POINTER(DfsphStepStats)], c_int32),
        "dfsph_set_rigid_init": ([vp, c_int32, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_get_rigid_init": ([vp, c_int32, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_get_rigid_state": ([vp, c_int32] + [POINTER(c_double)] * 4, c_int32),
        "dfsph_set_rigid_velocity": ([vp, c_int32, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_get_rigid_force": ([vp, c_int32, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_get_rigid_mass": ([vp, c_int32, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_get_rigid_grad": ([vp, c_int32, POINTER(c_double)], c_int32),
        "dfsph_get_net_jacobians": ([vp, c_int32, POINTER(c_double)], c_int32),
        "dfsph_get_manager_grad": ([vp, c_int32, c_int32, POINTER(c_double)], c_int32),
        "dfsph_get_manager_jacobians": ([vp, c_int32, c_int32, POINTER(c_double)], c_int32),
        "dfsph_get_contact_count": ([vp, POINTER(c_int64), POINTER(c_int64)], c_int32),
        "dfsph_reset_gradient": ([vp], c_int32),
        "dfsph_backward": ([vp, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_tape_length": ([vp, POINTER(c_int64)], c_int32),
        "dfsph_copy_field": ([vp, c_int32, POINTER(c_double), c_int64], c_int32),
        "dfsph_set_field": ([vp, c_int32, POINTER(c_double), c_int64], c_int32),
        "dfsph_num_particles": ([vp, POINTER(c_int64), POINTER(c_int64)], c_int32),
        "dfsph_get_neighbors": ([vp, c_int32, POINTER(c_int64), POINTER(c_int32), POINTER(c_int64)], c_int32),
        "dfsph_get_time": ([vp, POINTER(c_double), POINTER(c_int64)], c_int32),
        "dfsph_synchronize": ([vp], c_int32),
        "dfsph_launch_count": ([vp, POINTER(c_int64)], c_int32),
        "dfsph_record_event": ([vp, c_int32], c_int32),
        "dfsph_event_elapsed": ([vp, c_int32, c_int32, POINTER(c_double)], c_int32),
        "dfsph_profile_enable": ([vp, c_int32], c_int32),
        "dfsph_profile_read": ([vp, c_int32, POINTER(c_int64), POINTER(c_double), POINTER(c_int64)], c_int32),
        "dfsph_kernel_class_name": ([c_int32], c_char_p),
        "dfsph_set_device": ([c_int32], c_int32),
        "dfsph_density_error_noalloc": ([c_void_p, c_int32, c_int64, c_double, c_int32, c_void_p, c_void_p], c_int32),
        "dfsph_set_time": ([vp, c_double, c_int64], c_int32),
        "dfsph_set_rigid_state": ([vp, c_int32] + [POINTER(c_double)] * 4, c_int32),
        "dfsph_set_gradient_enabled": ([vp, c_int32], c_int32),
        "dfsph_checkpoint_save": ([vp, POINTER(c_int32)], c_int32),
        "dfsph_checkpoint_restore": ([vp, c_int32], c_int32),
        "dfsph_checkpoint_free": ([vp, c_int32], c_int32),
        "dfsph_adjoint_sweep": ([vp, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_mlp_create": ([c_int32, c_uint64, POINTER(vp)], c_int32),
        "dfsph_mlp_destroy": ([vp], c_int32),
        "dfsph_mlp_get_params": ([vp, POINTER(c_float), POINTER(c_float)], c_int32),
        "dfsph_mlp_set_params": ([vp, POINTER(c_float), POINTER(c_float)], c_int32),
        "dfsph_mlp_fit_normalization": ([vp, vp, vp, c_int64], c_int32),
        "dfsph_mlp_train_step": ([vp, vp, vp, c_int64, vp, c_int64, c_float, POINTER(c_double)], c_int32),
        "dfsph_mlp_gradient": ([vp, vp, vp, c_int64, POINTER(c_double), POINTER(c_double)], c_int32),
        "dfsph_mlp_predict": ([vp, vp, vp, c_int64], c_int32),
        "dfsph_mlp_set_wait_limit": ([vp, c_int32], c_int32),
        "dfsph_set_warmstart_model": ([vp, vp], c_int32),
        "dfsph_ml_record": ([vp, c_int32], c_int32),
        "dfsph_ml_capture": ([vp, vp, vp, c_int64, POINTER(c_int64)], c_int32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


EXPORTED_SYMBOLS = (
    "dfsph_abi_version", "dfsph_last_error", "dfsph_default_params", "dfsph_create", "dfsph_destroy",
    "dfsph_reset", "dfsph_step", "dfsph_set_rigid_init", "dfsph_get_rigid_init", "dfsph_get_rigid_state",
    "dfsph_set_rigid_velocity", "dfsph_get_rigid_force", "dfsph_get_rigid_mass", "dfsph_get_rigid_grad",
    "dfsph_get_net_jacobians", "dfsph_reset_gradient", "dfsph_backward", "dfsph_tape_length",
    "dfsph_copy_field", "dfsph_set_field", "dfsph_num_particles", "dfsph_get_neighbors", "dfsph_get_time",
    "dfsph_synchronize", "dfsph_launch_count", "dfsph_record_event", "dfsph_event_elapsed",
    "dfsph_profile_enable", "dfsph_profile_read", "dfsph_kernel_class_name", "dfsph_set_device",
    "dfsph_density_error_noalloc", "dfsph_set_time", "dfsph_set_rigid_state", "dfsph_set_gradient_enabled",
    "dfsph_checkpoint_save", "dfsph_checkpoint_restore", "dfsph_checkpoint_free", "dfsph_adjoint_sweep",
    "dfsph_mlp_create", "dfsph_mlp_destroy", "dfsph_mlp_get_params", "dfsph_mlp_set_params",
    "dfsph_mlp_fit_normalization", "dfsph_mlp_train_step", "dfsph_mlp_gradient", "dfsph_mlp_predict",
    "dfsph_mlp_set_wait_limit",
    "dfsph_set_warmstart_model", "dfsph_ml_record", "dfsph_ml_capture",
    "dfsph_get_manager_grad", "dfsph_get_manager_jacobians", "dfsph_get_contact_count",
)
KERNEL_CLASSES = ("sort", "lists_density_factor", "bf_lists", "density_pass", "velocity_pass",
                  "xsph_advect", "integrate", "pairs", "rigid", "mlp")
PHASES = ("divergence_solve", "pressure_solve")   # profile slots after the kernel classes
MLP_NPARAMS = 4545


def check(lib, rc, allow=()):
    if rc != DFSPH_OK and rc not in allow:
        msg = lib.dfsph_last_error()
        raise DfsphError(rc, msg.decode() if msg else "")
    return rc
