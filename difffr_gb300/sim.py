"""DiffDFSPH simulation handle: a thin wrapper over the libdfsph C ABI.

One ``DiffDFSPH`` owns one device context (all particle state in HBM; three CUDA
streams: the fluid solve, the rigid bodies, and the per-body chain rule). Arrays cross the boundary as float64 numpy arrays in the caller's particle
order. Every method raises ``DfsphError`` on a non-zero status; nothing falls back
to the CPU.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_double, c_int32, c_int64, c_void_p

import numpy as np

from . import _abi
from ._abi import check, dptr


def grad_blocks(g):
    """The 78 chain-state numbers (dfsph_get_rigid_grad layout) as named blocks."""
    return {
        "x_v0": g[0:9].reshape(3, 3), "x_w0": g[9:18].reshape(3, 3),
        "q_v0": g[18:30].reshape(4, 3), "q_w0": g[30:42].reshape(4, 3),
        "v_v0": g[42:51].reshape(3, 3), "v_w0": g[51:60].reshape(3, 3),
        "w_v0": g[60:69].reshape(3, 3), "w_w0": g[69:78].reshape(3, 3),
    }


class DiffDFSPH:
    def __init__(self, scene, lib_path=None):
        self.lib = _abi.load_library(lib_path)
        self.scene = scene
        self._cs = _abi.CScene(scene)
        h = c_void_p()
        check(self.lib, self.lib.dfsph_create(self._cs.ref(), byref(h)))
        self.h = h
        nf, nb = c_int64(), c_int64()
        check(self.lib, self.lib.dfsph_num_particles(self.h, byref(nf), byref(nb)))
        self.n_fluid, self.n_boundary = nf.value, nb.value
        self.n_bodies = len(scene.bodies)
        self.last_stats = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.dfsph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -------------------------------------------------------------- stepping
    def step(self, n=1, allow_not_converged=True):
        st = _abi.DfsphStepStats()
        allow = (_abi.DFSPH_ERR_NOT_CONVERGED,) if allow_not_converged else ()
        rc = check(self.lib, self.lib.dfsph_step(self.h, int(n), byref(st)), allow=allow)
        d = st.as_dict()
        d["rc"] = rc
        self.last_stats = d
        return d

    def reset(self):
        check(self.lib, self.lib.dfsph_reset(self.h))

    def synchronize(self):
        check(self.lib, self.lib.dfsph_synchronize(self.h))

    def time(self):
        t, sc = c_double(), c_int64()
        check(self.lib, self.lib.dfsph_get_time(self.h, byref(t), byref(sc)))
        return t.value, sc.value

    def launch_count(self):
        c = c_int64()
        check(self.lib, self.lib.dfsph_launch_count(self.h, byref(c)))
        return c.value

    # -------------------------------------------------------------- fields
    def field(self, f):
        n = self.n_boundary if f in _abi.BOUNDARY_FIELDS else self.n_fluid
        c = _abi.FIELD_COMPONENTS.get(f, 1)
        out = np.zeros(n * c, dtype=np.float64)
        check(self.lib, self.lib.dfsph_copy_field(self.h, int(f), dptr(out), out.size))
        return out.reshape(n, c) if c > 1 else out

    def set_field(self, f, data):
        d = np.ascontiguousarray(data, dtype=np.float64).ravel()
        check(self.lib, self.lib.dfsph_set_field(self.h, int(f), dptr(d), d.size))

    def positions(self):
        return self.field(_abi.FIELD_X)

    def velocities(self):
        return self.field(_abi.FIELD_V)

    def neighbor_total(self, which):
        """Number of (particle, neighbour) pairs of a set after the last step."""
        tot = c_int64()
        check(self.lib, self.lib.dfsph_get_neighbors(self.h, int(which), None, None, byref(tot)))
        return tot.value

    def neighbors(self, which):
        tot = c_int64()
        check(self.lib, self.lib.dfsph_get_neighbors(self.h, int(which), None, None, byref(tot)))
        rows = self.n_fluid if which in (_abi.NB_FLUID_FLUID, _abi.NB_FLUID_BOUNDARY) else self.n_boundary
        start = np.zeros(rows + 1, dtype=np.int64)
        idx = np.zeros(max(tot.value, 1), dtype=np.int32)
        check(self.lib, self.lib.dfsph_get_neighbors(self.h, int(which), start.ctypes.data_as(POINTER(c_int64)),
                                                     idx.ctypes.data_as(POINTER(c_int32)), byref(tot)))
        return start, idx[: tot.value]

    # -------------------------------------------------------------- rigid bodies
    def rigid_state(self, b):
        """(x, q (w, x, y, z), v, omega) of body b as new arrays."""
        if getattr(self, "_rs_ptrs", None) is None:
            # one output buffer and its four pointers, made once (the per-call ctypes
            # conversions otherwise dominate this call on slow hosts)
            self._rs_buf = np.zeros(13)
            base = self._rs_buf.ctypes.data
            self._rs_ptrs = tuple(ctypes.cast(base + 8 * o, POINTER(c_double)) for o in (0, 3, 7, 10))
        check(self.lib, self.lib.dfsph_get_rigid_state(self.h, int(b), *self._rs_ptrs))
        r = self._rs_buf.copy()
        return r[0:3], r[3:7], r[7:10], r[10:13]

    def rigid_force(self, b):
        F, T = np.zeros(3), np.zeros(3)
        check(self.lib, self.lib.dfsph_get_rigid_force(self.h, int(b), dptr(F), dptr(T)))
        return F, T

    def rigid_mass(self, b):
        m, I = np.zeros(1), np.zeros(9)
        check(self.lib, self.lib.dfsph_get_rigid_mass(self.h, int(b), dptr(m), dptr(I)))
        return m[0], I.reshape(3, 3)

    def set_rigid_init(self, b, v, w):
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        check(self.lib, self.lib.dfsph_set_rigid_init(self.h, int(b), dptr(v), dptr(w)))

    def rigid_init(self, b):
        v, w = np.zeros(3), np.zeros(3)
        check(self.lib, self.lib.dfsph_get_rigid_init(self.h, int(b), dptr(v), dptr(w)))
        return v, w

    def set_rigid_velocity(self, b, v, w):
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        check(self.lib, self.lib.dfsph_set_rigid_velocity(self.h, int(b), dptr(v), dptr(w)))

    def rigid_grad(self, b):
        """Forward-mode chain state (78 doubles, reference accessor order)."""
        o = np.zeros(78)
        check(self.lib, self.lib.dfsph_get_rigid_grad(self.h, int(b), dptr(o)))
        return o

    def rigid_grad_blocks(self, b):
        return grad_blocks(self.rigid_grad(b))

    @property
    def uses_manager(self):
        return bool(self.scene.params.use_rigid_gradient_manager)

    def manager_grad(self, b, b2):
        """The gradient manager's chain state [b][b2] (78 doubles, dfsph_get_rigid_grad layout):
        derivatives of body b's state with respect to body b2's initial (v, omega)."""
        o = np.zeros(78)
        check(self.lib, self.lib.dfsph_get_manager_grad(self.h, int(b), int(b2), dptr(o)))
        return o

    def manager_grad_blocks(self, b, b2):
        return grad_blocks(self.manager_grad(b, b2))

    def manager_jacobians(self, b, b2):
        """The manager's force / torque blocks [b][b2] (dfsph_get_net_jacobians layout)."""
        o = np.zeros(78)
        check(self.lib, self.lib.dfsph_get_manager_jacobians(self.h, int(b), int(b2), dptr(o)))
        return o

    def contact_count(self):
        """(samples of dynamic bodies in contact, samples that carried a penalty force) of the last step."""
        nc, na = c_int64(), c_int64()
        check(self.lib, self.lib.dfsph_get_contact_count(self.h, byref(nc), byref(na)))
        return nc.value, na.value

    def net_jacobians(self, b):
        o = np.zeros(78)
        check(self.lib, self.lib.dfsph_get_net_jacobians(self.h, int(b), dptr(o)))
        return o

    def reset_gradient(self):
        check(self.lib, self.lib.dfsph_reset_gradient(self.h))

    def backward(self, dL_dstate):
        """dL_dstate: (n_bodies, 13) = dL/d(x, q(w,x,y,z), v, omega) of the current state.
        Returns (n_bodies, 6) = dL/d(v0, omega0)."""
        g = np.ascontiguousarray(dL_dstate, dtype=np.float64).reshape(self.n_bodies, 13)
        out = np.zeros((self.n_bodies, 6))
        check(self.lib, self.lib.dfsph_backward(self.h, dptr(g), dptr(out)))
        return out

    def tape_length(self):
        n = c_int64()
        check(self.lib, self.lib.dfsph_tape_length(self.h, byref(n)))
        return n.value

    # -------------------------------------------------------------- timing
    def record_event(self, slot):
        check(self.lib, self.lib.dfsph_record_event(self.h, int(slot)))

    def event_elapsed_ms(self, a, b):
        ms = c_double()
        check(self.lib, self.lib.dfsph_event_elapsed(self.h, int(a), int(b), byref(ms)))
        return ms.value

    def profile_enable(self, on=True):
        check(self.lib, self.lib.dfsph_profile_enable(self.h, 1 if on else 0))

    def profile(self):
        """Per kernel class: launches, device ms, work units since profile_enable()."""
        out = {}
        for k, name in enumerate(_abi.KERNEL_CLASSES + _abi.PHASES):
            l, ms, u = c_int64(), c_double(), c_int64()
            check(self.lib, self.lib.dfsph_profile_read(self.h, k, byref(l), byref(ms), byref(u)))
            out[name] = {"launches": l.value, "ms": ms.value, "units": u.value}
        return out

    # -------------------------------------------------------------- state control
    def set_time(self, t, step_count=0):
        check(self.lib, self.lib.dfsph_set_time(self.h, float(t), int(step_count)))

    def set_rigid_state(self, b, x, q, v, w):
        a = [np.ascontiguousarray(z, dtype=np.float64) for z in (x, q, v, w)]
        check(self.lib, self.lib.dfsph_set_rigid_state(self.h, int(b), *[dptr(z) for z in a]))

    def set_gradient_enabled(self, on=True):
        check(self.lib, self.lib.dfsph_set_gradient_enabled(self.h, 1 if on else 0))

    def checkpoint_save(self):
        slot = c_int32()
        check(self.lib, self.lib.dfsph_checkpoint_save(self.h, byref(slot)))
        return slot.value

    def checkpoint_restore(self, slot):
        check(self.lib, self.lib.dfsph_checkpoint_restore(self.h, int(slot)))

    def checkpoint_free(self, slot):
        check(self.lib, self.lib.dfsph_checkpoint_free(self.h, int(slot)))

    def adjoint_sweep(self, lam):
        """Full 13-component adjoints (n_bodies, 13) pulled back over the recorded steps. With
        the gradient manager the v0 and omega0 columns have separate maps: lam is then
        (2, n_bodies, 13), the v0 sweep's adjoint and the omega0 sweep's."""
        shape = (2, self.n_bodies, 13) if self.uses_manager else (self.n_bodies, 13)
        g = np.ascontiguousarray(lam, dtype=np.float64).reshape(shape)
        out = np.zeros_like(g)
        check(self.lib, self.lib.dfsph_adjoint_sweep(self.h, dptr(g), dptr(out)))
        return out

    def rigid_state_vector(self, b):
        x, q, v, w = self.rigid_state(b)
        return np.concatenate([x, q, v, w])

    # -------------------------------------------------------------- learned warm start
    def set_warmstart_model(self, model):
        """Use a ``WarmStartModel`` for the pressure warm start (None: the reference formula)."""
        check(self.lib, self.lib.dfsph_set_warmstart_model(self.h, model.h if model is not None else None))
        self._ws_model = model  # keep the model alive while the context uses it

    def ml_record(self, on=True):
        check(self.lib, self.lib.dfsph_ml_record(self.h, 1 if on else 0))

    def ml_capture(self, x, y):
        """Copies the last step's training samples (features, target stiffness) into the
        device tensors x (float32 [cap, 4]) and y (float32 [cap]); returns the count."""
        import torch
        if not (x.is_cuda and y.is_cuda and x.dtype == torch.float32 and y.dtype == torch.float32
                and x.is_contiguous() and y.is_contiguous() and x.dim() == 2 and x.shape[1] == 4):
            raise ValueError("x: contiguous CUDA float32 [cap, 4]; y: contiguous CUDA float32 [cap]")
        torch.cuda.current_stream(x.device).synchronize()  # the library's stream is not ordered against PyTorch's
        cap = min(int(x.shape[0]), int(y.shape[0]))
        cnt = c_int64()
        check(self.lib, self.lib.dfsph_ml_capture(self.h, c_void_p(x.data_ptr()), c_void_p(y.data_ptr()), cap,
                                                  byref(cnt)))
        return cnt.value
