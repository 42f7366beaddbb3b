"""CPU oracle of the DiffDFSPH step — test infrastructure only.

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
package, as the checker. The product (``difffr_gb300``) never imports it.
"""
import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_int32, c_int64, c_void_p

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(_HERE, "dfsph_oracle.cpp")
SRCS = [SRC, os.path.join(_HERE, "mlp_oracle.cpp")]
DEPS = SRCS + [os.path.join(_HERE, "..", "include", "dfsph.h")]  # the scene structs it reads
LIB = os.path.join(_HERE, "_build", "liboracle_dfsph.so")

MODE_F32 = 0       # <float, float>   the reference's default float build
MODE_MIXED = 1     # <float, double>  FP32 fluid, FP64 rigid (the GPU split)
MODE_F64 = 2       # <double, double> the reference's USE_DOUBLE build


def build(force=False):
    """Compiles the oracle with g++ (OpenMP, no FMA contraction so x86 and Arm agree)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in DEPS):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB, *SRCS]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        from difffr_gb300 import _abi
        dp = POINTER(c_double)
        L.orc_create.argtypes = [POINTER(_abi.DfsphScene), c_int]
        L.orc_create.restype = c_void_p
        L.orc_destroy.argtypes = [c_void_p]
        L.orc_set_threads.argtypes = [c_int]
        L.orc_set_threads.restype = c_int
        L.orc_step.argtypes = [c_void_p, c_int, POINTER(_abi.DfsphStepStats)]
        L.orc_copy_field.argtypes = [c_void_p, c_int, dp]
        L.orc_set_field.argtypes = [c_void_p, c_int, dp]
        for n in ("orc_get_rigid_state",):
            getattr(L, n).argtypes = [c_void_p, c_int, dp, dp, dp, dp]
        for n in ("orc_get_rigid_force", "orc_get_rigid_mass", "orc_set_rigid_init", "orc_set_rigid_velocity"):
            getattr(L, n).argtypes = [c_void_p, c_int, dp, dp]
        for n in ("orc_get_rigid_grad", "orc_get_net_jacobians"):
            getattr(L, n).argtypes = [c_void_p, c_int, dp]
        for n in ("orc_get_manager_grad", "orc_get_manager_jacobians"):
            getattr(L, n).argtypes = [c_void_p, c_int, c_int, dp]
        L.orc_set_rigid_state.argtypes = [c_void_p, c_int, dp, dp, dp, dp]
        L.orc_set_time.argtypes = [c_void_p, c_double, c_int64]
        L.orc_get_contact_count.argtypes = [c_void_p, POINTER(c_int64), POINTER(c_int64)]
        L.orc_get_neighbors.argtypes = [c_void_p, c_int, POINTER(c_int64), POINTER(c_int32), POINTER(c_int64)]
        L.orc_reset.argtypes = [c_void_p]
        L.orc_reset_gradient.argtypes = [c_void_p]
        L.orc_num_particles.argtypes = [c_void_p, POINTER(c_int64), POINTER(c_int64)]
        L.orc_get_time.argtypes = [c_void_p]
        L.orc_get_time.restype = c_double
        L.orc_kernel_eval.argtypes = [c_double, c_int, dp, dp, dp, dp]
        fp = POINTER(c_float)
        L.orc_kernel_eval_f.argtypes = [c_float, c_int, fp, fp, fp, fp]
        L.orc_quat_eval.argtypes = [c_int, dp, dp, dp, dp, dp, dp]
        L.orc_mlp_eval.argtypes = [fp, fp, fp, fp, c_int64, fp, dp]
        L.orc_st_kernel_eval.argtypes = [c_double, c_int, dp, dp, dp]
        L.orc_st_kernel_eval_f.argtypes = [c_float, c_int, fp, fp, fp]
        L.orc_mlp_eval.restype = c_double
        _lib = L
    return _lib


def reference_root():
    """The DiffFR checkout the reference pins are built from, or None when it is absent.

    Taken from the DIFFFR_REFERENCE environment variable, else a directory named
    ``reference`` beside this repository. Only the pin recipes and the fixture scripts
    read it; GPU tests, ``smoke()`` and ``bench.py`` never do.
    """
    p = os.environ.get("DIFFFR_REFERENCE")
    if not p:
        p = os.path.join(os.path.dirname(_HERE), "..", "reference")
    p = os.path.abspath(p)
    return p if os.path.isdir(os.path.join(p, "SPlisHSPlasH")) else None


def _p(a):
    return a.ctypes.data_as(POINTER(c_double))


def grad_blocks(g):
    """The 78 chain-state numbers (dfsph_get_rigid_grad layout) as named blocks."""
    return {
        "x_v0": g[0:9].reshape(3, 3), "x_w0": g[9:18].reshape(3, 3),
        "q_v0": g[18:30].reshape(4, 3), "q_w0": g[30:42].reshape(4, 3),
        "v_v0": g[42:51].reshape(3, 3), "v_w0": g[51:60].reshape(3, 3),
        "w_v0": g[60:69].reshape(3, 3), "w_w0": g[69:78].reshape(3, 3),
    }


class Oracle:
    """The oracle simulation behind the same scene description as the GPU library."""

    def __init__(self, scene, mode=None, threads=None):
        from difffr_gb300 import _abi
        L = lib()
        if threads:
            L.orc_set_threads(int(threads))
        if mode is None:
            mode = MODE_F64 if scene.params.fluid_precision == _abi.DFSPH_FP64 else MODE_MIXED
        self._cs = _abi.CScene(scene)
        self.h = L.orc_create(self._cs.ref(), int(mode))
        if not self.h:
            raise RuntimeError("oracle creation failed")
        self.L = L
        self.scene = scene
        nf, nb = c_int64(), c_int64()
        L.orc_num_particles(self.h, ctypes.byref(nf), ctypes.byref(nb))
        self.n_fluid, self.n_boundary = nf.value, nb.value

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def step(self, n=1):
        from difffr_gb300 import _abi
        st = _abi.DfsphStepStats()
        rc = self.L.orc_step(self.h, int(n), ctypes.byref(st))
        d = st.as_dict()
        d["rc"] = rc
        return d

    def field(self, f):
        from difffr_gb300 import _abi
        n = self.n_boundary if f in _abi.BOUNDARY_FIELDS else self.n_fluid
        c = _abi.FIELD_COMPONENTS.get(f, 1)
        out = np.zeros(n * c, dtype=np.float64)
        rc = self.L.orc_copy_field(self.h, int(f), _p(out))
        assert rc == 0
        return out.reshape(n, c) if c > 1 else out

    def set_field(self, f, data):
        d = np.ascontiguousarray(data, dtype=np.float64).ravel()
        assert self.L.orc_set_field(self.h, int(f), _p(d)) == 0

    def rigid_state(self, b):
        x, q, v, w = (np.zeros(k) for k in (3, 4, 3, 3))
        assert self.L.orc_get_rigid_state(self.h, b, _p(x), _p(q), _p(v), _p(w)) == 0
        return x, q, v, w

    def rigid_force(self, b):
        F, T = np.zeros(3), np.zeros(3)
        assert self.L.orc_get_rigid_force(self.h, b, _p(F), _p(T)) == 0
        return F, T

    def rigid_mass(self, b):
        m, I = np.zeros(1), np.zeros(9)
        assert self.L.orc_get_rigid_mass(self.h, b, _p(m), _p(I)) == 0
        return m[0], I.reshape(3, 3)

    def rigid_grad(self, b):
        o = np.zeros(78)
        assert self.L.orc_get_rigid_grad(self.h, b, _p(o)) == 0
        return o

    def rigid_grad_blocks(self, b):
        return grad_blocks(self.rigid_grad(b))

    def manager_grad(self, b, b2):
        o = np.zeros(78)
        assert self.L.orc_get_manager_grad(self.h, b, b2, _p(o)) == 0
        return o

    def manager_jacobians(self, b, b2):
        o = np.zeros(78)
        assert self.L.orc_get_manager_jacobians(self.h, b, b2, _p(o)) == 0
        return o

    def contact_count(self):
        nc, na = c_int64(), c_int64()
        assert self.L.orc_get_contact_count(self.h, ctypes.byref(nc), ctypes.byref(na)) == 0
        return nc.value, na.value

    def net_jacobians(self, b):
        o = np.zeros(78)
        assert self.L.orc_get_net_jacobians(self.h, b, _p(o)) == 0
        return o

    def set_rigid_init(self, b, v, w):
        v = np.asarray(v, dtype=np.float64); w = np.asarray(w, dtype=np.float64)
        assert self.L.orc_set_rigid_init(self.h, b, _p(v), _p(w)) == 0

    def set_rigid_velocity(self, b, v, w):
        v = np.asarray(v, dtype=np.float64); w = np.asarray(w, dtype=np.float64)
        assert self.L.orc_set_rigid_velocity(self.h, b, _p(v), _p(w)) == 0

    def set_rigid_state(self, b, x, q, v, w):
        a = [np.ascontiguousarray(z, dtype=np.float64) for z in (x, q, v, w)]
        assert self.L.orc_set_rigid_state(self.h, int(b), *[_p(z) for z in a]) == 0

    def set_time(self, t, step_count=0):
        assert self.L.orc_set_time(self.h, float(t), int(step_count)) == 0

    def load_state(self, sim):
        """Takes over another run's fluid and rigid state (positions, velocities, both warm-start
        stiffness fields, every body's state, time and step count), e.g. a GPU context's state in
        the middle of a trajectory, so that both continue from the same inputs."""
        from difffr_gb300 import _abi
        for f in (_abi.FIELD_X, _abi.FIELD_V, _abi.FIELD_KAPPA, _abi.FIELD_KAPPA_V):
            self.set_field(f, sim.field(f))
        for b in range(sim.n_bodies):
            self.set_rigid_state(b, *sim.rigid_state(b))
        t, sc = sim.time()
        self.set_time(t, sc)

    def neighbors(self, which):
        tot = c_int64()
        rc = self.L.orc_get_neighbors(self.h, int(which), None, None, ctypes.byref(tot))
        assert rc == 0, rc
        rows = self.n_fluid if which in (0, 1) else self.n_boundary
        start = np.zeros(rows + 1, dtype=np.int64)
        idx = np.zeros(tot.value, dtype=np.int32)
        self.L.orc_get_neighbors(self.h, int(which), start.ctypes.data_as(POINTER(c_int64)),
                                 idx.ctypes.data_as(POINTER(c_int32)), ctypes.byref(tot))
        return start, idx

    def reset(self):
        self.L.orc_reset(self.h)

    def reset_gradient(self):
        self.L.orc_reset_gradient(self.h)

    def time(self):
        return self.L.orc_get_time(self.h)


def kernel_eval(h, r):
    """Oracle cubic kernel (double): W, gradW, gradGradW at offsets r[n,3]."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    n = r.shape[0]
    W, G, H = np.zeros(n), np.zeros((n, 3)), np.zeros((n, 3, 3))
    lib().orc_kernel_eval(float(h), n, _p(r), _p(W), _p(G), _p(H))
    return W, G, H


def kernel_eval_f(h, r):
    """Oracle cubic kernel (float)."""
    r = np.ascontiguousarray(r, dtype=np.float32)
    n = r.shape[0]
    W, G, H = np.zeros(n, np.float32), np.zeros((n, 3), np.float32), np.zeros((n, 3, 3), np.float32)
    fp = lambda a: a.ctypes.data_as(POINTER(c_float))
    lib().orc_kernel_eval_f(float(h), n, fp(r), fp(W), fp(G), fp(H))
    return W, G, H


def st_kernel_eval(h, r, single=False):
    """Oracle surface-tension kernels (cohesion, adhesion) at offsets r[n,3], in double or
    (single=True) float."""
    dt = np.float32 if single else np.float64
    r = np.ascontiguousarray(r, dtype=dt)
    n = r.shape[0]
    C, A = np.zeros(n, dt), np.zeros(n, dt)
    if single:
        fp = lambda a: a.ctypes.data_as(POINTER(c_float))
        lib().orc_st_kernel_eval_f(float(h), n, fp(r), fp(C), fp(A))
    else:
        lib().orc_st_kernel_eval(float(h), n, _p(r), _p(C), _p(A))
    return C, A


def quat_eval(q, p):
    q = np.ascontiguousarray(q, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    n = q.shape[0]
    a, b, c, d = np.zeros((n, 3, 4)), np.zeros((n, 3, 4)), np.zeros((n, 4, 4)), np.zeros((n, 4, 3))
    lib().orc_quat_eval(n, _p(q), _p(p), _p(a), _p(b), _p(c), _p(d))
    return a, b, c, d


def mlp_eval(params, norm, x, y=None, with_grad=True):
    """The warm-start MLP on the CPU: (prediction, gradient of the mean squared error or
    None, loss). params: 4545 floats; norm: 10 floats; x: (n, 4); y: (n,) or None."""
    fp = POINTER(c_float)
    params = np.ascontiguousarray(params, dtype=np.float32)
    norm = np.ascontiguousarray(norm, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 4)
    n = x.shape[0]
    pred = np.zeros(n, dtype=np.float32)
    yy = None if y is None else np.ascontiguousarray(y, dtype=np.float32)
    grad = np.zeros(4545) if (with_grad and y is not None) else None
    loss = lib().orc_mlp_eval(params.ctypes.data_as(fp), norm.ctypes.data_as(fp), x.ctypes.data_as(fp),
                              None if yy is None else yy.ctypes.data_as(fp), n, pred.ctypes.data_as(fp),
                              None if grad is None else _p(grad))
    return pred, grad, loss
