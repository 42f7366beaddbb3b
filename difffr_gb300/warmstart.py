"""Learned warm start for the DFSPH pressure stiffness.

``WarmStartModel`` owns one MLP (4 -> 64 -> 64 -> 1, GELU, BF16 weights) on the GPU; its
training and inference run in the library's tensor-core kernels. ``collect_samples``
records (features, target) pairs from a running simulation, ``train`` fits the model with
Adam on shuffled minibatches, and ``DiffDFSPH.set_warmstart_model`` switches a simulation's
pressure warm start from the reference formula (TimeStepDiffDFSPH.cpp:964-1059,
kappa <- 0.5 max(kappa, -0.00025) / h^2) to the model. The Jacobi solve always continues
to the configured tolerance, so the model only changes where the solve starts.

Tensors passed here are CUDA float32 tensors (PyTorch only holds the device memory).
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_double, c_float, c_void_p

import numpy as np

from . import _abi
from ._abi import check

NPARAMS = _abi.MLP_NPARAMS
FEATURES = ("density_error", "neighbour_count", "previous_kappa", "speed")


def _dev(t, dtype, cols=None):
    """Device pointer of a CUDA tensor for the library. The library's streams are not
    ordered against PyTorch's, so PyTorch's current stream is synchronised first: every
    kernel that writes the tensor has finished before the library reads it."""
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
        raise ValueError(f"expected a contiguous CUDA tensor of {dtype}")
    if cols is not None and (t.dim() != 2 or t.shape[1] != cols):
        raise ValueError(f"expected shape [n, {cols}]")
    torch.cuda.current_stream(t.device).synchronize()
    return c_void_p(t.data_ptr())


class WarmStartModel:
    def __init__(self, seed=0, device=0, lib=None):
        self.lib = lib or _abi.load_library()
        h = c_void_p()
        check(self.lib, self.lib.dfsph_mlp_create(int(device), int(seed), byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.dfsph_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- parameters
    def params(self):
        p = np.zeros(NPARAMS, dtype=np.float32)
        n = np.zeros(10, dtype=np.float32)
        check(self.lib, self.lib.dfsph_mlp_get_params(self.h, p.ctypes.data_as(POINTER(c_float)),
                                                      n.ctypes.data_as(POINTER(c_float))))
        return p, n

    def set_params(self, params=None, norm=None):
        fp = POINTER(c_float)
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        if p is not None and p.size != NPARAMS:
            raise ValueError(f"expected {NPARAMS} parameters")
        if n is not None and n.size != 10:
            raise ValueError("expected 10 normalisation values")
        check(self.lib, self.lib.dfsph_mlp_set_params(self.h, None if p is None else p.ctypes.data_as(fp),
                                                      None if n is None else n.ctypes.data_as(fp)))

    def save(self, path):
        p, n = self.params()
        np.savez(path, params=p, norm=n)

    def load(self, path):
        d = np.load(path)
        self.set_params(d["params"], d["norm"])

    # -------------------------------------------------------------- training / inference
    def fit_normalization(self, x, y):
        import torch
        check(self.lib, self.lib.dfsph_mlp_fit_normalization(self.h, _dev(x, torch.float32, 4),
                                                             _dev(y, torch.float32), int(x.shape[0])))

    def train_step(self, x, y, idx=None, lr=1e-3, n=None):
        import torch
        loss = c_double()
        n = int(idx.shape[0] if idx is not None else x.shape[0]) if n is None else int(n)
        check(self.lib, self.lib.dfsph_mlp_train_step(
            self.h, _dev(x, torch.float32, 4), _dev(y, torch.float32), int(min(x.shape[0], y.shape[0])),
            None if idx is None else _dev(idx, torch.int32), n, float(lr), byref(loss)))
        return loss.value

    def gradient(self, x, y):
        import torch
        g = np.zeros(NPARAMS)
        loss = c_double()
        check(self.lib, self.lib.dfsph_mlp_gradient(self.h, _dev(x, torch.float32, 4), _dev(y, torch.float32),
                                                    int(x.shape[0]), g.ctypes.data_as(POINTER(c_double)),
                                                    byref(loss)))
        return g, loss.value

    def predict(self, x):
        import torch
        out = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        check(self.lib, self.lib.dfsph_mlp_predict(self.h, _dev(x, torch.float32, 4), _dev(out, torch.float32),
                                                   int(x.shape[0])))
        return out


def collect_samples(sim, steps, every=1):
    """Runs `steps` steps of `sim` with the reference warm start and returns the recorded
    (features [m, 4], target [m]) of every `every`-th step as CUDA tensors."""
    import torch
    sim.ml_record(True)
    xb = torch.empty((sim.n_fluid, 4), dtype=torch.float32, device="cuda")
    yb = torch.empty(sim.n_fluid, dtype=torch.float32, device="cuda")
    xs, ys = [], []
    try:
        for s in range(int(steps)):
            sim.step(1)
            if s % every == 0:
                c = sim.ml_capture(xb, yb)
                xs.append(xb[:c].clone())
                ys.append(yb[:c].clone())
    finally:
        sim.ml_record(False)
    return torch.cat(xs), torch.cat(ys)


def train(model, x, y, epochs=4, batch=65536, lr=2e-3, lr_final=2e-4, seed=0, fit_norm=True):
    """Adam on shuffled minibatches with a geometric learning-rate decay; returns the mean
    training loss of each epoch (normalised units)."""
    import torch
    if fit_norm:
        model.fit_normalization(x, y)
    n = int(x.shape[0])
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    nb = max(1, n // batch)
    total = epochs * nb
    losses = []
    k = 0
    for _ in range(int(epochs)):
        perm = torch.randperm(n, generator=g, device="cuda").to(torch.int32)
        acc = 0.0
        for b in range(nb):
            lr_k = lr * (lr_final / lr) ** (k / max(total - 1, 1))
            idx = perm[b * batch:(b + 1) * batch] if nb > 1 else perm
            acc += model.train_step(x, y, idx=idx.contiguous(), lr=lr_k)
            k += 1
        losses.append(acc / nb)
    return losses
