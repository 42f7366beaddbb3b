"""The learned warm start on the GPU: tensor-core inference and training kernels against
the CPU restatement (oracle/mlp_oracle.cpp), training on a known map, and the solver
with the model in its pressure warm start.

Tolerances: predictions within 2e-3 of the target scale (the GPU contracts the 4-wide
input layer with FMA and sums the 64-wide products in the tensor core's order, which can
move a BF16 rounding); gradients per parameter block with cosine >= 0.999 and relative
L2 error <= 2e-2 against the oracle's FP64 sums of the same BF16-rounded products.
"""
import numpy as np
import pytest

from difffr_gb300 import _abi
from difffr_gb300 import scene as scn

pytestmark = pytest.mark.gpu

BLOCKS = {"W1": (0, 256), "b1": (256, 320), "W2": (320, 4416), "b2": (4416, 4480), "w3": (4480, 4544),
          "b3": (4544, 4545)}


def _model(seed=3):
    from difffr_gb300.warmstart import WarmStartModel
    return WarmStartModel(seed=seed)


def _data(n, seed=0):
    import torch
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 4)).astype(np.float32) * np.array([0.01, 8.0, 0.2, 0.5], np.float32) + \
        np.array([0.002, 35.0, 0.1, 0.3], np.float32)
    y = (0.9 * x[:, 2] + 3.0 * x[:, 0] + 0.01 * rng.normal(size=n)).astype(np.float32)
    return x, y, torch.tensor(x, device="cuda"), torch.tensor(y, device="cuda")


def test_mlp_predict_matches_oracle(gpu_lib, oracle_lib):
    m = _model()
    x, y, xt, yt = _data(1000)          # not a multiple of the 128-row tile
    m.fit_normalization(xt, yt)
    p, norm = m.params()
    got = m.predict(xt).cpu().numpy()
    ref, _, _ = oracle_lib.mlp_eval(p, norm, x)
    scale = float(norm[9])
    assert np.max(np.abs(got - ref)) <= 2e-3 * scale, np.max(np.abs(got - ref)) / scale


def test_mlp_predict_after_training_matches_oracle(gpu_lib, oracle_lib):
    """Inference reads the small weights from its parameter block, a host copy refreshed
    after every parameter change: predictions after Adam steps follow the new weights."""
    m = _model(seed=9)
    x, y, xt, yt = _data(3000, seed=4)
    m.fit_normalization(xt, yt)
    p0, _ = m.params()
    m.predict(xt)                       # the host copy is current for p0
    for _ in range(3):
        m.train_step(xt, yt, lr=1e-2)
    p, norm = m.params()
    assert np.max(np.abs(p - p0)) > 1e-3
    got = m.predict(xt).cpu().numpy()
    ref, _, _ = oracle_lib.mlp_eval(p, norm, x)
    scale = float(norm[9])
    assert np.max(np.abs(got - ref)) <= 2e-3 * scale, np.max(np.abs(got - ref)) / scale


def test_mlp_predict_rejects_overlapping_buffers(gpu_lib):
    import torch
    lib = gpu_lib
    m = _model()
    n = 1000
    buf = torch.zeros(5 * n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    x = buf.data_ptr()
    rc = lib.dfsph_mlp_predict(m.h, x, x + 4 * (4 * n - 1), n)   # y starts inside x
    assert rc == _abi.DFSPH_ERR_INVALID_ARG
    assert "overlap" in lib.dfsph_last_error().decode()
    _abi.check(lib, lib.dfsph_mlp_predict(m.h, x, x + 4 * (4 * n), n))   # y right after x
    torch.cuda.synchronize()
    assert torch.isfinite(buf[4 * n:]).all()


def test_mlp_gradient_matches_oracle(gpu_lib, oracle_lib):
    m = _model(seed=5)
    x, y, xt, yt = _data(2000, seed=1)
    m.fit_normalization(xt, yt)
    p, norm = m.params()
    g, loss = m.gradient(xt, yt)
    _, gr, lr_ = oracle_lib.mlp_eval(p, norm, x, y)
    assert abs(loss - lr_) <= 1e-3 * max(lr_, 1e-6)
    for name, (a, b) in BLOCKS.items():
        u, v = g[a:b], gr[a:b]
        rel = np.linalg.norm(u - v) / max(np.linalg.norm(v), 1e-30)
        assert rel <= 2e-2, (name, rel)
        if b - a > 1:
            cos = float(u @ v / (np.linalg.norm(u) * np.linalg.norm(v) + 1e-30))
            assert cos >= 0.999, (name, cos)


def test_mlp_training_fits_a_known_map(gpu_lib):
    import torch
    from difffr_gb300.warmstart import train
    m = _model(seed=7)
    x, y, xt, yt = _data(65536, seed=2)
    losses = train(m, xt, yt, epochs=30, batch=8192, lr=3e-3, lr_final=3e-4)
    assert losses[-1] < 0.1 * losses[0], losses
    assert losses[-1] < 0.02, losses
    pred = m.predict(xt).cpu().numpy()
    r2 = 1.0 - np.mean((pred - y) ** 2) / np.var(y)
    assert r2 > 0.98, r2


def test_learned_warm_start_in_the_solver(gpu_lib):
    """Samples recorded from the plain solver; the trained model predicts held-out steps'
    stiffness better than the reference warm-start formula, and a solve started from the
    model reaches the same tolerance."""
    import torch
    from difffr_gb300.sim import DiffDFSPH
    from difffr_gb300.warmstart import collect_samples, train
    # a small dam break (16^3 particles, r = 0.01) in its collapse phase
    sc = scn.dam_break_sphere(n=(16, 16, 16), r=0.01, box=(0.7, 0.45, 0.45), dt=0.001)
    sim = DiffDFSPH(sc)
    sim.set_gradient_enabled(False)
    sim.step(100)
    xtr, ytr = collect_samples(sim, 60)
    xte, yte = collect_samples(sim, 20)
    assert xtr.shape[0] > 1000 and torch.isfinite(xtr).all() and torch.isfinite(ytr).all()
    m = _model(seed=11)
    train(m, xtr, ytr, epochs=40, batch=4096, lr=3e-3, lr_final=3e-4)
    invH2 = 1.0 / sc.params.time_step ** 2
    plain = 0.5 * torch.clamp(xte[:, 2], min=-0.00025 * invH2)
    mse_plain = float(torch.mean((plain - yte) ** 2))
    mse_model = float(torch.mean((m.predict(xte) - yte) ** 2))
    assert mse_model < mse_plain, (mse_model, mse_plain)
    # the solver with the model: converges to the same tolerance
    slot = sim.checkpoint_save()
    st_plain = sim.step(5)
    sim.checkpoint_restore(slot)
    sim.set_warmstart_model(m)
    st_ml = sim.step(5)
    eta = sc.params.max_error * 0.01 * sc.params.density0
    assert st_ml["rc"] == 0 and st_ml["pressure_avg_error"] <= eta
    assert st_plain["rc"] == 0
    sim.set_warmstart_model(None)
    sim.close()
    m.close()
