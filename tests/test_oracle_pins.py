"""The oracle's kernel and quaternion algebra against golden vectors produced by the
reference's own SPHKernels.h / GradientUtils.cpp (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_kernels.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_cubic_kernel_double_bit_exact(oracle_lib, gold):
    W, G, H = oracle_lib.kernel_eval(float(gold["h"]), gold["r"])
    assert np.array_equal(W, gold["double_W"])
    assert np.array_equal(G, gold["double_gradW"])
    assert np.array_equal(H, gold["double_gradGradW"])


def test_cubic_kernel_float_bit_exact(oracle_lib, gold):
    W, G, H = oracle_lib.kernel_eval_f(float(gold["h"]), gold["r"].astype(np.float32))
    assert np.array_equal(W, gold["float_W"])
    assert np.array_equal(G, gold["float_gradW"])
    assert np.array_equal(H, gold["float_gradGradW"])


def test_surface_tension_kernels_bit_exact(oracle_lib, gold):
    """Cohesion and adhesion kernels (SPHKernels.h:437-559) against the reference's own
    compiled sources, double and float builds. At |r| = h exactly the float adhesion kernel
    takes the 0.25 power of a slightly negative number and both give NaN (compared as equal);
    the GPU kernel clamps that argument at zero, and neighbour pairs have |r| < h."""
    C, A = oracle_lib.st_kernel_eval(float(gold["h"]), gold["r"])
    assert np.array_equal(C, gold["double_cohesion"])
    assert np.array_equal(A, gold["double_adhesion"])
    Cf, Af = oracle_lib.st_kernel_eval(float(gold["h"]), gold["r"].astype(np.float32), single=True)
    assert np.array_equal(Cf, gold["float_cohesion"])
    assert np.array_equal(Af, gold["float_adhesion"], equal_nan=True)


def test_quaternion_jacobians_bit_exact(oracle_lib, gold):
    a, b, c, d = oracle_lib.quat_eval(gold["qp"][:, :4], gold["qp"][:, 4:])
    assert np.array_equal(a, gold["double_Rqp"])
    assert np.array_equal(b, gold["double_RqTp"])
    assert np.array_equal(c, gold["double_pq"])
    assert np.array_equal(d, gold["double_wq"])


def test_kernel_edge_cases(oracle_lib, gold):
    """Zero offset: W = W0 = 8/(pi h^3), gradient cut below 1e-5, zero outside support."""
    h = float(gold["h"])
    r = np.array([[0.0, 0.0, 0.0], [3e-6, 0, 0], [h * 1.0000001, 0, 0], [2 * h, 0, 0]])
    W, G, H = oracle_lib.kernel_eval(h, r)
    assert W[0] == pytest.approx(8.0 / (np.pi * h ** 3), rel=1e-15)
    assert np.all(G[:2] == 0) and np.all(H[:2] == 0)
    assert W[2] == 0 and W[3] == 0 and np.all(G[2:] == 0)


def test_kernel_normalisation_and_antisymmetry(oracle_lib):
    """Integral of W over its support is 1; grad W is odd."""
    h = 0.1
    g = np.linspace(-h, h, 61)
    dx = g[1] - g[0]
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    r = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    W, G, _ = oracle_lib.kernel_eval(h, r)
    assert W.sum() * dx ** 3 == pytest.approx(1.0, rel=2e-3)
    W2, G2, _ = oracle_lib.kernel_eval(h, -r)
    assert np.array_equal(W, W2) and np.allclose(G, -G2, atol=0, rtol=0)


# --------------------------------------------------------------------------- the step itself
# tests/golden/reference_step.npz holds what the reference's own DiffDFSPH step (its sources
# compiled by oracle/build_ref_step.sh) produced on small contact scenes: per step the sweep
# counts, the body's state, fluid force and torque and gradient chain state; after the last
# step the fluid fields and the boundary volumes. In FP64 the oracle reproduces it to the last
# bits (1e-12 relative allows for summation-order rounding; the fields were equal bit for bit
# when the fixture was made). In FP32 (the reference's float build against the oracle's float
# mode) the tolerance is 1e-5.
import ref_step_fixture as rsf  # noqa: E402

_STEP_GOLD, _STEP_META = rsf.load()


@pytest.mark.parametrize("case", sorted(_STEP_META))
def test_oracle_step_matches_reference_step(oracle_lib, case):
    m = _STEP_META[case]
    sc = rsf.scene_of(m)
    mode = oracle_lib.MODE_F64 if m["build"] == "double" else oracle_lib.MODE_F32
    o = oracle_lib.Oracle(sc, mode=mode)
    worst, iters_equal = rsf.compare(o, sc, _STEP_GOLD, case, m["steps"])
    assert iters_equal
    tol = 1e-12 if m["build"] == "double" else 1e-5
    bad = {k: v for k, v in worst.items() if v > tol}
    assert not bad, (case, bad)


def test_regular_triangle_sampling_bit_exact():
    """difffr_gb300.mesh_sampling's regular triangle pattern (samplingMode 1) against the
    reference's own RegularTriangleSampling::sampleMesh (tests/golden/make_golden.py): the
    same samples in the same order, bit for bit, on a cube at two spacings and on a seeded
    triangle soup."""
    from difffr_gb300.mesh_sampling import regular_triangle_samples
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_sampling.npz"))
    k = 0
    while f"{k}_samples" in g:
        s = regular_triangle_samples(g[f"{k}_vertices"], g[f"{k}_faces"], float(g[f"{k}_d"]))
        assert np.array_equal(s, g[f"{k}_samples"]), k
        k += 1
    assert k == 3
