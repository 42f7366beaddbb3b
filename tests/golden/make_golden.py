"""Generates golden vectors for the oracle from the reference's own sources.

Runs oracle/_ref/ref_pin_{double,float} (built by oracle/build_ref.sh from the
reference's SPHKernels.h/.cpp and GradientUtils.cpp) on seeded inputs and stores
inputs and outputs in tests/golden/reference_kernels.npz; runs oracle/_ref/ref_sampling_double
(the reference's RegularTriangleSampling.cpp) on a cube and a seeded triangle soup and stores
the meshes and samples in tests/golden/reference_sampling.npz. Run in a container that
has the reference checkout:

    sh oracle/build_ref.sh /path/to/DiffFR && python tests/golden/make_golden.py
"""
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "..", "..", "oracle", "_ref")


def inputs(seed=1234):
    rng = np.random.default_rng(seed)
    h = 0.1
    r = []
    # edge cases: zero offset, below the 1e-5 gradient cut, exactly q = 0.5 and q = 1, just outside
    for d in (0.0, 5e-6, 0.05, 0.1, 0.1000001, 0.0999999, 0.0500001, 0.12):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        r.append(d * u)
    r.append([0.05, 0.0, 0.0])
    r.append([0.0, 0.1, 0.0])
    # random offsets inside and around the support
    dirs = rng.normal(size=(400, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rad = rng.uniform(0.0, 1.1 * h, size=(400, 1))
    r = np.vstack([np.array(r), dirs * rad])
    q = rng.normal(size=(64, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    p = rng.uniform(-0.2, 0.2, size=(64, 3))
    return h, r, np.hstack([q, p])


def run(binary, h, r, qp, dtype):
    blob = struct.pack("<di", h, r.shape[0]) + r.astype("<f8").tobytes() + struct.pack("<i", qp.shape[0])
    blob += qp.astype("<f8").tobytes()
    out = subprocess.run([binary], input=blob, capture_output=True, check=True).stdout
    a = np.frombuffer(out, dtype=dtype)
    nk = r.shape[0] * 13
    nq = qp.shape[0] * 52
    k = a[:nk].reshape(-1, 13)
    qq = a[nk:nk + nq].reshape(-1, 52)
    st = a[nk + nq:].reshape(-1, 2)
    return {"W": k[:, 0], "gradW": k[:, 1:4], "gradGradW": k[:, 4:13].reshape(-1, 3, 3),
            "Rqp": qq[:, 0:12].reshape(-1, 3, 4), "RqTp": qq[:, 12:24].reshape(-1, 3, 4),
            "pq": qq[:, 24:40].reshape(-1, 4, 4), "wq": qq[:, 40:52].reshape(-1, 4, 3),
            "cohesion": st[:, 0], "adhesion": st[:, 1]}


def sampling_meshes(seed=3):
    """A unit cube (12 triangles) and a seeded triangle soup, with the spacings they are
    sampled at."""
    v = np.array([[x, y, z] for x in (-.5, .5) for y in (-.5, .5) for z in (-.5, .5)])
    f = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6], [0, 2, 6],
                  [0, 6, 4], [1, 5, 7], [1, 7, 3]])
    rng = np.random.default_rng(seed)
    sv = rng.normal(size=(12, 3))
    sf = rng.integers(0, 12, size=(14, 3))
    sf = sf[(sf[:, 0] != sf[:, 1]) & (sf[:, 1] != sf[:, 2]) & (sf[:, 0] != sf[:, 2])]
    return [("cube", v, f, 0.0375), ("cube", v, f, 0.1), ("soup", sv, sf, 0.15)]


def run_sampling(v, f, d):
    """The reference's RegularTriangleSampling::sampleMesh (oracle/_ref/ref_sampling_double)."""
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        np.concatenate([np.array([len(v), len(f), d], np.float64), np.asarray(v, np.float64).ravel(),
                        np.asarray(f, np.float64).ravel()]).tofile(fin)
        subprocess.run([os.path.join(REF, "ref_sampling_double"), fin, fout], check=True)
        return np.fromfile(fout, np.float64).reshape(-1, 3)


def main():
    samp = {}
    for k, (name, v, f, d) in enumerate(sampling_meshes()):
        samp[f"{k}_vertices"], samp[f"{k}_faces"], samp[f"{k}_d"] = v, f, np.array(d)
        samp[f"{k}_samples"] = run_sampling(v, f, d)
    np.savez_compressed(os.path.join(HERE, "reference_sampling.npz"), **samp)
    print("wrote", os.path.join(HERE, "reference_sampling.npz"))
    h, r, qp = inputs()
    res = {"h": np.array(h), "r": r, "qp": qp}
    for prec, dt in (("double", "<f8"), ("float", "<f4")):
        o = run(os.path.join(REF, f"ref_pin_{prec}"), h, r, qp, dt)
        for k, v in o.items():
            res[f"{prec}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "reference_kernels.npz"), **res)
    print("wrote", os.path.join(HERE, "reference_kernels.npz"))


if __name__ == "__main__":
    main()
