"""Generates golden vectors for the oracle from the reference's own sources.

Runs oracle/_ref/ref_pin_{double,float} (built by oracle/build_ref.sh from the
reference's SPHKernels.h/.cpp and GradientUtils.cpp) on seeded inputs and stores
inputs and outputs in tests/golden/reference_kernels.npz. Run in a container that
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


def main():
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
