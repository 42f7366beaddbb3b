"""Rigid-body records of the reference's binary state files (host-side I/O).

SimulatorBase::saveState (Simulator/SimulatorBase.cpp:1899-2005) writes two binary files
per state besides the fluid's BGEO file:

* ``state_<n>.bin``: the scene file's MD5, frame counters, every GenericParameters value
  of the simulator objects, the time manager's and the simulation's state, then the
  rigid records;
* ``state_<n>_dynamicRB.bin``: the rigid records alone.

A rigid record is written for every dynamic or animated body in boundary-model order as
four raw Eigen matrices in the build's scalar type (float by default, double with
USE_DOUBLE; BinaryFileWriter::writeMatrix, Utilities/BinaryFileReaderWriter.h:53-56):
position (3), rotation coefficients in Eigen's (x, y, z, w) order (4), velocity (3) and
angular velocity (3). Nothing follows the records in either file, so they are read from
the end; loadStateWithRigidExisted (SimulatorBase.cpp:2124-2201) reads the same records
after the parameter block. The parameter block itself depends on the full
GenericParameters registry of the reference's build and is not interpreted here.

The scalar type is detected from the records: the one whose quaternions all have unit
norm.
"""
from __future__ import annotations

import numpy as np

RECORD = 13  # x(3) q(4: x, y, z, w) v(3) omega(3)


def read_rigid_records(path, n_bodies, real=None):
    """The last ``n_bodies`` rigid records of a state file as a list of
    (x, q (w, x, y, z), v, omega) in float64, and the scalar type they were stored in."""
    data = open(path, "rb").read()
    cands = [np.dtype(real)] if real is not None else [np.dtype(np.float32), np.dtype(np.float64)]
    for dt in cands:
        nbytes = RECORD * n_bodies * dt.itemsize
        if nbytes > len(data):
            continue
        a = np.frombuffer(data[len(data) - nbytes:], dtype=dt.newbyteorder("<")).reshape(n_bodies, RECORD)
        a = a.astype(np.float64)
        qn = np.linalg.norm(a[:, 3:7], axis=1)
        if real is not None or (np.all(np.isfinite(a)) and np.all(np.abs(qn - 1.0) < 1e-4)):
            out = [(r[0:3].copy(), np.array([r[6], r[3], r[4], r[5]]), r[7:10].copy(), r[10:13].copy()) for r in a]
            return out, dt
    raise ValueError(f"{path}: no {n_bodies} rigid records with unit quaternions at the end of the file")


def write_dynamic_rb(path, records, real=np.float32):
    """Writes ``state_<n>_dynamicRB.bin``: records (x, q (w, x, y, z), v, omega) per dynamic
    or animated body, in the scalar type ``real``, little-endian."""
    rows = []
    for x, q, v, w in records:
        q = np.asarray(q, dtype=np.float64)
        rows.append(np.concatenate([np.asarray(x, float), [q[1], q[2], q[3], q[0]], np.asarray(v, float),
                                    np.asarray(w, float)]))
    a = np.asarray(rows, dtype=np.float64).reshape(-1, RECORD)
    with open(path, "wb") as f:
        f.write(a.astype(np.dtype(real).newbyteorder("<")).tobytes())
