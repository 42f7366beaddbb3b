"""OBJ meshes and their boundary samples for Akinci2012 rigid bodies (host-side set-up).

- ``load_obj``: vertices and triangles of a Wavefront OBJ file ("v x y z" and "f a b c ..."
  lines, 1-based or negative indices, "a/b/c" index groups; polygons become triangle fans),
  scaled per axis as the reference's loadObj does with the body's "scale".
- ``regular_triangle_samples``: the reference's RegularTriangleSampling
  (SPlisHSPlasH/Utilities/RegularTriangleSampling.cpp:13-117), restated: every vertex; each
  unique edge at ceil(l / d) + 1 evenly spaced points without its end points; each
  triangle in lines parallel to its longest edge, ceil(h / d) + 1 lines from the base to
  the opposite vertex without the first and last, each line at ceil(len / d) + 1 evenly
  spaced points without its end points. The reference samples rigid bodies with
  d = 1.5 r in this mode (RigidBody3dBoundarySimulator.cpp:149-156).

The reference's default surface sampling for rigid bodies is its Poisson-disk sampler
(samplingMode 0), which draws from std::default_random_engine; this library samples
every OBJ body with the regular triangle pattern (samplingMode 1) instead, so boundary
sample sets of mode-0 scenes differ from the reference's.
"""
from __future__ import annotations

import math

import numpy as np


def load_obj(path, scale=(1.0, 1.0, 1.0)):
    verts, faces = [], []
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "v" and len(p) >= 4:
                verts.append([float(p[1]), float(p[2]), float(p[3])])
            elif p[0] == "f" and len(p) >= 4:
                idx = []
                for tok in p[1:]:
                    k = int(tok.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(verts) + k)
                for t in range(1, len(idx) - 1):
                    faces.append([idx[0], idx[t], idx[t + 1]])
    v = np.asarray(verts, dtype=np.float64).reshape(-1, 3) * np.asarray(scale, dtype=np.float64)
    fa = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    if fa.size and (fa.min() < 0 or fa.max() >= v.shape[0]):
        raise ValueError(f"{path}: face index out of range")
    return v, fa


def _unique_edges(faces):
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]], axis=0)
    e = np.sort(e, axis=1)
    return np.unique(e, axis=0)  # sorted by (first, second) index


def regular_triangle_samples(vertices, faces, d):
    v = np.asarray(vertices, dtype=np.float64)
    faces = np.asarray(faces, dtype=np.int64)
    out = [v.copy()]
    # edges without their end points (:27-46)
    for a, b in _unique_edges(faces):
        v0 = v[a]
        direction = v[b] - v0
        n = int(math.ceil(np.linalg.norm(direction) / d)) + 1
        if n == 1:
            out.append(v0[None, :])
            continue
        i = np.arange(1, n - 1, dtype=np.float64)
        if i.size:
            out.append(v0 + (i / (n - 1))[:, None] * direction)
    # faces, lines parallel to the longest edge, without the edge samples (:48-94)
    for f in faces:
        l2, v0, base, top = 0.0, None, None, None
        for c in range(3):
            e = v[f[(c + 1) % 3]] - v[f[c]]
            le2 = float(e @ e)
            if le2 > l2:
                l2, v0, base, top = le2, v[f[c]], e, v[f[(c + 2) % 3]] - v[f[c]]
        if v0 is None:
            continue
        length = math.sqrt(l2)
        bn = base / length
        height = float(np.linalg.norm(top - (bn @ top) * bn))
        num_lines = int(math.ceil(height / d)) + 1
        for line in range(1, num_lines - 1):
            alpha = line / (num_lines - 1)
            start = v0 + alpha * top
            line_len = (1.0 - alpha) * length
            ns = int(math.ceil(line_len / d)) + 1
            if ns < 3:
                continue
            i = np.arange(1, ns - 1, dtype=np.float64)
            out.append(start + ((i * line_len) / (ns - 1))[:, None] * bn)
    return np.vstack(out)


def sample_obj(path, scale, particle_radius):
    """Boundary samples of an OBJ body in its local frame (regular triangle pattern, d = 1.5 r)."""
    v, f = load_obj(path, scale)
    return regular_triangle_samples(v, f, 1.5 * particle_radius)
