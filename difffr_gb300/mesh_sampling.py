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

- ``poisson_disk_samples``: the reference's default (samplingMode 0,
  SPlisHSPlasH/Utilities/PoissonDiskSampling.cpp:20-435, called with the minimum distance
  r, 10 trials and the geodesic distance norm from RigidBody3dBoundarySimulator.cpp:140-146),
  restated: 40 candidates per pi r^2 of surface, drawn with square-root barycentric
  coordinates on triangles picked with probability proportional to area (stochastic
  acceptance); cells of size r / sqrt(3) indexed floor((x - min) / size) + 1 and sorted
  lexicographically; then for each trial k and each of the 27 phase groups
  (cx mod 3 + 3 (cy mod 3) + 9 (cz mod 3)) the k-th candidate of every cell of the group
  is accepted unless an accepted sample within two cells lies closer than r, with the
  distance between points of different triangles stretched by
  (asin c1 - asin c2) / (c1 - c2) (c = the triangles' normals against the joining
  direction). Cells of one phase group are three cells apart, so their candidates never
  conflict with each other and a group is tested at once. The reference seeds its
  generators from std::random_device, so its sample sets differ from run to run; here the
  generator is numpy's, seeded, so a scene samples the same way every time.
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


def _dot3(a, b):
    """a . b summed as Eigen sums a 3-vector of doubles: (a0 b0 + a1 b1) + a2 b2."""
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def regular_triangle_samples(vertices, faces, d):
    v = np.asarray(vertices, dtype=np.float64)
    faces = np.asarray(faces, dtype=np.int64)
    out = [v.copy()]
    # edges without their end points (:27-46)
    for a, b in _unique_edges(faces):
        v0 = v[a]
        direction = v[b] - v0
        n = int(math.ceil(math.sqrt(_dot3(direction, direction)) / d)) + 1
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
            le2 = float(_dot3(e, e))
            if le2 > l2:
                l2, v0, base, top = le2, v[f[c]], e, v[f[(c + 2) % 3]] - v[f[c]]
        if v0 is None:
            continue
        length = math.sqrt(l2)
        bn = base / length
        hv = top - _dot3(bn, top) * bn
        height = math.sqrt(_dot3(hv, hv))
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


def _tri_pick(areas, n, rng):
    """n triangle indices with probability proportional to area (stochastic acceptance,
    PoissonDiskSampling.cpp:171-195)."""
    out = np.empty(n, dtype=np.int64)
    todo = np.arange(n)
    amax = areas.max()
    while todo.size:
        idx = np.minimum((areas.size * rng.random(todo.size)).astype(np.int64), areas.size - 1)
        ok = rng.random(todo.size) < areas[idx] / amax
        out[todo[ok]] = idx[ok]
        todo = todo[~ok]
    return out


def poisson_disk_samples(vertices, faces, r, num_trials=10, distance_norm=1, seed=0):
    v = np.asarray(vertices, dtype=np.float64)
    f = np.asarray(faces, dtype=np.int64)
    if f.size == 0:
        return np.zeros((0, 3))
    rng = np.random.default_rng(seed)
    cell = r / math.sqrt(3.0)
    minv = v.min(axis=0)
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    cr = np.cross(b - a, c - a)
    crn = np.linalg.norm(cr, axis=1)
    areas = crn / 2.0
    normals = cr / np.where(crn > 0, crn, 1.0)[:, None]
    n0 = int(40.0 * (areas.sum() / (math.pi * r * r)))
    if n0 == 0:
        return np.zeros((0, 3))
    # initial candidates (:120-169)
    rn1 = np.sqrt(rng.random(n0))
    bc1 = 1.0 - rn1
    bc2 = rng.random(n0) * rn1
    bc3 = 1.0 - bc1 - bc2
    tri = _tri_pick(areas, n0, rng)
    pos = bc1[:, None] * a[tri] + bc2[:, None] * b[tri] + bc3[:, None] * c[tri]
    cp = np.floor((pos - minv) / cell).astype(np.int64) + 1
    order = np.lexsort((cp[:, 2], cp[:, 1], cp[:, 0]))
    pos, tri, cp = pos[order], tri[order], cp[order]
    new_cell = np.ones(n0, dtype=bool)
    new_cell[1:] = np.any(cp[1:] != cp[:-1], axis=1)
    starts = np.flatnonzero(new_cell)                  # first candidate of each cell
    ucell = cp[starts]                                 # the cells, in sorted order
    run = np.diff(np.append(starts, n0))               # candidates per cell
    uid_of = np.cumsum(new_cell) - 1                   # candidate -> cell id
    # cell id lookup on a padded dense grid (neighbours reach two cells out)
    dims = ucell.max(axis=0) + 5
    lin = ((ucell[:, 0] + 2) * dims[1] + (ucell[:, 1] + 2)) * dims[2] + (ucell[:, 2] + 2)
    grid = np.full(int(dims[0] * dims[1] * dims[2]), -1, dtype=np.int32)
    grid[lin] = np.arange(ucell.shape[0])
    occ = np.full(ucell.shape[0] + 1, -1, dtype=np.int64)  # accepted candidate of each cell (+ a -1 slot)
    phase = ucell[:, 0] % 3 + 3 * (ucell[:, 1] % 3) + 9 * (ucell[:, 2] % 3)
    groups = [np.flatnonzero(phase == g) for g in range(27)]
    off = np.stack(np.meshgrid(np.arange(-2, 3), np.arange(-2, 3), np.arange(-2, 3), indexing="ij"), -1).reshape(-1, 3)
    off = off[np.sum(np.abs(off) == 2, axis=1) < 3]  # the corners lie farther than r
    off_lin = (off[:, 0] * dims[1] + off[:, 1]) * dims[2] + off[:, 2]
    accepted = []
    for k in range(num_trials):
        for g in groups:
            cells = g[run[g] > k]
            if cells.size == 0:
                continue
            cand = starts[cells] + k
            nid = grid[lin[cells][:, None] + off_lin[None, :]]        # neighbour cell ids, -1 = empty
            other = occ[nid]                                          # accepted neighbour candidates
            conflict = np.zeros(cells.size, dtype=bool)
            mi, ni = np.nonzero(other >= 0)
            if mi.size:
                pi, pj = cand[mi], other[mi, ni]
                d = pos[pj] - pos[pi]
                e = np.linalg.norm(d, axis=1)
                dist = e.copy()
                if distance_norm == 1:
                    diff = tri[pi] != tri[pj]
                    u = d / np.where(e > 0, e, 1.0)[:, None]
                    c1 = np.clip(np.einsum("ij,ij->i", normals[tri[pi]], u), -1.0, 1.0)
                    c2 = np.clip(np.einsum("ij,ij->i", normals[tri[pj]], u), -1.0, 1.0)
                    dc = c1 - c2
                    with np.errstate(divide="ignore", invalid="ignore"):
                        stretch = np.where(np.abs(dc) > 1e-5, (np.arcsin(c1) - np.arcsin(c2)) / np.where(dc != 0, dc, 1.0),
                                           1.0 / np.sqrt(np.maximum(1.0 - c1 * c1, 0.0)))
                    dist = np.where(diff, e * stretch, e)
                hit = dist < r
                conflict[mi[hit]] = True
            take = cells[~conflict]
            occ[take] = starts[take] + k
            accepted.append(starts[take] + k)
    idx = np.concatenate(accepted) if accepted else np.zeros(0, dtype=np.int64)
    return pos[idx]


def sample_obj(path, scale, particle_radius, mode=1, seed=0):
    """Boundary samples of an OBJ body in its local frame: mode 0 the Poisson-disk pattern
    with minimum distance r (the reference's default), mode 1 the regular triangle pattern
    at d = 1.5 r."""
    v, f = load_obj(path, scale)
    if mode == 0:
        return poisson_disk_samples(v, f, particle_radius, seed=seed)
    return regular_triangle_samples(v, f, 1.5 * particle_radius)
