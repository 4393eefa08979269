"""Mesh bodies: a scene's "Bodies" entries voxelised into particles (eng/particle_func.py:265-294
``load_body``, used by eng/particle_system.py:82-91 and :175-200 ``init_body``).

The reference loads the geometry file with the ``trimesh`` package (not installed here) and
calls, in order, ``apply_scale(scale)``, ``apply_transform(rotation_matrix(angle, axis,
vertices.mean(axis=-1)))``, ``voxelized(pitch=particle_diameter).fill()`` and takes the
voxel centres plus the body's translation.  This module restates those steps:

* Wavefront OBJ geometry (``v`` and ``f`` records; polygons split into a fan of triangles
  from their first vertex; ``a/b/c`` references and negative indices resolved) or STL
  (ASCII or binary);
* the rotation about an axis through a point (Rodrigues' formula as a 4 x 4 homogeneous
  matrix).  The reference passes ``vertices.mean(axis=-1)`` as the point: the mean of each
  vertex's three coordinates, of which the rotation takes the first three values.  That is
  kept as written;
* voxelisation by subdivision: the triangles are split at their edge midpoints (a
  triangle into four) until no edge is longer than half the pitch, every vertex is rounded
  to the nearest multiple of the pitch (numpy's round half to even), and the occupied
  cells, indexed from their smallest index per axis, form a dense grid;
* ``fill``: the grid's enclosed cavities filled (scipy.ndimage.binary_fill_holes);
* the voxel centres (cell index x pitch + origin, origin = smallest index x pitch) in the
  grid's C order, plus the translation.

No golden vectors exist for this path (the reference ships no tests and trimesh cannot be
run here); tests/test_mesh_body.py checks it on shapes whose voxelisation is known in
closed form.
"""
import math

import numpy as np


def load_obj(path):
    """(vertices (V, 3) float64, triangles (F, 3) int64) of a Wavefront OBJ file."""
    verts, faces = [], []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v":
                verts.append([float(c) for c in parts[1:4]])
            elif parts[0] == "f":
                idx = []
                for ref in parts[1:]:
                    k = int(ref.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(verts) + k)
                for q in range(1, len(idx) - 1):
                    faces.append([idx[0], idx[q], idx[q + 1]])
    v = np.asarray(verts, dtype=np.float64).reshape(-1, 3)
    fa = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
    if fa.size and (fa.min() < 0 or fa.max() >= len(v)):
        raise ValueError(f"{path}: face references a missing vertex")
    return v, fa


def load_stl(path):
    """(vertices (3F, 3) float64, triangles (F, 3) int64) of an STL file, ASCII or binary
    (each triangle keeps its own three vertices)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:5].lower() == b"solid" and b"facet" in data[:1024]:
        pts = [[float(c) for c in line.split()[1:4]] for line in data.decode("ascii", "replace").splitlines()
               if line.strip().startswith("vertex")]
        v = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
    else:
        n = int(np.frombuffer(data[80:84], dtype="<u4")[0])
        rec = np.dtype([("normal", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")])
        if len(data) < 84 + n * rec.itemsize:
            raise ValueError(f"{path}: truncated binary STL")
        tri = np.frombuffer(data[84:84 + n * rec.itemsize], dtype=rec)
        v = tri["v"].reshape(-1, 3).astype(np.float64)
    if len(v) % 3:
        raise ValueError(f"{path}: vertex count not a multiple of three")
    return v, np.arange(len(v), dtype=np.int64).reshape(-1, 3)


def load_mesh(path):
    """OBJ or STL geometry by the file's extension."""
    if str(path).lower().endswith(".stl"):
        return load_stl(path)
    return load_obj(path)


def rotation_matrix(angle, direction, point=None):
    """4 x 4 matrix of the rotation by angle (radians) about the axis `direction` through
    `point` (the first three values of it are used)."""
    s, c = math.sin(angle), math.cos(angle)
    d = np.asarray(direction[:3], dtype=np.float64)
    d = d / math.sqrt(float(np.dot(d, d)))
    m = np.diag([c, c, c, 1.0])
    m[:3, :3] += np.outer(d, d) * (1.0 - c)
    ds = d * s
    m[:3, :3] += np.array([[0.0, -ds[2], ds[1]], [ds[2], 0.0, -ds[0]], [-ds[1], ds[0], 0.0]])
    if point is not None:
        p = np.asarray(point[:3], dtype=np.float64)
        m[:3, 3] = p - np.dot(m[:3, :3], p)
    return m


def transform_points(points, matrix):
    """points (N, 3) through a 4 x 4 homogeneous matrix."""
    h = np.column_stack((points, np.ones(len(points))))
    return np.dot(matrix, h.T).T[:, :3]


def _split(vertices, faces):
    """Each triangle into four at its edge midpoints (a midpoint shared by the triangles of
    an edge is one vertex)."""
    e = np.sort(np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]]), axis=1)
    uniq, inv = np.unique(e, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    mids = (vertices[uniq[:, 0]] + vertices[uniq[:, 1]]) / 2.0
    base = len(vertices)
    nf = len(faces)
    m01, m12, m20 = (inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base)
    a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
    new = np.concatenate([np.column_stack((a, m01, m20)), np.column_stack((m01, b, m12)),
                          np.column_stack((m20, m12, c)), np.column_stack((m01, m12, m20))])
    return np.vstack((vertices, mids)), new


def subdivide_to_size(vertices, faces, max_edge, max_iter=10):
    """Vertices of the mesh split until no triangle edge is longer than max_edge: the
    triangles short enough are kept, the others split (up to max_iter rounds)."""
    done = []
    v, f = vertices, faces
    for it in range(max_iter + 1):
        tri = v[f]
        edge = np.sqrt(((np.diff(tri[:, [0, 1, 2, 0]], axis=1)) ** 2).sum(axis=2))
        too_long = (edge > max_edge).any(axis=1)
        ok = f[~too_long]
        if len(ok):
            done.append(v[np.unique(ok.reshape(-1))])
        if not too_long.any():
            break
        if it == max_iter:
            raise ValueError("mesh body: edges still longer than half the particle diameter after "
                             f"{max_iter} subdivisions (scale the mesh or split it)")
        v, f = _split(v, f[too_long])
    return np.vstack(done) if done else np.zeros((0, 3))


def voxel_points(vertices, faces, pitch):
    """Centres of the filled voxel grid of a closed triangle mesh (see the module docstring)."""
    from scipy.ndimage import binary_fill_holes
    v = subdivide_to_size(vertices, faces, pitch / 2.0)
    hit = np.round(v / pitch).astype(np.int64)
    occupied = np.unique(hit, axis=0)
    origin = occupied.min(axis=0)
    idx = occupied - origin
    grid = np.zeros(idx.max(axis=0) + 1, dtype=bool)
    grid[idx[:, 0], idx[:, 1], idx[:, 2]] = True
    grid = binary_fill_holes(grid)
    cells = np.column_stack(np.nonzero(grid)).astype(np.float64)
    return cells * pitch + origin.astype(np.float64) * pitch


def load_body(body, pitch, base_dir=None):
    """Particle positions of one "Bodies" entry (eng/particle_func.py:265-294): the mesh
    scaled, rotated, voxelised at the particle diameter and filled, plus its translation."""
    import os
    path = body["geometryFile"]
    if base_dir is not None and not os.path.isabs(path) and not os.path.exists(path):
        path = os.path.join(base_dir, path)
    v, f = load_mesh(path)
    v = v * np.asarray(body.get("scale", 1.0), dtype=np.float64)
    angle = float(body.get("rotationAngle", 0.0)) / 180 * math.pi
    axis = body.get("rotationAxis", [0.0, 0.0, 1.0])
    v = transform_points(v, rotation_matrix(angle, axis, v.mean(axis=-1)))
    return voxel_points(v, f, pitch) + np.asarray(body["translation"], dtype=np.float64)
