"""Host-side particle generators (numpy), restating the reference's scene construction.

The reference builds its initial particle set on the host with numpy and uploads it
once (eng/particle_func.py:176-208, eng/particle_system.py:289-314).  The functions
here produce the same arrays in the same order, so that particle ``id0`` values match
the reference's ``set_id0`` numbering (eng/particle_system.py:208-211):

* ``calc_cube_particle_num`` - lattice coordinates per axis:
  ``arange(t + off/2, t + size + 1e-5, off)`` (eng/particle_func.py:253-259).
* ``cube_lattice`` - ``meshgrid(indexing='ij')`` flattened with x slowest; in 2D the z
  list is ``[0.0]`` (eng/particle_func.py:189-196).
* ``calc_dummy_boundary`` - the wall boxes of dummy particles: 3 boxes in 2D (left,
  floor, right) and 5 in 3D (back, right, front, left, floor), no top wall
  (eng/particle_func.py:316-343).
* ``calc_rep_boundary`` - repulsive-particle boxes (eng/particle_func.py:346-374).
"""
from functools import reduce

import numpy as np

MAT_REP = -2
MAT_DUMMY = -1
MAT_FLUID = 1
MAT_SOIL = 2
MAT_RIGID = 11


def calc_cube_particle_num(translation, size, dim=3, offset=None):
    """Per-axis lattice coordinates and their product count (eng/particle_func.py:253-259)."""
    step = offset if offset is not None else 0.1
    axes = []
    for d in range(dim):
        s = step if size[d] >= 0 else -step
        axes.append(np.arange(translation[d] + s / 2.0, translation[d] + size[d] + 1e-5, s))
    count = reduce(lambda a, b: a * b, [len(a) for a in axes])
    return count, axes


def cube_lattice(lower_corner, cube_size, dim, offset):
    """(n, 3) f64 lattice positions of one cube, x slowest (eng/particle_func.py:189-196)."""
    n, axes = calc_cube_particle_num(lower_corner, cube_size, dim, offset=offset)
    if dim == 2:
        axes = axes + [np.array([0.0])]
    grid = np.array(np.meshgrid(*axes, sparse=False, indexing="ij"), dtype=np.float64)
    pts = grid.reshape(grid.shape[0], -1).transpose().copy()
    assert pts.shape[0] == n
    return pts


def count_cube_num(pos_bld, pos_fru, dim, offset):
    n, _ = calc_cube_particle_num(pos_bld, np.asarray(pos_fru) - np.asarray(pos_bld), dim, offset=offset)
    return n


def count_boundary(boundary, dim, offset):
    return sum(count_cube_num(b[0], b[1], dim, offset) for b in boundary)


def chk_block_in_domain(domain_start, domain_end, translation, size, dim):
    """Raise when a block leaves the domain (eng/particle_func.py:246-251)."""
    ok_start = all(translation[d] - domain_start[d] >= 0.0 for d in range(dim))
    ok_end = all(translation[d] + size[d] - domain_end[d] <= 0.0 for d in range(dim))
    if not (ok_start and ok_end):
        raise ValueError("Block is not in domain!")


def calc_dummy_boundary(dim, ds, de, vs, ve):
    """Dummy wall boxes [lower, upper] (eng/particle_func.py:316-343); no top wall."""
    if dim == 3:
        return [
            [np.array([vs[0], ds[1], vs[2]]), np.array([ds[0], de[1], de[2]])],  # back  (x < 0)
            [np.array([vs[0], ds[1], de[2]]), np.array([de[0], de[1], ve[2]])],  # right (z > end)
            [np.array([de[0], ds[1], ds[2]]), np.array([ve[0], de[1], ve[2]])],  # front (x > end)
            [np.array([ds[0], ds[1], vs[2]]), np.array([ve[0], de[1], ds[2]])],  # left  (z < 0)
            [np.array(vs, dtype=np.float64), np.array([ve[0], ds[1], ve[2]])],   # floor
        ]
    return [
        [np.array([vs[0], ds[1], ds[2]]), np.array([ds[0], de[1], de[2]])],      # left wall
        [np.array([vs[0], vs[1], ds[2]]), np.array([ve[0], ds[1], de[2]])],      # floor
        [np.array([de[0], ds[1], ds[2]]), np.array([ve[0], de[1], de[2]])],      # right wall
    ]


def calc_rep_boundary(dim, ds, de, radius):
    """Repulsive-particle boxes (eng/particle_func.py:346-374)."""
    t = radius / 2
    if dim == 3:
        return [
            [np.array([ds[0] - t, ds[1] + t, ds[2] - t]), np.array([ds[0] + t, de[1] - t, de[2] - t])],
            [np.array([ds[0] - t, ds[1] + t, de[2] - t]), np.array([de[0] - t, de[1] - t, de[2] + t])],
            [np.array([de[0] - t, ds[1] + t, ds[2] + t]), np.array([de[0] + t, de[1] - t, de[2] + t])],
            [np.array([ds[0] + t, ds[1] + t, ds[2] - t]), np.array([de[0] + t, de[1] - t, ds[2] + t])],
            [np.asarray(ds, dtype=np.float64) - t, np.array([de[0], ds[1], de[2]]) + t],
        ]
    return [
        [np.array([ds[0] - t, ds[1] + t, ds[2]]), np.array([ds[0] + t, de[1] - t, de[2]])],
        [np.array([ds[0] - t, ds[1] - t, ds[2]]), np.array([de[0] + t, ds[1] + t, de[2]])],
        [np.array([de[0] - t, ds[1] + t, ds[2]]), np.array([de[0] + t, de[1] - t, de[2]])],
    ]
