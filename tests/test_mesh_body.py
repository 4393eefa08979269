"""Mesh bodies (eng/particle_func.py:265-294, load_body): OBJ geometry, the rotation, the
voxelisation by subdivision and filling, and their place in the scene (after the blocks,
before the boundary particles, eng/particle_system.py:135-148).

No golden vectors exist (the reference ships no tests, and trimesh, which it calls, is not
installed), so the voxelisation is checked on shapes with a known answer: an axis-aligned
box voxelises to every grid point of [0, size] (the surface vertices round onto the grid
planes and the fill closes the inside), a rotated box to its volume within the surface
layer's share, and the rotation against its closed form.
"""
import math

import numpy as np
import pytest

from helpers import cfg_of, mesh_box_scene_3d, write_box_obj
from tisphi_gb300 import mesh_body


def test_obj_quads_become_triangle_fans(tmp_path):
    path = write_box_obj(tmp_path / "box.obj", (1.0, 2.0, 3.0))
    v, f = mesh_body.load_obj(path)
    assert v.shape == (8, 3) and f.shape == (12, 3)
    assert np.array_equal(v.max(axis=0), [1.0, 2.0, 3.0]) and np.array_equal(v.min(axis=0), [0.0, 0.0, 0.0])
    # every edge of the closed surface is shared by exactly two triangles
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert np.all(counts == 2)


def test_negative_obj_indices(tmp_path):
    p = tmp_path / "tri.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf -3 -2 -1\n")
    v, f = mesh_body.load_obj(str(p))
    assert f.tolist() == [[0, 1, 2]]


def test_box_voxelises_to_every_grid_point(tmp_path):
    v, f = mesh_body.load_obj(write_box_obj(tmp_path / "box.obj"))
    size = np.array([0.1, 0.06, 0.08])
    pitch = 0.01
    pts = mesh_body.voxel_points(v * size, f, pitch)
    n = np.rint(size / pitch).astype(int) + 1
    assert pts.shape == (int(np.prod(n)), 3)
    grid = np.stack(np.meshgrid(*[np.arange(k) * pitch for k in n], indexing="ij"), -1).reshape(-1, 3)
    np.testing.assert_allclose(pts, grid, rtol=0, atol=1e-15)  # C order of the grid


def test_rotation_matrix_closed_form():
    m = mesh_body.rotation_matrix(math.pi / 2, [0.0, 0.0, 2.0], point=[1.0, 0.0, 0.0])
    out = mesh_body.transform_points(np.array([[2.0, 0.0, 0.0], [1.0, 0.0, 5.0]]), m)
    np.testing.assert_allclose(out, [[1.0, 1.0, 0.0], [1.0, 0.0, 5.0]], atol=1e-15)
    a, d = 0.7, np.array([1.0, 2.0, 2.0]) / 3.0
    r = mesh_body.rotation_matrix(a, d)[:3, :3]
    np.testing.assert_allclose(r @ r.T, np.eye(3), atol=1e-15)
    np.testing.assert_allclose(r @ d, d, atol=1e-15)
    assert abs(np.trace(r) - (1 + 2 * math.cos(a))) < 1e-14


def test_rotated_box_keeps_its_volume(tmp_path):
    v, f = mesh_body.load_obj(write_box_obj(tmp_path / "box.obj"))
    v = v * 0.2
    m = mesh_body.rotation_matrix(math.radians(30.0), [0.0, 0.0, 1.0], v.mean(axis=-1))
    pitch = 0.01
    pts = mesh_body.voxel_points(mesh_body.transform_points(v, m), f, pitch)
    # the voxel centres fill the box grown by about half a pitch on every side (as the
    # axis-aligned box's 21^3 centres on [0, 0.2] do)
    vol = (0.2 + pitch) ** 3
    assert abs(len(pts) * pitch ** 3 - vol) < 0.05 * vol
    assert len(np.unique(np.round(pts / pitch), axis=0)) == len(pts)


def test_subdivision_refuses_unbounded_meshes():
    v = np.array([[0.0, 0.0, 0.0], [1e6, 0.0, 0.0], [0.0, 1e6, 0.0]])
    with pytest.raises(ValueError):
        mesh_body.subdivide_to_size(v, np.array([[0, 1, 2]]), 1e-3, max_iter=3)


def test_scene_places_bodies_after_blocks(tmp_path):
    from tisphi_gb300.scene import build_scene
    obj = write_box_obj(tmp_path / "unit_box.obj")
    d = mesh_box_scene_3d(obj)
    s = build_scene(cfg_of(d))
    body = np.nonzero(s.obj_id == 1)[0]
    fluid = np.nonzero(s.mat_type == 1)[0]
    dummy = np.nonzero(s.mat_type == -1)[0]
    assert len(body) == 6 * 4 * 5  # 0.1 x 0.06 x 0.08 m at a 0.02 m pitch, both ends included
    assert fluid.max() < body.min() and body.max() < dummy.min()
    assert np.all(s.mat_type[body] == 11) and np.all(s.is_dynamic[body] == 1)
    np.testing.assert_allclose(s.x[body].min(axis=0), [0.1, 0.2, 0.04], atol=1e-15)
    np.testing.assert_allclose(s.x[body].max(axis=0), [0.2, 0.26, 0.12], atol=1e-12)
    assert np.all(s.density[body] == 500.0)


def test_two_dimensional_scene_rejects_bodies(tmp_path):
    from tisphi_gb300 import scenes
    from tisphi_gb300.scene import build_scene
    d = scenes.floating_box_2d()
    d["Bodies"] = [{"objectId": 2, "geometryFile": write_box_obj(tmp_path / "b.obj"), "translation": [0, 0, 0],
                    "scale": 0.1, "rotationAngle": 0.0, "rotationAxis": [0, 0, 1], "velocity": [0, 0, 0],
                    "materialId": 1, "isDynamic": True}]
    with pytest.raises(NotImplementedError):
        build_scene(cfg_of(d))


def _stl_ascii(path, v, f):
    with open(path, "w") as out:
        out.write("solid box\n")
        for t in f:
            out.write("  facet normal 0 0 0\n    outer loop\n")
            for k in t:
                out.write("      vertex %.17g %.17g %.17g\n" % tuple(v[k]))
            out.write("    endloop\n  endfacet\n")
        out.write("endsolid box\n")


def _stl_binary(path, v, f):
    rec = np.zeros(len(f), dtype=[("normal", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")])
    rec["v"] = v[f]
    with open(path, "wb") as out:
        out.write(b"binary box".ljust(80, b" "))
        out.write(np.uint32(len(f)).tobytes())
        out.write(rec.tobytes())


def test_stl_ascii_and_binary_voxelise_like_obj(tmp_path):
    v, f = mesh_body.load_obj(write_box_obj(tmp_path / "box.obj", (0.1, 0.06, 0.08)))
    want = mesh_body.voxel_points(v, f, 0.02)
    _stl_ascii(tmp_path / "a.stl", v, f)
    _stl_binary(tmp_path / "b.stl", v, f)
    for name in ("a.stl", "b.stl"):
        vs, fs = mesh_body.load_mesh(str(tmp_path / name))
        assert fs.shape == (12, 3)
        got = mesh_body.voxel_points(vs, fs, 0.02)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-9)  # binary STL holds f32 coordinates
