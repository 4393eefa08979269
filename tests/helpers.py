"""Shared test helpers: scenes at test sizes and oracle-vs-GPU field comparison."""
import numpy as np

from tisphi_gb300 import scenes
from tisphi_gb300.configer_builder import SimConfiger

SCALAR = ["density", "m_V", "pressure", "mass"]
VECTOR = ["x", "v"]


def cfg_of(d):
    return SimConfiger(config=d)


def small_dambreak_2d(**kw):
    base = dict(spacing=0.02, width=0.6, height=0.4, domain=(1.2, 0.8))
    base.update(kw)
    return scenes.dambreak_2d(**base)


def small_dambreak_3d(**kw):
    base = dict(spacing=0.02, domain=(0.6, 0.4, 0.2), size=(0.3, 0.2, 0.1), jitter_frac=0.01)
    base.update(kw)
    return scenes.dambreak_3d(**base)


def small_column(method, **kw):
    base = dict(spacing=0.004, width=0.2, height=0.1, domain=(0.5, 0.15))
    base.update(kw)
    return scenes.column_2d(method=method, **base)


def describe_diff(name, a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        return f"{name}: shape {a.shape} vs {b.shape}"
    d = np.abs(a - b)
    bad = np.count_nonzero(~((a == b) | (np.isnan(a) & np.isnan(b))))
    scale = np.maximum(np.abs(b), 1e-300)
    return (f"{name}: {bad} / {a.size} differ, max abs {np.nanmax(d) if d.size else 0:.3e}, "
            f"max rel {np.nanmax(d / scale) if d.size else 0:.3e}")


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.maximum(np.abs(b), floor)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(scale > 0, np.abs(a - b) / scale, np.abs(a - b))
    return float(np.nanmax(r)) if r.size else 0.0


def write_box_obj(path, size=(1.0, 1.0, 1.0)):
    """A closed box [0, size] as a Wavefront OBJ file: eight corners, six quads."""
    sx, sy, sz = size
    corners = [(x, y, z) for x in (0.0, sx) for y in (0.0, sy) for z in (0.0, sz)]
    # corner index = 4 * ix + 2 * iy + iz (1-based in the file), quads wound outwards
    quads = [(1, 2, 4, 3), (5, 7, 8, 6), (1, 5, 6, 2), (3, 4, 8, 7), (1, 3, 7, 5), (2, 6, 8, 4)]
    with open(path, "w") as f:
        for c in corners:
            f.write("v %r %r %r\n" % c)
        for q in quads:
            f.write("f " + " ".join(f"{k}/{k}/{k}" for k in q) + "\n")
    return str(path)


def mesh_box_scene_3d(obj_path, box_density=500.0, steps_dt=2e-5):
    """floating_box_3d with the rigid box given as a mesh body (a unit-box OBJ scaled to
    0.1 x 0.06 x 0.08 m) instead of a block."""
    d = scenes.floating_box_3d(dt=steps_dt, box_density=box_density)
    d["Blocks"] = [b for b in d["Blocks"] if b["objectId"] != 1]
    d["Bodies"] = [{"objectId": 1, "geometryFile": obj_path, "translation": [0.1, 0.2, 0.04],
                    "scale": [0.1, 0.06, 0.08], "rotationAngle": 0.0, "rotationAxis": [0.0, 0.0, 1.0],
                    "velocity": [0.0, 0.0, 0.0], "materialId": 1, "isDynamic": True}]
    return d
