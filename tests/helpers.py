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
