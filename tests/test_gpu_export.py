"""Headless outputs: CSV / VTK export files and the device visual buffer.

* export_csv: the reference's 17 columns (eng/ui_sim.py:293-298), values equal to dump();
* export_vtk: a VTK XML unstructured grid whose points and point-data arrays equal dump();
* visual buffer: values, range, jet colours and scaled positions equal a numpy
  restatement of assign_value_color / v_maxmin / set_color / copy2vis (colours to 1 f32
  ulp, positions exact), in both precision forms.
"""
import re

import numpy as np
import pytest

from helpers import cfg_of, small_column, small_dambreak_2d

pytestmark = pytest.mark.gpu


def _read_vtu(path):
    blob = open(path, "rb").read()
    head, _, raw = blob.partition(b"\n_")
    text = head.decode()
    arrays = {}
    types = {"Float64": np.float64, "Float32": np.float32, "Int64": np.int64, "Int32": np.int32, "UInt8": np.uint8}
    for m in re.finditer(r'<DataArray type="(\w+)"(?: Name="([^"]+)")?(?: NumberOfComponents="(\d)")? '
                         r'format="appended" offset="(\d+)"/>', text):
        t, name, comps, off = m.group(1), m.group(2) or "Points", m.group(3), int(m.group(4))
        nbytes = int(np.frombuffer(raw[off:off + 8], dtype=np.uint64)[0])
        a = np.frombuffer(raw[off + 8:off + 8 + nbytes], dtype=types[t])
        arrays[name] = a.reshape(-1, int(comps)) if comps else a
    return arrays


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_csv_and_vtk_match_dump(native, tmp_path, precision):
    from tisphi_gb300.export import CSV_COLUMNS, export_csv, export_vtk
    from tisphi_gb300.simulation import Simulation
    sim = Simulation(cfg_of(small_column(3)), precision=precision)
    sim.solver.step(3)
    pos, data = sim.ps.dump()
    merged = {**data, **pos}
    table = np.loadtxt(export_csv("000003", str(tmp_path), sim), delimiter=",")
    for k, c in enumerate(CSV_COLUMNS):
        np.testing.assert_array_equal(table[:, k], np.asarray(merged[c], dtype=np.float64), err_msg=c)
    arrays = _read_vtu(export_vtk("000003", str(tmp_path), sim))
    np.testing.assert_array_equal(arrays["Points"][:, 0], pos["pos.x"])
    np.testing.assert_array_equal(arrays["Points"][:, 1], pos["pos.y"])
    for k in ("density", "stress.yy", "id0", "vel.norm"):
        np.testing.assert_array_equal(arrays[k], data[k], err_msg=k)


def _jet(x):
    def cm(x, h, wl, wr, c):
        w = np.where(x < c, wl, wr)
        return np.clip((w - np.abs(np.clip(x, 0, 1) - c)) / w * h, 0, 1)
    return np.stack([cm(x, 1.5, .37, .37, .75), cm(x, 1.5, .37, .37, .5), cm(x, 1.5, .37, .37, .25)], axis=1)


def _values(ps, title):
    f = lambda nm: ps.field(nm).cpu().numpy().astype(np.float64)
    if title == 2:
        return f("density")
    if title == 3:
        v = f("v")
        return np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])
    if title == 52:
        return -f("stress")[:, 1, 1]
    if title == 41:
        return f("x")[:, 0]
    raise ValueError(title)


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
@pytest.mark.parametrize("scene,title,group,show", [("wc", 2, 0, 0), ("wc", 3, 2, 1), ("dp", 52, 1, 0),
                                                    ("dp", 41, 2, 1)])
def test_visual_buffer(native, precision, scene, title, group, show):
    from tisphi_gb300.simulation import Simulation
    d = small_dambreak_2d() if scene == "wc" else small_column(3)
    sim = Simulation(cfg_of(d), precision=precision)
    sim.solver.step(4)
    ps = sim.ps
    w2s = 1.0 / max(ps.domain_size)
    pos, col, (vmax, vmin) = ps.visual(color_title=title, color_group=group, show_bdy=show)
    pos, col = pos.cpu().numpy(), col.cpu().numpy()
    ids = ps.field("id0").cpu().numpy().astype(np.int64)
    mt = ps.field("mat_type").cpu().numpy()
    x = ps.field("x").cpu().numpy().astype(np.float64)
    val = _values(ps, title)
    flow = (mt == 1) | (mt == 2)
    assert vmax == val[flow].max() and vmin == val[flow].min()
    real = mt > 0
    bdy = (mt == -1) | (mt == -2)
    shown = real | (bdy if show else np.zeros_like(real))
    np.testing.assert_array_equal(pos[ids[shown]], (x[shown] * w2s).astype(np.float32))
    assert np.all(pos[ids[~shown]] == 0)
    pick = {0: flow, 1: real, 2: real | ((mt == -1) if show else np.zeros_like(real))}[group]
    ref = _jet((val[pick] - vmin) * (1.0 / (vmax - vmin))).astype(np.float32)
    np.testing.assert_allclose(col[ids[pick]], ref, rtol=0, atol=1.2e-7)
    assert np.all(col[ids[~pick]] == 0)
