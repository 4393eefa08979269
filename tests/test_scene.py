"""Host-side scene construction: counts, geometry and order follow the reference generators."""
import numpy as np
import pytest

from helpers import cfg_of
from tisphi_gb300 import scenes
from tisphi_gb300.scene import build_scene, scene_geometry


def test_dambreak_2d_counts_and_grid():
    s = build_scene(cfg_of(scenes.dambreak_2d()))
    assert s.count(1) == 7200 and s.count(-1) == 1944 and s.n == 9144
    g = s.geom
    assert list(g.grid_num[:2]) == [110, 56] and g.grid_num_total == 6160
    assert g.smoothing_len == pytest.approx(0.015) and g.support_radius == pytest.approx(0.03)


def test_column_counts():
    s = build_scene(cfg_of(scenes.column_2d()))
    assert s.count(2) == 20000 and s.count(-1) == 2418
    assert s.geom.grid_num_total == 169 * 52


def test_dambreak_3d_counts():
    g = scene_geometry(cfg_of(scenes.dambreak_3d()))
    assert list(g.grid_num) == [201, 101, 33] and g.grid_num_total == 669933


def test_lattice_order_and_dummy_defaults():
    s = build_scene(cfg_of(scenes.dambreak_2d(jitter=0.0)))
    fluid = s.x[s.mat_type == 1]
    # x slowest, y fastest (meshgrid 'ij'), first point at half a spacing from the corner
    assert fluid[0, 0] == pytest.approx(0.005) and fluid[0, 1] == pytest.approx(0.005)
    assert fluid[1, 0] == pytest.approx(0.005) and fluid[1, 1] == pytest.approx(0.015)
    d = s.mat_type == -1
    assert np.all(s.density[d] == 0) and np.all(s.mass[d] == 0) and np.all(s.obj_id[d] == -1)
    assert np.all(s.x[:, 2] == 0.0)


def test_jitter_seeded_and_flow_only():
    a = build_scene(cfg_of(scenes.dambreak_2d(jitter=1e-4, seed=7)))
    b = build_scene(cfg_of(scenes.dambreak_2d(jitter=1e-4, seed=7)))
    c = build_scene(cfg_of(scenes.dambreak_2d(jitter=0.0)))
    np.testing.assert_array_equal(a.x, b.x)
    f = a.mat_type == 1
    dev = np.abs(a.x[f] - c.x[f])
    assert dev[:, :2].max() <= 1e-4 and dev[:, :2].max() > 5e-5 and np.all(dev[:, 2] == 0)
    np.testing.assert_array_equal(a.x[~f], c.x[~f])


def test_block_outside_domain_rejected():
    d = scenes.dambreak_2d()
    d["Blocks"][0]["size"] = [4.0, 0.6, 0.1]
    with pytest.raises(ValueError):
        build_scene(cfg_of(d))
