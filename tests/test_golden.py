"""Pin the f64 oracle (and, on a GPU, the FP64 CUDA form) to the reference's own code.

tests/golden/*.npz were produced by tests/golden/make_golden.py, which runs the
reference's unmodified Python/Taichi source (Simulation -> solver.step()) under a serial
Taichi-API emulator.  The oracle restates the same arithmetic; the only intended
differences are constant powers written as products (q1**4 as (q1*q1)*(q1*q1) instead of
libm pow), so fields agree to a few ulp (tested at 1e-12 normwise) after a few steps, and
to 1e-11 after the 40-step fixtures (the Drucker-Prager equivalent plastic strain, a sum
over the few particles that yield, moves by 1e-12 of its largest value there).  The
particle order after the last sort and the cell offsets must agree exactly.
"""
import glob
import json
import os

import numpy as np
import pytest

from tisphi_gb300.configer_builder import SimConfiger

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
RTOL = 1e-12

FLOAT_FIELDS = ["x", "v", "density", "pressure", "m_V", "CSPM_f", "d_density", "d_vel", "v_tmp", "density_tmp"]
SOIL_FIELDS = ["stress", "strain_equ", "strain_equ_p"]


def _close(name, a, b, scale, rtol=RTOL):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    err = np.max(np.abs(a - b)) if a.size else 0.0
    assert err <= rtol * scale, f"{name}: max abs diff {err:.3e} vs scale {scale:.3e}"


def _scale(b):
    m = np.max(np.abs(b)) if b.size else 0.0
    return m if m > 0 else 1.0


def _check(get, g, soil, dp):
    np.testing.assert_array_equal(get("id0").astype(np.int64), g["id0"])
    np.testing.assert_array_equal(get("mat_type").astype(np.int64), g["mat_type"])
    rtol = RTOL if int(g["steps"]) < 40 else 10 * RTOL
    for name in FLOAT_FIELDS + (SOIL_FIELDS if soil else []):
        b = g[name]
        a = get(name).reshape(b.shape)
        mask = np.ones(b.shape[0], dtype=bool)
        if name in ("d_density", "d_vel", "v_tmp", "density_tmp"):
            mask = g["mat_type"] > 0  # transient fields of boundary particles are stale copies
        _close(name, a[mask], b[mask], _scale(b[mask]), rtol)
    if dp:
        np.testing.assert_array_equal(get("flag_retmap").astype(np.int64), g["flag_retmap"])


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_scene_builder_matches_reference_generator(path):
    """Initial particles (lattice + boundary boxes, then the seeded jitter) match exactly."""
    from tisphi_gb300.scene import build_scene
    g = np.load(path)
    s = build_scene(SimConfiger(config=json.loads(str(g["scene_json"]))))
    np.testing.assert_array_equal(s.x, g["x_init"])


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_oracle_matches_reference_source(oracle_lib, path):
    g = np.load(path)
    scene = json.loads(str(g["scene_json"]))
    orc = oracle_lib.OracleSim(SimConfiger(config=scene))
    assert orc.params.dt == float(g["dt"])
    orc.step(int(g["steps"]))
    np.testing.assert_array_equal(orc.grid()[:-1], g["grid_end"])
    method = scene["Configuration"]["simulationMethod"]
    _check(orc.get, g, method != 1, method == 3)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_fp64_gpu_matches_reference_source(native, path):
    from tisphi_gb300.simulation import Simulation
    g = np.load(path)
    scene = json.loads(str(g["scene_json"]))
    sim = Simulation(SimConfiger(config=scene))
    sim.solver.step(int(g["steps"]))
    np.testing.assert_array_equal(sim.ps.grid_particle_num, g["grid_end"])
    method = scene["Configuration"]["simulationMethod"]

    def get(name):
        return sim.ps.field(name).cpu().numpy()

    _check(get, g, method != 1, method == 3)
