"""Boundary modes and kernel functions beyond the default scene (dummy particles, Wendland
C2): collision (boundary 1), repulsive particles (3), dummy + repulsive particles (4), each
with the Wendland C2 and the cubic spline kernel, on the 2D WCSPH dambreak, against the
f64 oracle after 10 steps.

* FP64 form: every field bit-identical (eng/solver_sph_base.py:525-601 collision,
  :675-689 repulsive force, :721-... kernel functions in the oracle's order).
* FP32-mixed form: density within 1e-5 relative and positions within 1e-6 m, the bounds of
  the default scene; these scenes run the list kernels' compile-time variants for the cubic
  spline and for repulsive particles, and (collision) a scene without a static block.
"""
import numpy as np
import pytest

from helpers import cfg_of, describe_diff, small_dambreak_2d

pytestmark = pytest.mark.gpu

MODES = [(1, 1), (1, 0), (3, 1), (3, 0), (4, 1), (4, 0)]


def _scene(boundary, kernel):
    d = small_dambreak_2d(kernel=kernel)
    d["Configuration"]["boundary"] = boundary
    return d


def _pair(d, oracle_lib, precision):
    from tisphi_gb300.simulation import Simulation
    cfg = cfg_of(d)
    return Simulation(cfg, precision=precision), oracle_lib.OracleSim(cfg)


@pytest.mark.parametrize("boundary,kernel", MODES)
def test_fp64_bit_exact(oracle_lib, native, boundary, kernel):
    sim, orc = _pair(_scene(boundary, kernel), oracle_lib, "fp64")
    sim.solver.step(10)
    orc.step(10)
    bad = []
    for nm in ("x", "v", "density", "pressure", "m_V", "id0", "mat_type"):
        a = sim.ps.field(nm).detach().cpu().numpy().astype(np.float64)
        b = orc.get(nm)
        if not np.all((a == b) | (np.isnan(a) & np.isnan(b))):
            bad.append(describe_diff(nm, a, b))
    assert not bad, f"boundary={boundary} kernel={kernel}: " + "; ".join(bad)


@pytest.mark.parametrize("boundary,kernel", MODES)
def test_fp32_close(oracle_lib, native, boundary, kernel):
    sim, orc = _pair(_scene(boundary, kernel), oracle_lib, "fp32_mixed")
    sim.solver.step(10)
    orc.step(10)
    gid = sim.ps.field("id0").cpu().numpy()
    oid = orc.get("id0").astype(np.int64)
    inv = np.empty_like(gid)
    inv[gid] = np.arange(gid.size)
    take = inv[oid]
    f = orc.get("mat_type") == 1
    rho = sim.ps.field("density").cpu().numpy().astype(np.float64)[take][f]
    rho_o = orc.get("density")[f]
    x = sim.ps.field("x").cpu().numpy().astype(np.float64)[take][f]
    e_rho = float(np.max(np.abs(rho - rho_o) / rho_o))
    e_x = float(np.max(np.abs(x - orc.get("x")[f])))
    assert e_rho < 1e-5 and e_x < 1e-6, f"boundary={boundary} kernel={kernel}: density {e_rho:.3e}, x {e_x:.3e}"
    sim.ps.check_errors()
