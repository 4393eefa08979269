"""FP64 GPU form vs the f64 CPU oracle: bit-exact cell lists, neighbour sets and physics.

The FP64 kernels evaluate every expression in the oracle's order and are compiled without
FMA contraction, so every comparison here is exact (``==`` on f64 values, NaN-aware).
"""
import numpy as np
import pytest

from helpers import cfg_of, describe_diff, small_column, small_dambreak_2d, small_dambreak_3d

pytestmark = pytest.mark.gpu

FIELDS_WC = ["x", "v", "density", "m_V", "pressure", "mass", "id0", "mat_type"]
FIELDS_SOIL = FIELDS_WC + ["stress", "strain_equ", "strain_equ_p"]


def _pair(d, oracle_lib, native, precision="fp64"):
    from tisphi_gb300.simulation import Simulation
    cfg = cfg_of(d)
    sim = Simulation(cfg, precision=precision)
    orc = oracle_lib.OracleSim(cfg)
    return sim, orc


def _gpu(sim, name):
    return sim.ps.field(name).detach().cpu().numpy()


def _compare(sim, orc, names, where):
    bad = []
    for nm in names:
        a = _gpu(sim, nm).astype(np.float64)
        b = orc.get(nm)
        same = (a == b) | (np.isnan(a) & np.isnan(b))
        if not np.all(same):
            bad.append(describe_diff(nm, a, b))
    assert not bad, f"{where}: " + "; ".join(bad)


def test_sort_and_grid_bit_exact(oracle_lib, native):
    sim, orc = _pair(small_dambreak_2d(), oracle_lib, native)
    sim.ps.initialize_particle_system()
    orc.sort()
    _compare(sim, orc, ["x", "id0", "mat_type"], "after sort")
    np.testing.assert_array_equal(sim.ps.grid_particle_num, orc.grid()[:-1])


@pytest.mark.parametrize("scene", ["2d", "3d"])
def test_neighbor_sets_bit_exact(oracle_lib, native, scene):
    d = small_dambreak_2d() if scene == "2d" else small_dambreak_3d()
    sim, orc = _pair(d, oracle_lib, native)
    sim.ps.initialize_particle_system()
    orc.sort()
    gc, gl = sim.ps.neighbors()
    oc, ol = orc.neighbors()
    np.testing.assert_array_equal(gc, oc)
    np.testing.assert_array_equal(gl, ol)
    assert gc.sum() > 0


@pytest.mark.parametrize("corr", [0, 1])
def test_kernel_corr_bit_exact(oracle_lib, native, corr):
    sim, orc = _pair(small_dambreak_3d(corr=corr), oracle_lib, native)
    sim.ps.initialize_particle_system()
    orc.sort()
    sim.solver.calc_kernel_corr()
    orc.call(oracle_lib.ORC_KERNEL_CORR)
    names = ["CSPM_f"] + (["CSPM_L"] if corr else [])
    _compare(sim, orc, names, f"kernel_corr corr={corr}")


def _one_step(sim, orc, oracle_lib):
    sim.ps.initialize_particle_system()
    orc.sort()
    sim.solver.calc_kernel_corr()
    orc.call(oracle_lib.ORC_KERNEL_CORR)
    sim.solver.init_real2tmp()
    orc.call(oracle_lib.ORC_INIT_TMP)
    sim.solver.one_step()
    orc.call(oracle_lib.ORC_ONE_STEP)


def test_wc_one_step_bit_exact(oracle_lib, native):
    sim, orc = _pair(small_dambreak_2d(), oracle_lib, native)
    # two full steps first so that velocities and pressures are non-trivial
    sim.solver.step(2)
    orc.step(2)
    _one_step(sim, orc, oracle_lib)
    _compare(sim, orc, ["d_density", "d_vel", "pressure", "v_tmp", "density_tmp"], "WC one_step")


@pytest.mark.parametrize("ti", [1, 2, 4])
def test_wc_2d_steps_bit_exact(oracle_lib, native, ti):
    sim, orc = _pair(small_dambreak_2d(integration=ti), oracle_lib, native)
    sim.solver.step(20)
    orc.step(20)
    _compare(sim, orc, FIELDS_WC, f"WC 2D ti={ti} after 20 steps")


@pytest.mark.parametrize("kernel,xsph", [(0, False), (1, True)])
def test_wc_kernel_xsph_variants(oracle_lib, native, kernel, xsph):
    sim, orc = _pair(small_dambreak_2d(kernel=kernel, xsph=xsph), oracle_lib, native)
    sim.solver.step(10)
    orc.step(10)
    _compare(sim, orc, FIELDS_WC, f"WC kernel={kernel} xsph={xsph}")


def test_wc_3d_cspm_steps_bit_exact(oracle_lib, native):
    sim, orc = _pair(small_dambreak_3d(corr=1), oracle_lib, native)
    sim.solver.step(5)
    orc.step(5)
    _compare(sim, orc, FIELDS_WC, "WC 3D CSPM after 5 steps")


@pytest.mark.parametrize("method", [2, 3])
def test_soil_steps_bit_exact(oracle_lib, native, method):
    sim, orc = _pair(small_column(method), oracle_lib, native)
    sim.solver.step(10)
    orc.step(10)
    names = FIELDS_SOIL + (["flag_retmap"] if method == 3 else [])
    _compare(sim, orc, names, f"soil method={method} after 10 steps")


@pytest.mark.parametrize("method", [2, 3])
def test_soil_lf_xsph_corr(oracle_lib, native, method):
    sim, orc = _pair(small_column(method, integration=2, xsph=True, corr=1), oracle_lib, native)
    sim.solver.step(5)
    orc.step(5)
    _compare(sim, orc, FIELDS_SOIL, f"soil method={method} LF+XSPH+CSPM")


def test_determinism_two_runs(oracle_lib, native):
    from tisphi_gb300.simulation import Simulation
    d = small_dambreak_2d()
    a = Simulation(cfg_of(d))
    b = Simulation(cfg_of(d))
    a.solver.step(15)
    b.solver.step(15)
    for nm in ["x", "v", "density", "pressure"]:
        np.testing.assert_array_equal(_gpu(a, nm), _gpu(b, nm))
