"""Solver attributes that the reference's kernels read, assigned after construction.

The reference's Taichi kernels read the solver's material attributes when they are first
compiled (eng/solver_sph_wc.py:12-15, eng/solver_sph_muI.py:13-20,
eng/solver_sph_dp.py:13-27), so a script may change them between construction and the
first step.  Here the attributes push the new values to the device: a scene built with one
value and switched to another must step exactly like a scene built with the other value
(FP64 form: bit-identical; FP32-mixed form: bit-identical as well, both run the same
kernels on the same constants).  substep_RK runs the reference's RK4 sequence on a handle
of any integrator, bit-identical to a handle created for RK4.
"""
import math

import numpy as np
import pytest

from helpers import cfg_of, small_column, small_dambreak_2d

pytestmark = pytest.mark.gpu

FIELDS = ["x", "v", "density", "pressure"]


def _sim(d, precision):
    from tisphi_gb300.simulation import Simulation
    return Simulation(cfg_of(d), precision=precision)


def _same(a, b, names):
    for nm in names:
        x = a.ps.field(nm).cpu().numpy()
        y = b.ps.field(nm).cpu().numpy()
        assert np.array_equal(x, y), f"{nm} differs"


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_wcsph_stiffness_viscosity_assignment(native, precision):
    want = _sim(small_dambreak_2d(stiffness=2.0e4, viscosity=0.01), precision)
    got = _sim(small_dambreak_2d(stiffness=5.0e4, viscosity=0.005), precision)
    got.solver.stiffness = 2.0e4
    got.solver.viscosity = 0.01
    assert got.solver.stiffness == 2.0e4 and got.solver.viscosity == 0.01
    want.solver.step(5)
    got.solver.step(5)
    _same(want, got, FIELDS)
    # a change between steps takes effect at the next step
    other = _sim(small_dambreak_2d(stiffness=2.0e4, viscosity=0.01), precision)
    other.solver.step(5)
    other.solver.stiffness = 3.0e4
    got.solver.stiffness = 3.0e4
    other.solver.step(3)
    got.solver.step(3)
    _same(other, got, FIELDS)


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_mui_friction_cohesion_assignment(native, precision):
    def column(fric, coh):
        d = small_column(2)
        d["Materials"][0]["friction"] = fric
        d["Materials"][0]["cohesion"] = coh
        return d
    want = _sim(column(30.0, 50.0), precision)
    got = _sim(column(21.9, 0.0), precision)
    got.solver.fric = 30.0 / 180 * math.pi
    got.solver.coh = 50.0
    assert abs(got.solver.mu - math.tan(30.0 / 180 * math.pi)) < 1e-15
    want.solver.step(5)
    got.solver.step(5)
    _same(want, got, FIELDS + ["stress"])
    # assigning mu sets the friction angle atan(mu)
    got.solver.mu = math.tan(25.0 / 180 * math.pi)
    assert abs(got.solver.fric - 25.0 / 180 * math.pi) < 1e-15


def test_dp_cohesion_assignment(native):
    # cohesion does not enter the geostatic initial stress, so the two scenes start alike
    def column(coh):
        d = small_column(3)
        d["Materials"][0]["cohesion"] = coh
        return d
    want = _sim(column(200.0), "fp64")
    got = _sim(column(0.0), "fp64")
    got.solver.coh = 200.0
    t = math.tan(got.solver.fric)
    assert abs(got.solver.k_c - 600.0 / math.sqrt(9 + 12 * t * t)) < 1e-12
    want.solver.step(5)
    got.solver.step(5)
    _same(want, got, FIELDS + ["stress", "flag_retmap"])


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_substep_rk_on_any_handle(native, precision):
    rk = _sim(small_dambreak_2d(integration=4), precision)
    lf = _sim(small_dambreak_2d(integration=2), precision)
    for s in (rk, lf):
        s.ps.initialize_particle_system()
        s.solver.calc_kernel_corr()
        s.solver.init_real2tmp()
    rk.solver.substep()
    lf.solver.substep_RK()
    _same(rk, lf, ["v", "density"])
