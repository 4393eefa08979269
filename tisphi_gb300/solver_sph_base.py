"""SPHBase with the reference's method names, dispatching to the GB300 library.

Mirrors eng/solver_sph_base.py:10-61: ``step()`` runs sort, kernel correction,
``init_real2tmp``, ``substep`` (SE / LF / RK4 by ``timeIntegration``), ``advect_pos``,
``advect_something`` and ``enforce_boundary``; each of those is also callable on its own.
``dt[None]`` is the fixed time step from ``calc_dt_CFL`` (eng/solver_sph_base.py:209-212).
"""
import ctypes

import numpy as np

from . import _native as nat
from .particle_system import ParticleSystem, _Scalar, _stream
from .params import calc_dt_cfl


class SPHBase:
    def __init__(self, particle_system: ParticleSystem):
        self.ps = particle_system
        cfg = self.ps.cfg
        self.g = np.array(cfg.get_cfg("gravitation"), dtype=np.float64)
        self.flagKernel = cfg.get_cfg("kernel")
        self.flagKernelCorr = cfg.get_cfg("kernelCorrection")
        self.flagTI = cfg.get_cfg("timeIntegration")
        self.flagXSPH = cfg.get_cfg("xsph")
        self.dt_min = cfg.get_cfg("timeStepSizeMin")
        self.dt = _Scalar(lambda: self.ps.dt_value)
        self.epsilon = 1e-8
        self.I3 = np.eye(3)
        self._lib = self.ps._lib
        self._h = self.ps._h

    def calc_dt_CFL(self, CFL_component, vsound, dt_min):
        return calc_dt_cfl(CFL_component, self.ps.smoothing_len, vsound, dt_min)

    def _call(self, fn, *args):
        return nat.check(getattr(self._lib, fn)(self._h, *args, _stream()), fn)

    # ---- time integration -------------------------------------------------------
    def step(self, nsteps=1):
        self._call("tsg_step", nsteps)

    def substep(self):
        self._call("tsg_substep")

    def one_step(self):
        self._call("tsg_one_step")

    def init_real2tmp(self):
        self._call("tsg_init_tmp")

    def calc_kernel_corr(self):
        self._call("tsg_kernel_corr")

    def advect_SE(self):
        self._call("tsg_advect", nat.TSG_ADVECT_FULL)

    def advect_LF(self):
        self._call("tsg_advect", nat.TSG_ADVECT_FULL)

    def advect_LF_half(self):
        self._call("tsg_advect", nat.TSG_ADVECT_LF_HALF)

    def init_RK(self):
        self._call("tsg_advect", nat.TSG_RK_INIT)

    def advect_RK_4(self):
        self._call("tsg_advect", nat.TSG_RK_STAGE)

    def advect_RK(self):
        self._call("tsg_advect", nat.TSG_RK_FINAL)

    def substep_SE(self):
        self.one_step()
        self.advect_SE()

    def substep_LF(self):
        self.one_step()
        self.advect_LF_half()
        self.one_step()
        self.advect_LF()

    def update_RK(self, m):
        self._call("tsg_rk_update", int(m))

    def substep_RK(self):
        """The reference's RK4 sequence (eng/solver_sph_base.py:172-180), on a handle of any
        integrator: every handle holds the RK accumulators."""
        self.init_RK()
        for q, m in enumerate((1, 2, 2, 1)):
            self.one_step()
            self.update_RK(m)
            if q < 3:
                self.advect_RK_4()
        self.advect_RK()

    def advect_pos(self):
        self._call("tsg_advect", nat.TSG_ADVECT_POS)

    def advect_something(self):
        self._call("tsg_advect", nat.TSG_ADVECT_SOMETHING)

    def enforce_boundary(self):
        self._call("tsg_advect", nat.TSG_ENFORCE_BOUNDARY)

    def solve_rigid_body(self):
        """Shape matching of the dynamic rigid bodies (eng/solver_sph_base.py:472-500); step()
        calls it after advect_something."""
        self._call("tsg_solve_rigid_body")
