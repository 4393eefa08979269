"""MUISPHSolver: mu(I) rheology SPH for granular flow (eng/solver_sph_muI.py:6-156).

The reference's kernels read ``mu`` (= tan(fric), set in the constructor,
eng/solver_sph_muI.py:20) and ``coh`` when they are first compiled.  Here ``fric``, ``mu``
and ``coh`` are properties that push the material to the device (``tsg_set_soil``):
assigning ``fric`` (radians) recomputes ``mu`` as the constructor does, assigning ``mu``
sets the friction angle atan(mu), and the next step uses the new values.
"""
import math

from . import _native as nat
from .solver_sph_base import SPHBase


class MUISPHSolver(SPHBase):
    def __init__(self, particle_system):
        super().__init__(particle_system)
        m = self.ps.mat_soil[0]
        self.density0 = m["density0"]
        self._coh = float(m["cohesion"])
        self._fric = m["friction"] / 180 * math.pi
        self.E = m["EYoungMod"]
        self.poi = m["poison"]
        self.dila = m["dilatancy"] / 180 * math.pi
        self.eta_0 = 0.0
        self.vsound = 24.0
        self.vsound2 = self.vsound ** 2

    def _push(self):
        nat.check(self._lib.tsg_set_soil(self._h, self._fric, self._coh), "tsg_set_soil")

    @property
    def fric(self):
        return self._fric

    @fric.setter
    def fric(self, value):
        self._fric = float(value)
        self._push()

    @property
    def mu(self):
        return math.tan(self._fric)

    @mu.setter
    def mu(self, value):
        self._fric = math.atan(float(value))
        self._push()

    @property
    def coh(self):
        return self._coh

    @coh.setter
    def coh(self, value):
        self._coh = float(value)
        self._push()
