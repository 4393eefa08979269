"""DPSPHSolver: Drucker-Prager elastoplastic SPH (eng/solver_sph_dp.py:6-296).

The reference's kernels read ``alpha_fric`` and ``k_c``, which the constructor derives from
the friction angle and the cohesion (eng/solver_sph_dp.py:26-27).  Here ``fric`` (radians)
and ``coh`` are properties: assigning one recomputes both constants as the constructor does
and pushes them to the device (``tsg_set_soil``); the next step uses them.  The geostatic
initial stress (init_stress, from the friction angle at construction) is not redone, as in
the reference.
"""
import math

from . import _native as nat
from .solver_sph_base import SPHBase


class DPSPHSolver(SPHBase):
    def __init__(self, particle_system):
        super().__init__(particle_system)
        m = self.ps.mat_soil[0]
        self.density0 = m["density0"]
        self._coh = float(m["cohesion"])
        self._fric = m["friction"] / 180 * math.pi
        self.E = m["EYoungMod"]
        self.poi = m["poison"]
        self.dila = m["dilatancy"] / 180 * math.pi
        self.vsound2 = self.E / self.density0
        self.vsound = math.sqrt(self.vsound2)
        self.eps_f = 1e-4
        self.G = self.E / (2 * (1 + self.poi))
        self.K = self.E / (3 * (1 - 2 * self.poi))

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
    def coh(self):
        return self._coh

    @coh.setter
    def coh(self, value):
        self._coh = float(value)
        self._push()

    @property
    def alpha_fric(self):
        t = math.tan(self._fric)
        return t / math.sqrt(9 + 12 * t ** 2)

    @property
    def k_c(self):
        t = math.tan(self._fric)
        return 3 * self._coh / math.sqrt(9 + 12 * t ** 2)
