"""DPSPHSolver: Drucker-Prager elastoplastic SPH (eng/solver_sph_dp.py:6-296)."""
import math

from .solver_sph_base import SPHBase


class DPSPHSolver(SPHBase):
    def __init__(self, particle_system):
        super().__init__(particle_system)
        m = self.ps.mat_soil[0]
        self.density0 = m["density0"]
        self.coh = m["cohesion"]
        self.fric = m["friction"] / 180 * math.pi
        self.E = m["EYoungMod"]
        self.poi = m["poison"]
        self.dila = m["dilatancy"] / 180 * math.pi
        self.vsound2 = self.E / self.density0
        self.vsound = math.sqrt(self.vsound2)
        self.eps_f = 1e-4
        t = math.tan(self.fric)
        self.alpha_fric = t / math.sqrt(9 + 12 * t ** 2)
        self.k_c = 3 * self.coh / math.sqrt(9 + 12 * t ** 2)
        self.G = self.E / (2 * (1 + self.poi))
        self.K = self.E / (3 * (1 - 2 * self.poi))
