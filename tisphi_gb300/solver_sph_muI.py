"""MUISPHSolver: mu(I) rheology SPH for granular flow (eng/solver_sph_muI.py:6-156)."""
import math

from .solver_sph_base import SPHBase


class MUISPHSolver(SPHBase):
    def __init__(self, particle_system):
        super().__init__(particle_system)
        m = self.ps.mat_soil[0]
        self.density0 = m["density0"]
        self.coh = m["cohesion"]
        self.fric = m["friction"] / 180 * math.pi
        self.E = m["EYoungMod"]
        self.poi = m["poison"]
        self.dila = m["dilatancy"] / 180 * math.pi
        self.eta_0 = 0.0
        self.mu = math.tan(self.fric)
        self.vsound = 24.0
        self.vsound2 = self.vsound ** 2
