"""WCSPHSolver: weakly compressible SPH (eng/solver_sph_wc.py:6-132)."""
from .solver_sph_base import SPHBase


class WCSPHSolver(SPHBase):
    def __init__(self, particle_system):
        super().__init__(particle_system)
        m = self.ps.mat_fluid[0]
        self.density0 = m["density0"]
        self.viscosity = m["viscosity"]
        self.stiffness = m["stiffness"]
        self.exponent = m["exponent"]
        self.vsound = 60
