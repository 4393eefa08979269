"""Simulation: particle system + solver by ``simulationMethod`` (eng/simulation.py:7-22)."""
from .configer_builder import SimConfiger
from .particle_system import ParticleSystem
from .solver_sph_dp import DPSPHSolver
from .solver_sph_muI import MUISPHSolver
from .solver_sph_wc import WCSPHSolver


class Simulation:
    def __init__(self, config: SimConfiger, precision=None) -> None:
        self.cfg = config
        self.solver_type = self.cfg.get_cfg("simulationMethod")
        if self.solver_type not in (1, 2, 3):
            raise NotImplementedError(f"Solver type {self.solver_type} has not been implemented.")
        self.ps = ParticleSystem(self.cfg, precision=precision)
        self.solver = self.build_solver()

    def build_solver(self):
        if self.solver_type == 1:
            return WCSPHSolver(self.ps)
        if self.solver_type == 2:
            return MUISPHSolver(self.ps)
        return DPSPHSolver(self.ps)
