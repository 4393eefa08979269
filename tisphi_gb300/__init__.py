"""tisphi_gb300: GB300-native (sm_103a) implementation of tiSPHi's per-substep SPH path.

Public objects mirror the reference's API: ``SimConfiger``, ``Simulation``,
``ParticleSystem``, ``WCSPHSolver``, ``MUISPHSolver``, ``DPSPHSolver``.  Compute runs in
libtisphi_gb300.so (hand-written CUDA for sm_103a) through its C ABI.
"""
from .configer_builder import SimConfiger  # noqa: F401


def __getattr__(name):
    # GPU-backed classes import torch and the native library lazily, so that the host-side
    # scene tools stay importable on machines without a GPU.
    if name in ("Simulation",):
        from .simulation import Simulation
        return Simulation
    if name == "ParticleSystem":
        from .particle_system import ParticleSystem
        return ParticleSystem
    if name in ("WCSPHSolver", "MUISPHSolver", "DPSPHSolver", "SPHBase"):
        from . import solver_sph_base, solver_sph_dp, solver_sph_muI, solver_sph_wc
        return {"WCSPHSolver": solver_sph_wc.WCSPHSolver, "MUISPHSolver": solver_sph_muI.MUISPHSolver,
                "DPSPHSolver": solver_sph_dp.DPSPHSolver, "SPHBase": solver_sph_base.SPHBase}[name]
    raise AttributeError(name)
